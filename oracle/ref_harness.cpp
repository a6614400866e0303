// Harness that drives the AdaM-DG reference library (compiled from its own
// sources, unmodified, against the Eigen stand-in in oracle/shim) and dumps
// its results keyed by element multi-index.  Test infrastructure only: its
// output pins the C restatement in oracle/amdg_oracle.c and becomes the
// committed golden fixtures under tests/golden/.
//
// Usage:
//   ref_harness linear <dim> <N> <k> <sparse 0|1> <ic> <engine> <steps> <dt> <c_0> ... <c_{dim-1}>
//     ic     : sin_sum  -> u0 = sin(2 pi sum x_d)  (init_separable_scalar_sum, as in
//                          example/02_hyperbolic_01_scalar_const_coefficient.cpp); the final
//                          L1/L2/Linf errors against the translated solution ("NORMERR")
//              sin_prod -> u0 = prod_d sin(2 pi x_d) (init_separable_scalar)
//     engine : assembled -> HyperbolicAlpt::assemble_matrix_scalar + RK3SSP::step_rk
//              matfree   -> FastRHS::transform_ucoe_alpt_to_rhs per dim with
//                           c_d*(u_vx + ulft_vjp | urgt_vjp) on the "flx" sets,
//                           RK3SSP::step_stage (the 4D/6D CPU baseline path)
//   ref_harness burgers <dim> <N> <alpha> <steps> <dt>
//     u_t + sum_d (u^2/2)_{x_d} = 0, u0 = 0.5 + 0.25 sin(2 pi sum x_d), Alpert k=2,
//     Lagrange degree 3 (msh_case 1) interpolation of the flux
//     (LagrInterpolation::nonlinear_Lagr_fast), HyperbolicLagrRHS volume and
//     interface terms, HyperbolicAlptRHS::rhs_flx_penalty_scalar(alpha), RK3SSP
//     step_stage, sparse grid without adaptivity (07_vlasov_maxwell_adapt.cpp
//     stage loop).  Dumps u0, up0 (point values), fu0_d (interpolation
//     coefficients of the flux in dimension d), rhs0 and uT; then DGSolution::val
//     and the exact solution at 48 fixed points ("vals") and the L1/L2/Linf errors
//     of get_error_no_separable_scalar with 1 and 2 Gauss points ("NORMERR").
//   ref_harness burgers_herm <N> <alpha> <steps> <dt>
//     the 2D version with the flux interpolated by cubic Hermite interpolation
//     (HermInterpolation::nonlinear_Herm_2D_fast, HyperbolicSameFluxHermRHS), see run_burgers_herm.
//   ref_harness burgers_herm_adapt <N_init> <NMAX> <eps> <eta> <alpha> <cfl> <steps> [time [t_end]]
//     the 2D adaptive Burgers loop of example/02_hyperbolic_05_burgers_adapt.cpp as that driver
//     runs it (Hermite flux interpolation, assembled LxF matrix), see run_burgers_herm_adapt.
//   ref_harness burgers_adapt <dim> <N_init> <NMAX> <eps> <eta> <alpha> <cfl> <umax> <steps>
//     adaptive version of the above, following the time loop of
//     example/02_hyperbolic_05_burgers_adapt.cpp:223-476 with the Lagrange
//     right-hand side: adaptive separable initialisation, then per step
//     dt = cfl / sum_d umax 2^maxlevel_d, copy_ucoe_to_predict, ForwardEuler
//     predictor, refine, copy_predict_to_ucoe, three RK3SSP stages, coarsen.
//     Dumps the element set and coefficients after init (u_init) and after
//     every step (u_step<i>), with the step sizes and the largest level sum of
//     any element (Hash::hash_key overflows int32 in 3D once it reaches 23,
//     Hash.cpp:55-114; such a step is flagged "HASH_OVERFLOW").
//   ref_harness burgers_adapt ... <steps> time [t_end]
//     the same loop without dumps: wall time of every time step (the evolution
//     loop only, initialisation excluded) with the DOF the step's RK stages
//     advanced (get_dof after refine), "TSTEP <i> <seconds> <dof> <elements>";
//     with t_end the last step is shortened to land on it, as
//     02_hyperbolic_05_burgers_adapt.cpp does (dt = min(dt, final_time - t)).
//   ref_harness wave <dim> <N> <sigma> <steps> <dt> [a]
//     u_tt = div(K grad u), K = (1 + a prod_d sin(2 pi x_d))^2 (a = 0.5 by default), u0 = Gaussian
//     bump, u_t(0) = 0:
//     DiffusionRHS with Lagrange-interpolated (degree 4, msh_case 2) K grad u and K u, IPDG
//     penalty, RK4ODE2nd (03_wave_06_var_coeff_adapt.cpp:154-279). Dumps u0, rhs0, uT, vT.
//   ref_harness wave_adapt <dim> <N_init> <NMAX> <eps> <eta> <sigma> <cfl> <steps> [a]
//     the adaptive loop of 03_wave_06_var_coeff_adapt.cpp:181-297 for the same problem (no
//     source); dumps u and u_t after the adaptive initialisation and after every step.
//   ref_harness matrices <N> <k>
//     dumps the 1D operator matrices u_v, u_vx, ulft_vjp, urgt_vjp.
//   ref_harness intp_init <dim> <N_init> <NMAX> <eps> <degree> <width>
//     DGAdaptIntp::init_adaptive_intp (k = 2, Lagrange degree 3 with msh_case 1 or 4 with
//     msh_case 2) of exp(-width |x - (0.3, 0.4, 0.5)|^2); dumps the element set and the Alpert
//     coefficients (u_init).
//   ref_harness intp_error <dim> <N_init> <NMAX> <eps_a> <eps_b> <degree> <width>
//     two such initialisations (refine eps_a and eps_b) and
//     DGAdaptIntp::get_L2_error_split_adaptive_intp_scalar of the first against the second
//     (dumps u_a, u_b and the 1 x 1 block err).
//
// Output (text, %.17g): blocks "BEGIN <name> <rows> <cols>" ... "END".
// Element blocks have one row per element: level[dim] suppt[dim] coeff[(k+1)^dim]
// where coeff is VecMultiD row-major order (last dimension fastest).
#include "AllBasis.h"
#include "AlptBasis.h"
#include "BilinearForm.h"
#include "DGAdapt.h"
#include "DGAdaptIntp.h"
#include "DGSolution.h"
#include "Element.h"
#include "ExactSolution.h"
#include "FastMultiplyLU.h"
#include "Hash.h"
#include "HermBasis.h"
#include "Interpolation.h"
#include "LagrBasis.h"
#include "ODESolver.h"
#include "OperatorMatrix1D.h"
#include "Timer.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

namespace {

void set_statics(int dim, int k, int lagr_degree = 3) {
    AlptBasis::PMAX = k;
    LagrBasis::PMAX = lagr_degree;
    LagrBasis::msh_case = lagr_degree == 4 ? 2 : 1;
    HermBasis::PMAX = 3;
    HermBasis::msh_case = 1;
    Element::PMAX_alpt = AlptBasis::PMAX;
    Element::PMAX_intp = LagrBasis::PMAX;
    Element::DIM = dim;
    Element::VEC_NUM = 1;
    DGSolution::DIM = dim;
    DGSolution::VEC_NUM = 1;
    Interpolation::DIM = dim;
    Interpolation::VEC_NUM = 1;
    DGSolution::ind_var_vec = {0};
    DGAdapt::indicator_var_adapt = {0};
    Element::is_intp.assign(1, std::vector<bool>(dim, true));
}

void dump_elements(const char* name, DGSolution& dg, int which) {
    const int dim = DGSolution::DIM;
    const int nb = (int)dg.dg.begin()->second.size_alpt();
    std::printf("BEGIN %s %zu %d\n", name, dg.dg.size(), 2 * dim + nb);
    for (auto& it : dg.dg) {
        const Element& e = it.second;
        for (int d = 0; d < dim; ++d) std::printf("%d ", e.level[d]);
        for (int d = 0; d < dim; ++d) std::printf("%d ", e.suppt[d]);
        const VecMultiD<double>& v = (which == 0) ? e.ucoe_alpt[0] : (which == 1 ? e.rhs[0] : e.ucoe_ut[0]);
        for (int i = 0; i < nb; ++i) std::printf("%.17g ", v.at(i));
        std::printf("\n");
    }
    std::printf("END\n");
}

void dump_elements_vec(const char* name, DGSolution& dg, const std::function<const VecMultiD<double>&(const Element&)>& get) {
    const int dim = DGSolution::DIM;
    const int nb = (int)get(dg.dg.begin()->second).get_index_iterator().size();
    std::printf("BEGIN %s %zu %d\n", name, dg.dg.size(), 2 * dim + nb);
    for (auto& it : dg.dg) {
        const Element& e = it.second;
        for (int d = 0; d < dim; ++d) std::printf("%d ", e.level[d]);
        for (int d = 0; d < dim; ++d) std::printf("%d ", e.suppt[d]);
        const VecMultiD<double>& v = get(e);
        for (int i = 0; i < nb; ++i) std::printf("%.17g ", v.at(i));
        std::printf("\n");
    }
    std::printf("END\n");
}

void dump_matrix(const char* name, const VecMultiD<double>& m, int rows, int cols) {
    std::printf("BEGIN %s %d %d\n", name, rows, cols);
    for (int r = 0; r < rows; ++r) {
        for (int c = 0; c < cols; ++c) std::printf("%.17g ", m.at(r, c));
        std::printf("\n");
    }
    std::printf("END\n");
}

// The reference's FastRHS transforms are protected; this subclass exposes the
// single-dimension Alpert->Alpert transform that a linear constant-coefficient
// operator needs (FastMultiplyLU.cpp:46-59).
class LinearMatFree : public FastRHS {
public:
    explicit LinearMatFree(DGSolution& dg) : FastRHS(dg), dg_(dg) {}
    void apply_dim(const VecMultiD<double>* mat, int d, double c) {
        transform_ucoe_alpt_to_rhs(mat, std::string("flx"), d, c, 0);
    }
    void zero_rhs() { dg_.set_rhs_zero(); }
private:
    DGSolution& dg_;
};

int run_linear(int argc, char** argv) {
    if (argc < 10) { std::fprintf(stderr, "linear: bad args\n"); return 2; }
    const int dim = std::atoi(argv[2]);
    const int N = std::atoi(argv[3]);
    const int k = std::atoi(argv[4]);
    const bool sparse = std::atoi(argv[5]) != 0;
    const std::string ic = argv[6];
    const std::string engine = argv[7];
    const int steps = std::atoi(argv[8]);
    const double dt = std::atof(argv[9]);
    if (argc < 10 + dim) { std::fprintf(stderr, "linear: need %d coefficients\n", dim); return 2; }
    std::vector<double> c(dim);
    for (int d = 0; d < dim; ++d) c[d] = std::atof(argv[10 + d]);

    set_statics(dim, k);
    Hash hash;
    LagrBasis::set_interp_msh01();
    HermBasis::set_interp_msh01();
    AllBasis<AlptBasis> all_bas_alpt(N);
    AllBasis<LagrBasis> all_bas_lagr(N);
    AllBasis<HermBasis> all_bas_herm(N);
    OperatorMatrix1D<AlptBasis, AlptBasis> oper(all_bas_alpt, all_bas_alpt, "period");

    const double refine_eps = 1e10, coarsen_eta = -1;
    DGAdapt dg(sparse, N, N, all_bas_alpt, all_bas_lagr, all_bas_herm, hash, refine_eps, coarsen_eta, true, false);

    const double PI = Const::PI;
    if (ic == "sin_sum") {
        // sin(2 pi sum x) expanded into 2^(dim-1) separable products of sin/cos
        std::vector<std::function<double(double, int)>> funcs;
        const int nterm = 1 << dim;
        for (int mask = 0; mask < nterm; ++mask) {
            // a product with an odd number of sin factors contributes with sign
            int nsin = __builtin_popcount(mask);
            if (nsin % 2 == 0) continue;
            const double sign = ((nsin - 1) / 2) % 2 == 0 ? 1.0 : -1.0;
            funcs.push_back([=](double x, int d) {
                double v = ((mask >> d) & 1) ? std::sin(2 * PI * x) : std::cos(2 * PI * x);
                return d == 0 ? sign * v : v;
            });
        }
        dg.init_separable_scalar_sum(funcs);
    } else if (ic == "sin_prod") {
        dg.init_separable_scalar([=](double x, int) { return std::sin(2 * PI * x); });
    } else {
        std::fprintf(stderr, "unknown ic\n");
        return 2;
    }
    std::printf("META dim=%d N=%d k=%d sparse=%d elements=%zu dof=%d\n", dim, N, k, (int)sparse, dg.dg.size(), dg.get_dof());
    dump_elements("u0", dg, 0);

    double t_evolve = 0;
    if (engine == "assembled") {
        HyperbolicAlpt op(dg, oper);
        op.assemble_matrix_scalar(c);
        RK3SSP ode(op, dt);
        ode.init();
        // one operator application on u0, written back into Element::rhs
        op.multi(ode.ucoe, ode.rhs);
        ode.eigenvec_to_rhs();
        dump_elements("rhs0", dg, 1);
        ode.rhs.setZero();
        auto t0 = std::chrono::steady_clock::now();
        for (int s = 0; s < steps; ++s) ode.step_rk();
        auto t1 = std::chrono::steady_clock::now();
        t_evolve = std::chrono::duration<double>(t1 - t0).count();
        ode.final();
    } else if (engine == "matfree") {
        std::vector<VecMultiD<double>> mats;
        for (int d = 0; d < dim; ++d) {
            VecMultiD<double> m = oper.u_vx;
            const VecMultiD<double>& f = (c[d] >= 0) ? oper.ulft_vjp : oper.urgt_vjp;
            for (int r = 0; r < oper.row; ++r)
                for (int q = 0; q < oper.col; ++q) m.at(r, q) = oper.u_vx.at(r, q) + f.at(r, q);
            mats.push_back(m);
        }
        LinearMatFree fast(dg);
        auto rhs_eval = [&]() {
            fast.zero_rhs();
            for (int d = 0; d < dim; ++d) fast.apply_dim(&mats[d], d, c[d]);
        };
        rhs_eval();
        dump_elements("rhs0", dg, 1);
        auto t0 = std::chrono::steady_clock::now();
        for (int s = 0; s < steps; ++s) {
            RK3SSP ode(dg, dt);
            ode.init();
            for (int stage = 0; stage < 3; ++stage) {
                rhs_eval();
                ode.set_rhs_zero();
                ode.add_rhs_to_eigenvec();
                ode.step_stage(stage);
                ode.final();
            }
        }
        auto t1 = std::chrono::steady_clock::now();
        t_evolve = std::chrono::duration<double>(t1 - t0).count();
    } else {
        std::fprintf(stderr, "unknown engine\n");
        return 2;
    }
    dump_elements("uT", dg, 0);
    if (ic == "sin_prod") {
        // exact solution: translation by c*t
        const double T = steps * dt;
        auto f = [=](double x, int d) { return std::sin(2 * PI * (x - c[d] * T)); };
        const double err = dg.get_L2_error_split_separable_scalar(f, std::pow(0.5, 0.5 * dim));
        std::printf("L2ERR %.17g\n", err);
    } else if (ic == "sin_sum") {
        // exact solution sin(2 pi sum_d (x_d - c_d t)): DGSolution::get_error_no_separable_scalar
        // (DGSolution.cpp:326-335) with 1 and 2 Gauss points
        const double T = steps * dt;
        double shift = 0.0;
        for (int d = 0; d < dim; ++d) shift += c[d] * T;
        auto f = [=](std::vector<double> x) {
            double s = -shift;
            for (double xd : x) s += xd;
            return std::sin(2 * PI * s);
        };
        for (int gp = 1; gp <= 2; ++gp) {
            std::vector<double> err = dg.get_error_no_separable_scalar(f, gp);
            std::printf("NORMERR %d %.17g %.17g %.17g\n", gp, err[0], err[1], err[2]);
        }
    }
    std::printf("TIME evolve_s=%.9g dof_stage=%.17g\n", t_evolve, 3.0 * steps * dg.get_dof());
    return 0;
}

int run_burgers(int argc, char** argv) {
    if (argc < 7) { std::fprintf(stderr, "burgers: bad args\n"); return 2; }
    const int dim = std::atoi(argv[2]);
    const int N = std::atoi(argv[3]);
    const double alpha = std::atof(argv[4]);
    const int steps = std::atoi(argv[5]);
    const double dt = std::atof(argv[6]);
    const int k = 2;
    set_statics(dim, k);
    Hash hash;
    LagrBasis::set_interp_msh01();
    HermBasis::set_interp_msh01();
    AllBasis<AlptBasis> all_bas_alpt(N);
    AllBasis<LagrBasis> all_bas_lagr(N);
    AllBasis<HermBasis> all_bas_herm(N);
    OperatorMatrix1D<AlptBasis, AlptBasis> oper_alpt(all_bas_alpt, all_bas_alpt, "period");
    OperatorMatrix1D<LagrBasis, AlptBasis> oper_lagr(all_bas_lagr, all_bas_alpt, "period");
    DGAdapt dg(true, N, N, all_bas_alpt, all_bas_lagr, all_bas_herm, hash, 1e10, -1, true, false);

    const double PI = Const::PI;
    std::vector<std::function<double(double, int)>> funcs;
    funcs.push_back([](double, int d) { return d == 0 ? 0.5 : 1.0; });
    for (int mask = 0; mask < (1 << dim); ++mask) {
        int nsin = __builtin_popcount(mask);
        if (nsin % 2 == 0) continue;
        const double sign = ((nsin - 1) / 2) % 2 == 0 ? 0.25 : -0.25;
        funcs.push_back([=](double x, int d) {
            double v = ((mask >> d) & 1) ? std::sin(2 * PI * x) : std::cos(2 * PI * x);
            return d == 0 ? sign * v : v;
        });
    }
    dg.init_separable_scalar_sum(funcs);
    std::printf("META dim=%d N=%d k=%d sparse=1 elements=%zu dof=%d\n", dim, N, k, dg.dg.size(), dg.get_dof());
    dump_elements("u0", dg, 0);

    auto flux = [](std::vector<double> u, int, int) -> double { return FluxFunction::burgers_flux_scalar(u[0]); };
    std::vector<std::vector<bool>> is_intp(1, std::vector<bool>(dim, true));
    LagrInterpolation interp(dg);
    FastLagrIntp fast_lagr(dg, interp.Lag_pt_Alpt_1D, interp.Lag_pt_Alpt_1D_d1);
    HyperbolicLagrRHS rhs_lagr(dg, oper_lagr);
    HyperbolicAlptRHS rhs_alpt(dg, oper_alpt);
    const std::vector<double> lxf(dim, alpha);
    auto rhs_eval = [&]() {
        interp.nonlinear_Lagr_fast(flux, is_intp, fast_lagr);
        dg.set_rhs_zero();
        rhs_lagr.rhs_vol_scalar();
        rhs_lagr.rhs_flx_intp_scalar();
        rhs_alpt.rhs_flx_penalty_scalar(lxf);
    };
    rhs_eval();
    dump_elements_vec("up0", dg, [](const Element& e) -> const VecMultiD<double>& { return e.up_intp[0]; });
    for (int d = 0; d < dim; ++d) {
        char nm[32];
        std::snprintf(nm, sizeof nm, "fu0_%d", d);
        dump_elements_vec(nm, dg, [d](const Element& e) -> const VecMultiD<double>& { return e.fucoe_intp[0][d]; });
    }
    dump_elements("rhs0", dg, 1);
    auto t0 = std::chrono::steady_clock::now();
    for (int s = 0; s < steps; ++s) {
        RK3SSP ode(dg, dt);
        ode.init();
        for (int stage = 0; stage < 3; ++stage) {
            rhs_eval();
            ode.set_rhs_zero();
            ode.add_rhs_to_eigenvec();
            ode.step_stage(stage);
            ode.final();
        }
    }
    auto t1 = std::chrono::steady_clock::now();
    dump_elements("uT", dg, 0);
    std::printf("TIME evolve_s=%.9g dof_stage=%.17g\n", std::chrono::duration<double>(t1 - t0).count(),
                3.0 * steps * dg.get_dof());
    // exact solution u(x, T) = exact_1d(sum_d x_d, dim T) of BurgersExact(0.5, 0.25, 0)
    // (ExactSolution.h:13-19: a + b v(X - a T' + c, b T') with X = sum x_d, T' = dim T)
    BurgersExact burgers(0.5, 0.25, 0.0);
    const double T = steps * dt;
    auto exact = [&](std::vector<double> x) -> double {
        double s = 0.0;
        for (int d = 0; d < dim; ++d) s += x[d];
        return burgers.exact_1d(s, dim * T);
    };
    // DGSolution::val and the exact solution at fixed quasi-random points
    const int npts = 48;
    std::printf("BEGIN vals %d %d\n", npts, dim + 2);
    for (int i = 0; i < npts; ++i) {
        std::vector<double> x(dim);
        for (int d = 0; d < dim; ++d) {
            const double a = 0.7548776662466927 * (d + 1) + 0.5698402909980532 * d * d;
            x[d] = std::fmod(0.5 + a * (i + 1), 1.0);
        }
        for (int d = 0; d < dim; ++d) std::printf("%.17g ", x[d]);
        std::printf("%.17g %.17g\n", dg.val(x, std::vector<int>(dim, 0))[0], exact(x));
    }
    std::printf("END\n");
    // DGSolution::get_error_no_separable_scalar (DGSolution.cpp:326-335) with 1 and 2 Gauss points
    for (int gp = 1; gp <= 2; ++gp) {
        std::vector<double> err = dg.get_error_no_separable_scalar(exact, gp);
        std::printf("NORMERR %d %.17g %.17g %.17g\n", gp, err[0], err[1], err[2]);
    }
    return 0;
}

// 2D Burgers with the flux interpolated by cubic Hermite interpolation (HermBasis::PMAX = 3,
// msh_case 1), as example/02_hyperbolic_05_burgers_adapt.cpp:192-263 composes it:
// HermInterpolation::nonlinear_Herm_2D_fast (flux, its first and second derivative; interpolation
// in x only, the flux being the same in every direction), HyperbolicSameFluxHermRHS::rhs_vol_scalar
// and rhs_flx_intp_scalar, HyperbolicAlptRHS::rhs_flx_penalty_scalar(alpha); RK3SSP step_stage on
// the sparse grid of level N.  Dumps u0, up0 (u and its x / y / xy derivatives at the Hermite
// points), fu0 (the flux's Hermite coefficients), rhs0 and uT.
int run_burgers_herm(int argc, char** argv) {
    if (argc < 6) { std::fprintf(stderr, "burgers_herm: bad args\n"); return 2; }
    const int dim = 2;
    const int N = std::atoi(argv[2]);
    const double alpha = std::atof(argv[3]);
    const int steps = std::atoi(argv[4]);
    const double dt = std::atof(argv[5]);
    const int k = 2;
    set_statics(dim, k);
    Hash hash;
    LagrBasis::set_interp_msh01();
    HermBasis::set_interp_msh01();
    AllBasis<AlptBasis> all_bas_alpt(N);
    AllBasis<LagrBasis> all_bas_lagr(N);
    AllBasis<HermBasis> all_bas_herm(N);
    OperatorMatrix1D<AlptBasis, AlptBasis> oper_alpt(all_bas_alpt, all_bas_alpt, "period");
    OperatorMatrix1D<HermBasis, AlptBasis> oper_herm(all_bas_herm, all_bas_alpt, "period");
    DGAdapt dg(true, N, N, all_bas_alpt, all_bas_lagr, all_bas_herm, hash, 1e10, -1, true, false);
    const double PI = Const::PI;
    std::vector<std::function<double(double, int)>> funcs;
    funcs.push_back([](double, int d) { return d == 0 ? 0.5 : 1.0; });
    funcs.push_back([=](double x, int d) { return d == 0 ? 0.25 * std::sin(2 * PI * x) : std::cos(2 * PI * x); });
    funcs.push_back([=](double x, int d) { return d == 0 ? 0.25 * std::cos(2 * PI * x) : std::sin(2 * PI * x); });
    dg.init_separable_scalar_sum(funcs);
    std::printf("META dim=%d N=%d k=%d sparse=1 elements=%zu dof=%d\n", dim, N, k, dg.dg.size(), dg.get_dof());
    dump_elements("u0", dg, 0);
    auto flux = [](std::vector<double> u, int, int) -> double { return FluxFunction::burgers_flux_scalar(u[0]); };
    auto flux_d1 = [](std::vector<double> u, int, int, int) -> double {
        return FluxFunction::burgers_flux_1st_derivative_scalar(u[0]);
    };
    auto flux_d2 = [](std::vector<double> u, int, int, int, int) -> double {
        return FluxFunction::burgers_flux_2nd_derivative_scalar(u[0]);
    };
    std::vector<std::vector<bool>> is_intp_herm{std::vector<bool>{true, false}};
    HermInterpolation interp(dg);
    FastHermIntp fast_herm(dg, interp.Her_pt_Alpt_1D);
    HyperbolicSameFluxHermRHS rhs_herm(dg, oper_herm);
    HyperbolicAlptRHS rhs_alpt(dg, oper_alpt);
    const std::vector<double> lxf(dim, alpha);
    auto rhs_eval = [&]() {
        interp.nonlinear_Herm_2D_fast(flux, flux_d1, flux_d2, is_intp_herm, fast_herm);
        dg.set_rhs_zero();
        rhs_herm.rhs_vol_scalar();
        rhs_herm.rhs_flx_intp_scalar();
        rhs_alpt.rhs_flx_penalty_scalar(lxf);
    };
    rhs_eval();
    dump_elements_vec("up0", dg, [](const Element& e) -> const VecMultiD<double>& { return e.up_intp[0]; });
    dump_elements_vec("fu0", dg, [](const Element& e) -> const VecMultiD<double>& { return e.fucoe_intp[0][0]; });
    dump_elements("rhs0", dg, 1);
    for (int s = 0; s < steps; ++s) {
        RK3SSP ode(dg, dt);
        ode.init();
        for (int stage = 0; stage < 3; ++stage) {
            rhs_eval();
            ode.set_rhs_zero();
            ode.add_rhs_to_eigenvec();
            ode.step_stage(stage);
            ode.final();
        }
    }
    dump_elements("uT", dg, 0);
    return 0;
}

// The time loop of example/02_hyperbolic_05_burgers_adapt.cpp:223-476 as that driver runs it
// without artificial viscosity: 2D, u0 = sin(2 pi (x+y)) by init_separable_scalar_sum, cubic
// Hermite interpolation of the flux (HermInterpolation::nonlinear_Herm_2D_fast, built once before
// the loop, as the driver does), HyperbolicSameFluxHermRHS volume and interface terms, the LxF
// penalty as the assembled HyperbolicAlpt matrix (assemble_matrix_flx_scalar(d, -1, alpha/2) and
// (d, 1, -alpha/2)) added by add_rhs_matrix, dt = cfl / sum_d 2^maxlevel_d (wave speed 1),
// predictor, refine, SSP-RK3, coarsen.  Dumps u after init and after every step; with "time" the
// step wall times instead (as burgers_adapt).
int run_burgers_herm_adapt(int argc, char** argv) {
    if (argc < 9) { std::fprintf(stderr, "burgers_herm_adapt: bad args\n"); return 2; }
    const int dim = 2;
    const int N_init = std::atoi(argv[2]);
    const int NMAX = std::atoi(argv[3]);
    const double eps = std::atof(argv[4]);
    const double eta = std::atof(argv[5]);
    const double alpha = std::atof(argv[6]);
    const double cfl = std::atof(argv[7]);
    const int steps = std::atoi(argv[8]);
    const bool timing = argc > 9 && std::string(argv[9]) == "time";
    const double t_end = argc > 10 ? std::atof(argv[10]) : 0.0;
    const int k = 2;
    set_statics(dim, k);
    Hash hash;
    LagrBasis::set_interp_msh01();
    HermBasis::set_interp_msh01();
    AllBasis<AlptBasis> all_bas_alpt(NMAX);
    AllBasis<LagrBasis> all_bas_lagr(NMAX);
    AllBasis<HermBasis> all_bas_herm(NMAX);
    OperatorMatrix1D<AlptBasis, AlptBasis> oper_alpt(all_bas_alpt, all_bas_alpt, "period");
    OperatorMatrix1D<HermBasis, AlptBasis> oper_herm(all_bas_herm, all_bas_alpt, "period");
    DGAdapt dg(true, N_init, NMAX, all_bas_alpt, all_bas_lagr, all_bas_herm, hash, eps, eta, true, true);
    const double PI = Const::PI;
    std::vector<std::function<double(double, int)>> funcs;
    funcs.push_back([=](double x, int d) { return d == 0 ? std::sin(2. * PI * x) : std::cos(2. * PI * x); });
    funcs.push_back([=](double x, int d) { return d == 0 ? std::cos(2. * PI * x) : std::sin(2. * PI * x); });
    dg.init_separable_scalar_sum(funcs);
    std::printf("META dim=%d N=%d k=%d sparse=1 elements=%zu dof=%d\n", dim, NMAX, k, dg.dg.size(), dg.get_dof());
    if (!timing) dump_elements("u_init", dg, 0);
    auto flux = [](std::vector<double> u, int, int) -> double { return FluxFunction::burgers_flux_scalar(u[0]); };
    auto flux_d1 = [](std::vector<double> u, int, int, int) -> double {
        return FluxFunction::burgers_flux_1st_derivative_scalar(u[0]);
    };
    auto flux_d2 = [](std::vector<double> u, int, int, int, int) -> double {
        return FluxFunction::burgers_flux_2nd_derivative_scalar(u[0]);
    };
    HyperbolicSameFluxHermRHS rhs_herm(dg, oper_herm);
    HermInterpolation interp(dg);
    std::vector<std::vector<bool>> is_intp_herm{std::vector<bool>{true, false}};
    FastHermIntp fast_herm(dg, interp.Her_pt_Alpt_1D);
    auto assemble = [&](HyperbolicAlpt& lin) {
        for (int d = 0; d < dim; ++d) {
            lin.assemble_matrix_flx_scalar(d, -1, alpha / 2);
            lin.assemble_matrix_flx_scalar(d, 1, -alpha / 2);
        }
    };
    auto herm_rhs = [&]() {
        interp.nonlinear_Herm_2D_fast(flux, flux_d1, flux_d2, is_intp_herm, fast_herm);
        dg.set_rhs_zero();
        rhs_herm.rhs_vol_scalar();
        rhs_herm.rhs_flx_intp_scalar();
    };
    double t = 0.0;
    for (int step = 0; step < steps; ++step) {
        if (t_end > 0.0 && t >= t_end) break;
        const auto t0 = std::chrono::steady_clock::now();
        const std::vector<int> max_mesh = dg.max_mesh_level_vec();
        double sum_c_dx = 0.;
        for (int d = 0; d < dim; ++d) sum_c_dx += 1.0 * std::pow(2., max_mesh[d]);
        double dt = cfl / sum_c_dx;
        if (t_end > 0.0) dt = std::min(dt, t_end - t);
        {
            dg.copy_ucoe_to_predict();
            HyperbolicAlpt linear(dg, oper_alpt);
            assemble(linear);
            ForwardEuler ode(linear, dt);
            ode.init();
            herm_rhs();
            ode.set_rhs_zero();
            ode.add_rhs_to_eigenvec();
            ode.add_rhs_matrix(linear);
            ode.step_stage(0);
            ode.final();
        }
        dg.refine();
        const int stage_dof = dg.get_dof();
        dg.copy_predict_to_ucoe();
        {
            HyperbolicAlpt linear(dg, oper_alpt);
            assemble(linear);
            RK3SSP ode(linear, dt);
            ode.init();
            for (int stage = 0; stage < ode.num_stage; ++stage) {
                herm_rhs();
                ode.set_rhs_zero();
                ode.add_rhs_to_eigenvec();
                ode.add_rhs_matrix(linear);
                ode.step_stage(stage);
                ode.final();
            }
        }
        dg.coarsen();
        t += dt;
        if (timing) {
            const double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            std::printf("TSTEP %d %.9g %d %zu\n", step, sec, stage_dof, dg.dg.size());
            std::fflush(stdout);
            continue;
        }
        std::printf("STEP %d dt=%.17g elements=%zu\n", step, dt, dg.dg.size());
        char nm[32];
        std::snprintf(nm, sizeof nm, "u_step%d", step);
        dump_elements(nm, dg, 0);
    }
    return 0;
}

int run_burgers_adapt(int argc, char** argv) {
    if (argc < 11) { std::fprintf(stderr, "burgers_adapt: bad args\n"); return 2; }
    const int dim = std::atoi(argv[2]);
    const int N_init = std::atoi(argv[3]);
    const int NMAX = std::atoi(argv[4]);
    const double eps = std::atof(argv[5]);
    const double eta = std::atof(argv[6]);
    const double alpha = std::atof(argv[7]);
    const double cfl = std::atof(argv[8]);
    const double umax = std::atof(argv[9]);
    const int steps = std::atoi(argv[10]);
    const bool timing = argc > 11 && std::string(argv[11]) == "time";
    const double t_end = argc > 12 ? std::atof(argv[12]) : 0.0;
    const int k = 2;
    set_statics(dim, k);
    Hash hash;
    LagrBasis::set_interp_msh01();
    HermBasis::set_interp_msh01();
    AllBasis<AlptBasis> all_bas_alpt(NMAX);
    AllBasis<LagrBasis> all_bas_lagr(NMAX);
    AllBasis<HermBasis> all_bas_herm(NMAX);
    OperatorMatrix1D<AlptBasis, AlptBasis> oper_alpt(all_bas_alpt, all_bas_alpt, "period");
    OperatorMatrix1D<LagrBasis, AlptBasis> oper_lagr(all_bas_lagr, all_bas_alpt, "period");
    DGAdapt dg(true, N_init, NMAX, all_bas_alpt, all_bas_lagr, all_bas_herm, hash, eps, eta, true, false);

    const double PI = Const::PI;
    std::vector<std::function<double(double, int)>> funcs;
    funcs.push_back([](double, int d) { return d == 0 ? 0.5 : 1.0; });
    for (int mask = 0; mask < (1 << dim); ++mask) {
        int nsin = __builtin_popcount(mask);
        if (nsin % 2 == 0) continue;
        const double sign = ((nsin - 1) / 2) % 2 == 0 ? 0.25 : -0.25;
        funcs.push_back([=](double x, int d) {
            double v = ((mask >> d) & 1) ? std::sin(2 * PI * x) : std::cos(2 * PI * x);
            return d == 0 ? sign * v : v;
        });
    }
    dg.init_separable_scalar_sum(funcs);
    std::printf("META dim=%d N=%d k=%d sparse=1 elements=%zu dof=%d\n", dim, NMAX, k, dg.dg.size(), dg.get_dof());
    if (!timing) dump_elements("u_init", dg, 0);

    auto flux = [](std::vector<double> u, int, int) -> double { return FluxFunction::burgers_flux_scalar(u[0]); };
    std::vector<std::vector<bool>> is_intp(1, std::vector<bool>(dim, true));
    HyperbolicLagrRHS rhs_lagr(dg, oper_lagr);
    HyperbolicAlptRHS rhs_alpt(dg, oper_alpt);
    const std::vector<double> lxf(dim, alpha);
    double t = 0.0;
    for (int step = 0; step < steps; ++step) {
        if (t_end > 0.0 && t >= t_end) break;
        const auto t0 = std::chrono::steady_clock::now();
        const std::vector<int> max_mesh = dg.max_mesh_level_vec();
        double sum_c_dx = 0.;
        for (int d = 0; d < dim; ++d) sum_c_dx += umax * std::pow(2., max_mesh[d]);
        double dt = cfl / sum_c_dx;
        if (t_end > 0.0) dt = std::min(dt, t_end - t);
        // LagrInterpolation and FastLagrIntp hold per-grid data: rebuild after adaptation
        auto rhs_eval = [&]() {
            LagrInterpolation interp(dg);
            FastLagrIntp fast_lagr(dg, interp.Lag_pt_Alpt_1D, interp.Lag_pt_Alpt_1D_d1);
            interp.nonlinear_Lagr_fast(flux, is_intp, fast_lagr);
            dg.set_rhs_zero();
            rhs_lagr.rhs_vol_scalar();
            rhs_lagr.rhs_flx_intp_scalar();
            rhs_alpt.rhs_flx_penalty_scalar(lxf);
        };
        dg.copy_ucoe_to_predict();
        {
            ForwardEuler ode(dg, dt);
            ode.init();
            rhs_eval();
            ode.set_rhs_zero();
            ode.add_rhs_to_eigenvec();
            ode.step_stage(0);
            ode.final();
        }
        dg.refine();
        dg.copy_predict_to_ucoe();
        const int stage_dof = dg.get_dof();
        {
            RK3SSP ode(dg, dt);
            ode.init();
            for (int stage = 0; stage < 3; ++stage) {
                rhs_eval();
                ode.set_rhs_zero();
                ode.add_rhs_to_eigenvec();
                ode.step_stage(stage);
                ode.final();
            }
        }
        dg.coarsen();
        t += dt;
        if (timing) {
            const double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            std::printf("TSTEP %d %.9g %d %zu\n", step, sec, stage_dof, dg.dg.size());
            std::fflush(stdout);
            continue;
        }
        int maxsum = 0;
        for (auto& it : dg.dg) {
            int s = 0;
            for (int d = 0; d < dim; ++d) s += it.second.level[d];
            maxsum = std::max(maxsum, s);
        }
        std::printf("STEP %d dt=%.17g elements=%zu maxlevsum=%d%s\n", step, dt, dg.dg.size(), maxsum,
                    (dim == 3 && maxsum >= 23) ? " HASH_OVERFLOW" : "");
        char nm[32];
        std::snprintf(nm, sizeof nm, "u_step%d", step);
        dump_elements(nm, dg, 0);
    }
    return 0;
}

// Wave equation u_tt = div(K grad u), K = (1 + a prod_d sin(2 pi x_d))^2, periodic, Alpert k = 2,
// Lagrange degree 4 (msh_case 2, as the example sets it) interpolation of K u_x and K u, DiffusionRHS terms and the IPDG
// penalty as 03_wave_06_var_coeff_adapt.cpp:154-279 (no source, no adaptivity): u0 a Gaussian bump,
// u_t = 0. Dumps u0, rhs0 (the right-hand side at u0, read through EulerODE2nd with dt = 1 on a
// second solution) and uT, vT after `steps` RK4ODE2nd steps.
int run_wave(int argc, char** argv) {
    if (argc < 7) { std::fprintf(stderr, "wave: bad args\n"); return 2; }
    const int dim = std::atoi(argv[2]);
    const int N = std::atoi(argv[3]);
    const double sigma = std::atof(argv[4]);
    const int steps = std::atoi(argv[5]);
    const double dt = std::atof(argv[6]);
    const double amp = argc > 7 ? std::atof(argv[7]) : 0.5;
    const int k = 2;
    set_statics(dim, k, 4);
    DGSolution::prob = "wave";
    Hash hash;
    LagrBasis::set_interp_msh01();
    HermBasis::set_interp_msh01();
    AllBasis<AlptBasis> all_bas_alpt(N);
    AllBasis<LagrBasis> all_bas_lagr(N);
    AllBasis<HermBasis> all_bas_herm(N);
    OperatorMatrix1D<AlptBasis, AlptBasis> oper_alpt(all_bas_alpt, all_bas_alpt, "period");
    OperatorMatrix1D<LagrBasis, AlptBasis> oper_lagr(all_bas_lagr, all_bas_alpt, "period");
    const double centre[3] = {0.3, 0.4, 0.5};
    auto zero = [](double, int) { return 0.0; };
    auto bump = [&](double x, int d) { return std::exp(-200.0 * (x - centre[d]) * (x - centre[d])); };
    const double PI = Const::PI;
    auto coe = [=](std::vector<double> x, int) -> double {
        double s = 1.0;
        for (int d = 0; d < dim; ++d) s *= std::sin(2 * PI * x[d]);
        const double c = 1.0 + amp * s;
        return c * c;
    };
    std::vector<std::vector<bool>> is_intp(1, std::vector<bool>(dim, true));
    std::vector<std::vector<bool>> is_intp_d0(1, std::vector<bool>(dim, false));
    is_intp_d0[0][0] = true;
    auto init = [&](DGAdapt& dg) {
        dg.init_separable_scalar(zero);
        dg.copy_ucoe_to_ucoe_ut();
        dg.init_separable_scalar(bump);
    };
    // right-hand side at u0: v1 = v0 + 1 * rhs with v0 = 0
    {
        DGAdapt dg(true, N, N, all_bas_alpt, all_bas_lagr, all_bas_herm, hash, 1e10, -1, true, false);
        init(dg);
        LagrInterpolation interp(dg);
        FastLagrIntp fast(dg, interp.Lag_pt_Alpt_1D, interp.Lag_pt_Alpt_1D_d1);
        DiffusionRHS diffuse(dg, oper_lagr);
        DiffusionAlpt ipdg(dg, oper_alpt, sigma);
        ipdg.assemble_matrix_flx_ujp_vjp();
        EulerODE2nd ode(ipdg, 1.0);
        ode.init();
        dg.set_rhs_zero();
        interp.var_coeff_gradu_Lagr_fast(coe, is_intp, fast);
        diffuse.rhs_flx_gradu();
        diffuse.rhs_vol();
        interp.var_coeff_u_Lagr_fast(coe, is_intp_d0, fast);
        diffuse.rhs_flx_u();
        ode.rhs_to_eigenvec();
        ode.add_rhs_matrix(ipdg);
        ode.step_stage(0);
        ode.final();
        dump_elements("rhs0", dg, 2);
    }
    DGAdapt dg(true, N, N, all_bas_alpt, all_bas_lagr, all_bas_herm, hash, 1e10, -1, true, false);
    init(dg);
    std::printf("META dim=%d N=%d k=%d sparse=1 elements=%zu dof=%d\n", dim, N, k, dg.dg.size(), dg.get_dof());
    dump_elements("u0", dg, 0);
    LagrInterpolation interp(dg);
    FastLagrIntp fast(dg, interp.Lag_pt_Alpt_1D, interp.Lag_pt_Alpt_1D_d1);
    DiffusionRHS diffuse(dg, oper_lagr);
    auto t0 = std::chrono::steady_clock::now();
    for (int s = 0; s < steps; ++s) {
        DiffusionAlpt ipdg(dg, oper_alpt, sigma);
        ipdg.assemble_matrix_flx_ujp_vjp();
        RK4ODE2nd ode(ipdg, dt);
        ode.init();
        for (int stage = 0; stage < 4; ++stage) {
            dg.set_rhs_zero();
            interp.var_coeff_gradu_Lagr_fast(coe, is_intp, fast);
            diffuse.rhs_flx_gradu();
            diffuse.rhs_vol();
            interp.var_coeff_u_Lagr_fast(coe, is_intp_d0, fast);
            diffuse.rhs_flx_u();
            ode.rhs_to_eigenvec();
            ode.add_rhs_matrix(ipdg);
            ode.step_stage(stage);
            ode.final();
        }
    }
    auto t1 = std::chrono::steady_clock::now();
    dump_elements("uT", dg, 0);
    dump_elements("vT", dg, 2);
    std::printf("TIME evolve_s=%.9g dof_stage=%.17g\n", std::chrono::duration<double>(t1 - t0).count(),
                4.0 * steps * dg.get_dof());
    return 0;
}

// The adaptive wave loop of 03_wave_06_var_coeff_adapt.cpp:181-297 (no source): dt from the
// finest level, EulerODE2nd predictor on copies of (u, u_t) through step_rk (the source-free
// step_rk_source: rhs recomputed as the IPDG matrix times u), refine, copy the predictions
// back, four RK4ODE2nd stages with the interpolated DiffusionRHS terms plus the IPDG matrix,
// coarsen. u0 the Gaussian bump, u_t(0) = 0, adaptive initialisation. Dumps u and u_t after
// the initialisation and after every step.
int run_wave_adapt(int argc, char** argv) {
    if (argc < 10) { std::fprintf(stderr, "wave_adapt: bad args\n"); return 2; }
    const int dim = std::atoi(argv[2]);
    const int N_init = std::atoi(argv[3]);
    const int NMAX = std::atoi(argv[4]);
    const double eps = std::atof(argv[5]);
    const double eta = std::atof(argv[6]);
    const double sigma = std::atof(argv[7]);
    const double cfl = std::atof(argv[8]);
    const int steps = std::atoi(argv[9]);
    const double amp = argc > 10 ? std::atof(argv[10]) : 0.5;
    const int k = 2;
    set_statics(dim, k, 4);
    DGSolution::prob = "wave";
    Hash hash;
    LagrBasis::set_interp_msh01();
    HermBasis::set_interp_msh01();
    AllBasis<AlptBasis> all_bas_alpt(NMAX);
    AllBasis<LagrBasis> all_bas_lagr(NMAX);
    AllBasis<HermBasis> all_bas_herm(NMAX);
    OperatorMatrix1D<AlptBasis, AlptBasis> oper_alpt(all_bas_alpt, all_bas_alpt, "period");
    OperatorMatrix1D<LagrBasis, AlptBasis> oper_lagr(all_bas_lagr, all_bas_alpt, "period");
    DGAdapt dg(true, N_init, NMAX, all_bas_alpt, all_bas_lagr, all_bas_herm, hash, eps, eta, true, false);
    const double centre[3] = {0.3, 0.4, 0.5};
    auto zero = [](double, int) { return 0.0; };
    auto bump = [&](double x, int d) { return std::exp(-200.0 * (x - centre[d]) * (x - centre[d])); };
    const double PI = Const::PI;
    auto coe = [=](std::vector<double> x, int) -> double {
        double s = 1.0;
        for (int d = 0; d < dim; ++d) s *= std::sin(2 * PI * x[d]);
        const double c = 1.0 + amp * s;
        return c * c;
    };
    std::vector<std::vector<bool>> is_intp(1, std::vector<bool>(dim, true));
    std::vector<std::vector<bool>> is_intp_d0(1, std::vector<bool>(dim, false));
    is_intp_d0[0][0] = true;
    dg.init_separable_scalar(zero);
    dg.copy_ucoe_to_ucoe_ut();
    dg.init_separable_scalar(bump);
    std::printf("META dim=%d N=%d k=%d sparse=1 elements=%zu dof=%d\n", dim, NMAX, k, dg.dg.size(), dg.get_dof());
    dump_elements("u_init", dg, 0);
    dump_elements("ut_init", dg, 2);
    DiffusionRHS diffuse(dg, oper_lagr);
    double t = 0.0;
    for (int step = 0; step < steps; ++step) {
        const std::vector<int> max_mesh = dg.max_mesh_level_vec();
        double sum_c_dx = 0.;
        for (int d = 0; d < dim; ++d) sum_c_dx += 1.0 * std::pow(2., max_mesh[d]);
        const double dt = cfl / sum_c_dx;
        dg.copy_ucoe_to_predict();
        dg.copy_ucoe_ut_to_predict();
        {
            DiffusionAlpt ipdg(dg, oper_alpt, sigma);
            ipdg.assemble_matrix_flx_ujp_vjp();
            EulerODE2nd ode(ipdg, dt);
            ode.init();
            ode.step_rk();
            ode.final();
        }
        dg.refine();
        dg.copy_predict_to_ucoe();
        dg.copy_predict_to_ucoe_ut();
        {
            DiffusionAlpt ipdg(dg, oper_alpt, sigma);
            ipdg.assemble_matrix_flx_ujp_vjp();
            RK4ODE2nd ode(ipdg, dt);
            ode.init();
            LagrInterpolation interp(dg);
            FastLagrIntp fast(dg, interp.Lag_pt_Alpt_1D, interp.Lag_pt_Alpt_1D_d1);
            for (int stage = 0; stage < 4; ++stage) {
                dg.set_rhs_zero();
                interp.var_coeff_gradu_Lagr_fast(coe, is_intp, fast);
                diffuse.rhs_flx_gradu();
                diffuse.rhs_vol();
                interp.var_coeff_u_Lagr_fast(coe, is_intp_d0, fast);
                diffuse.rhs_flx_u();
                ode.rhs_to_eigenvec();
                ode.add_rhs_matrix(ipdg);
                ode.step_stage(stage);
                ode.final();
            }
        }
        dg.coarsen();
        t += dt;
        std::printf("STEP %d dt=%.17g elements=%zu\n", step, dt, dg.dg.size());
        char nm[32];
        std::snprintf(nm, sizeof nm, "u_step%d", step);
        dump_elements(nm, dg, 0);
        std::snprintf(nm, sizeof nm, "ut_step%d", step);
        dump_elements(nm, dg, 2);
    }
    return 0;
}

int run_matrices(int argc, char** argv) {
    if (argc < 4) return 2;
    const int N = std::atoi(argv[2]);
    const int k = std::atoi(argv[3]);
    set_statics(1, k);
    AllBasis<AlptBasis> all_bas_alpt(N);
    OperatorMatrix1D<AlptBasis, AlptBasis> oper(all_bas_alpt, all_bas_alpt, "period");
    dump_matrix("u_v", oper.u_v, oper.row, oper.col);
    dump_matrix("u_vx", oper.u_vx, oper.row, oper.col);
    dump_matrix("ulft_vjp", oper.ulft_vjp, oper.row, oper.col);
    dump_matrix("urgt_vjp", oper.urgt_vjp, oper.row, oper.col);
    return 0;
}

int run_intp_init(int argc, char** argv) {
    if (argc < 8) { std::fprintf(stderr, "intp_init: bad args\n"); return 2; }
    const int dim = std::atoi(argv[2]);
    const int N_init = std::atoi(argv[3]);
    const int NMAX = std::atoi(argv[4]);
    const double eps = std::atof(argv[5]);
    const int degree = std::atoi(argv[6]);
    const double width = std::atof(argv[7]);
    const int k = 2;
    set_statics(dim, k, degree);
    Hash hash;
    LagrBasis::set_interp_msh01();
    HermBasis::set_interp_msh01();
    AllBasis<AlptBasis> all_bas_alpt(NMAX);
    AllBasis<LagrBasis> all_bas_lagr(NMAX);
    AllBasis<HermBasis> all_bas_herm(NMAX);
    OperatorMatrix1D<LagrBasis, LagrBasis> oper_ll(all_bas_lagr, all_bas_lagr, "period");
    OperatorMatrix1D<HermBasis, HermBasis> oper_hh(all_bas_herm, all_bas_herm, "period");
    DGAdaptIntp dg(true, N_init, NMAX, all_bas_alpt, all_bas_lagr, all_bas_herm, hash, eps, eps / 10, true, false,
                   oper_ll, oper_hh);
    const double centre[3] = {0.3, 0.4, 0.5};
    auto f = [=](std::vector<double> x, int) {
        double r2 = 0.0;
        for (int d = 0; d < dim; ++d) r2 += (x[d] - centre[d]) * (x[d] - centre[d]);
        return std::exp(-width * r2);
    };
    dg.init_adaptive_intp(f);
    std::printf("META dim=%d N=%d k=%d sparse=1 elements=%zu dof=%d\n", dim, NMAX, k, dg.dg.size(), dg.get_dof());
    dump_elements("u_init", dg, 0);
    return 0;
}

int run_intp_error(int argc, char** argv) {
    if (argc < 9) { std::fprintf(stderr, "intp_error: bad args\n"); return 2; }
    const int dim = std::atoi(argv[2]);
    const int N_init = std::atoi(argv[3]);
    const int NMAX = std::atoi(argv[4]);
    const double eps_a = std::atof(argv[5]);
    const double eps_b = std::atof(argv[6]);
    const int degree = std::atoi(argv[7]);
    const double width = std::atof(argv[8]);
    set_statics(dim, 2, degree);
    Hash hash;
    LagrBasis::set_interp_msh01();
    HermBasis::set_interp_msh01();
    AllBasis<AlptBasis> all_bas_alpt(NMAX);
    AllBasis<LagrBasis> all_bas_lagr(NMAX);
    AllBasis<HermBasis> all_bas_herm(NMAX);
    OperatorMatrix1D<LagrBasis, LagrBasis> oper_ll(all_bas_lagr, all_bas_lagr, "period");
    OperatorMatrix1D<HermBasis, HermBasis> oper_hh(all_bas_herm, all_bas_herm, "period");
    const double centre[3] = {0.3, 0.4, 0.5};
    auto f = [=](std::vector<double> x, int) {
        double r2 = 0.0;
        for (int d = 0; d < dim; ++d) r2 += (x[d] - centre[d]) * (x[d] - centre[d]);
        return std::exp(-width * r2);
    };
    DGAdaptIntp a(true, N_init, NMAX, all_bas_alpt, all_bas_lagr, all_bas_herm, hash, eps_a, eps_a / 10, true, false,
                  oper_ll, oper_hh);
    a.init_adaptive_intp(f);
    DGAdaptIntp b(true, N_init, NMAX, all_bas_alpt, all_bas_lagr, all_bas_herm, hash, eps_b, eps_b / 10, true, false,
                  oper_ll, oper_hh);
    b.init_adaptive_intp(f);
    const double err = a.get_L2_error_split_adaptive_intp_scalar(b);
    dump_elements("u_a", a, 0);
    dump_elements("u_b", b, 0);
    std::printf("BEGIN err 1 1\n%.17g\nEND\n", err);
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 2) { std::fprintf(stderr, "usage: ref_harness linear|matrices ...\n"); return 2; }
    const std::string mode = argv[1];
    if (mode == "linear") return run_linear(argc, argv);
    if (mode == "matrices") return run_matrices(argc, argv);
    if (mode == "burgers") return run_burgers(argc, argv);
    if (mode == "burgers_herm") return run_burgers_herm(argc, argv);
    if (mode == "burgers_adapt") return run_burgers_adapt(argc, argv);
    if (mode == "burgers_herm_adapt") return run_burgers_herm_adapt(argc, argv);
    if (mode == "wave") return run_wave(argc, argv);
    if (mode == "wave_adapt") return run_wave_adapt(argc, argv);
    if (mode == "intp_init") return run_intp_init(argc, argv);
    if (mode == "intp_error") return run_intp_error(argc, argv);
    std::fprintf(stderr, "unknown mode %s\n", mode.c_str());
    return 2;
}
