// Adaptive inviscid Burgers u_t + sum_d (u^2/2)_{x_d} = 0 with Lagrange interpolation of the flux,
// written like the reference drivers (the time loop of example/02_hyperbolic_05_burgers_adapt.cpp:
// 223-476 with the stage loop of example/07_vlasov_maxwell_adapt.cpp:278-320) and running on the
// GPU through amdg_dg.hpp: the same statics, DGAdapt, LagrInterpolation + FastLagrIntp,
// HyperbolicLagrRHS, HyperbolicAlptRHS with a global Lax-Friedrichs constant, ForwardEuler
// predictor, refine, RK3SSP stage by stage, coarsen.  u0 = 0.5 + 0.25 sin(2 pi (x_1 + ... + x_d)),
// periodic unit cube, Alpert degree 2, Lagrange degree 3 (msh_case 1).
//
//   burgers_adapt [DIM] [N_init] [NMAX] [steps] [refine_eps] [coarsen_eta] [lxf_alpha] [output]
// output (optional): one line per element, "level... suppt... coefficients..." (%.17g)
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>

#include "amdg_dg.hpp"

using namespace amdg_gpu;

int main(int argc, char* argv[]) {
    const int DIM = argc > 1 ? std::atoi(argv[1]) : 3;
    AlptBasis::PMAX = 2;
    LagrBasis::PMAX = 3;
    LagrBasis::msh_case = 1;
    HermBasis::PMAX = 3;
    HermBasis::msh_case = 1;
    Element::PMAX_alpt = AlptBasis::PMAX;
    Element::PMAX_intp = LagrBasis::PMAX;
    Element::DIM = DIM;
    Element::VEC_NUM = 1;
    DGSolution::DIM = Element::DIM;
    DGSolution::VEC_NUM = Element::VEC_NUM;
    Interpolation::DIM = DGSolution::DIM;
    Interpolation::VEC_NUM = DGSolution::VEC_NUM;
    DGSolution::ind_var_vec = {0};
    DGAdapt::indicator_var_adapt = {0};
    Element::is_intp.assign(Element::VEC_NUM, std::vector<bool>(DIM, true));

    const int N_init = argc > 2 ? std::atoi(argv[2]) : 3;
    const int NMAX = argc > 3 ? std::atoi(argv[3]) : 8;
    const int steps = argc > 4 ? std::atoi(argv[4]) : 36;
    const double refine_eps = argc > 5 ? std::atof(argv[5]) : 1e-5;
    const double coarsen_eta = argc > 6 ? std::atof(argv[6]) : 1e-6;
    const double alpha = argc > 7 ? std::atof(argv[7]) : 0.825;
    const std::string output = argc > 8 ? argv[8] : "";
    const bool sparse = true;
    const double cfl = 0.1;
    const std::vector<double> wave_speed(DIM, 0.75);
    const std::string boundary_type = "period";

    Hash hash;
    LagrBasis::set_interp_msh01();
    HermBasis::set_interp_msh01();
    AllBasis<LagrBasis> all_bas_lagr(NMAX);
    AllBasis<HermBasis> all_bas_herm(NMAX);
    AllBasis<AlptBasis> all_bas_alpt(NMAX);
    OperatorMatrix1D<AlptBasis, AlptBasis> oper_matx_alpt(all_bas_alpt, all_bas_alpt, boundary_type);
    OperatorMatrix1D<LagrBasis, AlptBasis> oper_matx_lagr(all_bas_lagr, all_bas_alpt, boundary_type);

    DGAdapt dg_solu(sparse, N_init, NMAX, all_bas_alpt, all_bas_lagr, all_bas_herm, hash, refine_eps, coarsen_eta,
                    true, false);
    // 0.5 + 0.25 sin(2 pi sum_d x_d) as a sum of separable terms: the constant, then every product
    // of sines and cosines with an odd number of sines (sin of a sum, expanded)
    std::vector<std::function<double(double, int)>> init_func;
    init_func.push_back([](double, int d) { return d == 0 ? 0.5 : 1.0; });
    for (int mask = 0; mask < (1 << DIM); ++mask) {
        int nsin = 0;
        for (int d = 0; d < DIM; ++d) nsin += (mask >> d) & 1;
        if (nsin % 2 == 0) continue;
        const double sign = ((nsin - 1) / 2) % 2 == 0 ? 0.25 : -0.25;
        init_func.push_back([=](double x, int d) {
            const double v = ((mask >> d) & 1) ? std::sin(2. * M_PI * x) : std::cos(2. * M_PI * x);
            return d == 0 ? sign * v : v;
        });
    }
    dg_solu.init_separable_scalar_sum(init_func);

    auto func_flux = [](std::vector<double> u, int, int) -> double { return FluxFunction::burgers_flux_scalar(u[0]); };
    const std::vector<std::vector<bool>> is_intp(1, std::vector<bool>(DIM, true));
    HyperbolicLagrRHS fast_rhs_lagr(dg_solu, oper_matx_lagr);
    HyperbolicAlptRHS fast_rhs_alpt(dg_solu, oper_matx_alpt);
    const std::vector<double> lxf_alpha(DIM, alpha);

    auto rhs_eval = [&]() {
        LagrInterpolation interp(dg_solu);
        FastLagrIntp fast_lagr_intp(dg_solu, interp.Lag_pt_Alpt_1D, interp.Lag_pt_Alpt_1D_d1);
        interp.nonlinear_Lagr_fast(func_flux, is_intp, fast_lagr_intp);
        dg_solu.set_rhs_zero();
        fast_rhs_lagr.rhs_vol_scalar();
        fast_rhs_lagr.rhs_flx_intp_scalar();
        fast_rhs_alpt.rhs_flx_penalty_scalar(lxf_alpha);
    };

    const auto t0 = std::chrono::steady_clock::now();
    double curr_time = 0.;
    for (int num_time_step = 0; num_time_step < steps; ++num_time_step) {
        // dt = cfl / (c_1 / dx_1 + ... + c_dim / dx_dim)
        const std::vector<int> max_mesh = dg_solu.max_mesh_level_vec();
        double sum_c_dx = 0.;
        for (int d = 0; d < DIM; d++) sum_c_dx += std::abs(wave_speed[d]) * std::pow(2., max_mesh[d]);
        const double dt = cfl / sum_c_dx;

        // predict by Euler forward, refine on the prediction, restore the solution
        dg_solu.copy_ucoe_to_predict();
        {
            ForwardEuler odeSolver(dg_solu, dt);
            odeSolver.init();
            rhs_eval();
            odeSolver.set_rhs_zero();
            odeSolver.add_rhs_to_eigenvec();
            odeSolver.step_stage(0);
            odeSolver.final();
        }
        dg_solu.refine();
        dg_solu.copy_predict_to_ucoe();

        // SSP-RK3, the right-hand side re-evaluated per stage
        {
            RK3SSP odeSolver(dg_solu, dt);
            odeSolver.init();
            for (int stage = 0; stage < odeSolver.num_stage; ++stage) {
                rhs_eval();
                odeSolver.set_rhs_zero();
                odeSolver.add_rhs_to_eigenvec();
                odeSolver.step_stage(stage);
                odeSolver.final();
            }
        }
        dg_solu.coarsen();
        curr_time += dt;
    }
    synchronize();
    const double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::printf("steps %d time %.17g elements %d dof %d seconds %.6f\n", steps, curr_time, dg_solu.size_elem(),
                dg_solu.get_dof(), sec);
    if (!output.empty()) {
        std::vector<int> level, suppt;
        dg_solu.elements(level, suppt);
        const std::vector<double> u = dg_solu.coefficients();
        const int E = dg_solu.size_elem(), B = int(u.size()) / std::max(E, 1);
        FILE* f = std::fopen(output.c_str(), "w");
        if (!f) return 1;
        for (int e = 0; e < E; ++e) {
            for (int d = 0; d < DIM; ++d) std::fprintf(f, "%d ", level[size_t(e) * DIM + d]);
            for (int d = 0; d < DIM; ++d) std::fprintf(f, "%d ", suppt[size_t(e) * DIM + d]);
            for (int q = 0; q < B; ++q) std::fprintf(f, "%.17g ", u[size_t(e) * B + q]);
            std::fprintf(f, "\n");
        }
        std::fclose(f);
    }
    return 0;
}
