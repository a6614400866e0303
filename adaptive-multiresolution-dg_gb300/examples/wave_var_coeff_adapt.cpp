// Variable-coefficient wave equation u_tt = div(K grad u) on the periodic unit square with
// adaptivity, written like the reference driver example/03_wave_06_var_coeff_adapt.cpp and running
// on the GPU through amdg_dg.hpp: the same statics (Alpert degree 2, Lagrange degree 4 with the
// msh_case 2 nodes, DGSolution::prob = "wave"), DGAdapt with a coarse start level, the Gaussian
// bump exp(-200 |x - (0.3, 0.4)|^2) at rest, IPDG sigma = 10, and the reference's time loop term
// by term: the EulerODE2nd predictor, refine, the four RK4ODE2nd stages (interpolation of K grad u,
// DiffusionRHS::rhs_flx_gradu / rhs_vol, interpolation of K u, rhs_flx_u, the IPDG matrix term),
// coarsen.  The problem has no source term, so the source assembly of the reference driver and
// the *_source variants of the steps are left out.
//
//   wave_var_coeff_adapt [N_init] [NMAX] [steps] [refine_eps] [coarsen_eta]
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "amdg_dg.hpp"

using namespace amdg_gpu;

int main(int argc, char* argv[]) {
    const int DIM = 2;
    AlptBasis::PMAX = 2;
    LagrBasis::PMAX = 4;
    LagrBasis::msh_case = 2;
    Element::PMAX_alpt = AlptBasis::PMAX;
    Element::DIM = DIM;
    Element::VEC_NUM = 1;
    DGSolution::DIM = Element::DIM;
    DGSolution::VEC_NUM = Element::VEC_NUM;
    DGSolution::prob = "wave";
    DGSolution::ind_var_vec = {0};
    DGAdapt::indicator_var_adapt = {0};

    const int N_init = argc > 1 ? std::atoi(argv[1]) : 3;
    const int NMAX = argc > 2 ? std::atoi(argv[2]) : 7;
    const int steps = argc > 3 ? std::atoi(argv[3]) : 20;
    const double refine_eps = argc > 4 ? std::atof(argv[4]) : 1e-5;
    const double coarsen_eta = argc > 5 ? std::atof(argv[5]) : 1e-6;
    const bool sparse = true;
    const double cfl = 0.1;
    const double sigma_ipdg = 10.0;
    const std::vector<double> waveConst(DIM, 1.0);

    Hash hash;
    LagrBasis::set_interp_msh01();
    HermBasis::set_interp_msh01();
    AllBasis<LagrBasis> all_bas_lagr(NMAX);
    AllBasis<HermBasis> all_bas_herm(NMAX);
    AllBasis<AlptBasis> all_bas_alpt(NMAX);
    OperatorMatrix1D<AlptBasis, AlptBasis> oper_matx_alpt(all_bas_alpt, all_bas_alpt, "period");
    OperatorMatrix1D<LagrBasis, AlptBasis> oper_matx_lagr(all_bas_lagr, all_bas_alpt, "period");

    DGAdapt dg_solu(sparse, N_init, NMAX, all_bas_alpt, all_bas_lagr, all_bas_herm, hash, refine_eps, coarsen_eta,
                    true, false);
    // u(0) the Gaussian bump, u_t(0) = 0
    const double centre[2] = {0.3, 0.4};
    dg_solu.init_separable_scalar([&](double x, int d) { return std::exp(-200.0 * (x - centre[d]) * (x - centre[d])); });
    dg_solu.set_ucoe_ut_zero();

    // K = (1 + 0.5 sin(2 pi x) sin(2 pi y))^2
    const double PI = 3.14159265358979323846;
    auto coe_func = [PI](std::vector<double> x, int) -> double {
        const double c = 1.0 + 0.5 * std::sin(2.0 * PI * x[0]) * std::sin(2.0 * PI * x[1]);
        return c * c;
    };
    const std::vector<std::vector<bool>> is_intp{std::vector<bool>(DIM, true)};
    LagrInterpolation interp(dg_solu);
    FastLagrIntp fastLagr(dg_solu, interp.Lag_pt_Alpt_1D, interp.Lag_pt_Alpt_1D_d1);
    DiffusionRHS diffuseRHS(dg_solu, oper_matx_lagr);

    double curr_time = 0.0;
    for (int num_time_step = 0; num_time_step < steps; ++num_time_step) {
        // --- part 1: time step dt = cfl / sum_d c_d 2^maxlevel_d
        const std::vector<int> max_mesh = dg_solu.max_mesh_level_vec();
        double sum_c_dx = 0.;
        for (int d = 0; d < DIM; d++) sum_c_dx += std::abs(waveConst[d]) * std::pow(2., max_mesh[d]);
        const double dt = cfl / sum_c_dx;

        // --- part 2: predict by Euler forward
        {
            dg_solu.copy_ucoe_to_predict();
            dg_solu.copy_ucoe_ut_to_predict();

            DiffusionAlpt operator_ujp_vjp(dg_solu, oper_matx_alpt, sigma_ipdg);
            operator_ujp_vjp.assemble_matrix_flx_ujp_vjp();

            dg_solu.set_source_zero();

            EulerODE2nd odesolver(operator_ujp_vjp, dt);
            odesolver.init();

            dg_solu.set_rhs_zero();

            interp.var_coeff_gradu_Lagr_fast(coe_func, is_intp, fastLagr);
            diffuseRHS.rhs_flx_gradu();
            diffuseRHS.rhs_vol();

            interp.var_coeff_u_Lagr_fast(coe_func, is_intp, fastLagr);
            diffuseRHS.rhs_flx_u();
            odesolver.rhs_to_eigenvec();

            odesolver.add_rhs_matrix(operator_ujp_vjp);

            // EulerODE2nd::step_rk: the rhs is recomputed as the IPDG matrix times u
            odesolver.step_rk();

            odesolver.final();
        }

        // --- part 3: refine on the prediction, then back to the state at t_n
        dg_solu.refine();
        dg_solu.copy_predict_to_ucoe();
        dg_solu.copy_predict_to_ucoe_ut();

        // --- part 4: time evolution
        DiffusionAlpt operator_ujp_vjp(dg_solu, oper_matx_alpt, sigma_ipdg);
        operator_ujp_vjp.assemble_matrix_flx_ujp_vjp();

        dg_solu.set_source_zero();

        RK4ODE2nd odesolver(operator_ujp_vjp, dt);
        odesolver.init();

        for (int stage = 0; stage < odesolver.num_stage; stage++) {
            dg_solu.set_rhs_zero();

            interp.var_coeff_gradu_Lagr_fast(coe_func, is_intp, fastLagr);
            diffuseRHS.rhs_flx_gradu();
            diffuseRHS.rhs_vol();

            interp.var_coeff_u_Lagr_fast(coe_func, is_intp, fastLagr);
            diffuseRHS.rhs_flx_u();
            odesolver.rhs_to_eigenvec();

            odesolver.add_rhs_matrix(operator_ujp_vjp);

            odesolver.step_stage(stage);

            odesolver.final();
        }

        // --- part 5: coarsen
        dg_solu.coarsen();

        curr_time += dt;
    }
    synchronize();

    const std::vector<double> u = dg_solu.coefficients(), ut = dg_solu.ucoe_ut();
    double su = 0.0, sut = 0.0;
    for (double v : u) su += v * v;
    for (double v : ut) sut += v * v;
    std::printf("steps %d time %.17g elements %d max level %d\n", steps, curr_time, dg_solu.size_elem(),
                dg_solu.max_mesh_level());
    std::printf("sum of squares u: %.17g\n", su);
    std::printf("sum of squares u_t: %.17g\n", sut);
    return 0;
}
