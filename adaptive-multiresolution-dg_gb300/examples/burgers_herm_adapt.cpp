// Adaptive 2D inviscid Burgers u_t + (u^2/2)_x + (u^2/2)_y = 0 with the flux interpolated by cubic
// Hermite interpolation: example/02_hyperbolic_05_burgers_adapt.cpp statement by statement, as that
// driver runs without artificial viscosity (viscosity_option 0: the SSP-RK3 branch), running on the
// GPU through amdg_dg.hpp -- the same statics, DGAdapt with init_separable_scalar_sum of
// sin(2 pi (x + y)), HermInterpolation + FastHermIntp built once before the loop,
// HyperbolicSameFluxHermRHS, the Lax-Friedrichs matrix assembled by HyperbolicAlpt::
// assemble_matrix_flx_scalar and added by add_rhs_matrix, ForwardEuler predictor, refine, RK3SSP
// stage by stage, coarsen.  The artificial-viscosity and IMEX branches and the profile output are
// left out.
//
//   burgers_herm_adapt [N_init] [NMAX] [final_time] [refine_eps] [coarsen_eta] [max_steps] [output]
// max_steps (not in the reference driver) stops the loop after that many steps; output (optional):
// one line per element, "level... suppt... coefficients..." (%.17g)
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>

#include "amdg_dg.hpp"

using namespace amdg_gpu;

int main(int argc, char* argv[]) {
    // constant variable
    const int DIM = 2;

    // static variables
    AlptBasis::PMAX = 2;

    LagrBasis::PMAX = 3;
    LagrBasis::msh_case = 1;

    HermBasis::PMAX = 3;
    HermBasis::msh_case = 1;

    Element::PMAX_alpt = AlptBasis::PMAX;
    Element::PMAX_intp = HermBasis::PMAX;
    Element::DIM = DIM;
    Element::VEC_NUM = 1;

    DGSolution::DIM = Element::DIM;
    DGSolution::VEC_NUM = Element::VEC_NUM;

    DGSolution::ind_var_vec = {0};
    DGAdapt::indicator_var_adapt = {0};

    Element::is_intp.resize(Element::VEC_NUM);
    for (size_t num = 0; num < size_t(Element::VEC_NUM); num++) Element::is_intp[num] = std::vector<bool>(Element::DIM, true);

    Interpolation::DIM = DGSolution::DIM;
    Interpolation::VEC_NUM = DGSolution::VEC_NUM;

    // computation parameters (the reference's defaults, overridable from the command line)
    int N_init = argc > 1 ? std::atoi(argv[1]) : 3;
    int NMAX = argc > 2 ? std::atoi(argv[2]) : 3;
    double final_time = argc > 3 ? std::atof(argv[3]) : 0.03;
    double refine_eps = argc > 4 ? std::atof(argv[4]) : 1e-2;
    double coarsen_eta = argc > 5 ? std::atof(argv[5]) : refine_eps / 10.;
    const int max_steps = argc > 6 ? std::atoi(argv[6]) : 1 << 30;
    const std::string output = argc > 7 ? argv[7] : "";
    const bool sparse = true;
    const double cfl_hyper = 0.2;  // cfl number when no shock, 0.2 for P2
    const std::string boundary_type = "period";
    const bool is_adapt_find_ptr_alpt = true;
    const bool is_adapt_find_ptr_intp = true;
    if (N_init > NMAX) {
        std::printf("Mesh level in initialization should not be larger than Maximum mesh level\n");
        return 1;
    }

    // initialize hash key
    Hash hash;

    // initialize interpolation points for Lagrange and Hermite interpolation basis
    LagrBasis::set_interp_msh01();
    HermBasis::set_interp_msh01();

    // initialize all basis functions in 1D for Alpert, Lagrange and Hermite basis
    AllBasis<LagrBasis> all_bas_lagr(NMAX);
    AllBasis<HermBasis> all_bas_herm(NMAX);
    AllBasis<AlptBasis> all_bas_alpt(NMAX);

    // operator matrix in 1D
    OperatorMatrix1D<AlptBasis, AlptBasis> oper_matx_alpt(all_bas_alpt, all_bas_alpt, boundary_type);
    OperatorMatrix1D<HermBasis, AlptBasis> oper_matx_herm(all_bas_herm, all_bas_alpt, boundary_type);

    // initialization of DG solution
    DGAdapt dg_solu(sparse, N_init, NMAX, all_bas_alpt, all_bas_lagr, all_bas_herm, hash, refine_eps, coarsen_eta,
                    is_adapt_find_ptr_alpt, is_adapt_find_ptr_intp);

    // project initial function into numerical solution
    // f(x,y) = sin(2*pi*(x+y)) = sin(2*pi*x) * cos(2*pi*y) + cos(2*pi*x) * sin(2*pi*y)
    auto init_func_1 = [](double x, int d) { return (d == 0) ? (std::sin(2. * M_PI * x)) : (std::cos(2. * M_PI * x)); };
    auto init_func_2 = [](double x, int d) { return (d == 0) ? (std::cos(2. * M_PI * x)) : (std::sin(2. * M_PI * x)); };
    std::vector<std::function<double(double, int)>> init_func{init_func_1, init_func_2};
    dg_solu.init_separable_scalar_sum(init_func);

    // physical flux and its first and second derivatives
    auto func_flux = [&](std::vector<double> u, int, int) -> double { return FluxFunction::burgers_flux_scalar(u[0]); };
    auto func_flux_d1 = [&](std::vector<double> u, int, int, int) -> double {
        return FluxFunction::burgers_flux_1st_derivative_scalar(u[0]);
    };
    auto func_flux_d2 = [&](std::vector<double> u, int, int, int, int) -> double {
        return FluxFunction::burgers_flux_2nd_derivative_scalar(u[0]);
    };

    // third and fourth derivatives of the physical flux (used by the PMAX 5 variant)
    auto func_flux_d3 = [&](std::vector<double> u, int i, int d, int i1, int i2, int i3) -> double { return 0.; };
    auto func_flux_d4 = [&](std::vector<double> u, int i, int d, int i1, int i2, int i3, int i4) -> double { return 0.; };

    // Hermite interpolation for the nonlinear physical flux
    HyperbolicSameFluxHermRHS fast_rhs_herm(dg_solu, oper_matx_herm);
    HermInterpolation interp_herm(dg_solu);

    // Burgers' equation has the same flux in x and y, so it is interpolated in x only
    std::vector<std::vector<bool>> is_intp_herm;
    is_intp_herm.push_back(std::vector<bool>{true, false});

    // fast hermite interpolation
    FastHermIntp fast_herm_intp(dg_solu, interp_herm.Her_pt_Alpt_1D);

    // constant in global Lax-Friedrich flux
    const std::vector<double> lxf_alpha{1.2, 1.2};
    // wave speed in x and y direction
    const std::vector<double> wave_speed{1., 1.};

    // begin time evolution
    const auto t0 = std::chrono::steady_clock::now();
    double curr_time = 0.;
    int num_time_step = 0;
    while (curr_time < final_time && num_time_step < max_steps) {
        // --- part 1: calculate time step dt ---
        const std::vector<int>& max_mesh = dg_solu.max_mesh_level_vec();

        // dt = cfl/(c1/dx1 + c2/dx2 + ... + c_dim/dx_dim)
        double sum_c_dx = 0.;
        for (size_t d = 0; d < size_t(DIM); d++) sum_c_dx += std::abs(wave_speed[d]) * std::pow(2., max_mesh[d]);
        double dt = cfl_hyper / sum_c_dx;
        dt = std::min(dt, final_time - curr_time);

        // --- part 2: predict by Euler forward
        {
            // before Euler forward, copy Element::ucoe_alpt to Element::ucoe_alpt_predict
            dg_solu.copy_ucoe_to_predict();

            HyperbolicAlpt linear(dg_solu, oper_matx_alpt);
            linear.assemble_matrix_flx_scalar(0, -1, lxf_alpha[0] / 2);
            linear.assemble_matrix_flx_scalar(0, 1, -lxf_alpha[0] / 2);
            linear.assemble_matrix_flx_scalar(1, -1, lxf_alpha[1] / 2);
            linear.assemble_matrix_flx_scalar(1, 1, -lxf_alpha[1] / 2);

            ForwardEuler odeSolver(linear, dt);
            odeSolver.init();

            // Hermite interpolation
            if (HermBasis::PMAX == 3) {
                interp_herm.nonlinear_Herm_2D_fast(func_flux, func_flux_d1, func_flux_d2, is_intp_herm, fast_herm_intp);
            } else if (HermBasis::PMAX == 5) {
                interp_herm.nonlinear_Herm_2D_PMAX5_scalar_fast(func_flux, func_flux_d1, func_flux_d2, func_flux_d3,
                                                                func_flux_d4, is_intp_herm, fast_herm_intp);
            }

            // calculate rhs
            dg_solu.set_rhs_zero();

            fast_rhs_herm.rhs_vol_scalar();
            fast_rhs_herm.rhs_flx_intp_scalar();

            odeSolver.set_rhs_zero();
            odeSolver.add_rhs_to_eigenvec();
            odeSolver.add_rhs_matrix(linear);

            // Euler forward time stepping
            odeSolver.step_stage(0);

            // the prediction of the solution at t^(n+1) is now the solution
            odeSolver.final();
        }

        // --- part 3: refine based on the prediction
        dg_solu.refine();

        // after refine, copy Element::ucoe_alpt_predict back to Element::ucoe_alpt
        dg_solu.copy_predict_to_ucoe();

        // --- part 4: time evolution
        HyperbolicAlpt linear(dg_solu, oper_matx_alpt);
        linear.assemble_matrix_flx_scalar(0, -1, lxf_alpha[0] / 2);
        linear.assemble_matrix_flx_scalar(0, 1, -lxf_alpha[0] / 2);
        linear.assemble_matrix_flx_scalar(1, -1, lxf_alpha[1] / 2);
        linear.assemble_matrix_flx_scalar(1, 1, -lxf_alpha[1] / 2);

        RK3SSP odeSolver(linear, dt);
        odeSolver.init();

        for (int stage = 0; stage < odeSolver.num_stage; ++stage) {
            // Hermite interpolation
            if (HermBasis::PMAX == 3) {
                interp_herm.nonlinear_Herm_2D_fast(func_flux, func_flux_d1, func_flux_d2, is_intp_herm, fast_herm_intp);
            } else if (HermBasis::PMAX == 5) {
                interp_herm.nonlinear_Herm_2D_PMAX5_scalar_fast(func_flux, func_flux_d1, func_flux_d2, func_flux_d3,
                                                                func_flux_d4, is_intp_herm, fast_herm_intp);
            }

            // calculate rhs and update Element::ucoe_alpt
            dg_solu.set_rhs_zero();

            fast_rhs_herm.rhs_vol_scalar();
            fast_rhs_herm.rhs_flx_intp_scalar();

            // add to rhs in odeSolver
            odeSolver.set_rhs_zero();
            odeSolver.add_rhs_to_eigenvec();
            odeSolver.add_rhs_matrix(linear);

            odeSolver.step_stage(stage);

            odeSolver.final();
        }

        // --- part 5: coarsen
        dg_solu.coarsen();

        // add current time and increase time steps
        curr_time += dt;
        num_time_step++;
    }
    synchronize();
    const double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::printf("steps %d time %.17g elements %d dof %d seconds %.6f\n", num_time_step, curr_time, dg_solu.size_elem(),
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
