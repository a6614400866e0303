// Constant-coefficient scalar hyperbolic equation u_t + sum_d u_{x_d} = 0 on the periodic unit
// square, written like the reference driver example/02_hyperbolic_01_scalar_const_coefficient.cpp
// and running on the GPU through amdg_dg.hpp: the same statics (Alpert degree 2, Lagrange degree 5
// with the msh_case 1 nodes), the non-separable initial value cos(2 pi sum_d x_d) by adaptive
// interpolation (DGAdaptIntp::init_adaptive_intp, no refinement: refine_eps = 1e10), SSP-RK3 with
// dt = dx cfl / DIM rounded to land on the final time, and the error against the exact solution
// interpolated adaptively (refine_eps 1e-6) through get_L2_error_split_adaptive_intp_scalar.
//
//   hyperbolic_const_coefficient_intp [NMAX] [final_time]
#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "amdg_dg.hpp"

using namespace amdg_gpu;

int main(int argc, char* argv[]) {
    const int DIM = 2;
    AlptBasis::PMAX = 2;
    LagrBasis::PMAX = 5;
    LagrBasis::msh_case = 1;
    HermBasis::PMAX = 3;
    HermBasis::msh_case = 1;
    Element::PMAX_alpt = AlptBasis::PMAX;
    Element::PMAX_intp = LagrBasis::PMAX;
    Element::DIM = DIM;
    Element::VEC_NUM = 1;
    DGSolution::DIM = Element::DIM;
    DGSolution::VEC_NUM = Element::VEC_NUM;
    DGSolution::ind_var_vec = {0};
    DGAdapt::indicator_var_adapt = {0};

    const int NMAX = argc > 1 ? std::atoi(argv[1]) : 4;
    const double final_time = argc > 2 ? std::atof(argv[2]) : 0.1;
    const int N_init = NMAX;
    const bool sparse = true;
    const double cfl = 0.1;
    const double refine_eps = 1e10, coarsen_eta = -1;
    const double PI = 3.14159265358979323846;

    Hash hash;
    LagrBasis::set_interp_msh01();
    HermBasis::set_interp_msh01();
    AllBasis<AlptBasis> all_bas_alpt(NMAX);
    AllBasis<LagrBasis> all_bas_lagr(NMAX);
    AllBasis<HermBasis> all_bas_herm(NMAX);
    OperatorMatrix1D<AlptBasis, AlptBasis> oper_matx(all_bas_alpt, all_bas_alpt, "period");
    OperatorMatrix1D<HermBasis, HermBasis> oper_matx_herm_herm(all_bas_herm, all_bas_herm, "period");
    OperatorMatrix1D<LagrBasis, LagrBasis> oper_matx_lagr_lagr(all_bas_lagr, all_bas_lagr, "period");

    DGAdaptIntp dg_solu(sparse, N_init, NMAX, all_bas_alpt, all_bas_lagr, all_bas_herm, hash, refine_eps, coarsen_eta,
                        true, false, oper_matx_lagr_lagr, oper_matx_herm_herm);
    auto init_func = [=](std::vector<double> x, int) {
        double sum_x = 0.;
        for (int d = 0; d < DIM; d++) sum_x += x[d];
        return std::cos(2 * PI * sum_x);
    };
    dg_solu.init_adaptive_intp(init_func);

    const std::vector<double> hyperbolicConst(DIM, 1.);
    const int max_mesh = dg_solu.max_mesh_level();
    const double dx = 1. / std::pow(2., max_mesh);
    double dt = dx * cfl / DIM;
    const int total_time_step = int(std::ceil(final_time / dt)) + 1;
    dt = final_time / total_time_step;

    HyperbolicAlpt dg_operator(dg_solu, oper_matx);
    dg_operator.assemble_matrix_scalar(hyperbolicConst);
    RK3SSP odesolver(dg_operator, dt);
    odesolver.init();
    for (int step = 0; step < total_time_step; ++step) odesolver.step_rk();
    odesolver.final();
    synchronize();

    DGAdaptIntp dg_solu_ext(sparse, N_init, NMAX, all_bas_alpt, all_bas_lagr, all_bas_herm, hash, 1e-6, -1, true, false,
                            oper_matx_lagr_lagr, oper_matx_herm_herm);
    auto final_func = [=](std::vector<double> x, int) {
        double sum_x = 0.;
        for (int d = 0; d < DIM; d++) sum_x += x[d];
        return std::cos(2. * PI * (sum_x - DIM * final_time));
    };
    dg_solu_ext.init_adaptive_intp(final_func);
    const double err_l2 = dg_solu_ext.get_L2_error_split_adaptive_intp_scalar(dg_solu);
    std::printf("elements %d dof %d steps %d dt %.17g elements_ext %d\n", dg_solu.size_elem(), dg_solu.get_dof(),
                total_time_step, dt, dg_solu_ext.size_elem());
    std::printf("L2 error at final time: %.17g\n", err_l2);
    return 0;
}
