// Constant-coefficient scalar hyperbolic equation on a sparse grid with
// periodic boundary conditions, written like the reference driver
// example/02_hyperbolic_01_scalar_const_coefficient.cpp but running on the
// GPU through amdg_dg.hpp.  Same statics, same object construction order,
// same time loop; the initial condition is the separable sum of
// sin(2 pi sum_d x_d) (init_separable_scalar_sum) so the error is computed
// with the split separable formula.
//
//   hyperbolic_const_coefficient [N] [final_time] [mixed]
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "amdg_dg.hpp"

using namespace amdg_gpu;

int main(int argc, char* argv[]) {
    const int DIM = 2;
    AlptBasis::PMAX = 2;
    LagrBasis::PMAX = 3;
    LagrBasis::msh_case = 1;
    Element::PMAX_alpt = AlptBasis::PMAX;
    Element::DIM = DIM;
    Element::VEC_NUM = 1;
    DGSolution::DIM = Element::DIM;
    DGSolution::VEC_NUM = Element::VEC_NUM;
    DGSolution::ind_var_vec = {0};
    DGAdapt::indicator_var_adapt = {0};

    int NMAX = argc > 1 ? std::atoi(argv[1]) : 7;
    double final_time = argc > 2 ? std::atof(argv[2]) : 0.1;
    const bool mixed = argc > 3 && std::strcmp(argv[3], "mixed") == 0;
    const double cfl = 0.1;
    const double PI = 3.14159265358979323846;

    Hash hash;
    LagrBasis::set_interp_msh01();
    HermBasis::set_interp_msh01();
    AllBasis<AlptBasis> all_bas_alpt(NMAX);
    AllBasis<LagrBasis> all_bas_lagr(NMAX);
    AllBasis<HermBasis> all_bas_herm(NMAX);
    OperatorMatrix1D<AlptBasis, AlptBasis> oper_matx(all_bas_alpt, all_bas_alpt, "period");

    DGAdapt dg_solu(true, NMAX, NMAX, all_bas_alpt, all_bas_lagr, all_bas_herm, hash, 1e10, -1, true, false);
    auto f1 = [=](double x, int d) { return d == 0 ? std::sin(2 * PI * x) : std::cos(2 * PI * x); };
    auto f2 = [=](double x, int d) { return d == 0 ? std::cos(2 * PI * x) : std::sin(2 * PI * x); };
    dg_solu.init_separable_scalar_sum({f1, f2});

    const std::vector<double> hyperbolicConst(DIM, 1.);
    const int max_mesh = dg_solu.max_mesh_level();
    const double dx = 1. / std::pow(2., max_mesh);
    double dt = dx * cfl / DIM;
    const int total_time_step = int(std::ceil(final_time / dt)) + 1;
    dt = final_time / total_time_step;

    HyperbolicAlpt dg_operator(dg_solu, oper_matx);
    dg_operator.assemble_matrix_scalar(hyperbolicConst);
    RK3SSP odesolver(dg_operator, dt, mixed ? AMDG_PREC_MIXED : AMDG_PREC_FP64);
    odesolver.init();
    for (int step = 0; step < total_time_step; ++step) odesolver.step_rk();
    odesolver.final();
    synchronize();

    // exact solution sin(2 pi (x + y - 2t)), compared term by term through the
    // separable split formula: |u - u_h|^2 = |u|^2 + sum(u_h^2 - 2 u u_h) with
    // u = sin(a)cos(b) + cos(a)sin(b); the cross term is linear in u so it is
    // summed over the two separable terms.
    const double T = final_time;
    auto e1 = [=](double x, int d) { return d == 0 ? std::sin(2 * PI * (x - 2 * T)) : std::cos(2 * PI * x); };
    auto e2 = [=](double x, int d) { return d == 0 ? std::cos(2 * PI * (x - 2 * T)) : std::sin(2 * PI * x); };
    const double n2 = dg_solu.get_L2_norm()[0];
    // with a reference norm of 1 the split formula stays positive:
    // a^2 = 1 + n2 - 2<u_h,e1>, b^2 = 1 + n2 - 2<u_h,e2>; |u|^2 = 1/2 over the unit square
    const double a = dg_solu.get_L2_error_split_separable_scalar(e1, 1.0);
    const double b = dg_solu.get_L2_error_split_separable_scalar(e2, 1.0);
    const double cross = 0.5 * ((1.0 + n2 - a * a) + (1.0 + n2 - b * b));
    const double err = std::sqrt(std::max(0.0, 0.5 + n2 - 2.0 * cross));
    std::printf("elements %d dof %d steps %d dt %.17g\n", dg_solu.size_elem(), dg_solu.get_dof(), total_time_step, dt);
    std::printf("L2 error at final time: %.17g\n", err);
    return 0;
}
