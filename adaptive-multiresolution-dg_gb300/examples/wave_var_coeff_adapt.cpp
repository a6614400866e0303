// Variable-coefficient wave equation u_tt = div(K grad u) on the periodic unit square with
// adaptivity, written like the reference driver example/03_wave_06_var_coeff_adapt.cpp but
// running on the GPU through amdg_dg.hpp: same statics (Alpert degree 2, Lagrange degree 4 with
// the msh_case 2 nodes), DGAdapt with a coarse start level, the Gaussian bump
// exp(-200 |x - (0.3, 0.4)|^2) at rest, IPDG sigma = 10, and the time loop of predictor, refine,
// RK4ODE2nd and coarsen (one WaveLagrRHS::adaptive_step per step; no source term).
//
//   wave_var_coeff_adapt [N_init] [NMAX] [steps] [refine_eps] [coarsen_eta]
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

    Hash hash;
    LagrBasis::set_interp_msh01();
    HermBasis::set_interp_msh01();
    AllBasis<LagrBasis> all_bas_lagr(NMAX);
    AllBasis<HermBasis> all_bas_herm(NMAX);
    AllBasis<AlptBasis> all_bas_alpt(NMAX);

    DGAdapt dg_solu(sparse, N_init, NMAX, all_bas_alpt, all_bas_lagr, all_bas_herm, hash, refine_eps, coarsen_eta,
                    true, false);
    // u(0) the Gaussian bump, u_t(0) = 0
    const double centre[2] = {0.3, 0.4};
    dg_solu.init_separable_scalar([&](double x, int d) { return std::exp(-200.0 * (x - centre[d]) * (x - centre[d])); });
    WaveLagrRHS wave(dg_solu, sigma_ipdg);

    double curr_time = 0.0;
    for (int num_time_step = 0; num_time_step < steps; ++num_time_step)
        curr_time += wave.adaptive_step(cfl, 1.0, refine_eps, coarsen_eta);
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
