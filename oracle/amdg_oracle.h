/*
 * CPU oracle for the adaptive sparse-grid DG right-hand side: a plain C
 * restatement of the reference algorithm (AdaM-DG), used ONLY as test
 * infrastructure -- the checker in tests/, smoke() and the cpu_baseline leg of
 * bench.py.  Nothing in the product library links or calls it.
 *
 * Conventions (shared with the reference):
 *   - 1D element (level n, suppt j): n = 0..N, j odd; n<=1 -> support [0,1],
 *     n>=2 -> [2^(1-n) (j-1)/2, 2^(1-n) (j+1)/2].  1D element order
 *     o(n,j) = 0 for n=0, else 2^(n-1) + (j-1)/2  (Element.cpp:386-389).
 *   - 1D basis order = o * (k+1) + p  (AllBasis.h:81-84).
 *   - Per-element coefficient block: (k+1)^dim doubles, row-major over dims,
 *     last dimension fastest (VecMultiD.h:114-116).
 *   - 1D operator matrices are stored row = solution basis, col = test basis,
 *     as OperatorMatrix1D::u_vx.at(row_idx, col_idx) (OperatorMatrix1D.h:166-199).
 */
#ifndef AMDG_ORACLE_H
#define AMDG_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef double (*amdg_oracle_fn1d)(double x, int d, int term, void* user);

/* Alpert basis value (or derivative) at x, limit sgn in {-1,0,1}. */
double amdg_oracle_alpert_val(int k, int level, int suppt, int p, int deriv, double x, int sgn);

/* Gauss-Legendre rule on [-1,1] (n <= 16 points). */
int amdg_oracle_gauss_legendre(int n, double* x, double* w);

/* 1D operator matrices, each (2^N (k+1))^2, row = solution basis, col = test basis.
 * Any pointer may be NULL. */
int amdg_oracle_oper1d(int N, int k, double* u_v, double* u_vx, double* ulft_vjp, double* urgt_vjp);

/* Number of elements of the sparse (sum of levels <= N) or full grid. */
int64_t amdg_oracle_grid_count(int dim, int N, int sparse);
/* Elements in lexicographic order of (order_0,...,order_{dim-1}); level/suppt are E x dim. */
int64_t amdg_oracle_grid(int dim, int N, int sparse, int32_t* level, int32_t* suppt);

/* 1D projections onto all Alpert basis functions (Basis::product_function):
 * out[term][d][basis] for nterms separable terms. */
int amdg_oracle_project_separable(int N, int k, int dim, int nterms, amdg_oracle_fn1d f, void* user, double* out);

/* Expand separable 1D projections into element coefficients: u[e][q] = sum_term prod_d coef. */
int amdg_oracle_init_separable(int dim, int N, int k, int64_t E, const int32_t* level, const int32_t* suppt,
                               int nterms, const double* coef1d, double* u);

/* Linear constant-coefficient operator (HyperbolicAlpt::assemble_matrix_scalar, upwind flux),
 * rhs = L u.  c has dim entries. nthreads <= 0 -> OpenMP default. */
int amdg_oracle_linear_rhs(int dim, int N, int k, int64_t E, const int32_t* level, const int32_t* suppt,
                           const double* c, const double* u, double* rhs, int nthreads);

/* SSP-RK3 steps of the linear operator, in place on u (RK3SSP::step_rk). */
int amdg_oracle_linear_rk3(int dim, int N, int k, int64_t E, const int32_t* level, const int32_t* suppt,
                           const double* c, double dt, int steps, double* u, int nthreads);

/* One linear RHS evaluation restricted to the test elements [e_begin, e_end) (timing samples). */
int amdg_oracle_linear_rhs_range(int dim, int N, int k, int64_t E, const int32_t* level, const int32_t* suppt,
                                 const double* c, const double* u, double* rhs, int64_t e_begin, int64_t e_end,
                                 int nthreads);

/* Operator handle for repeated evaluations (level/suppt must outlive it). */
void* amdg_oracle_linop_create(int dim, int N, int k, int64_t E, const int32_t* level, const int32_t* suppt,
                               const double* c);
int amdg_oracle_linop_apply_range(void* handle, const double* u, double* rhs, int64_t e_begin, int64_t e_end, int nthreads);
void amdg_oracle_linop_destroy(void* handle);

/* L2 error against a separable exact solution (DGSolution::get_L2_error_split_separable_scalar). */
double amdg_oracle_l2_error_split(int dim, int N, int k, int64_t E, const int32_t* level, const int32_t* suppt,
                                  const double* u, const double* coef1d_exact, double l2_norm_exact);

/* ---- Lagrange interpolation path (degree-3 hierarchical Lagrange, msh_case 1) ---- */
/* Lagrange interpolation degree of the calls that follow: 3 (node layout msh_case 1,
 * the default) or 4 (msh_case 2); -1 for anything else */
int amdg_oracle_set_lagr_degree(int degree);
int amdg_oracle_lagr_points_per_dim(void);
double amdg_oracle_lagr_val(int level, int suppt, int p, double x, int sgn);
double amdg_oracle_lagr_point(int level, int suppt, int p);
/* Lagrange (rows) x Alpert (cols) 1D matrices: u_v, u_vx, ulft_vjp + urgt_vjp. */
int amdg_oracle_oper1d_lagr(int N, int k, double* u_v, double* u_vx, double* uave2_vjp);
/* u_h at every interpolation point (E x 4^dim). */
int amdg_oracle_lagr_point_values(int dim, int N, int k, int64_t E, const int32_t* level, const int32_t* suppt,
                                  const double* u, double* up);
/* Hierarchical surplus of point values (E x 4^dim). */
int amdg_oracle_lagr_surplus(int dim, int N, int64_t E, const int32_t* level, const int32_t* suppt, const double* fp,
                             double* out);
/* Alpert coefficients (E x (k+1)^dim) of the Lagrange interpolant with coefficients coe
 * (E x p1^dim) by the fast transforms with u_v (Lagrange x Alpert) in every dimension. */
int amdg_oracle_lagr_to_alpert_fast(int dim, int N, int k, int64_t E, const int32_t* level, const int32_t* suppt,
                                    const double* coe, double* out);
/* Burgers right-hand side from flux interpolation coefficients (dim x E x 4^dim) and u. */
int amdg_oracle_burgers_rhs(int dim, int N, int k, int64_t E, const int32_t* level, const int32_t* suppt,
                            const double* fucoe, const double* u, double alpha, double* rhs);

/* The same two quantities by the reference's fast L/U partial-sum transforms
 * (the reference's operator on adaptive grids; equal to the direct sums on
 * sparse grids). */
int amdg_oracle_lagr_point_values_fast(int dim, int N, int k, int64_t E, const int32_t* level, const int32_t* suppt,
                                       const double* u, double* up);
int amdg_oracle_burgers_rhs_fast(int dim, int N, int k, int64_t E, const int32_t* level, const int32_t* suppt,
                                 const double* fucoe, const double* u, double alpha, double* rhs);

/* ---- point values and quadrature errors ---- */
/* DGSolution::val (DGSolution.cpp:613-625, Element::val Element.cpp:123-147): the sum over
 * the elements whose closed support contains x.  x is npts x dim. */
int amdg_oracle_eval_points(int dim, int N, int k, int64_t E, const int32_t* level, const int32_t* suppt,
                            const double* u, int64_t npts, const double* x, double* out);
/* BurgersExact::norm_1d (ExactSolution.cpp:8-66): v(x, t) with v = sin(2 pi (x - v t)); NaN when
 * Newton's iteration does not converge within 10 steps (the reference exits there). */
double amdg_oracle_burgers_wave(double x, double t);
/* a + b v(X - a T + c, b T) with X = sum_d x_d, T = dim t (BurgersExact::exact_1d, ExactSolution.cpp:68-71) */
double amdg_oracle_burgers_exact(int dim, const double* x, double a, double b, double c, double t);
/* L1, L2, Linf of u_h - u_exact by `gauss` Gauss-Legendre points per dimension on the uniform
 * mesh of the finest element level (DGSolution::get_error_no_separable_scalar, DGSolution.cpp:326-335;
 * Quad::norm_multiD, Quad.cpp:261-318). */
int amdg_oracle_error_burgers(int dim, int N, int k, int64_t E, const int32_t* level, const int32_t* suppt,
                              const double* u, int gauss, double a, double b, double c, double t, double* err3);

/* ---- wave equation u_tt = div(K grad u), K = (1 + a prod_d sin(2 pi x_d))^2 ---- */
/* Lagrange x Alpert ujp_vxlft + ujp_vxrgt, (2^N*4) x (2^N*(k+1)). */
int amdg_oracle_oper1d_lagr_ujp_vx(int N, int k, double* ujp_vxave);
double amdg_oracle_wave_coef(int dim, const double* x, double amp);
/* right-hand side of the semi-discrete wave equation (fast transforms), rhs = E x (k+1)^dim */
int amdg_oracle_wave_rhs_fast(int dim, int N, int k, int64_t E, const int32_t* level, const int32_t* suppt,
                              const double* u, double sigma, double amp, double* rhs);
/* the IPDG term alone (the adaptive wave loop's predictor right-hand side) */
int amdg_oracle_wave_penalty(int dim, int N, int k, int64_t E, const int32_t* level, const int32_t* suppt,
                             const double* u, double sigma, double* rhs);

/* ---- cubic Hermite interpolation of the flux (2D Burgers, 02_hyperbolic_05_burgers_adapt.cpp) ---- */
/* dof p of a 1D Hermite element: point p % 2, derivative order p / 2 */
double amdg_oracle_herm_val(int level, int suppt, int p, int deriv, double x, int sgn);
double amdg_oracle_herm_point(int level, int suppt, int p);
/* Hermite (2^N*4 rows) x Alpert (2^N*(k+1) cols): u_v, u_vx, ulft_vjp + urgt_vjp (any may be NULL) */
int amdg_oracle_oper1d_herm(int N, int k, double* u_v, double* u_vx, double* uave2_vjp);
/* u_h and its derivatives at the Hermite points, E x 4^dim: direct sums and fast transforms */
int amdg_oracle_herm_point_values(int dim, int N, int k, int64_t E, const int32_t* level, const int32_t* suppt,
                                  const double* u, double* up);
int amdg_oracle_herm_point_values_fast(int dim, int N, int k, int64_t E, const int32_t* level, const int32_t* suppt,
                                       const double* u, double* up);
/* f = u^2/2 and its derivatives at the 2D Hermite points from up (E x 16) */
int amdg_oracle_herm_flux_burgers2d(int64_t E, const double* up, double* fp);
/* hierarchical Hermite surplus of point data fp (E x 4^dim) */
int amdg_oracle_herm_surplus(int dim, int N, int64_t E, const int32_t* level, const int32_t* suppt, const double* fp,
                             double* out);
/* Burgers right-hand side from the flux's Hermite coefficients (fast transforms) plus the LxF penalty */
int amdg_oracle_burgers_herm_rhs_fast(int dim, int N, int k, int64_t E, const int32_t* level, const int32_t* suppt,
                                      const double* fucoe, const double* u, double alpha, double* rhs);

#ifdef __cplusplus
}
#endif
#endif
