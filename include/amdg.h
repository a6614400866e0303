/*
 * amdg.h -- C-ABI of the GB300-native adaptive sparse-grid DG right-hand-side
 * library (libamdg_gb300.so).
 *
 * Plain C types only: opaque handles, pointers and sizes.  Every call returns
 * an amdg_status; no C++ exception crosses this boundary.  The caller owns
 * host buffers; the library owns device memory.  A context and the handles
 * created from it are not thread-safe: use one host thread per context.
 *
 * Each entry point names the AdaM-DG reference interface it replaces
 * (file:line in the reference tree).
 *
 * Data layout shared by every call:
 *   - element e of a grid has a level and a support index per dimension
 *     (Element::level / Element::suppt, Element.h:24-25); elements are kept
 *     sorted by their per-dimension 1D element orders o_d = 0 for level 0,
 *     2^(n-1) + (j-1)/2 otherwise (Element.cpp:386-389), first dimension most
 *     significant;
 *   - the coefficient block of an element holds (k+1)^dim doubles, row-major
 *     over dimensions, last dimension fastest (VecMultiD.h:114-116), i.e. the
 *     layout of Element::ucoe_alpt[0];
 *   - a grid's coefficient vector is the concatenation of its element blocks
 *     in element order (num_elements * (k+1)^dim doubles).
 */
#ifndef AMDG_H
#define AMDG_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AMDG_ABI_VERSION 6

typedef enum amdg_status {
    AMDG_OK = 0,
    AMDG_ERR_ARG = 1,       /* invalid argument (bad size, null pointer, unsupported degree/dimension) */
    AMDG_ERR_CAPACITY = 2,  /* a size exceeds what the handle was built for */
    AMDG_ERR_NONFINITE = 3, /* a reduction met NaN or Inf */
    AMDG_ERR_TIMEOUT = 4,   /* a bounded device-side wait gave up */
    AMDG_ERR_CUDA = 5,      /* a CUDA runtime call failed (see amdg_last_error) */
    AMDG_ERR_STATE = 6,     /* call out of order (e.g. state not initialised) */
    AMDG_ERR_NOMEM = 7,     /* device or host allocation failed */
    AMDG_ERR_IO = 8,        /* a file could not be opened, read or written */
    AMDG_ERR_FORMAT = 9     /* a file is not a valid checkpoint (magic, version, range, checksum) */
} amdg_status;

/* Arithmetic of the operator applies.  The state and the RK stage
 * accumulation stay FP64 in both modes. */
typedef enum amdg_precision {
    AMDG_PREC_FP64 = 0,  /* plain FP64 everywhere */
    AMDG_PREC_MIXED = 1  /* operator blocks and products in FP32, FP32 accumulation */
} amdg_precision;

typedef struct amdg_context amdg_context;
typedef struct amdg_grid amdg_grid;
typedef struct amdg_linear_op amdg_linear_op;
typedef struct amdg_burgers_op amdg_burgers_op;
typedef struct amdg_batch amdg_batch;
typedef struct amdg_mlp amdg_mlp;
typedef struct amdg_wave_op amdg_wave_op;

/* Separable 1D factor g_d(x) of term `term` (the std::function<double(double,int)>
 * the reference takes, DGAdapt.h:17-38). */
typedef double (*amdg_fn1d)(double x, int d, int term, void* user);
/* The same factor at n points at once: out[i] = g_d(x[i]) for term `term` (one call per
 * dimension and term, for callers whose functions are cheap to evaluate in bulk). */
typedef void (*amdg_fn1d_batch)(const double* x, int64_t n, int d, int term, double* out, void* user);
/* A function of the point at n points at once: out[i] = f(x[i*dim], ..., x[i*dim + dim - 1]) (the
 * std::function<double(std::vector<double>, int)> of DGAdaptIntp::init_adaptive_intp,
 * DGAdaptIntp.h:33-50, for one unknown). */
typedef void (*amdg_fn_points)(const double* x, int64_t n, int dim, double* out, void* user);

/* ---- library / context ------------------------------------------------- */
int amdg_abi_version(void);
const char* amdg_status_string(amdg_status s);
/* Message of the last failing call on this host thread ("" if none). */
const char* amdg_last_error(void);

/* Binds a CUDA device and creates the library's stream.  No reference
 * counterpart: the reference is single-process CPU code. */
amdg_status amdg_context_create(int device, amdg_context** out);
amdg_status amdg_context_destroy(amdg_context* ctx);
/* Run all later work of this context on an existing cudaStream_t (NULL = the
 * context's own stream). */
amdg_status amdg_context_set_stream(amdg_context* ctx, void* cuda_stream);
amdg_status amdg_context_get_stream(amdg_context* ctx, void** cuda_stream);
amdg_status amdg_context_synchronize(amdg_context* ctx);
/* Number of kernels this context has launched so far. */
amdg_status amdg_context_launch_count(amdg_context* ctx, int64_t* count);

/* Host phase profile (no counterpart in the reference): wall time spent in the
 * library's host phases, including the waits on the stream they contain. */
enum {
    AMDG_PHASE_TOPOLOGY = 0,   /* neighbour lists / ancestors rebuilt for a new element set, uploads */
    AMDG_PHASE_SET_KEYS = 1,   /* element set replaced, coefficients carried over */
    AMDG_PHASE_NORMS = 2,      /* element indicator norms computed and read back */
    AMDG_PHASE_ADAPT_HOST = 3, /* refine / coarsen / hole filling on the host key set */
    AMDG_PHASE_RHS = 4,        /* Burgers right-hand sides enqueued */
    AMDG_PHASE_RK3 = 5,        /* Burgers SSP-RK3 steps enqueued (graph capture included) */
    AMDG_PHASE_CLASSIFIER = 6, /* learned refine/coarsen: features, network, probabilities read back */
    AMDG_PHASE_ADAPT_STEP = 7, /* whole adaptive steps (plain or learned) */
    AMDG_PHASE_ADAPT_DEVICE = 8, /* refine / coarsen on the device, including the one wait for the new element count */
    AMDG_PHASE_COUNT = 9
};
/* enable != 0 starts (and resets) the profile, 0 stops it. */
amdg_status amdg_context_profile(amdg_context* ctx, int enable);

/* Where the element set changes of this context's grids run (no reference counterpart; the
 * reference's DGAdapt::refine / coarsen and DGSolution::find_ptr_* are host code):
 * AMDG_ADAPT_DEVICE (default) -- refine, coarsen, hole filling and the fast transforms' neighbour
 * lists and surplus ancestors are computed on the device from the sorted element keys, with one
 * stream synchronisation per change (the new element count); AMDG_ADAPT_HOST -- the same on
 * the host key set, uploaded after every change.  Both give the same element sets and lists. */
enum { AMDG_ADAPT_DEVICE = 0, AMDG_ADAPT_HOST = 1 };
amdg_status amdg_context_set_adapt_mode(amdg_context* ctx, int mode);

/* Test hook (no reference counterpart): after `after` more device allocations by the library,
 * every allocation fails as if the device were out of memory (the calls report AMDG_ERR_NOMEM);
 * -1 turns it off.  Process-wide. */
amdg_status amdg_debug_fail_device_allocations(int64_t after);
/* seconds[AMDG_PHASE_COUNT] and calls[AMDG_PHASE_COUNT] (either may be NULL). */
amdg_status amdg_context_profile_read(const amdg_context* ctx, double* seconds, int64_t* calls);

/* ---- host-side set-up (no device needed) -------------------------------- */
/* OperatorMatrix1D<AlptBasis,AlptBasis>(all_bas, all_bas, "period")
 * (OperatorMatrix1D.h:125-199): dense 1D matrices of the (2^nmax)(k+1) Alpert
 * basis functions, row = solution basis, column = test basis, row-major.  Any
 * output pointer may be NULL. */
amdg_status amdg_oper1d_build(int nmax, int k, double* u_v, double* u_vx, double* ulft_vjp, double* urgt_vjp);
/* Element multi-indices of the sparse or full grid in the library's element
 * order (DGSolution.cpp:17-54).  Call with level == NULL to get the count. */
amdg_status amdg_grid_enumerate(int dim, int nmax, int sparse, int64_t* num_elements, int32_t* level, int32_t* suppt);

/* ---- grid (DGSolution / DGAdapt) --------------------------------------- */
/* Sparse (sum of levels <= nmax) or full grid of Alpert degree k.
 * Replaces DGSolution::DGSolution (DGSolution.cpp:10-57) and the
 * DGAdapt constructor with find_ptr_alpt (DGAdapt.cpp:5-37,
 * DGSolution.cpp:675-728).  dim 1..6, nmax*dim <= 60, k 1..3. */
amdg_status amdg_grid_create(amdg_context* ctx, int dim, int nmax, int k, int sparse, amdg_grid** out);
amdg_status amdg_grid_destroy(amdg_grid* g);
/* DGAdapt(sparse, level_init, NMAX, ...) with level_init < NMAX: the sparse
 * (or full) grid of level level_init whose elements may later refine up to
 * level nmax (DGAdapt.cpp:5-37). */
amdg_status amdg_grid_create_ex(amdg_context* ctx, int dim, int level_init, int nmax, int k, int sparse, amdg_grid** out);
/* DGSolution::size_elem / get_dof (DGSolution.cpp:836-849). */
amdg_status amdg_grid_size(const amdg_grid* g, int64_t* num_elements, int64_t* dof);
/* level and suppt of every element, num_elements x dim each (host buffers). */
amdg_status amdg_grid_elements(const amdg_grid* g, int32_t* level, int32_t* suppt);
/* DGSolution::max_mesh_level_vec (DGSolution.cpp:948-959): dim entries. */
amdg_status amdg_grid_max_mesh_level(const amdg_grid* g, int32_t* levels);
/* Element::ucoe_alpt of every element, host <-> device (n = dof doubles). */
amdg_status amdg_grid_set_coefficients(amdg_grid* g, const double* host, int64_t n);
amdg_status amdg_grid_get_coefficients(const amdg_grid* g, double* host, int64_t n);
/* Device pointer of the grid's FP64 coefficient vector (valid until destroy). */
amdg_status amdg_grid_coefficients_device(amdg_grid* g, double** device_ptr);
/* DGAdapt::init_separable_scalar_sum / init_separable_scalar
 * (DGAdapt.cpp:63-147; DGSolution.cpp:150-184): coefficients of
 * sum_term prod_d f(x_d, d, term).  The 1D projections run on the host, the
 * expansion into element blocks on the device.  Without adaptivity
 * (refine threshold not reached), as in the reference drivers that pass
 * refine_eps = 1e10. */
amdg_status amdg_grid_init_separable(amdg_grid* g, int nterms, amdg_fn1d f, void* user);
/* DGAdapt::init_separable_scalar_sum with adaptivity (DGAdapt.cpp:120-147,
 * 850-894): every leaf whose projected block has norm > eps gets its children,
 * holes are filled, until nothing changes; then the coefficients are set. */
amdg_status amdg_grid_init_separable_adaptive(amdg_grid* g, int nterms, amdg_fn1d f, void* user, double eps);
/* amdg_grid_init_separable / _adaptive / amdg_grid_l2_error_separable_sum with the factors given
 * in bulk (same points, same arithmetic). */
amdg_status amdg_grid_init_separable_batch(amdg_grid* g, int nterms, amdg_fn1d_batch f, void* user);
amdg_status amdg_grid_init_separable_adaptive_batch(amdg_grid* g, int nterms, amdg_fn1d_batch f, void* user,
                                                    double eps);
amdg_status amdg_grid_l2_error_separable_sum_batch(const amdg_grid* g, int nterms, amdg_fn1d_batch f, void* user,
                                                   double l2_norm_exact, double* out);
/* DGAdaptIntp::init_adaptive_intp (DGAdaptIntp.cpp:35-46, 184-270; FastLagrInit,
 * FastMultiplyLU.cpp:1617-1620): starting from the grid's element set (the sparse grid of the
 * initial level), f is interpolated at the Lagrange points (degree 3 or 5 with the msh_case 1
 * nodes, or 4 with msh_case 2) and turned into hierarchical surpluses on the device; every leaf whose
 * indicator sqrt(sum_points prod_d M_d * surplus^2) exceeds eps (M the 1D Lagrange mass diagonal,
 * DGAdaptIntp::indicator_norm_intp_Lag) gets its children, holes are filled, and this repeats
 * until nothing changes.  The grid's coefficients are then the Alpert coefficients of the
 * interpolant, by the fast transforms with u_v (Lagrange x Alpert) in every dimension.  f is
 * called once per round on all points of the current element set.  k must be 2.  rounds (may
 * be NULL): refinement rounds that changed the element set. */
amdg_status amdg_grid_init_adaptive_intp(amdg_grid* g, int lagr_degree, amdg_fn_points f, void* user, double eps,
                                         int* rounds);
/* DGAdaptIntp::get_L2_error_split_adaptive_intp_scalar (DGAdaptIntp.cpp:57-102): the L2 distance
 * between the solutions on g and on `exact` (same dimension, finest level and degree), from the
 * orthonormality of the Alpert basis: err^2 = |u_exact|^2 + |u|^2 - 2 * (sum over the elements
 * both grids hold of u . u_exact).  The block products run on the device.  *out = sqrt(err^2),
 * or err^2 itself when it is negative, as the reference returns it. */
amdg_status amdg_grid_l2_error_split_grid(const amdg_grid* g, const amdg_grid* exact, double* out);
/* DGAdapt::refine (DGAdapt.cpp:371-404): one pass -- leaves whose indicator
 * (the 2-norm of the element block of d_indicator, or of the grid's own
 * coefficients when NULL; DGAdapt::indicator_norm :1018-1030) exceeds eps get
 * all their children up to level nmax, then holes are filled (check_hole).
 * The grid's coefficients are carried over, new elements start at zero
 * (copy_predict_to_ucoe).  Operators built on the grid rebuild themselves on
 * their next call.  num_elements may be NULL. */
amdg_status amdg_grid_refine(amdg_grid* g, const double* d_indicator, double eps, int64_t* num_elements);
/* DGAdapt::coarsen (DGAdapt.cpp:675-688, 982-1016): childless elements with
 * indicator < eta and a level > 0 in some dimension are removed, repeatedly. */
amdg_status amdg_grid_coarsen(amdg_grid* g, double eta, int64_t* num_elements);
/* Counter bumped on every change of the element set. */
amdg_status amdg_grid_version(const amdg_grid* g, int64_t* version);
/* DGSolution::get_L2_norm (DGSolution.cpp:933-946): sum of squares of all
 * coefficients (the reference returns the squared norm). */
amdg_status amdg_grid_l2_norm(const amdg_grid* g, double* out);
/* DGSolution::get_L2_error_split_separable_scalar (DGSolution.cpp:217-256). */
amdg_status amdg_grid_l2_error_separable(const amdg_grid* g, amdg_fn1d f, void* user, double l2_norm_exact,
                                         double* out);

/* Same for an exact solution given as a sum of nterms separable terms
 * (|u - u_h|^2 = |u|^2 + sum u_h^2 - 2 sum_terms <u_h, term>). */
amdg_status amdg_grid_l2_error_separable_sum(const amdg_grid* g, int nterms, amdg_fn1d f, void* user,
                                             double l2_norm_exact, double* out);

/* Values of the solution on the tensor mesh x1d^dim (x1d: n1 host coordinates,
 * the same in every dimension): d_out[i_0]...[i_{dim-1}] (device, n1^dim
 * doubles, last index fastest) = u_h(x1d[i_0], ..., x1d[i_{dim-1}]), summed over
 * every element whose closed support holds the point (DGSolution::val,
 * DGSolution.cpp:613-625; Element::val, Element.cpp:123-147).  At most 2^31
 * points per call. */
amdg_status amdg_grid_eval_tensor(const amdg_grid* g, int n1, const double* x1d, double* d_out);

/* err[3] = L1, L2, Linf of u_h - u at time t, u the exact solution of
 * u_t + sum_d (u^2/2)_{x_d} = 0 with u(x,0) = a + b sin(2 pi (sum_d x_d + c)),
 * by gauss_points (1..10) Gauss-Legendre points per dimension in every cell of
 * the uniform mesh of the finest element level
 * (DGSolution::get_error_no_separable_scalar, DGSolution.cpp:326-335;
 * Quad::norm_multiD, Quad.cpp:261-318; BurgersExact::exact_1d / norm_1d,
 * ExactSolution.cpp:8-71, with x -> sum_d x_d and t -> dim t).
 * AMDG_ERR_NONFINITE when the exact solution's Newton iteration fails (past
 * the shock time). */
amdg_status amdg_grid_error_burgers(const amdg_grid* g, double a, double b, double c, double t, int gauss_points,
                                    double* err);

/* ---- linear constant-coefficient operator (HyperbolicAlpt) -------------- */
/* HyperbolicAlpt::assemble_matrix_scalar (BilinearForm.cpp:691-710): volume
 * term c_d * u_vx plus upwind flux c_d * ulft_vjp (c_d >= 0) or c_d * urgt_vjp
 * (c_d < 0) in each dimension, entries below 1e-13 dropped as in
 * BilinearFormAlpt::assemble_matrix_alpt (BilinearForm.cpp:25-87).  Matrix
 * free: the 1D blocks and the per-(element, dimension) neighbour lists live on
 * the device.  coef has dim entries. */
amdg_status amdg_linear_create(amdg_grid* g, const double* coef, amdg_linear_op** out);
amdg_status amdg_linear_destroy(amdg_linear_op* op);
/* Number of nonzero (element, neighbour, dimension) block pairs and the
 * algorithmic flops of one apply (2 * (k+1)^(dim+1) per pair). */
amdg_status amdg_linear_stats(const amdg_linear_op* op, int64_t* pairs, double* flops_per_apply);
/* Kernel variant per precision (variants[0] FP64, variants[1] mixed; 0 = one
 * thread per output coefficient, 1 = column variant, 2 = column variant whose
 * neighbour blocks arrive in shared memory by bulk asynchronous copies, mixed
 * only, 3 = the same bulk-copy ring with the per-dimension contraction
 * (FastMultiplyLU::transform_1D, FastMultiplyLU.cpp:436-512) on the tensor pipe
 * as 3xTF32 mma.sync with FP32 accumulation, mixed only), chosen when the
 * operator is built by timing the candidates on its grid, and the measured stage
 * times stage_ms[precision*4 + variant] (0 where not timed).  No reference
 * counterpart.  Either pointer may be NULL. */
amdg_status amdg_linear_tuning(const amdg_linear_op* op, int* variants, float* stage_ms);
/* Override the autotuner's choice (kept until the grid changes). */
amdg_status amdg_linear_set_variant(amdg_linear_op* op, amdg_precision prec, int variant);
/* Configuration of the bulk-copy variant (variant 2), picked by the same autotuner: 0 = 3-slot
 * ring with the 1D operator block copied into the slot, 1 = 3 slots with the operator block read
 * from the (L1-resident) table, 2 / 3 / 4 / 5 = 6 / 2 / 4 / 1 slots with the table read, 6 / 7 =
 * 1 slot with 2 / 4 elements (warps) per CTA.  stage_ms[8]: measured stage time per configuration
 * (0 where not timed).  All configurations sum in the same order. */
amdg_status amdg_linear_copy_config(const amdg_linear_op* op, int* config, float* stage_ms);
amdg_status amdg_linear_set_copy_config(amdg_linear_op* op, int config);
/* Polls of the bulk-copy variant's bounded waits before a wait gives up (no reference
 * counterpart; default 4194304 = 2^22).  A wait that gives up makes the kernel drain its copies in
 * flight (with its own bound) and return without writing; the call then fails with
 * AMDG_ERR_TIMEOUT and leaves the state as it was.  0 makes every wait give up at once, for
 * testing that path. */
amdg_status amdg_linear_set_wait_limit(amdg_linear_op* op, uint32_t polls);
/* BilinearForm::multi (BilinearForm.h:23): d_rhs = L d_u, device pointers of
 * dof doubles each. */
amdg_status amdg_linear_apply(amdg_linear_op* op, const double* d_u, double* d_rhs, amdg_precision prec);
/* RK3SSP::step_rk (ODESolver.cpp:261-271), nsteps steps of size dt on the
 * grid's device state; stage updates fused into the operator kernel. */
amdg_status amdg_rk3ssp_steps(amdg_linear_op* op, double dt, int nsteps, amdg_precision prec);
/* Same, through host memory: uploads host_u (dof doubles), steps, and writes
 * the result back into host_u.  The call a host-side driver makes per step
 * when it keeps Element::ucoe_alpt on the host (ODESolver::init/final,
 * ODESolver.cpp:25-60). */
amdg_status amdg_rk3ssp_steps_host(amdg_linear_op* op, double dt, int nsteps, double* host_u, amdg_precision prec);
/* Serving form of amdg_rk3ssp_steps_host, no reference counterpart: nreq independent requests
 * on the operator's grid, request r stepped from host_in[r] (dof doubles) into host_out[r]
 * (host_out[r] may equal host_in[r]).  Request r + 1 is copied in and request r - 1 copied out
 * while request r is stepped (three device states, one copy stream per direction); pinned host
 * buffers let the copies overlap.  Requests are independent: an output buffer must not be the
 * input of a later request of the same call.  The grid's own coefficients are left unchanged. */
amdg_status amdg_rk3ssp_serve_host(amdg_linear_op* op, double dt, int nsteps, amdg_precision prec, int nreq,
                                   const double* const* host_in, double* const* host_out);

/* Allocation-free variant of amdg_rk3ssp_steps, with no counterpart in the
 * reference: for callers that cannot call cudaMalloc (host callbacks, which may
 * not call CUDA, processes whose device memory belongs to another allocator,
 * loops that must not allocate).  d_u is the caller's device state (dof doubles, input
 * and output).  The stage vectors live in a fixed 4 MiB device array shared by
 * every call, so the grid may hold at most 262,144 coefficients (larger grids
 * get AMDG_ERR_CAPACITY) and calls that overlap on the GPU race.  The first
 * call on a device looks up the array's address; make it before any stream
 * capture.  The address is kept until the library is unloaded: a device reset
 * in between is not supported.  With AMDG_PREC_MIXED this call keeps its stage
 * vectors in FP64 (the operator converts each value it loads to FP32), where
 * amdg_rk3ssp_steps keeps them as FP32 (hi, lo) pairs: the two agree to about
 * 1e-6 relative, not bitwise; in FP64 they agree bitwise. */
amdg_status amdg_rk3ssp_steps_noalloc(amdg_linear_op* op, double* d_u, double dt, int nsteps, amdg_precision prec);

/* ---- the reference driver's per-element vectors and explicit integrators ----
 * (no separate reference entry points: these are the Element members and ODESolver calls a
 * driver's stage loop uses, e.g. example/07_vlasov_maxwell_adapt.cpp:278-320) */
/* DGSolution::set_rhs_zero (DGSolution.h:153): Element::rhs of every element = 0.  The grid's rhs
 * vector (dof doubles) is what the *_rhs_add calls accumulate into; it restarts at zero whenever
 * the element set changes. */
amdg_status amdg_grid_set_rhs_zero(amdg_grid* g);
amdg_status amdg_grid_rhs_device(amdg_grid* g, double** device_ptr);
/* Element::rhs of every element into host memory (n = dof doubles). */
amdg_status amdg_grid_get_rhs(amdg_grid* g, double* host, int64_t n);
/* DGSolution::copy_ucoe_to_predict / copy_predict_to_ucoe (DGSolution.h:171-174): the prediction
 * vector follows refine / coarsen like the coefficients (new elements zero, as the reference's
 * new Element objects are). */
amdg_status amdg_grid_copy_ucoe_to_predict(amdg_grid* g);
amdg_status amdg_grid_copy_predict_to_ucoe(amdg_grid* g);
/* DGSolution::copy_ucoe_ut_to_predict / copy_predict_to_ucoe_ut: the same for u_t (the grid's
 * velocity field, created as zero when absent). */
amdg_status amdg_grid_copy_ucoe_ut_to_predict(amdg_grid* g);
amdg_status amdg_grid_copy_predict_to_ucoe_ut(amdg_grid* g);
/* Element indicator of amdg_grid_refine / amdg_grid_coarsen: AMDG_INDICATOR_U (default) the block
 * norm of u; AMDG_INDICATOR_U_UT that plus the block norm of u_t, as DGAdapt::indicator_norm
 * computes it when DGSolution::prob is "wave" (DGAdapt.cpp:1018-1030). */
enum { AMDG_INDICATOR_U = 0, AMDG_INDICATOR_U_UT = 1 };
amdg_status amdg_grid_set_indicator(amdg_grid* g, int mode);
/* y += a x on device vectors of n doubles (Eigen's vector update). */
amdg_status amdg_vector_axpy(amdg_context* ctx, double a, const double* d_x, double* d_y, int64_t n);

/* ODESolver (ODESolver.h:5-38) for ForwardEuler (ODESolver.h:115-127, ODESolver.cpp:209-213) and
 * RK3SSP (ODESolver.h:183-198, ODESolver.cpp:285-301) on a grid's device state: create = the
 * constructor + ExplicitRK::init() (ODESolver.h:93: the coefficients at t_n are kept, the
 * solver's rhs is zero); set_rhs_zero / add_rhs_to_eigenvec (:38, :24) act on the solver's rhs
 * vector (add: += the grid's Element::rhs); step_stage(stage) updates the grid's coefficients;
 * final() (:17) zeroes the solver's rhs (the state already is the grid's).  The element set must not change between create and step_stage. */
/* Second-order-in-time schemes on (u, u_t) (RKODE2nd, ODESolver.h:257-283): AMDG_ODE_EULER_ODE2ND
 * (EulerODE2nd::step_stage, ODESolver.cpp:409-414: u += dt u_t, u_t += dt rhs) and
 * AMDG_ODE_RK4ODE2ND (RK4ODE2nd::step_stage, ODESolver.cpp:579-615: the stage state from (u, u_t)
 * at t_n and the stage increments, the step's end at stage 3); create keeps u and u_t at t_n
 * (the grid's velocity field, created as zero when absent), step_stage writes the grid's u and
 * u_t. */
typedef struct amdg_ode amdg_ode;
enum { AMDG_ODE_FORWARD_EULER = 0, AMDG_ODE_RK3SSP = 1, AMDG_ODE_EULER_ODE2ND = 2, AMDG_ODE_RK4ODE2ND = 3 };
amdg_status amdg_ode_create(amdg_grid* g, int scheme, double dt, amdg_ode** out);
amdg_status amdg_ode_destroy(amdg_ode* ode);
amdg_status amdg_ode_set_rhs_zero(amdg_ode* ode);
amdg_status amdg_ode_add_rhs_to_eigenvec(amdg_ode* ode);
amdg_status amdg_ode_step_stage(amdg_ode* ode, int stage);
amdg_status amdg_ode_final(amdg_ode* ode);

/* ---- stage updates for an externally computed right-hand side ----------- */
/* RK3SSP::step_stage / ForwardEuler::step_stage (ODESolver.cpp:209-213,
 * 285-301) on device vectors of n doubles: stage 0 u = un + dt*rhs,
 * stage 1 u = 3/4 un + 1/4 (u + dt*rhs), stage 2 u = 1/3 un + 2/3 (u + dt*rhs). */
amdg_status amdg_rk3_stage_update(amdg_context* ctx, int stage, double dt, const double* d_un, double* d_u,
                                  const double* d_rhs, int64_t n);

/* ---- nonlinear flux through Lagrange interpolation (Burgers) ------------- */
/* Scalar inviscid Burgers u_t + sum_d (u^2/2)_{x_d} = 0 with global
 * Lax-Friedrichs flux, the flux interpolated by degree-3 hierarchical
 * Lagrange interpolation (msh_case 1).  Replaces the set-up of
 * LagrInterpolation(dg) + FastLagrIntp + HyperbolicLagrRHS +
 * HyperbolicAlptRHS (Interpolation.h:36-47, FastMultiplyLU.h:194-205,
 * 575-629) for the registered flux u^2/2 (FluxFunction::burgers_flux_scalar,
 * Interplation.cpp:5070-5073).  alpha has dim entries (lxf_alpha).  The grid
 * must be free of holes (every element's parents present, DGAdapt::check_hole);
 * otherwise AMDG_ERR_STATE. */
amdg_status amdg_burgers_create(amdg_grid* g, const double* alpha, amdg_burgers_op** out);
/* The same operator with the flux interpolated by cubic Hermite interpolation (HermBasis with
 * PMAX 3, msh_case 1: value and slope at two points per 1D element), 2D only, as
 * example/02_hyperbolic_05_burgers_adapt.cpp runs Burgers: replaces the set-up of
 * HermInterpolation(dg) + FastHermIntp(dg, Her_pt_Alpt_1D) + HyperbolicSameFluxHermRHS(dg,
 * oper_matx_herm) (Interpolation.h:251-283, FastMultiplyLU.h:224-235, 477-498) for the registered
 * flux u^2/2 with f' = u, f'' = 1.  Every amdg_burgers_* and amdg_lagr_* call below takes it:
 * point values are then u_h and its slopes at the Hermite points (4^2 per element,
 * Element::up_intp), flux coefficients the Hermite coefficients of the flux
 * (HermInterpolation::eval_fp_to_coe_D_Her, Interplation.cpp:3651-3849), amdg_lagr_interpolate
 * is HermInterpolation::nonlinear_Herm_2D_fast (Interplation.cpp:4609-4621) and the
 * AMDG_LAGR_RHS_VOL / _FLX groups are HyperbolicSameFluxHermRHS::rhs_vol_scalar /
 * rhs_flx_intp_scalar (FastMultiplyLU.cpp:970-1016).  The LxF penalty group is the driver's
 * assembled HyperbolicAlpt::assemble_matrix_flx_scalar(d, -1, alpha/2) + (d, 1, -alpha/2)
 * (BilinearForm.cpp:759-769), equal to rhs_flx_penalty_scalar(alpha) up to rounding.
 * AMDG_ERR_ARG unless the grid is 2D. */
amdg_status amdg_burgers_create_herm(amdg_grid* g, const double* alpha, amdg_burgers_op** out);
amdg_status amdg_burgers_destroy(amdg_burgers_op* op);
/* One right-hand-side evaluation, d_rhs = R(d_u) (device vectors of dof doubles).
 * Point values and the hierarchical surplus run in FP64 in both modes; with
 * AMDG_PREC_MIXED the transforms back to Alpert coefficients and the penalty
 * run in FP32.  Composition:
 * LagrInterpolation::nonlinear_Lagr_fast (Interplation.cpp:4033-4047),
 * DGSolution::set_rhs_zero, HyperbolicLagrRHS::rhs_vol_scalar and
 * rhs_flx_intp_scalar (FastMultiplyLU.cpp:1125-1189),
 * HyperbolicAlptRHS::rhs_flx_penalty_scalar (FastMultiplyLU.cpp:1269-1276). */
amdg_status amdg_burgers_rhs(amdg_burgers_op* op, const double* d_u, double* d_rhs, amdg_precision prec);
/* Values of u_h at every Lagrange interpolation point, num_elements x 4^dim
 * (FastLagrIntp::eval_up_Lagr, FastMultiplyLU.cpp:1362; Element::up_intp). */
amdg_status amdg_burgers_point_values(amdg_burgers_op* op, const double* d_u, double* d_up, amdg_precision prec);
/* Interpolation coefficients of the flux, num_elements x 4^dim, identical in
 * every dimension for this flux (Element::fucoe_intp after
 * LagrInterpolation::eval_fp_to_coe_D_Lag, Interplation.cpp:1222-1434). */
amdg_status amdg_burgers_flux_coefficients(amdg_burgers_op* op, const double* d_u, double* d_fu, amdg_precision prec);
/* nsteps SSP-RK3 steps of size dt on the grid's device state, the RHS
 * re-evaluated per stage (RK3SSP::step_stage, ODESolver.cpp:285-301, in the
 * stage loop of example/07_vlasov_maxwell_adapt.cpp:278-320). */
amdg_status amdg_burgers_rk3_steps(amdg_burgers_op* op, double dt, int nsteps, amdg_precision prec);
/* The right-hand side call by call, as a reference driver composes it:
 * LagrInterpolation::nonlinear_Lagr_fast (Interplation.cpp:4033-4047) for the registered flux
 * u^2/2 -- point values of the grid's coefficients, the flux there and its hierarchical surpluses,
 * kept in the operator -- then each group added into the grid's rhs (amdg_grid_rhs_device):
 * AMDG_LAGR_RHS_VOL = HyperbolicLagrRHS::rhs_vol_scalar, AMDG_LAGR_RHS_FLX = rhs_flx_intp_scalar
 * (FastMultiplyLU.cpp:1125-1189; both need the interpolation of the current element set and
 * precision), AMDG_LAGR_RHS_PENALTY = HyperbolicAlptRHS::rhs_flx_penalty_scalar(alpha)
 * (:1269-1276) on the grid's coefficients; alpha (dim entries) replaces the operator's LxF
 * constants, NULL keeps them.  vol + flx + penalty added in that order equal amdg_burgers_rhs. */
enum { AMDG_LAGR_RHS_VOL = 0, AMDG_LAGR_RHS_FLX = 1, AMDG_LAGR_RHS_PENALTY = 2 };
/* Algorithmic work of one right-hand side on the current element set (no reference counterpart):
 * the multiply-adds of every 1D transform sweep the right-hand side runs (2 flops each, from the
 * neighbour lists' L / full / U counts; terms whose first sweeps coincide share them) plus the
 * surplus passes, and the (element, neighbour) pairs the sweeps visit.  Reads the lists back (synchronises): for measurement, not for the step loop. */
amdg_status amdg_burgers_work(amdg_burgers_op* op, double* flops, double* transform_pairs);
/* Kernel of the transform sweeps (no reference counterpart): 0 one thread per output entry; 1 one
 * thread per column of the transformed dimension, all its entries from one load of each input
 * value; 2 / 3 / 4 one warp per (term, element), its lanes over (column, neighbour phase), the
 * phases' partial sums added by shuffles, each warp serving 1 / 2 / 4 elements; -1 (default) 2 for
 * the FP32 sweeps of the mixed mode and 0 for the FP64 and double-float sweeps.  0 and 1 sum every
 * output in the same order (identical results); 2-4 sum in another fixed order (deterministic,
 * equal to rounding). */
amdg_status amdg_burgers_set_sweep_variant(amdg_burgers_op* op, int variant);
amdg_status amdg_lagr_interpolate(amdg_burgers_op* op, amdg_precision prec);
amdg_status amdg_lagr_rhs_add(amdg_burgers_op* op, int group, const double* alpha, amdg_precision prec);

/* ---- batched independent linear solves ------------------------------------ */
/* Many independent constant-coefficient solves (one HyperbolicAlpt + RK3SSP
 * per grid in the reference, run one after the other) advanced together: the
 * grids' element tables are concatenated and every SSP-RK3 stage of all
 * solves is one fused launch.  No reference counterpart for the batching
 * itself.  grids: n grids sharing dim, nmax and k (their current
 * coefficients are copied in); coef: n x dim velocities.  The batch does not
 * follow later changes of the grids' element sets. */
amdg_status amdg_batch_create(amdg_context* ctx, int n, amdg_grid* const* grids, const double* coef, amdg_batch** out);
amdg_status amdg_batch_destroy(amdg_batch* b);
amdg_status amdg_batch_size(const amdg_batch* b, int64_t* num_elements, int64_t* dof, int64_t* pairs);
/* Per-solve time step sizes (n doubles). */
amdg_status amdg_batch_set_dt(amdg_batch* b, const double* dt);
/* nsteps SSP-RK3 steps of every solve; use_graph != 0 captures one step's
 * launches into a CUDA graph on first use and replays it. */
amdg_status amdg_batch_rk3_steps(amdg_batch* b, int nsteps, amdg_precision prec, int use_graph);
/* Copy solve `solve`'s coefficients back into its grid (for norms, errors, IO). */
amdg_status amdg_batch_store(amdg_batch* b, int solve);
/* Device pointer of the concatenated state and the element offsets (n+1 entries, may be NULL). */
amdg_status amdg_batch_coefficients_device(amdg_batch* b, double** device_ptr, int64_t* elem_offsets);
/* Adaptivity inside the batch (no reference counterpart for the batching), the part of the
 * reference's refine -> step -> coarsen loop that falls between two steps: every solve's state is
 * written back to its grid; the elements to refine are chosen on the current state -- by the
 * surplus criterion (leaves with block norm > eps, DGAdapt::refine), or, with a classifier, by
 * its "refine" class where its largest class probability is at least tau and by the criterion
 * elsewhere (as amdg_burgers_adaptive_step_learned); the grid is coarsened on the criterion
 * (leaves with norm < eta, DGAdapt::coarsen), then the chosen elements still present get their
 * children (zero coefficients: the next steps give them values, and the next call's coarsening
 * removes those that stay small); and the batch is rebuilt on the new element sets (neighbour
 * lists, state; step graphs re-captured).  The solves' time steps are kept: set them again if
 * the finest levels changed.  stats (may be NULL): [refined by the classifier, uncertain,
 * elements after].  When replacing a solve's element set fails (AMDG_ERR_NOMEM), the solves
 * before it keep their new sets and the batch is rebuilt on the sets the grids hold, so it stays
 * usable. */
amdg_status amdg_batch_adapt(amdg_batch* b, amdg_mlp* mlp, double eps, double eta, double tau, int64_t* stats);
/* Stage kernel of the batch: amdg_batch_create times one stage with every candidate and keeps
 * the fastest per precision (batches under 100,000 DOF keep candidate 2).  Candidates 0-4: the
 * column kernel with CTAs of 64, 128, 256, 512 and 1024 threads (threads / (k+1)^(dim-1) elements
 * per CTA; dim <= 3, 256 only above) on the FP64 state (mixed: FP32 contraction, FP32 shadows of
 * the stage inputs).  Mixed only: candidates 5-9, the same column kernel with the stage vectors
 * kept as FP32 (hi, lo) pairs for the whole amdg_batch_rk3_steps call (split once, merged once,
 * a double-float stage update); candidates 10-15, one warp per element with the neighbour blocks
 * streamed into shared memory by bulk asynchronous copies, on the same FP32-pair state, in (ring
 * slots, elements per CTA) = (1, 1), (1, 2), (1, 4), (2, 1), (2, 2), (2, 4) -- its waits are
 * bounded, and a wait that gives up fails the call with AMDG_ERR_TIMEOUT and leaves the state as it
 * was; candidates 16-18, the column kernel on the FP32-pair state as one persistent launch (a grid
 * of the CTAs that fit on the device at once, each taking tile after tile) in (CTA threads,
 * schedule) = (64, static tile order), (128, static), (64, tiles taken from a device counter);
 * candidate 19 (blocks of at most 32 coefficients), one warp per element with a lane per
 * coefficient, each neighbour block one coalesced load and the 1D contraction by warp shuffles.
 * Every FP32-pair candidate sums in the same order (identical results).  kernel[2] = chosen
 * candidate (FP64, mixed); stage_ms[2][AMDG_BATCH_KERNELS] = measured stage times per candidate, 0
 * where not timed. */
#define AMDG_BATCH_KERNELS 20
amdg_status amdg_batch_tuning(const amdg_batch* b, int* kernel, float* stage_ms);
/* Override the stage kernel of one precision (AMDG_ERR_ARG where it is not offered). */
amdg_status amdg_batch_set_kernel(amdg_batch* b, amdg_precision prec, int kernel);
/* The column kernel with the given CTA size (candidates 0-4). */
amdg_status amdg_batch_set_tile(amdg_batch* b, amdg_precision prec, int threads);

/* Work counters since creation: RK-stage DOF updates (3 x DOF per SSP-RK3
 * step) and right-hand-side evaluations (including adaptive predictors).  No
 * counterpart in the reference. */
amdg_status amdg_burgers_counters(const amdg_burgers_op* op, int64_t* stage_dof_updates, int64_t* rhs_evaluations);

/* One adaptive time step of the Burgers solver, the loop body of
 * example/02_hyperbolic_05_burgers_adapt.cpp:223-476 with the Lagrange
 * right-hand side: dt = cfl / sum_d wave_speed 2^maxlevel_d, forward-Euler
 * prediction, amdg_grid_refine on the prediction (eps), one SSP-RK3 step,
 * amdg_grid_coarsen (eta).  dt_out may be NULL. */
amdg_status amdg_burgers_adaptive_step(amdg_burgers_op* op, double cfl, double wave_speed, double eps, double eta,
                                       amdg_precision prec, double* dt_out);
/* Same, and records what the surplus criterion decided for every element of
 * the grid at the start of the step: decisions[e] = 1 refined, 2 coarsened
 * away, 0 kept (host buffer of num_elements entries, may be NULL).  These are
 * the labels the learned classifier is trained on. */
amdg_status amdg_burgers_adaptive_step_ex(amdg_burgers_op* op, double cfl, double wave_speed, double eps, double eta,
                                          amdg_precision prec, double* dt_out, int8_t* decisions);

/* ---- second-order wave equation (config of 03_wave_06_var_coeff_adapt.cpp) ---- */
/* Second field v = u_t of the grid (Element::ucoe_ut), dof entries, remapped with u when the
 * element set changes (new elements zero).  A grid without one reads as v = 0 in the wave
 * calls below, which create it. */
amdg_status amdg_grid_set_velocity(amdg_grid* g, const double* host, int64_t n);
amdg_status amdg_grid_get_velocity(const amdg_grid* g, double* host, int64_t n);

/* ---- checkpoint / restart (no reference counterpart: the reference's IO writes text only) ---- */
/* Binary checkpoint of the grid: sorted element keys, FP64 coefficients, u_t when the grid has
 * one, and `time` as given, with an FNV-1a checksum; written to path.tmp and renamed. */
amdg_status amdg_grid_save(const amdg_grid* g, const char* path, double time);
/* A new grid with the checkpoint's element set, coefficients and u_t; *time gets the stored time
 * (may be null).  AMDG_ERR_FORMAT for a bad magic, version, header, size, key order or checksum. */
amdg_status amdg_grid_load(amdg_context* ctx, const char* path, amdg_grid** out, double* time);
/* Text dump of IO::output_element_level_support (IO.cpp:502-517): one line per element, in key
 * order, "level xl xr " per dimension (xl, xr its support, printed as %g). */
amdg_status amdg_grid_write_level_support(const amdg_grid* g, const char* path);
/* The grid's dimension, finest level, Alpert degree and sparse flag (any pointer may be null). */
amdg_status amdg_grid_config(const amdg_grid* g, int* dim, int* nmax, int* k, int* sparse);

/* u_tt = div(K grad u) on the periodic unit cube, K = (1 + a prod_d sin(2 pi x_d))^2 (a = amplitude), Alpert
 * k = 2: K u_{x_d} and K u interpolated by degree-4 Lagrange with the msh_case 2 nodes, as
 * 03_wave_06_var_coeff_adapt.cpp:53-54 sets it (LagrInterpolation::
 * var_coeff_gradu_Lagr_fast / var_coeff_u_Lagr_fast, Interplation.cpp:4159-4212), the
 * DiffusionRHS terms rhs_flx_gradu, rhs_vol, rhs_flx_u (FastMultiplyLU.cpp:1691-1765) and the
 * IPDG penalty -sigma/dx [u][v], dx the finest element size
 * (DiffusionAlpt::assemble_matrix_flx_ujp_vjp, BilinearForm.cpp:920-929), evaluated matrix free. */
amdg_status amdg_wave_create(amdg_grid* g, double sigma, double amplitude, amdg_wave_op** out);
amdg_status amdg_wave_destroy(amdg_wave_op* op);
/* d_rhs = L(d_u) (device arrays, dof entries). */
amdg_status amdg_wave_rhs(amdg_wave_op* op, const double* d_u, double* d_rhs, amdg_precision prec);
/* The wave right-hand side term by term, as the reference's driver composes it
 * (03_wave_06_var_coeff_adapt.cpp:258-276): amdg_wave_interpolate interpolates K du/dx_d for every
 * d (AMDG_WAVE_INTERP_GRADU: LagrInterpolation::var_coeff_gradu_Lagr_fast) or K u
 * (AMDG_WAVE_INTERP_U: var_coeff_u_Lagr_fast) of the grid's current u; amdg_wave_rhs_add adds a
 * term group into the grid's rhs vector (Element::rhs): AMDG_WAVE_RHS_FLX_GRADU
 * (DiffusionRHS::rhs_flx_gradu) and AMDG_WAVE_RHS_VOL (rhs_vol) read the K grad u interpolation,
 * AMDG_WAVE_RHS_FLX_U (rhs_flx_u) the K u one, AMDG_WAVE_RHS_IPDG the IPDG term -sigma/dx [u][v]
 * of the current u (DiffusionAlpt::assemble_matrix_flx_ujp_vjp times u).  AMDG_ERR_STATE when the
 * interpolation a group reads is missing for this element set and precision. */
/* The IPDG parameter sigma of the operator (DiffusionAlpt's, BilinearForm.cpp:922-923). */
amdg_status amdg_wave_set_sigma(amdg_wave_op* op, double sigma);
enum { AMDG_WAVE_INTERP_GRADU = 0, AMDG_WAVE_INTERP_U = 1 };
amdg_status amdg_wave_interpolate(amdg_wave_op* op, int which, amdg_precision prec);
enum { AMDG_WAVE_RHS_FLX_GRADU = 0, AMDG_WAVE_RHS_VOL = 1, AMDG_WAVE_RHS_FLX_U = 2, AMDG_WAVE_RHS_IPDG = 3 };
amdg_status amdg_wave_rhs_add(amdg_wave_op* op, int group, amdg_precision prec);
/* RKODE2nd::add_rhs_matrix (the solver's rhs += the IPDG term of the grid's current u, FP64), and
 * the rhs of EulerODE2nd::step_rk (the solver's rhs = that term alone, ODESolver.cpp:394-399). */
amdg_status amdg_ode_add_wave_penalty(amdg_ode* ode, amdg_wave_op* op);
/* amdg_burgers_set_sweep_variant for the wave operator's transform sweeps. */
amdg_status amdg_wave_set_sweep_variant(amdg_wave_op* op, int variant);
/* nsteps RK4ODE2nd steps of u' = v, v' = L u on the grid's (u, v)
 * (RK4ODE2nd::step_stage, ODESolver.cpp:579-615). */
amdg_status amdg_wave_rk4_steps(amdg_wave_op* op, double dt, int nsteps, amdg_precision prec);
/* One adaptive step, the loop body of 03_wave_06_var_coeff_adapt.cpp:195-265 without source:
 * dt = cfl / sum_d wave_speed 2^maxlevel_d; EulerODE2nd predictor as step_rk_source runs it (the
 * predicted u_t takes the IPDG term of u alone, ODESolver.cpp:402-407); refine on the predicted
 * ||u|| + ||u_t|| (DGAdapt::indicator_norm for prob "wave", DGAdapt.cpp:1018-1030); one RK4ODE2nd
 * step; coarsen on ||u|| + ||u_t||. */
amdg_status amdg_wave_adaptive_step(amdg_wave_op* op, double cfl, double wave_speed, double eps, double eta,
                                    amdg_precision prec, double* dt_out);
/* As amdg_burgers_adaptive_step_ex / amdg_burgers_features / amdg_burgers_adaptive_step_learned for
 * the wave operator: the step is RK4ODE2nd, the criterion ||u|| + ||u_t||, and the classifier reads
 * the features of u followed by those of the grid's u_t, 2 (k+1)^dim (1 + 2 dim) floats per
 * element. */
amdg_status amdg_wave_adaptive_step_ex(amdg_wave_op* op, double cfl, double wave_speed, double eps, double eta,
                                       amdg_precision prec, double* dt_out, int8_t* decisions);
amdg_status amdg_wave_features(amdg_wave_op* op, const double* d_u, float* d_features);
amdg_status amdg_wave_adaptive_step_learned(amdg_wave_op* op, amdg_mlp* mlp, double cfl, double wave_speed, double eps,
                                            double eta, double tau, amdg_precision prec, double* dt_out, int64_t* stats);
amdg_status amdg_wave_adaptive_steps_learned(amdg_wave_op* op, amdg_mlp* mlp, double cfl, double wave_speed,
                                             double eps, double eta, double tau, amdg_precision prec, int horizon,
                                             double t_left, double* t_advanced, int* steps, int64_t* stats);
/* As amdg_burgers_counters (4 x DOF per RK4ODE2nd step). */
amdg_status amdg_wave_counters(const amdg_wave_op* op, int64_t* stage_dof_updates, int64_t* rhs_evaluations);

/* ---- learned refine/coarsen (no reference counterpart) -------------------- */
/* Per-element classifier refine / keep / coarsen: n_in -> n_hidden_layers x
 * hidden (ReLU) -> n_out (softmax), FP32, He-initialised from seed.  Judged
 * against DGAdapt::refine / coarsen (DGAdapt.cpp:371-404, 675-688). */
amdg_status amdg_mlp_create(amdg_context* ctx, int n_in, int hidden, int n_hidden_layers, int n_out, uint64_t seed,
                            amdg_mlp** out);
amdg_status amdg_mlp_destroy(amdg_mlp* m);
/* Flat parameters: per layer W[out][in] row-major, then b[out]. */
amdg_status amdg_mlp_num_params(const amdg_mlp* m, int64_t* n);
amdg_status amdg_mlp_get_params(const amdg_mlp* m, float* host, int64_t n);
amdg_status amdg_mlp_set_params(amdg_mlp* m, const float* host, int64_t n);
/* Class probabilities of n samples (device arrays n x n_in -> n x n_out). */
amdg_status amdg_mlp_predict(amdg_mlp* m, const float* d_x, int64_t n, float* d_probs);
/* Mean cross entropy of n labelled samples and its gradient (host, num_params floats; may be NULL). */
amdg_status amdg_mlp_loss_grad(amdg_mlp* m, const float* d_x, const int32_t* d_labels, int64_t n, double* loss,
                               float* host_grad);
/* Adam (0.9, 0.999, 1e-8) on minibatches of a seeded shuffle; mean loss of the last epoch in final_loss. */
amdg_status amdg_mlp_train(amdg_mlp* m, const float* d_x, const int32_t* d_labels, int64_t n, int epochs, int batch,
                           float lr, uint64_t seed, double* final_loss);
/* Classifier inputs of every element: |coefficients| of the element and of its
 * parent and grandparent in each dimension, log-scaled (log10(|c| + 1e-20)/20 + 1),
 * (k+1)^dim * (1 + 2 dim) floats per element (device). */
amdg_status amdg_burgers_features(amdg_burgers_op* op, const double* d_u, float* d_features);
/* Adaptive step with learned pre-adaptation: the classifier (3 classes: 0
 * refine, 1 keep, 2 coarsen, i.e. the decisions 1, 0, 2 of
 * amdg_burgers_adaptive_step_ex) decides which leaves to refine before the
 * step (no forward-Euler predictor); on elements whose largest class
 * probability is below tau the surplus criterion on the current coefficients
 * decides.  After the SSP-RK3 step the grid is coarsened as amdg_grid_coarsen
 * and the surplus criterion judges the result: leaves still above eps are
 * missed refinements, refined at the start of the next learned step.  stats
 * (may be NULL): [refined by the network, uncertain, missed refinements,
 * elements after the step]. */
amdg_status amdg_burgers_adaptive_step_learned(amdg_burgers_op* op, amdg_mlp* mlp, double cfl, double wave_speed,
                                               double eps, double eta, double tau, amdg_precision prec, double* dt_out,
                                               int64_t* stats);
/* The learned step over a horizon: the classifier (trained on the plain criterion's refinements
 * within the next `horizon` steps) pre-adapts the grid once, then `horizon` SSP-RK3 steps of one dt
 * (cfl / sum_d wave_speed 2^maxlevel_d of the grid before the pre-adaptation, as the plain step
 * takes it before its refinement) run on that grid (a CUDA graph
 * replays them), then coarsening and the criterion's check for
 * missed refinements as above.  mlp may be NULL: the surplus criterion on the current coefficients
 * then pre-adapts the grid alone (the same horizon without a network, the ablation of the
 * classifier).  With t_left > 0 no step passes t_left: the horizon is cut and its
 * last step shortened to land on it.  *t_advanced = the time stepped, *steps = the steps taken
 * (either may be NULL). */
amdg_status amdg_burgers_adaptive_steps_learned(amdg_burgers_op* op, amdg_mlp* mlp, double cfl, double wave_speed,
                                                double eps, double eta, double tau, amdg_precision prec, int horizon,
                                                double t_left, double* t_advanced, int* steps, int64_t* stats);

#ifdef __cplusplus
}
#endif
#endif /* AMDG_H */
