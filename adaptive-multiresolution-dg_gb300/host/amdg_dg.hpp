// C++ mirror of the AdaM-DG driver-facing API for the sparse-grid DG
// right-hand side, implemented over the C-ABI in include/amdg.h.
//
// A driver written against the reference (example/*.cpp) keeps its structure:
// the same class names, constructor arguments and method names, with the
// element table, coefficients and operators living on the GPU.  Classes whose
// reference role is host-side bookkeeping (AllBasis, OperatorMatrix1D, Hash)
// keep their constructors but hold only what the device needs; the 1D tables
// are built inside the library.  Errors throw amdg_gpu::Error (the reference
// prints and calls exit(1)).
//
// Mirrors: DGSolution/DGAdapt (DGAdapt.h:10-91, DGSolution.h:21-214),
// HyperbolicAlpt (BilinearForm.h:137-152), RK3SSP/ForwardEuler (ODESolver.h:5-205),
// LagrInterpolation + FastLagrIntp + HyperbolicLagrRHS + HyperbolicAlptRHS
// (Interpolation.h:36-129, FastMultiplyLU.h:194-205, 575-629), FluxFunction
// (Interplation.cpp:5070-5073).
//
// A host std::function cannot run on the device: LagrInterpolation recognises the
// fluxes the library registers by evaluating the given function at a few states
// (u^2/2, the Burgers flux of FluxFunction::burgers_flux_scalar) and throws
// AMDG_ERR_ARG for any other.  Arithmetic: amdg_gpu::precision (FP64 by default;
// AMDG_PREC_MIXED runs the back transforms in FP32).
#pragma once

#include <cmath>
#include <functional>
#include <stdexcept>
#include <string>
#include <vector>

#include "amdg.h"

namespace amdg_gpu {

struct Error : std::runtime_error {
    amdg_status status;
    Error(amdg_status s, const std::string& where)
        : std::runtime_error(where + ": " + amdg_status_string(s) + ": " + amdg_last_error()), status(s) {}
};

inline void check(amdg_status s, const char* where) {
    if (s != AMDG_OK) throw Error(s, where);
}

// arithmetic of the Lagrange-path classes below (a process-wide setting, like the reference's
// static configuration)
inline amdg_precision precision = AMDG_PREC_FP64;

// ---- static configuration, as set by the reference drivers ----------------
struct AlptBasis { static inline int PMAX = 2; };
struct LagrBasis {
    static inline int PMAX = 3;
    static inline int msh_case = 1;
    static void set_interp_msh01() {}
};
struct HermBasis {
    static inline int PMAX = 3;
    static inline int msh_case = 1;
    static void set_interp_msh01() {}
};
struct Element {
    static inline int DIM = 1, VEC_NUM = 1, PMAX_alpt = 2, PMAX_intp = 3;
    static inline std::vector<std::vector<bool>> is_intp;
};
struct Interpolation { static inline int DIM = 1, VEC_NUM = 1; };
struct Hash {};

template <class T>
struct AllBasis {
    explicit AllBasis(int max_level) : NMAX(max_level), PMAX(T::PMAX) {}
    const int NMAX;
    const int PMAX;
};

template <class U, class V>
struct OperatorMatrix1D {
    OperatorMatrix1D(const AllBasis<U>& u, const AllBasis<V>&, const std::string& boundary_type) : nmax(u.NMAX) {
        if (boundary_type != "period") throw Error(AMDG_ERR_ARG, "OperatorMatrix1D: only periodic boundaries are supported");
    }
    const int nmax;
};

// ---- library context (one per process and device) ---------------------------
class Runtime {
public:
    static amdg_context* context(int device = 0) {
        static Runtime rt(device);
        return rt.ctx_;
    }
private:
    explicit Runtime(int device) { check(amdg_context_create(device, &ctx_), "amdg_context_create"); }
    ~Runtime() { amdg_context_destroy(ctx_); }
    amdg_context* ctx_ = nullptr;
};

namespace detail {
struct SepFns {
    const std::vector<std::function<double(double, int)>>* fns;
};
inline double sep_trampoline(double x, int d, int term, void* user) {
    return (*static_cast<SepFns*>(user)->fns)[term](x, d);
}
}  // namespace detail

// ---- DGSolution / DGAdapt ------------------------------------------------------
class DGSolution {
public:
    static inline int DIM = 1;
    static inline int VEC_NUM = 1;
    static inline std::vector<int> ind_var_vec{0};
    // "wave": the refine / coarsen indicator adds the norm of u_t (DGAdapt.cpp:1018-1030)
    static inline std::string prob;

    // the grid starts with the elements of levels up to level_init (sum of levels for a sparse grid)
    DGSolution(bool sparse, int level_init, int NMAX, AllBasis<AlptBasis>& all_bas, AllBasis<LagrBasis>&,
               AllBasis<HermBasis>&, Hash&)
        : nmax_(NMAX) {
        check(amdg_grid_create_ex(Runtime::context(), DIM, level_init, NMAX, all_bas.PMAX, sparse ? 1 : 0, &grid_),
              "amdg_grid_create_ex");
    }
    DGSolution(const DGSolution&) = delete;
    DGSolution& operator=(const DGSolution&) = delete;
    virtual ~DGSolution() {
        release_lagr();
        amdg_grid_destroy(grid_);
    }

    int size_elem() const { int64_t e = 0; check(amdg_grid_size(grid_, &e, nullptr), "amdg_grid_size"); return int(e); }
    int size_basis_alpt() const { int64_t d = 0; check(amdg_grid_size(grid_, nullptr, &d), "amdg_grid_size"); return int(d); }
    int get_dof() const { return size_basis_alpt() * int(ind_var_vec.size()); }
    int nmax_level() const { return nmax_; }
    std::vector<int> max_mesh_level_vec() const {
        std::vector<int32_t> lv(DIM);
        check(amdg_grid_max_mesh_level(grid_, lv.data()), "amdg_grid_max_mesh_level");
        return std::vector<int>(lv.begin(), lv.end());
    }
    int max_mesh_level() const {
        int m = 0;
        for (int v : max_mesh_level_vec()) m = std::max(m, v);
        return m;
    }
    // sum of squares of all coefficients (DGSolution::get_L2_norm)
    std::vector<double> get_L2_norm() const {
        double s = 0;
        check(amdg_grid_l2_norm(grid_, &s), "amdg_grid_l2_norm");
        return {s};
    }
    double get_L2_error_split_separable_scalar(std::function<double(double, int)> func, double l2_norm_exact_soln) const {
        std::vector<std::function<double(double, int)>> fns{func};
        detail::SepFns sf{&fns};
        double err = 0;
        check(amdg_grid_l2_error_separable(grid_, detail::sep_trampoline, &sf, l2_norm_exact_soln, &err),
              "amdg_grid_l2_error_separable");
        return err;
    }
    // level and support index of every element (size_elem() x DIM each, Element::level / suppt)
    void elements(std::vector<int>& level, std::vector<int>& suppt) const {
        std::vector<int32_t> lv(size_t(size_elem()) * DIM), sp(lv.size());
        check(amdg_grid_elements(grid_, lv.data(), sp.data()), "amdg_grid_elements");
        level.assign(lv.begin(), lv.end());
        suppt.assign(sp.begin(), sp.end());
    }
    // coefficients of all elements, element blocks in the library's element order
    std::vector<double> coefficients() const {
        std::vector<double> u(size_basis_alpt());
        check(amdg_grid_get_coefficients(grid_, u.data(), int64_t(u.size())), "amdg_grid_get_coefficients");
        return u;
    }
    // Element::ucoe_ut of every element (second-order-in-time problems)
    std::vector<double> ucoe_ut() const {
        std::vector<double> v(size_basis_alpt());
        check(amdg_grid_get_velocity(grid_, v.data(), int64_t(v.size())), "amdg_grid_get_velocity");
        return v;
    }
    void copy_ucoe_to_ucoe_ut() {
        const std::vector<double> u = coefficients();
        check(amdg_grid_set_velocity(grid_, u.data(), int64_t(u.size())), "amdg_grid_set_velocity");
    }
    void set_ucoe_ut_zero() {
        const std::vector<double> z(size_basis_alpt(), 0.0);
        check(amdg_grid_set_velocity(grid_, z.data(), int64_t(z.size())), "amdg_grid_set_velocity");
    }
    void set_ucoe_alpt_zero() {
        const std::vector<double> z(size_basis_alpt(), 0.0);
        check(amdg_grid_set_coefficients(grid_, z.data(), int64_t(z.size())), "amdg_grid_set_coefficients");
    }
    amdg_grid* handle() const { return grid_; }

    // Element::rhs / ucoe_alpt_predict of every element (DGSolution.h:153, 171-174)
    void set_rhs_zero() { check(amdg_grid_set_rhs_zero(grid_), "amdg_grid_set_rhs_zero"); }
    void copy_ucoe_to_predict() { check(amdg_grid_copy_ucoe_to_predict(grid_), "amdg_grid_copy_ucoe_to_predict"); }
    void copy_predict_to_ucoe() { check(amdg_grid_copy_predict_to_ucoe(grid_), "amdg_grid_copy_predict_to_ucoe"); }
    void copy_ucoe_ut_to_predict() {
        check(amdg_grid_copy_ucoe_ut_to_predict(grid_), "amdg_grid_copy_ucoe_ut_to_predict");
    }
    void copy_predict_to_ucoe_ut() {
        check(amdg_grid_copy_predict_to_ucoe_ut(grid_), "amdg_grid_copy_predict_to_ucoe_ut");
    }
    // Element::source: the registered problems have no source term; drivers' source assembly drops out
    void set_source_zero() {}
    std::vector<double> rhs() const {
        std::vector<double> r(size_basis_alpt());
        check(amdg_grid_get_rhs(grid_, r.data(), int64_t(r.size())), "amdg_grid_get_rhs");
        return r;
    }
    // the device operator behind the Lagrange-path classes of this solution (one per grid, as the
    // reference keeps the interpolation data in the elements)
    amdg_burgers_op* lagr_op() {
        if (!lagr_) {
            const std::vector<double> zero(DIM, 0.0);
            check(amdg_burgers_create(grid_, zero.data(), &lagr_), "amdg_burgers_create");
        }
        return lagr_;
    }
    // ... and behind the Hermite-path classes (HermInterpolation, HyperbolicSameFluxHermRHS; 2D)
    amdg_burgers_op* herm_op() {
        if (!herm_) {
            const std::vector<double> zero(DIM, 0.0);
            check(amdg_burgers_create_herm(grid_, zero.data(), &herm_), "amdg_burgers_create_herm");
        }
        return herm_;
    }
    // the operator an LxF penalty is added through (either Burgers operator computes it alike)
    amdg_burgers_op* penalty_op() { return herm_ ? herm_ : lagr_op(); }
    // ... and behind the wave-path classes (the registered K = (1 + a prod_d sin 2 pi x_d)^2, IPDG
    // parameter from the last DiffusionAlpt built on this solution)
    amdg_wave_op* wave_op() {
        if (!wave_) check(amdg_wave_create(grid_, wave_sigma_, 0.5, &wave_), "amdg_wave_create");
        return wave_;
    }
    void set_wave_sigma(double sigma) {
        wave_sigma_ = sigma;
        if (wave_) check(amdg_wave_set_sigma(wave_, sigma), "amdg_wave_set_sigma");
    }
    // the refine / coarsen indicator for DGSolution::prob
    void apply_indicator() {
        check(amdg_grid_set_indicator(grid_, prob == "wave" ? AMDG_INDICATOR_U_UT : AMDG_INDICATOR_U),
              "amdg_grid_set_indicator");
    }

protected:
    void release_lagr() {
        amdg_burgers_destroy(lagr_);
        lagr_ = nullptr;
        amdg_burgers_destroy(herm_);
        herm_ = nullptr;
        amdg_wave_destroy(wave_);
        wave_ = nullptr;
    }
    amdg_grid* grid_ = nullptr;
    amdg_burgers_op* lagr_ = nullptr;
    amdg_burgers_op* herm_ = nullptr;
    amdg_wave_op* wave_ = nullptr;
    double wave_sigma_ = 0.0;
    int nmax_;
};

class DGAdapt : public DGSolution {
public:
    static inline std::vector<int> indicator_var_adapt{0};
    DGAdapt(bool sparse, int level_init, int NMAX, AllBasis<AlptBasis>& a, AllBasis<LagrBasis>& l, AllBasis<HermBasis>& h,
            Hash& hash, double eps, double eta, bool /*is_find_ptr_alpt*/, bool /*is_find_ptr_intp*/,
            bool /*is_find_ptr_general*/ = false)
        : DGSolution(sparse, level_init, NMAX, a, l, h, hash), eps_(eps), eta_(eta) {}
    void init_separable_scalar(std::function<double(double, int)> f) { init_separable_scalar_sum({f}); }
    // projection with adaptive refinement from the starting level (DGAdapt.cpp:120-147); drivers
    // that pass refine_eps = 1e10 get no refinement
    void init_separable_scalar_sum(std::vector<std::function<double(double, int)>> fns) {
        detail::SepFns sf{&fns};
        check(amdg_grid_init_separable_adaptive(grid_, int(fns.size()), detail::sep_trampoline, &sf, eps_),
              "amdg_grid_init_separable_adaptive");
    }
    void refine() {
        apply_indicator();
        check(amdg_grid_refine(grid_, nullptr, eps_, nullptr), "amdg_grid_refine");
    }
    void coarsen() {
        apply_indicator();
        check(amdg_grid_coarsen(grid_, eta_, nullptr), "amdg_grid_coarsen");
    }
    double refine_eps() const { return eps_; }
    double coarsen_eta() const { return eta_; }

protected:
    double eps_, eta_;
};

namespace detail {
struct PointFn {
    const std::function<double(std::vector<double>, int)>* f;
};
inline void point_trampoline(const double* x, int64_t n, int dim, double* out, void* user) {
    const auto& f = *static_cast<PointFn*>(user)->f;
    std::vector<double> p(dim);
    for (int64_t i = 0; i < n; ++i) {
        p.assign(x + i * dim, x + (i + 1) * dim);
        out[i] = f(p, 0);
    }
}
}  // namespace detail

// DGAdaptIntp (DGAdaptIntp.h): initialisation by adaptive Lagrange interpolation, with the
// degree and node layout of LagrBasis (PMAX 3 or 5 with msh_case 1, or 4 with msh_case 2)
class DGAdaptIntp : public DGAdapt {
public:
    DGAdaptIntp(bool sparse, int level_init, int NMAX, AllBasis<AlptBasis>& a, AllBasis<LagrBasis>& l,
                AllBasis<HermBasis>& h, Hash& hash, double eps, double eta, bool find_alpt, bool find_intp,
                const OperatorMatrix1D<LagrBasis, LagrBasis>&, const OperatorMatrix1D<HermBasis, HermBasis>&)
        : DGAdapt(sparse, level_init, NMAX, a, l, h, hash, eps, eta, find_alpt, find_intp) {}
    void init_adaptive_intp(std::function<double(std::vector<double>, int)> f) {
        const bool ok = ((LagrBasis::PMAX == 3 || LagrBasis::PMAX == 5) && LagrBasis::msh_case == 1) ||
                        (LagrBasis::PMAX == 4 && LagrBasis::msh_case == 2);
        if (!ok) throw Error(AMDG_ERR_ARG, "init_adaptive_intp: Lagrange PMAX 3 or 5 (msh_case 1) or 4 (msh_case 2) only");
        detail::PointFn pf{&f};
        check(amdg_grid_init_adaptive_intp(grid_, LagrBasis::PMAX, detail::point_trampoline, &pf, eps_, nullptr),
              "amdg_grid_init_adaptive_intp");
    }
    // L2 distance to the solution held by `exact_solu` (the reference's name for the argument;
    // its drivers pass the numerical solution to the interpolated exact one)
    double get_L2_error_split_adaptive_intp_scalar(DGSolution& exact_solu) const {
        double err = 0.0;
        check(amdg_grid_l2_error_split_grid(grid_, exact_solu.handle(), &err), "amdg_grid_l2_error_split_grid");
        return err;
    }
};

// ---- linear constant-coefficient operator + explicit RK ----------------------
class HyperbolicAlpt {
public:
    HyperbolicAlpt(DGSolution& dg, OperatorMatrix1D<AlptBasis, AlptBasis>&) : dg_(dg) {}
    HyperbolicAlpt(const HyperbolicAlpt&) = delete;
    ~HyperbolicAlpt() { amdg_linear_destroy(op_); }
    void assemble_matrix_scalar(const std::vector<double>& coef) {
        amdg_linear_destroy(op_);
        op_ = nullptr;
        check(amdg_linear_create(dg_.handle(), coef.data(), &op_), "amdg_linear_create");
    }
    // assemble_matrix_flx_scalar(dim, sign, coef) (BilinearForm.cpp:759-769): coef times ulft_vjp
    // (sign -1) or urgt_vjp (sign 1) along dim.  The terms are recorded; the pair
    // (d, -1, alpha_d / 2) + (d, 1, -alpha_d / 2) for every d is the global Lax-Friedrichs penalty
    // -alpha_d / 2 [u][v], which add_rhs_matrix applies on the device (lxf_alpha)
    void assemble_matrix_flx_scalar(int dim, int sign, double coefficient) {
        if (dim < 0 || dim >= DGSolution::DIM || (sign != -1 && sign != 1))
            throw Error(AMDG_ERR_ARG, "assemble_matrix_flx_scalar: bad dimension or sign");
        if (flx_.empty()) flx_.assign(size_t(2 * DGSolution::DIM), 0.0);
        flx_[size_t(2 * dim + (sign == 1 ? 1 : 0))] += coefficient;
    }
    std::vector<double> lxf_alpha() const {
        std::vector<double> alpha(DGSolution::DIM);
        for (int d = 0; d < DGSolution::DIM && !flx_.empty(); ++d) {
            alpha[size_t(d)] = 2.0 * flx_[size_t(2 * d)];
            if (flx_[size_t(2 * d + 1)] != -flx_[size_t(2 * d)])
                throw Error(AMDG_ERR_ARG, "HyperbolicAlpt: only Lax-Friedrichs pairs (d, -1, a/2), (d, 1, -a/2) are supported");
        }
        if (flx_.empty()) throw Error(AMDG_ERR_ARG, "HyperbolicAlpt: no flux terms assembled");
        return alpha;
    }
    amdg_linear_op* handle() const { return op_; }
    DGSolution& solution() const { return dg_; }

private:
    DGSolution& dg_;
    amdg_linear_op* op_ = nullptr;
    std::vector<double> flx_;  // [dim][sign -1, +1] coefficients of assemble_matrix_flx_scalar
};

// ExplicitRK on a DGSolution (ODESolver.h:5-38, 93): init() keeps the coefficients at t_n,
// set_rhs_zero / add_rhs_to_eigenvec act on the solver's own rhs vector, step_stage updates the
// solution, final() zeroes the solver's rhs.
class ExplicitRK {
public:
    ExplicitRK(DGSolution& dg, double dt, int scheme, int stages) : dg_(dg), dt_(dt), scheme_(scheme), num_stage(stages) {}
    ExplicitRK(const ExplicitRK&) = delete;
    virtual ~ExplicitRK() { amdg_ode_destroy(ode_); }
    void init() {
        amdg_ode_destroy(ode_);
        ode_ = nullptr;
        check(amdg_ode_create(dg_.handle(), scheme_, dt_, &ode_), "amdg_ode_create");
    }
    void set_rhs_zero() { check(amdg_ode_set_rhs_zero(need()), "amdg_ode_set_rhs_zero"); }
    void add_rhs_to_eigenvec() { check(amdg_ode_add_rhs_to_eigenvec(need()), "amdg_ode_add_rhs_to_eigenvec"); }
    void step_stage(int stage) { check(amdg_ode_step_stage(need(), stage), "amdg_ode_step_stage"); }
    void final() { check(amdg_ode_final(need()), "amdg_ode_final"); }
    // ODESolver::add_rhs_matrix (ODESolver.h:30): the solver's rhs += the operator's matrix times
    // the current solution, for the Lax-Friedrichs matrix a driver assembles with
    // assemble_matrix_flx_scalar.  The penalty is computed into Element::rhs (zeroed first, so it
    // holds the penalty alone afterwards) and added to the solver's rhs.
    void add_rhs_matrix(const HyperbolicAlpt& lin) {
        const std::vector<double> alpha = lin.lxf_alpha();
        dg_.set_rhs_zero();
        check(amdg_lagr_rhs_add(dg_.penalty_op(), AMDG_LAGR_RHS_PENALTY, alpha.data(), precision), "add_rhs_matrix");
        check(amdg_ode_add_rhs_to_eigenvec(need()), "amdg_ode_add_rhs_to_eigenvec");
    }

private:
    amdg_ode* need() {
        if (!ode_) throw Error(AMDG_ERR_STATE, "ExplicitRK: init() first");
        return ode_;
    }
    DGSolution& dg_;
    double dt_;
    int scheme_;
    amdg_ode* ode_ = nullptr;

public:
    const int num_stage;
};

class ForwardEuler : public ExplicitRK {
public:
    ForwardEuler(DGSolution& dg, double dt) : ExplicitRK(dg, dt, AMDG_ODE_FORWARD_EULER, 1) {}
    // on a flux-assembled linear form (the Lax-Friedrichs matrix): stage by stage, the matrix
    // added by add_rhs_matrix
    ForwardEuler(HyperbolicAlpt& lin, double dt) : ExplicitRK(lin.solution(), dt, AMDG_ODE_FORWARD_EULER, 1) {}
};

class RK3SSP : public ExplicitRK {
public:
    // on a DGSolution, stage by stage (ODESolver.h:183-198)
    RK3SSP(DGSolution& dg, double dt) : ExplicitRK(dg, dt, AMDG_ODE_RK3SSP, 3), op_(nullptr) {}
    // on an assembled linear operator: whole steps (RK3SSP::step_rk, ODESolver.cpp:261-271); on a
    // linear form with only flux terms assembled (the Lax-Friedrichs matrix of the Burgers
    // drivers), stage by stage with add_rhs_matrix
    RK3SSP(HyperbolicAlpt& op, double dt, amdg_precision prec = AMDG_PREC_FP64)
        : ExplicitRK(op.solution(), dt, AMDG_ODE_RK3SSP, 3), op_(op.handle() ? &op : nullptr), dt_(dt), prec_(prec) {}
    void init() {
        if (!op_) ExplicitRK::init();  // the linear form keeps its state on the device
    }
    void step_rk() {
        if (!op_) throw Error(AMDG_ERR_STATE, "RK3SSP::step_rk needs the operator form");
        check(amdg_rk3ssp_steps(op_->handle(), dt_, 1, prec_), "amdg_rk3ssp_steps");
    }
    void final() {
        if (!op_) ExplicitRK::final();
    }

private:
    HyperbolicAlpt* op_;
    double dt_ = 0.0;
    amdg_precision prec_ = AMDG_PREC_FP64;
};

// ---- Lagrange interpolation of the nonlinear flux, term by term --------------------
struct FluxFunction {
    static double burgers_flux_scalar(const double u) { return u * u * 0.5; }
    static double burgers_flux_1st_derivative_scalar(const double u) { return u; }
    static double burgers_flux_2nd_derivative_scalar(const double) { return 1.; }
};

// FastLagrIntp(dg, Lag_pt_Alpt_1D, Lag_pt_Alpt_1D_d1) (FastMultiplyLU.h:194-205): the tables
// live in the device operator; the object only carries the solution.
class FastLagrIntp {
public:
    FastLagrIntp(DGSolution& dg, const std::vector<std::vector<double>>&, const std::vector<std::vector<double>>&)
        : dg_(dg) {}
    DGSolution& solution() const { return dg_; }

private:
    DGSolution& dg_;
};

namespace detail {
// the registered coefficient of the wave operator, K = (1 + a prod_d sin(2 pi x_d))^2, a = 0.5
inline double wave_coefficient(const std::vector<double>& x) {
    double prod = 1.0;
    for (double xd : x) prod *= std::sin(2.0 * 3.14159265358979323846 * xd);
    const double c = 1.0 + 0.5 * prod;
    return c * c;
}
inline void require_wave_coefficient(const std::function<double(std::vector<double>, int)>& coe, const char* where) {
    const std::vector<std::vector<double>> xs{{0.125, 0.3, 0.7}, {0.61, 0.2, 0.45}, {0.9, 0.35, 0.15}};
    for (const auto& x3 : xs) {
        const std::vector<double> x(x3.begin(), x3.begin() + DGSolution::DIM);
        for (int d = 0; d < DGSolution::DIM; ++d)
            if (std::abs(coe(x, d) - wave_coefficient(x)) > 1e-12 * wave_coefficient(x))
                throw Error(AMDG_ERR_ARG, std::string(where) +
                                              ": only the coefficient (1 + 0.5 prod_d sin(2 pi x_d))^2 is registered");
    }
}
}  // namespace detail

// LagrInterpolation (Interpolation.h:36-129)
class LagrInterpolation {
public:
    explicit LagrInterpolation(DGSolution& dg) : dg_(dg) {}
    // the 1D tables the reference exposes for FastLagrIntp (built on the device instead)
    std::vector<std::vector<double>> Lag_pt_Alpt_1D, Lag_pt_Alpt_1D_d1;
    // LagrInterpolation::nonlinear_Lagr_fast (Interplation.cpp:4033-4047): flux coefficients of
    // the current solution, kept for the HyperbolicLagrRHS calls that follow
    void nonlinear_Lagr_fast(std::function<double(std::vector<double>, int, int)> func,
                             const std::vector<std::vector<bool>>& /*is_intp: the flux is the same in every dimension*/,
                             FastLagrIntp& /*fast*/) {
        for (double u : {0.375, -1.3125, 2.25})
            for (int d = 0; d < DGSolution::DIM; ++d)
                if (func(std::vector<double>{u}, 0, d) != FluxFunction::burgers_flux_scalar(u))
                    throw Error(AMDG_ERR_ARG, "LagrInterpolation::nonlinear_Lagr_fast: only the Burgers flux u^2/2 is registered");
        check(amdg_lagr_interpolate(dg_.lagr_op(), precision), "amdg_lagr_interpolate");
    }
    // LagrInterpolation::var_coeff_gradu_Lagr_fast / var_coeff_u_Lagr_fast (Interpolation.h:40-47):
    // K du/dx_d (every d) or K u of the current solution at the interpolation points and their
    // interpolation coefficients, kept for the DiffusionRHS calls that follow
    void var_coeff_gradu_Lagr_fast(std::function<double(std::vector<double>, int)> coe,
                                   const std::vector<std::vector<bool>>& /*is_intp*/, FastLagrIntp& /*fast*/) {
        detail::require_wave_coefficient(coe, "LagrInterpolation::var_coeff_gradu_Lagr_fast");
        check(amdg_wave_interpolate(dg_.wave_op(), AMDG_WAVE_INTERP_GRADU, precision), "amdg_wave_interpolate");
    }
    void var_coeff_u_Lagr_fast(std::function<double(std::vector<double>, int)> coe,
                               const std::vector<std::vector<bool>>& /*is_intp*/, FastLagrIntp& /*fast*/) {
        detail::require_wave_coefficient(coe, "LagrInterpolation::var_coeff_u_Lagr_fast");
        check(amdg_wave_interpolate(dg_.wave_op(), AMDG_WAVE_INTERP_U, precision), "amdg_wave_interpolate");
    }

private:
    DGSolution& dg_;
};

// HyperbolicLagrRHS (FastMultiplyLU.h:575-586): adds into Element::rhs
class HyperbolicLagrRHS {
public:
    HyperbolicLagrRHS(DGSolution& dg, const OperatorMatrix1D<LagrBasis, AlptBasis>&) : dg_(dg) {}
    void rhs_vol_scalar() { check(amdg_lagr_rhs_add(dg_.lagr_op(), AMDG_LAGR_RHS_VOL, nullptr, precision), "rhs_vol_scalar"); }
    void rhs_flx_intp_scalar() {
        check(amdg_lagr_rhs_add(dg_.lagr_op(), AMDG_LAGR_RHS_FLX, nullptr, precision), "rhs_flx_intp_scalar");
    }

private:
    DGSolution& dg_;
};

// HyperbolicAlptRHS (FastMultiplyLU.h:623-629): the LxF penalty, added into Element::rhs
class HyperbolicAlptRHS {
public:
    HyperbolicAlptRHS(DGSolution& dg, const OperatorMatrix1D<AlptBasis, AlptBasis>&) : dg_(dg) {}
    void rhs_flx_penalty_scalar(const std::vector<double>& lax_alpha) {
        if (int(lax_alpha.size()) != DGSolution::DIM) throw Error(AMDG_ERR_ARG, "rhs_flx_penalty_scalar: one alpha per dimension");
        check(amdg_lagr_rhs_add(dg_.lagr_op(), AMDG_LAGR_RHS_PENALTY, lax_alpha.data(), precision),
              "rhs_flx_penalty_scalar");
    }

private:
    DGSolution& dg_;
};

// ---- cubic Hermite interpolation of the flux, term by term (02_hyperbolic_05_burgers_adapt.cpp) ----
// FastHermIntp(dg, Her_pt_Alpt_1D) (FastMultiplyLU.h:224-235): the table lives in the device operator
class FastHermIntp {
public:
    FastHermIntp(DGSolution& dg, const std::vector<std::vector<double>>&) : dg_(dg) {}
    DGSolution& solution() const { return dg_; }

private:
    DGSolution& dg_;
};

// HermInterpolation (Interpolation.h:251-311), HermBasis PMAX 3 with msh_case 1, 2D
class HermInterpolation {
public:
    explicit HermInterpolation(DGSolution& dg) : dg_(dg) {}
    std::vector<std::vector<double>> Her_pt_Alpt_1D;  // built on the device instead
    // HermInterpolation::nonlinear_Herm_2D_fast (Interplation.cpp:4609-4621): u_h and its slopes at
    // the Hermite points, f, f' u_x, f' u_y, f'' u_x u_y + f' u_xy there and their Hermite
    // surpluses, kept for the HyperbolicSameFluxHermRHS calls that follow.  The registered flux is
    // Burgers' (f = u^2/2, f' = u, f'' = 1); other functions are refused.
    void nonlinear_Herm_2D_fast(std::function<double(std::vector<double>, int, int)> func,
                                std::function<double(std::vector<double>, int, int, int)> func_d1,
                                std::function<double(std::vector<double>, int, int, int, int)> func_d2,
                                const std::vector<std::vector<bool>>& /*is_intp: the same flux in x and y*/,
                                FastHermIntp& /*fast*/) {
        if (DGSolution::DIM != 2 || HermBasis::PMAX != 3)
            throw Error(AMDG_ERR_ARG, "HermInterpolation::nonlinear_Herm_2D_fast: 2D with HermBasis::PMAX = 3");
        for (double u : {0.375, -1.3125, 2.25})
            for (int d = 0; d < DGSolution::DIM; ++d)
                if (func(std::vector<double>{u}, 0, d) != FluxFunction::burgers_flux_scalar(u) ||
                    func_d1(std::vector<double>{u}, 0, d, 0) != FluxFunction::burgers_flux_1st_derivative_scalar(u) ||
                    func_d2(std::vector<double>{u}, 0, d, 0, 0) != FluxFunction::burgers_flux_2nd_derivative_scalar(u))
                    throw Error(AMDG_ERR_ARG, "HermInterpolation::nonlinear_Herm_2D_fast: only the Burgers flux is registered");
        check(amdg_lagr_interpolate(dg_.herm_op(), precision), "amdg_lagr_interpolate (Hermite)");
    }
    // HermInterpolation::nonlinear_Herm_2D_PMAX5_scalar_fast (Interplation.cpp:5001-5017), the quintic
    // Hermite variant a driver selects with HermBasis::PMAX = 5: declared so such drivers compile
    // unchanged; not built on the device, so it reports AMDG_ERR_ARG
    void nonlinear_Herm_2D_PMAX5_scalar_fast(std::function<double(std::vector<double>, int, int)>,
                                             std::function<double(std::vector<double>, int, int, int)>,
                                             std::function<double(std::vector<double>, int, int, int, int)>,
                                             std::function<double(std::vector<double>, int, int, int, int, int)>,
                                             std::function<double(std::vector<double>, int, int, int, int, int, int)>,
                                             const std::vector<std::vector<bool>>&, FastHermIntp&) {
        throw Error(AMDG_ERR_ARG, "HermInterpolation::nonlinear_Herm_2D_PMAX5_scalar_fast: only HermBasis::PMAX = 3 is built");
    }

private:
    DGSolution& dg_;
};

// HyperbolicSameFluxHermRHS (FastMultiplyLU.h:477-499): adds into Element::rhs
class HyperbolicSameFluxHermRHS {
public:
    HyperbolicSameFluxHermRHS(DGSolution& dg, const OperatorMatrix1D<HermBasis, AlptBasis>&) : dg_(dg) {}
    void rhs_vol_scalar() { check(amdg_lagr_rhs_add(dg_.herm_op(), AMDG_LAGR_RHS_VOL, nullptr, precision), "rhs_vol_scalar"); }
    void rhs_flx_intp_scalar() {
        check(amdg_lagr_rhs_add(dg_.herm_op(), AMDG_LAGR_RHS_FLX, nullptr, precision), "rhs_flx_intp_scalar");
    }

private:
    DGSolution& dg_;
};

// ---- variable-coefficient wave equation, term by term (03_wave_06_var_coeff_adapt.cpp) -------
// DiffusionAlpt(dg, oper, sigma) + assemble_matrix_flx_ujp_vjp (BilinearForm.h): the IPDG term
// -sigma/dx [u][v]; on the device it is the operator's last term group, applied to the current u.
class DiffusionAlpt {
public:
    DiffusionAlpt(DGSolution& dg, OperatorMatrix1D<AlptBasis, AlptBasis>&, double sigma) : dg_(dg) {
        dg_.set_wave_sigma(sigma);
    }
    void assemble_matrix_flx_ujp_vjp() {}
    DGSolution& solution() const { return dg_; }

private:
    DGSolution& dg_;
};


// DiffusionRHS (FastMultiplyLU.h:655-676): the interface and volume terms of div(K grad u), added
// into Element::rhs from the interpolations of K grad u and K u
class DiffusionRHS {
public:
    DiffusionRHS(DGSolution& dg, OperatorMatrix1D<LagrBasis, AlptBasis>&) : dg_(dg) {}
    void rhs_flx_gradu() { add(AMDG_WAVE_RHS_FLX_GRADU, "DiffusionRHS::rhs_flx_gradu"); }
    void rhs_vol() { add(AMDG_WAVE_RHS_VOL, "DiffusionRHS::rhs_vol"); }
    void rhs_flx_u() { add(AMDG_WAVE_RHS_FLX_U, "DiffusionRHS::rhs_flx_u"); }

private:
    void add(int group, const char* where) { check(amdg_wave_rhs_add(dg_.wave_op(), group, precision), where); }
    DGSolution& dg_;
};

// The second-order-in-time integrators on (u, u_t) (ODESolver.h:257-371): init keeps the state at
// t_n; rhs_to_eigenvec takes Element::rhs as the solver's rhs, add_rhs_matrix adds the IPDG term of
// the current u; step_stage writes the stage state into the solution; final zeroes the solver's rhs.
class RKODE2nd {
public:
    RKODE2nd(DiffusionAlpt& op, double dt, int scheme, int stages)
        : op_(op), dg_(op.solution()), dt_(dt), scheme_(scheme), num_stage(stages) {}
    RKODE2nd(const RKODE2nd&) = delete;
    virtual ~RKODE2nd() { amdg_ode_destroy(ode_); }
    void init() {
        amdg_ode_destroy(ode_);
        ode_ = nullptr;
        check(amdg_ode_create(dg_.handle(), scheme_, dt_, &ode_), "amdg_ode_create");
    }
    void rhs_to_eigenvec() {
        check(amdg_ode_set_rhs_zero(need()), "amdg_ode_set_rhs_zero");
        check(amdg_ode_add_rhs_to_eigenvec(need()), "amdg_ode_add_rhs_to_eigenvec");
    }
    void add_rhs_matrix(DiffusionAlpt& op) {
        check(amdg_ode_add_wave_penalty(need(), op.solution().wave_op()), "RKODE2nd::add_rhs_matrix");
    }
    void step_stage(int stage) { check(amdg_ode_step_stage(need(), stage), "amdg_ode_step_stage"); }
    void final() { check(amdg_ode_final(need()), "amdg_ode_final"); }

protected:
    amdg_ode* need() {
        if (!ode_) throw Error(AMDG_ERR_STATE, "RKODE2nd: init() first");
        return ode_;
    }
    DiffusionAlpt& op_;
    DGSolution& dg_;
    double dt_;
    int scheme_;
    amdg_ode* ode_ = nullptr;

public:
    const int num_stage;
};

class EulerODE2nd : public RKODE2nd {
public:
    EulerODE2nd(DiffusionAlpt& op, double dt) : RKODE2nd(op, dt, AMDG_ODE_EULER_ODE2ND, 1) {}
    // EulerODE2nd::step_rk (ODESolver.cpp:394-399): the rhs is recomputed as the operator matrix
    // (the IPDG term) times u, whatever was assembled before
    void step_rk() {
        check(amdg_ode_set_rhs_zero(need()), "amdg_ode_set_rhs_zero");
        add_rhs_matrix(op_);
        step_stage(0);
    }
};

class RK4ODE2nd : public RKODE2nd {
public:
    RK4ODE2nd(DiffusionAlpt& op, double dt) : RKODE2nd(op, dt, AMDG_ODE_RK4ODE2ND, 4) {}
};

// ---- nonlinear flux (Burgers) through Lagrange interpolation ------------------
// The reference composes LagrInterpolation::nonlinear_Lagr_fast,
// HyperbolicLagrRHS::rhs_vol_scalar / rhs_flx_intp_scalar and
// HyperbolicAlptRHS::rhs_flx_penalty_scalar per stage; on the device the
// whole right-hand side is one call for the registered flux u^2/2.
class BurgersLagrRHS {
public:
    BurgersLagrRHS(DGSolution& dg, const std::vector<double>& lxf_alpha) {
        check(amdg_burgers_create(dg.handle(), lxf_alpha.data(), &op_), "amdg_burgers_create");
    }
    BurgersLagrRHS(const BurgersLagrRHS&) = delete;
    ~BurgersLagrRHS() { amdg_burgers_destroy(op_); }
    void rk3_step(double dt, amdg_precision prec = AMDG_PREC_FP64) {
        check(amdg_burgers_rk3_steps(op_, dt, 1, prec), "amdg_burgers_rk3_steps");
    }
    amdg_burgers_op* handle() const { return op_; }

private:
    amdg_burgers_op* op_ = nullptr;
};

// ---- variable-coefficient wave equation (example/03_wave_06_var_coeff_adapt.cpp) ----
// DiffusionRHS with the Lagrange-interpolated K grad u and K u, the IPDG penalty -sigma/dx [u][v]
// and RK4ODE2nd, K = (1 + a prod_d sin(2 pi x_d))^2: the library registers the coefficient
// function (a device function cannot be a host std::function).  adaptive_step runs the loop body
// of the example (EulerODE2nd predictor, refine, four RK4ODE2nd stages, coarsen).
class WaveLagrRHS {
public:
    WaveLagrRHS(DGSolution& dg, double sigma_ipdg, double amplitude = 0.5) {
        check(amdg_wave_create(dg.handle(), sigma_ipdg, amplitude, &op_), "amdg_wave_create");
    }
    WaveLagrRHS(const WaveLagrRHS&) = delete;
    ~WaveLagrRHS() { amdg_wave_destroy(op_); }
    void rk4_step(double dt, amdg_precision prec = AMDG_PREC_FP64) {
        check(amdg_wave_rk4_steps(op_, dt, 1, prec), "amdg_wave_rk4_steps");
    }
    // one adaptive step; returns the dt taken (cfl / sum_d wave_speed 2^maxlevel_d)
    double adaptive_step(double cfl, double wave_speed, double eps, double eta, amdg_precision prec = AMDG_PREC_FP64) {
        double dt = 0;
        check(amdg_wave_adaptive_step(op_, cfl, wave_speed, eps, eta, prec, &dt), "amdg_wave_adaptive_step");
        return dt;
    }
    amdg_wave_op* handle() const { return op_; }

private:
    amdg_wave_op* op_ = nullptr;
};

inline void synchronize() { check(amdg_context_synchronize(Runtime::context()), "amdg_context_synchronize"); }

}  // namespace amdg_gpu
