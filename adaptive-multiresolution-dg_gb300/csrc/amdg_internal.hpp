// Internal declarations shared by the host set-up code and the CUDA
// translation units of libamdg_gb300.
#pragma once

#include <cstdint>
#include <string>
#include <unordered_map>
#include <vector>

#include "amdg.h"

namespace amdg {

constexpr double kRoundOff = 1e-13;  // Const::ROUND_OFF (libs.h:28)
constexpr int kMaxDim = 6;

// ---- error plumbing ------------------------------------------------------
void set_error(const std::string& msg);
amdg_status fail(amdg_status s, const std::string& msg);

// ---- 1D Alpert basis and operator matrices (host, FP64) -------------------
struct Basis1D {
    int k;     // polynomial degree
    int nmax;  // finest level
    int num_elem() const { return 1 << nmax; }
    int num_basis() const { return num_elem() * (k + 1); }
    // value (or derivative) of basis function `order` at x; sgn -1/0/+1 = left limit / value / right limit
    double eval(int order, int deriv, double x, int sgn) const;
};

// level n and odd support index j of 1D element order o
inline void elem_of_order(int o, int* n, int* j) {
    if (o == 0) { *n = 0; *j = 1; return; }
    int lev = 0;
    while ((1 << lev) <= o) ++lev;
    *n = lev;
    *j = 2 * (o - (1 << (lev - 1))) + 1;
}
inline int order_of_elem(int n, int j) { return n == 0 ? 0 : (1 << (n - 1)) + (j - 1) / 2; }
inline int level_of_order(int o) { int lev = 0; while ((1 << lev) <= o) ++lev; return lev; }
// support of 1D element order o in units of 2^-nmax
inline void support_units(int o, int nmax, int64_t* a, int64_t* b) {
    int n, j;
    elem_of_order(o, &n, &j);
    if (n <= 1) { *a = 0; *b = int64_t(1) << nmax; return; }
    const int64_t w = int64_t(1) << (nmax - n + 1);
    *a = int64_t((j - 1) / 2) * w;
    *b = *a + w;
}

// Dense 1D matrices, row = solution basis, col = test basis (OperatorMatrix1D layout).
struct Oper1D {
    int nb = 0;
    std::vector<double> u_v, u_vx, ulft_vjp, urgt_vjp;
};
void build_oper1d(const Basis1D& b, Oper1D* out, bool want_u_v);

// n-point Gauss-Legendre nodes and weights on [-1, 1] (n <= 16)
void gauss_legendre(int n, double* x, double* w);

// A separable factor given point by point or in bulk.
struct Fn1d {
    amdg_fn1d f = nullptr;
    amdg_fn1d_batch fb = nullptr;
    void* user = nullptr;
    void eval(const double* x, int64_t n, int d, int term, double* out) const {
        if (fb) {
            fb(x, n, d, term, out, user);
            return;
        }
        for (int64_t i = 0; i < n; ++i) out[i] = f(x[i], d, term, user);
    }
};
// 1D projection of f(., d, term) onto every basis function (Basis::product_function).
void project_1d(const Basis1D& b, const Fn1d& f, int d, int term, double* out);

// ---- Lagrange interpolation path (hierarchical Lagrange of degree 3 or 4) ----
constexpr int kMaxLagrPoints = 6;  // points per element and dimension (degree 5)

// Node layout of a hierarchical Lagrange basis (LagrBasis.cpp:33-155): degree 3
// with msh_case 1 (the Burgers examples) or degree 4 with msh_case 2 (the wave
// example, 03_wave_06_var_coeff_adapt.cpp:53-54).
struct LagrSpec {
    int p1 = 4;                               // points per element and dimension
    double pt0[kMaxLagrPoints];               // level-0 interpolation points on [-1, 1]
    double pt1[kMaxLagrPoints];               // level >= 1 points, in the element's own [-1, 1]
    double node0[kMaxLagrPoints];             // level-0 polynomial nodes
    double half[2][kMaxLagrPoints];           // level-1 polynomial nodes of the left / right half
    int side[kMaxLagrPoints];                 // level-1 function p lives on the left (0) / right (1) half
    int node[kMaxLagrPoints];                 // ... and interpolates at half[side][node]
};
// the layout of the given degree (3 or 4); nullptr for any other
const LagrSpec* lagr_spec(int degree);

struct LagrTables {
    const LagrSpec* spec = nullptr;
    int p1 = 4;
    int n_lagr = 0, n_alpt = 0;
    std::vector<double> a2p;    // [n_alpt][n_lagr]: Alpert basis at Lagrange points
    std::vector<double> lv;     // [n_lagr][n_alpt]: u_v   (Lagrange x Alpert)
    std::vector<double> lvx;    // [n_lagr][n_alpt]: u_vx
    std::vector<double> lflx;   // [n_lagr][n_alpt]: ulft_vjp + urgt_vjp
    std::vector<double> ajump;  // [n_alpt][n_alpt]: ujp_vjp (Alpert x Alpert)
    // diffusion terms (built when asked for)
    std::vector<double> a2pd;   // [n_alpt][n_lagr]: Alpert basis derivative at Lagrange points
    std::vector<double> ljv;    // [n_lagr][n_alpt]: ujp_vxlft + ujp_vxrgt
    std::vector<double> pts;    // [n_lagr]: coordinate of each Lagrange point
    std::vector<int32_t> anc_order;  // [n_elem1d][p1]: 1D order of the ancestor owning surplus point ic
    std::vector<int32_t> anc_point;  // [n_elem1d][p1]: its point index
    std::vector<int32_t> anc_rank;   // [n_elem1d][p1]: rank of its position among the p1
    double weight[kMaxLagrPoints * kMaxLagrPoints] = {0};  // [p0][rank]
    bool herm = false;  // Hermite weights: scaled per element level (build_herm_tables)
};
// basis function `order` (1D element order * p1 + p) at x, one-sided for sgn = -1 / 1
double lagr_eval(const LagrSpec& s, int order, double x, int sgn);
double lagr_point(const LagrSpec& s, int o, int p);
// integral of the square of every 1D Lagrange basis function (order * p1 + p) over its support,
// 10-point Gauss on each half (the diagonal of the Lagrange x Lagrange u_v)
void lagr_mass_diag(const LagrSpec& S, int nmax, std::vector<double>* out);
// all tables for Lagrange degree `degree` (3 or 4)
void build_lagr_tables(const Basis1D& alpt, int degree, LagrTables* t, bool diffusion = false);
// anc_order/anc_point/anc_rank only (t->spec and t->p1 set from `degree`)
void build_lagr_ancestors(const Basis1D& alpt, int degree, LagrTables* t);
// interpolation basis (S: Lagrange; nullptr: cubic Hermite) x Alpert products lv, lvx, lflx
void build_interp_products(const Basis1D& alpt, const LagrSpec* S, int P1, LagrTables* t);
// Cubic Hermite interpolation (HermBasis with PMAX 3, msh_case 1): dof p of a 1D element is
// point p % 2 and derivative order p / 2.  Basis function `order` (1D order * 4 + p), or its
// derivative, at x (one-sided for sgn = -1 / 1), the point of dof p of 1D element o, and the
// tables of the Hermite path (a2p: Alpert values or slopes at the Hermite points; the Hermite x
// Alpert products; ancestors with anc_rank = the ancestor's dof number ic0 and weight[p0][ic0]
// the level-1 weights, scaled by 2^((level - 1)(p0 / 2 - ic0 / 2)) per element level)
double herm_eval(int order, int deriv, double x, int sgn);
double herm_point(int o, int p);
void build_herm_tables(const Basis1D& alpt, LagrTables* t);
// dimension orders and L(0)/full(1)/U(2) tags of the 2^(dim-1) partial sums
void transform_schedule(int dim, std::vector<std::vector<int>>* dim_order, std::vector<std::vector<int>>* lu);

// ---- grid topology (host build, device copy) -------------------------------
struct HostGrid {
    int dim = 0, nmax = 0, k = 0, sparse = 1;
    int64_t num_elements = 0;
    std::vector<int32_t> order;  // num_elements x dim, 1D element orders, sorted lexicographically
    std::vector<uint64_t> key;   // packed orders (nmax bits per dimension), ascending
    // open-addressing index key -> element (load <= 1/2; built with the element set)
    std::vector<uint64_t> hkey;
    std::vector<int32_t> hval;   // -1: empty slot
    int hbits = 0;
    int64_t index_of(uint64_t k) const {
        if (hval.empty()) return -1;
        const uint64_t mask = (uint64_t(1) << hbits) - 1;
        for (uint64_t h = (k * 0x9E3779B97F4A7C15ull) >> (64 - hbits);; h = (h + 1) & mask) {
            const int32_t v = hval[h];
            if (v < 0) return -1;
            if (hkey[h] == k) return v;
        }
    }
};
// (re)build g->hkey / hval / hbits from g->key
void build_key_index(HostGrid* g);
void build_grid(int dim, int nmax, int sparse, HostGrid* g, int level_init = -1);
int64_t find_element(const HostGrid& g, const int32_t* orders);  // binary search, -1 if absent

// Batched independent grids sharing nmax, k and dim.  The 1D part depends on k and nmax only
// and is built once per batch; the element part on every element set.
struct BatchTables {
    std::vector<std::vector<int>> rel1d;  // 1D order -> related 1D orders (nonzero block)
    std::vector<int> blk_base;            // 1D order -> first block index of its row
    std::vector<double> blocks;           // [2][num_blocks][k+1][k+1]
    int num_blocks = 0;
};
void build_batch_tables(const Oper1D& op, int nmax, int np, BatchTables* out);
struct BatchTopology {
    std::vector<int64_t> row_ptr, src;   // CSR over (global element, dimension)
    std::vector<int32_t> blk;
    std::vector<double> blocks;          // [2][num_blocks][k+1][k+1]
    std::vector<int32_t> solve_of;       // global element -> solve
    std::vector<int64_t> elem_offset;    // solves + 1
    int num_blocks = 0;
};
// rows of every solve built in parallel, then concatenated in solve order
void build_batch_topology(const std::vector<const HostGrid*>& grids, const BatchTables& t, BatchTopology* out);

// Adaptivity on packed keys (one refine pass with hole filling; repeated coarsening).
// refined (optional): per element, 1 where the element was refined; force (optional): refine
// the leaves flagged instead of those with norm > eps
std::vector<uint64_t> refine_keys(const HostGrid& g, const double* norms, double eps, std::vector<uint8_t>* refined = nullptr,
                                  const uint8_t* force = nullptr);
void leaf_flags(const HostGrid& g, std::vector<uint8_t>* leaf);
// [e][d][2]: parent and grandparent in dimension d, -1 when absent
void parent_table(const HostGrid& g, std::vector<int32_t>* pg);
// parent tables of several grids whose elements are concatenated (offsets: grids + 1), with
// indices into the concatenation
void batch_parent_table(const std::vector<const HostGrid*>& grids, const std::vector<int64_t>& offset,
                        std::vector<int32_t>* pg);
// the adaptation between two steps on the host key set: coarsen (norm < eta), then give the
// chosen elements (force, or norm > eps without it) that the coarsening kept their children;
// carry[e] = 0 for the old elements that the coarsening removed (they start at zero if the
// refinement adds them back).  norms and force are per old element.
void adapt_keys_between_steps(const HostGrid& g, const double* norms, const uint8_t* force, double eps, double eta,
                              std::vector<uint64_t>* keys, std::vector<uint8_t>* carry);
// the same for several grids in parallel (norms and force over the concatenation)
void batch_adapt_keys(const std::vector<const HostGrid*>& grids, const std::vector<int64_t>& offset,
                      const double* norms, const uint8_t* force, double eps, double eta,
                      std::vector<std::vector<uint64_t>>* keys, std::vector<std::vector<uint8_t>>* carry);
// input and output widths of a classifier (capi_mlp.cu)
void mlp_shape(const amdg_mlp* m, int* n_in, int* n_out);
std::vector<uint64_t> coarsen_keys(const HostGrid& g, const double* norms, double eta);
void grid_from_keys(int dim, int nmax, int k, std::vector<uint64_t> keys, HostGrid* g);
// element norms of the separable expansion sum_t prod_d coef1d[t][d] (host, same arithmetic order as the device init)
void element_separable_norms(const HostGrid& g, const std::vector<double>& coef1d, int nterms, std::vector<double>* norms);

// Matrix-free linear operator topology: for every (element, dimension) the
// neighbours whose 1D block is nonzero, and the deduplicated 1D blocks.
struct LinearTopology {
    std::vector<int32_t> row_ptr;   // num_elements*dim + 1
    std::vector<int32_t> src;       // neighbour element
    std::vector<int32_t> blk;       // block id within its dimension
    std::vector<double> blocks;     // [dim][num_blocks][k+1][k+1] (row = solution p, col = test q)
    int num_blocks = 0;
};
void build_linear_topology(const HostGrid& g, const Oper1D& op, const double* coef, LinearTopology* out);

// Per-(element, dimension) neighbour lists of the fast transforms:
// vol = supports intersect in the dimension, flx = intersect or adjacent
// (periodic), identical indices elsewhere (Element.cpp:265-299).  Each entry
// carries the neighbour's level in that dimension for the L/U filters.
struct TransformTopology {
    std::vector<int32_t> vol_ptr, flx_ptr;       // CSR over (element, dimension): num_elements*dim + 1
    std::vector<int32_t> vol_nbr, flx_nbr;       // (element, 1D order along t) pairs, increasing order
    std::vector<int32_t> vol_split, flx_split;   // [e*dim+t]: first neighbour finer than e in t
};
void build_transform_topology(const HostGrid& g, TransformTopology* out);

// Matrices of the Lagrange path, indexed by PartialSum::mat.
enum LagrMat { kMatA2P = 0, kMatLV = 1, kMatLVX = 2, kMatLFLX = 3, kMatAJump = 4, kMatA2PD = 5, kMatLJV = 6,
               kNumLagrMats = 7 };
constexpr int kMaxTermSources = kMaxDim + 1;  // inputs a term's first sweep can read

// One term of a right-hand side or of the point values: either a partial sum
// of dim successive 1D transforms (FastRHS::transform_multiD_partial_sum,
// FastMultiplyLU.cpp:121-213; FastInterpolation, :904-968) -- in sweep j the
// transform runs along dims[j] with matrix mat[j] over the "vol" or "flx"
// (flx[j]) neighbour sets restricted by lu[j] (0 "L": finer neighbours, 1
// all, 2 "U": coarser or equal), the first sweep scaled by coef -- or (kind 1)
// the single full transform of the LxF penalty along dims[0] with the jump
// matrix on the flx sets (FastRHS::transform_ucoe_alpt_to_rhs, :46-59).
struct PartialSum {
    int8_t dims[kMaxDim], lu[kMaxDim], mat[kMaxDim], flx[kMaxDim];
    int8_t src;    // input of the first sweep (index into the launch's sources)
    int32_t kind;
    double coef;
    // as a node of a launch's sweep tree: the slice of the previous sweep this node reads (sweeps
    // after the first), and coef is the scale this sweep applies
    int32_t parent;
};
// The sweeps of a range of terms as a tree: terms whose first j sweeps coincide (same source,
// dimensions, L/U tags, matrices and neighbour sets, power-of-two coefficients moved to their last
// sweep) share those sweeps.  Nodes of sweep j at nodes[offset[j] .. offset[j] + count[j]); the last
// sweep has one node per term, in term order.
struct SweepTree {
    int offset[kMaxDim] = {0}, count[kMaxDim] = {0};
};
// nodes of the tree of terms [first, first + count) of `terms`, appended to `nodes`
SweepTree build_sweep_tree(const std::vector<PartialSum>& terms, int first, int count, int dim,
                           std::vector<PartialSum>* nodes);
// surplus ancestors: [e][d][ic] element index, ic < t.p1 (-1 for level 0 in d); false if a hole is found
bool build_surplus_ancestors(const HostGrid& g, const LagrTables& t, std::vector<int32_t>* anc);

}  // namespace amdg

// ---- opaque handle layouts (plain structs, owned by the C-ABI layer) ------
struct amdg_context {
    int device = 0;
    void* stream = nullptr;        // cudaStream_t in use
    void* own_stream = nullptr;    // stream created by the context
    int64_t launches = 0;
    int adapt_mode = 0;            // AMDG_ADAPT_DEVICE or AMDG_ADAPT_HOST (amdg_context_set_adapt_mode)
    // host phase profile (amdg_context_profile): wall seconds and calls per phase
    bool profile = false;
    double phase_sec[AMDG_PHASE_COUNT] = {0};
    int64_t phase_calls[AMDG_PHASE_COUNT] = {0};
};

namespace amdg {
// Adds the wall time of its scope to a phase of the context's profile (when enabled).
class PhaseTimer {
public:
    PhaseTimer(amdg_context* ctx, int phase);
    ~PhaseTimer();
    PhaseTimer(const PhaseTimer&) = delete;
    PhaseTimer& operator=(const PhaseTimer&) = delete;
private:
    amdg_context* ctx_;
    int phase_;
    double t0_;
};
}  // namespace amdg

namespace amdg {
// Device side of the element set (adapt_device.cu): the sorted packed keys, an open-addressing
// key -> element hash, and the grow-only work arrays of the device refine / coarsen.  Plain
// pointers so host translation units can hold it.
struct GridDevice {
    uint64_t* key = nullptr;         // sorted packed keys of the current element set
    uint64_t* key_alt = nullptr;     // the next element set is assembled here, then swapped in
    int64_t key_cap = 0;
    unsigned long long* hkey = nullptr;  // hash slots (all bits set: empty)
    int32_t* hval = nullptr;         // element index of the slot's key (-1: a key added by refinement)
    int64_t hcap = 0;                // slots (a power of two)
    int hbits = 0;
    int64_t hash_version = -1;       // element set the hash holds
    uint64_t* newk = nullptr;        // keys added by a refinement
    int64_t new_cap = 0;
    uint8_t* flag = nullptr;         // per element: refined / removed / forced
    uint8_t* force = nullptr;
    int32_t* pos = nullptr;          // exclusive scan of the kept elements (coarsen)
    int64_t flag_cap = 0;
    uint64_t* missed = nullptr;      // learned steps: leaves the criterion found above eps
    int64_t missed_cap = 0, n_missed = 0;
    void* stats = nullptr;           // device AdaptStats
    void* host_stats = nullptr;      // pinned host copy
    void* temp = nullptr;            // sort / scan scratch
    size_t temp_bytes = 0;
};
}  // namespace amdg

struct amdg_grid {
    int64_t version = 0;             // bumped whenever the element set changes
    // element-set statistics kept with every change: largest level and sum of levels per
    // dimension, largest level sum of an element (time step, coarsening passes, list bounds)
    int lev_max[amdg::kMaxDim] = {0};
    int64_t lev_sum[amdg::kMaxDim] = {0};
    int levsum_max = 0;
    // the device holds the element set (dev.key); after a device-side refine / coarsen the host
    // mirror `host` keeps only num_elements current until grid_ensure_host refreshes it
    bool host_stale = false;
    amdg::GridDevice dev;
    int64_t capacity = 0;            // elements the device arrays can hold
    amdg_context* ctx = nullptr;
    int device = 0;                  // kept so destroy never dereferences ctx
    amdg::HostGrid host;
    int block = 0;                   // (k+1)^dim
    int64_t dof = 0;
    int32_t* d_order = nullptr;      // device copy of host.order
    double* d_u = nullptr;           // FP64 coefficients (capacity elements)
    double* d_scratch = nullptr;     // reduction scratch
    size_t scratch_bytes = 0;
    // grow-only buffers of element-set changes: the spare coefficient array the
    // remap writes into (then swapped with d_u), the old-to-new index map, the
    // indicator norms
    int64_t order_capacity = 0;
    double* d_u_spare = nullptr;
    int64_t spare_capacity = 0;
    int32_t* d_map = nullptr;
    int64_t map_capacity = 0;
    double* d_norms = nullptr;
    int64_t norms_capacity = 0;
    // Element::ucoe_alpt_predict, remapped with u (new elements zero); Element::rhs, zeroed
    // when the element set changes
    double* d_pred = nullptr;
    double* d_pred_spare = nullptr;
    int64_t pred_capacity = 0, pred_spare_capacity = 0;
    double* d_rhs = nullptr;
    int64_t rhs_capacity = 0, rhs_version = -1;
    // second field v = u_t of second-order-in-time problems (Element::ucoe_ut), remapped with u
    double* d_v = nullptr;           // v_capacity elements, null until set
    double* d_v_spare = nullptr;
    int64_t v_capacity = 0, v_spare_capacity = 0;
    // Element::ucoe_ut_predict, remapped with u like d_pred
    double* d_pred_v = nullptr;
    double* d_pred_v_spare = nullptr;
    int64_t pred_v_capacity = 0, pred_v_spare_capacity = 0;
    int indicator = 0;               // AMDG_INDICATOR_U / AMDG_INDICATOR_U_UT for amdg_grid_refine / _coarsen
};

// ODESolver on a grid (ode.cu): the state at t_n (u, and u_t for the second-order schemes), the
// solver's rhs vector and the RK4ODE2nd running sums of the stage increments
struct amdg_ode {
    amdg_grid* grid = nullptr;
    int device = 0;
    int scheme = 0;        // AMDG_ODE_*
    double dt = 0.0;
    int64_t version = -1;  // element set of init()
    int64_t n = 0;         // dof
    double* d_un = nullptr;
    double* d_rhs = nullptr;
    double *d_vn = nullptr, *d_su = nullptr, *d_sv = nullptr;  // second-order schemes
};

struct amdg_linear_op {
    int64_t built_version = -1;      // grid version the topology was built for
    int64_t capacity = 0;            // dof the stage vectors can hold (a multiple of 4, with 4 spare)
    amdg_grid* grid = nullptr;
    int device = 0;                  // kept so destroy never dereferences grid
    std::vector<double> coef;
    int64_t pairs = 0;
    int num_blocks = 0;              // 1D blocks per dimension in the table
    // CSR over (element, dimension): row_ptr[e*dim + t] .. row_ptr[e*dim + t + 1]
    int32_t* d_row_ptr = nullptr;
    int32_t* d_src = nullptr;        // neighbour element index
    int32_t* d_blk = nullptr;        // block index within the dimension's table
    double* d_blocks64 = nullptr;    // [dim][num_blocks][k+1][k+1], row = solution p, col = test q
    float* d_blocks32 = nullptr;
    int32_t* d_pairs = nullptr;      // column variant: (src, blk) interleaved
    double* d_blocks64p = nullptr;   // column variant: blocks padded to a multiple of 4 entries
    float* d_blocks32p = nullptr;
    double* d_u1 = nullptr;          // RK stage vectors
    double* d_u2 = nullptr;
    float* d_shadow = nullptr;       // mixed mode: hi parts of u, u1, u2 (3 x capacity)
    float* d_lo = nullptr;           // mixed mode: lo parts of u, u1, u2 (3 x capacity)
    int* d_err = nullptr;            // set by a bounded copy wait that gave up (variant 2)
    uint32_t wait_limit = 1u << 22;  // polls of a bulk-copy wait before it gives up
    int variant[2] = {0, 0};         // kernel variant per precision, picked by the autotuner
    float variant_ms[2][4] = {{0, 0, 0, 0}, {0, 0, 0, 0}};  // measured stage time [precision][variant]
    int tma_cfg = 0;                 // configuration of the bulk-copy variant (ring depth, operator-block source)
    float tma_ms[8] = {0, 0, 0, 0, 0, 0, 0, 0};  // its measured stage time per configuration (kTmaConfigs)
    // request pipeline of amdg_rk3ssp_serve_host: three device states, copy-in / copy-out
    // streams, events (in_done[3], stepped[3], out_done[3]); created on first use
    double* d_io[3] = {nullptr, nullptr, nullptr};
    int64_t io_capacity = 0;
    void* io_stream[2] = {nullptr, nullptr};
    void* io_event[9] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
};

struct amdg_burgers_op {
    int kind = 0;                    // 0: Burgers flux u^2/2; 1: wave u_tt = div(K grad u) (amdg_wave_op)
    double sigma = 0.0;              // wave: IPDG penalty parameter
    double amp = 0.5;                // wave: K = (1 + amp prod_d sin(2 pi x_d))^2
    int64_t built_version = -1;
    int64_t capacity = 0;            // elements the work buffers can hold
    amdg_grid* grid = nullptr;
    int device = 0;
    std::vector<double> alpha;
    int p1 = 4;                      // Lagrange points per element and dimension (degree + 1)
    int points = 0;                  // p1^dim interpolation points per element
    int n1 = 0;                      // 1D elements
    // 1D matrices, FP64 and FP32 copies
    double *d_a2p = nullptr, *d_lv = nullptr, *d_lvx = nullptr, *d_lflx = nullptr, *d_ajump = nullptr;
    float *f_a2p = nullptr, *f_lv = nullptr, *f_lvx = nullptr, *f_lflx = nullptr, *f_ajump = nullptr;
    double *d_a2pd = nullptr, *d_ljv = nullptr, *d_pts = nullptr;  // wave: derivative and jump tables, point coordinates
    void *df_a2p = nullptr, *df_a2pd = nullptr;  // double-float (float2 hi, lo) copies for the mixed point values
    float *f_a2pd = nullptr, *f_ljv = nullptr;
    void* w_fields = nullptr;        // wave: (dim+1) coefficient-weighted point fields and their surpluses, 2 (dim+1) x E x p1^dim doubles
    double *d_v1 = nullptr, *d_su = nullptr, *d_sv = nullptr;  // wave: RK4ODE2nd stage v and running sums
    // neighbour lists of the fast transforms and the surplus ancestors
    int32_t *d_vol_ptr = nullptr, *d_vol_nbr = nullptr;  // nbr: (element, 1D order along t) pairs
    int32_t *d_flx_ptr = nullptr, *d_flx_nbr = nullptr;
    int32_t *d_vol_split = nullptr, *d_flx_split = nullptr;
    int32_t *d_anc = nullptr, *d_anc_point = nullptr, *d_anc_rank = nullptr;
    double weight[amdg::kMaxLagrPoints * amdg::kMaxLagrPoints] = {0};
    std::vector<std::vector<int>> sched_dims, sched_lu;
    // terms of the point values (first n_pv_terms) and of the right-hand side, in summation order
    std::vector<amdg::PartialSum> terms;
    amdg::PartialSum* d_terms = nullptr;
    int n_pv_terms = 0;
    int grp_first[3] = {0, 0, 0}, grp_count[3] = {0, 0, 0};  // Burgers: volume, interface, penalty terms
    // sweep trees of the term ranges launched so far, keyed by (first, count), their nodes on the
    // host and (uploaded whenever a tree is added or a coefficient changes) on the device
    std::vector<std::pair<std::pair<int, int>, amdg::SweepTree>> trees;
    std::vector<amdg::PartialSum> nodes;
    amdg::PartialSum* d_nodes = nullptr;
    size_t nodes_cap = 0;
    int64_t interp_version = -1;     // element set of the flux coefficients amdg_lagr_interpolate kept
    int interp_prec = -1;            // ... and their arithmetic
    // wave: element set and arithmetic of the K grad u [0] and K u [1] interpolations amdg_wave_interpolate kept
    int64_t wave_interp_version[2] = {-1, -1};
    int wave_interp_prec[2] = {-1, -1};
    int chunk = 1;  // terms per launch
    int sweep_variant = -1;  // transform sweep kernel: -1 by precision, 0 thread per output entry, 1 thread per
                             // column, 2 / 3 / 4 warp per (node, element) with 1 / 2 / 4 elements per warp
    // work buffers sized for FP64: E x p1^dim doubles each, the sweep buffers and
    // term slices chunk times that
    void *w_up = nullptr, *w_fu = nullptr, *w_a = nullptr, *w_b = nullptr, *w_u = nullptr;
    void *w_s0 = nullptr, *w_s1 = nullptr, *w_slots = nullptr;
    double *d_u1 = nullptr, *d_u2 = nullptr, *d_rhs64 = nullptr, *d_pred = nullptr;
    std::vector<double> host_norms;
    // one SSP-RK3 step captured as a CUDA graph, valid for (grid version, precision, dt)
    int32_t* d_anc_order = nullptr;  // device copy of anc_order (the device-built ancestors)
    int32_t* d_topo_cnt = nullptr;   // per (element, dimension) list lengths of the device build
    unsigned long long* d_cls = nullptr;  // learned step: [refined by the network, unsure] (device)
    unsigned long long* h_cls = nullptr;  // pinned host copy
    int32_t* d_pg = nullptr;         // [e][d][2] parent / grandparent (learned adaptivity features)
    float *d_feat = nullptr, *d_prob = nullptr;  // classifier features / probabilities
    int64_t feat_cap = 0;                        // elements the two hold
    int64_t pg_version = -1;                     // element set d_pg was built for
    std::vector<uint64_t> missed_keys;           // leaves the criterion found above eps after the last learned step
    void* graph_exec = nullptr;
    int64_t graph_version = -1;
    int graph_prec = -1;
    double graph_dt = 0.0;
    int64_t graph_launches = 0;
    int64_t stage_dof_updates = 0;  // RK stages x DOF advanced since creation
    int64_t rhs_evaluations = 0;    // right-hand sides evaluated since creation
    int64_t last_version = -1;  // configuration of the previous rk3 call
    int last_prec = -1;
    double last_dt = 0.0;
    std::vector<int32_t> anc_order;                   // surplus ancestor 1D orders (depend on nmax only)
    std::unordered_map<const void*, size_t> dev_cap;  // bytes held by each grow-only device array
};

// wave-equation operator: the Lagrange-path operator of kind 1
struct amdg_wave_op {
    amdg_burgers_op* lagr = nullptr;
};

namespace amdg {
// replace a grid's element set (coefficients carried over, new elements zero; bumps the version);
// with `carry`, only old elements e with (*carry)[e] != 0 keep their coefficients (the others
// start at zero if they are in the new set)
amdg_status grid_set_keys(amdg_grid* g, std::vector<uint64_t> keys, const std::vector<uint8_t>* carry = nullptr);
// indicator norms of a device coefficient vector on the grid's element set, plus those of a
// second vector when d_u2 is given (the wave problem's u_t) (synchronises)
amdg_status grid_norms(amdg_grid* g, const double* d_u, std::vector<double>* norms, const double* d_u2 = nullptr);
// coarsen the grid on the indicator ||u|| (+ ||u2|| when d_u2 is given)
amdg_status grid_coarsen(amdg_grid* g, double eta, const double* d_u2, int64_t* num_elements);

// ---- device-side element-set changes (adapt_device.cu) ------------------------
// refresh the host mirror (keys, orders, key index) after device-side changes
amdg_status grid_ensure_host(const amdg_grid* g);
// lev_max / lev_sum / levsum_max of the host element set
void grid_host_level_stats(amdg_grid* g);
// upload the host element set's keys (after a host-side change)
amdg_status grid_upload_keys(amdg_grid* g);
// the key -> element hash of the current element set (rebuilt when the set changed)
amdg_status grid_hash(amdg_grid* g);
// element indicators into g->d_norms: ||u_e|| (+ ||u2_e|| when d_u2 is given), summed as
// DGAdapt::indicator_norm does; a non-finite indicator is reported by the next refine / coarsen
amdg_status grid_device_norms(amdg_grid* g, const double* d_u, const double* d_u2);
// DGAdapt::refine on the device: leaves with indicator > eps (g->d_norms), or those flagged in
// d_force (device, one byte per element) when given, get all their children, holes are filled;
// new elements start at zero.  refined (host, may be null): per old element, 1 if refined.
// *added: elements added.  One stream synchronisation (the new element count).
amdg_status grid_device_refine(amdg_grid* g, double eps, const uint8_t* d_force, int8_t* refined, int64_t* added);
// DGAdapt::coarsen on the device on the indicators in g->d_norms.  With missed_eps > 0 the leaves
// of the coarsened set whose indicator exceeds it are recorded as missed refinements
// (g->dev.missed).  One stream synchronisation.
amdg_status grid_device_coarsen(amdg_grid* g, double eta, double missed_eps, int64_t* removed);
// 1 in d_force (device) for every element whose key is a recorded missed refinement
amdg_status grid_mark_missed(amdg_grid* g, uint8_t* d_force);
// the learned pre-adaptation flags into the grid's force buffer (*d_force): the classifier's
// refine class where confident (d_prob: E x 3, may be null), the criterion on g->d_norms elsewhere;
// d_counts[0] += refined by the classifier, d_counts[1] += unsure (device counters)
amdg_status grid_learned_flags(amdg_grid* g, const float* d_prob, double tau, double eps, uint8_t** d_force,
                               unsigned long long* d_counts);
// device flag the neighbour-list kernels set (reported by the next refine / coarsen or check)
int* grid_topology_error_flag(amdg_grid* g);
// synchronise and report a neighbour-list or ancestor error of the last device build
amdg_status grid_check_topology(amdg_grid* g);
// the element-set change of a remap: grow the spare arrays for E_new elements and move u (and v)
// through g->d_map (new -> old, -1 new element); bumps the version
amdg_status grid_apply_remap(amdg_grid* g, int64_t E_new);
// the spare arrays of that remap, allocated ahead of any change
amdg_status grid_reserve_remap(amdg_grid* g, int64_t E_new);
// device neighbour lists of the fast transforms and surplus ancestors for the current element set
struct DeviceTopoOut {
    int32_t *vol_ptr, *vol_nbr, *vol_split, *flx_ptr, *flx_nbr, *flx_split, *anc;
    int64_t vol_cap, flx_cap;        // pairs the nbr arrays hold
    const int32_t* anc_order;        // device [n1][p1]
    int p1;
    int* err;                        // device flag: a surplus ancestor is missing / a list overflowed
};
// bounds on the number of (element, neighbour) pairs of the vol and flx lists over all dimensions
void transform_topology_bounds(const amdg_grid* g, int64_t* vol_pairs, int64_t* flx_pairs);
amdg_status device_transform_topology(amdg_grid* g, const DeviceTopoOut& out, int32_t* d_cnt, void* stream);
// [e][d][2] parent / grandparent table on the device
amdg_status device_parent_table(amdg_grid* g, int32_t* d_pg, void* stream);
// the grid's Element::rhs vector (dof entries, zero after every element-set change)
amdg_status grid_rhs(amdg_grid* g, double** d_rhs);
// the grid's velocity field (u_t), created as zero when absent
amdg_status grid_ensure_velocity(amdg_grid* g);
}  // namespace amdg

struct amdg_batch {
    amdg_context* ctx = nullptr;
    int device = 0;
    int dim = 0, nmax = 0, k = 0, block = 0, nsolves = 0;
    std::vector<amdg_grid*> grids;
    amdg::BatchTables tables;  // built on the first rebuild
    std::vector<int64_t> elem_offset;
    int64_t num_elements = 0, dof = 0, pairs = 0;
    int num_blocks = 0;
    int64_t *d_row_ptr = nullptr, *d_src = nullptr;
    int32_t *d_blk = nullptr, *d_solve = nullptr;
    double *d_blocks64 = nullptr, *d_coef64 = nullptr, *d_dt = nullptr;
    float *d_blocks32 = nullptr, *d_coef32 = nullptr;
    double *d_u = nullptr, *d_u1 = nullptr, *d_u2 = nullptr;
    // mixed-mode stage state: three FP32 high and three FP32 low arrays at stride sstride (16-byte
    // aligned bases, 16 bytes of slack); the column kernel uses the high arrays as FP32 shadows
    float* d_shadow = nullptr;            // 3 x sstride
    float* d_lo = nullptr;                // 3 x sstride
    int64_t sstride = 0;
    int32_t* d_pairs = nullptr;           // (src, blk) interleaved per neighbour pair (bulk-copy ring kernel)
    float* d_blocks32p = nullptr;         // [2][num_blocks][(np^2 + 3) / 4 * 4]
    double* d_blocks64p = nullptr;        // the same in FP64
    float* d_dt32 = nullptr;              // [solve]
    int* d_err = nullptr;                 // bulk-copy wait gave up (device flag)
    unsigned long long* d_queue = nullptr;  // [3] chunk counters of the warp kernel's queue schedule, one per stage
    int sms = 0;                          // multiprocessors of the device (persistent grids)
    void* graph_exec[2] = {nullptr, nullptr};  // cudaGraphExec_t per precision
    int64_t launches_per_graph = 0;
    // stage kernel per precision (FP64, mixed), candidates as amdg_batch_tuning numbers them (the
    // column kernel at each CTA size, on the FP64 state or, mixed, on the FP32-pair state, the
    // bulk-copy ring and the warp-per-element kernel configurations); picked by the autotuner
    int kernel[2] = {2, 2};
    float kernel_ms[2][AMDG_BATCH_KERNELS] = {{0}};  // autotuner: one stage per candidate (0: not timed)
    // amdg_batch_adapt scratch over all elements (grow-only): norms, parent table, classifier
    // features and probabilities
    double* d_norms = nullptr;
    int32_t* d_pg = nullptr;
    float *d_feat = nullptr, *d_prob = nullptr;
    int64_t scratch_elems = 0, norms_elems = 0;
};
