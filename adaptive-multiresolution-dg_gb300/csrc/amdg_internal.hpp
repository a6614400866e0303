// Internal declarations shared by the host set-up code and the CUDA
// translation units of libamdg_gb300.
#pragma once

#include <cstdint>
#include <string>
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

// 1D projection of f(., d, term) onto every basis function (Basis::product_function).
void project_1d(const Basis1D& b, amdg_fn1d f, void* user, int d, int term, double* out);

// ---- grid topology (host build, device copy) -------------------------------
struct HostGrid {
    int dim = 0, nmax = 0, k = 0, sparse = 1;
    int64_t num_elements = 0;
    std::vector<int32_t> order;  // num_elements x dim, 1D element orders, sorted lexicographically
    std::vector<uint64_t> key;   // packed orders (nmax bits per dimension), ascending
};
void build_grid(int dim, int nmax, int sparse, HostGrid* g);
int64_t find_element(const HostGrid& g, const int32_t* orders);  // binary search, -1 if absent

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

}  // namespace amdg

// ---- opaque handle layouts (plain structs, owned by the C-ABI layer) ------
struct amdg_context {
    int device = 0;
    void* stream = nullptr;        // cudaStream_t in use
    void* own_stream = nullptr;    // stream created by the context
    int64_t launches = 0;
};

struct amdg_grid {
    amdg_context* ctx = nullptr;
    amdg::HostGrid host;
    int block = 0;                   // (k+1)^dim
    int64_t dof = 0;
    int32_t* d_order = nullptr;      // device copy of host.order
    double* d_u = nullptr;           // FP64 coefficients
    double* d_scratch = nullptr;     // reduction scratch
    size_t scratch_bytes = 0;
};

struct amdg_linear_op {
    amdg_grid* grid = nullptr;
    std::vector<double> coef;
    int64_t pairs = 0;
    int num_blocks = 0;              // 1D blocks per dimension in the table
    // CSR over (element, dimension): row_ptr[e*dim + t] .. row_ptr[e*dim + t + 1]
    int32_t* d_row_ptr = nullptr;
    int32_t* d_src = nullptr;        // neighbour element index
    int32_t* d_blk = nullptr;        // block index within the dimension's table
    double* d_blocks64 = nullptr;    // [dim][num_blocks][k+1][k+1], row = solution p, col = test q
    float* d_blocks32 = nullptr;
    double* d_u1 = nullptr;          // RK stage vectors
    double* d_u2 = nullptr;
};
