// Element-set changes on the device: the adaptive loop's refine and coarsen
// (DGAdapt::refine DGAdapt.cpp:371-404, coarsen :675-688 and :982-1016,
// check_hole :1351-1385, update_leaf :1036-1063) and the neighbour lists of
// the fast transforms (DGSolution::find_ptr_vol/flx_alpt, DGSolution.cpp:675-728,
// with the predicates of Element.cpp:265-348) built from the sorted packed keys
// without a round trip through the host.
//
// The element set lives on the device as sorted packed keys (1D orders, nmax
// bits per dimension, first dimension most significant).  A key -> element
// open-addressing hash answers "is this multi-index present" in O(1); it is
// rebuilt after every change.  A refinement marks the missing children of the
// refined leaves into the hash and a list (atomic append), fills holes in one
// CTA (rounds of "every parent of a new key must exist"), and the new sorted
// key set is the sort of old and new keys.  A coarsening decides removal by
// passes over the level sums from the finest down (an element goes when its
// indicator is below eta, it is not the root, and all its present children
// went), then compacts by a scan.  Each change synchronises the stream once to
// learn the new element count; everything else stays on the device.  The
// results are the host implementation's (csrc/adapt.cpp, csrc/grid.cpp): the
// same element sets, the same neighbour lists in the same order.
#include <cuda_runtime.h>

#include <cub/cub.cuh>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "amdg_internal.hpp"
#include "kernels.cuh"
#include "device_alloc.cuh"

using namespace amdg;

#define AMDG_CK(...)                                                                                    \
    do {                                                                                                \
        cudaError_t amdg_err_ = (__VA_ARGS__);                                                          \
        if (amdg_err_ != cudaSuccess)                                                                   \
            return fail(AMDG_ERR_CUDA, std::string(#__VA_ARGS__) + ": " + cudaGetErrorString(amdg_err_)); \
    } while (0)

namespace {

constexpr unsigned long long kEmptyKey = ~0ull;
constexpr int kMaxLevels = 17;  // nmax <= 16

cudaStream_t stream_of(const amdg_grid* g) { return static_cast<cudaStream_t>(g->ctx->stream); }

// Statistics of one element-set change, read back by the host in one copy.
struct AdaptStats {
    unsigned long long count;     // refine: keys added; coarsen: elements kept
    unsigned long long lev_sum[kMaxDim];
    int lev_max[kMaxDim];
    int levsum_max;
    int err;                      // bit 0: a list overflowed; bit 1: hole filling did not finish
    unsigned long long missed;    // coarsen: missed refinements recorded
    int nonfinite;                // set by the indicator kernel (cleared with the indicators only)
    int topo_err;                 // set by the neighbour-list kernels (cleared when reported)
};
// refine / coarsen restart everything before `nonfinite`
constexpr size_t kStatsReset = offsetof(AdaptStats, nonfinite);

template <class T>
amdg_status grow(T** p, int64_t* cap, int64_t need, int64_t want) {
    if (need <= *cap) return AMDG_OK;
    cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    if (amdg::device_malloc(reinterpret_cast<void**>(p), size_t(want) * sizeof(T)) != cudaSuccess) {
        *p = nullptr;
        return fail(AMDG_ERR_NOMEM, "cudaMalloc failed (device adaptivity buffers)");
    }
    *cap = want;
    return AMDG_OK;
}

amdg_status grow_temp(GridDevice& d, size_t bytes) {
    if (bytes <= d.temp_bytes) return AMDG_OK;
    cudaFree(d.temp);
    d.temp = nullptr;
    d.temp_bytes = 0;
    const size_t want = bytes + bytes / 2 + 4096;
    if (amdg::device_malloc(&d.temp, want) != cudaSuccess) {
        d.temp = nullptr;
        return fail(AMDG_ERR_NOMEM, "cudaMalloc failed (sort / scan scratch)");
    }
    d.temp_bytes = want;
    return AMDG_OK;
}

amdg_status ensure_stats(GridDevice& d) {
    if (d.stats && d.host_stats) return AMDG_OK;
    if (!d.host_stats && cudaMallocHost(&d.host_stats, sizeof(AdaptStats)) != cudaSuccess) {
        d.host_stats = nullptr;
        return fail(AMDG_ERR_NOMEM, "cudaMallocHost failed (adaptivity statistics)");
    }
    if (!d.stats && amdg::device_malloc(&d.stats, sizeof(AdaptStats)) != cudaSuccess) {
        d.stats = nullptr;
        return fail(AMDG_ERR_NOMEM, "cudaMalloc failed (adaptivity statistics)");
    }
    // every field starts at zero (the error flags are only ever set, and cleared when reported)
    if (cudaMemset(d.stats, 0, sizeof(AdaptStats)) != cudaSuccess)
        return fail(AMDG_ERR_CUDA, "cudaMemset failed (adaptivity statistics)");
    std::memset(d.host_stats, 0, sizeof(AdaptStats));
    return AMDG_OK;
}

// ---- packed keys and 1D orders ------------------------------------------------
struct KeyShape {
    int dim, nmax;
    __host__ __device__ int field(uint64_t key, int d) const {
        return int((key >> (uint64_t(nmax) * (dim - 1 - d))) & ((uint64_t(1) << nmax) - 1));
    }
    __host__ __device__ uint64_t with(uint64_t key, int d, int o) const {
        const uint64_t shift = uint64_t(nmax) * (dim - 1 - d);
        const uint64_t mask = ((uint64_t(1) << nmax) - 1) << shift;
        return (key & ~mask) | (uint64_t(o) << shift);
    }
};

__host__ __device__ __forceinline__ int level_of(int o) {
#ifdef __CUDA_ARCH__
    return o == 0 ? 0 : 32 - __clz(o);
#else
    int l = 0;
    while ((1 << l) <= o) ++l;
    return l;
#endif
}
__device__ __forceinline__ int parent_of(int o) { return o == 1 ? 0 : o / 2; }
// children of 1D order o below level nmax: {1} for o = 0, {2o, 2o+1} otherwise
__device__ __forceinline__ int children_of(int o, int nmax, int* ch) {
    const int n = level_of(o);
    if (n >= nmax) return 0;
    if (o == 0) { ch[0] = 1; return 1; }
    ch[0] = 2 * o;
    ch[1] = 2 * o + 1;
    return 2;
}

// ---- key -> element hash ---------------------------------------------------------
struct KeyHash {
    unsigned long long* key;
    int32_t* val;
    uint64_t mask;
    int bits;
};

__device__ __forceinline__ uint64_t hslot(uint64_t k, int bits) { return (k * 0x9E3779B97F4A7C15ull) >> (64 - bits); }

// element index of key k (>= 0), -1 when absent or added by the current refinement
__device__ __forceinline__ int32_t hfind(const KeyHash& h, uint64_t k) {
    uint64_t s = hslot(k, h.bits);
    for (uint64_t i = 0; i <= h.mask; ++i, s = (s + 1) & h.mask) {
        const unsigned long long v = h.key[s];
        if (v == kEmptyKey) return -1;
        if (v == k) return h.val[s];
    }
    return -1;
}
__device__ __forceinline__ bool hcontains(const KeyHash& h, uint64_t k) {
    uint64_t s = hslot(k, h.bits);
    for (uint64_t i = 0; i <= h.mask; ++i, s = (s + 1) & h.mask) {
        const unsigned long long v = *(volatile unsigned long long*)&h.key[s];
        if (v == kEmptyKey) return false;
        if (v == k) return true;
    }
    return false;
}
// inserts k; true when this call inserted it (slot in *slot), false when it was there
__device__ __forceinline__ bool hinsert(const KeyHash& h, uint64_t k, uint64_t* slot) {
    uint64_t s = hslot(k, h.bits);
    for (uint64_t i = 0; i <= h.mask; ++i, s = (s + 1) & h.mask) {
        const unsigned long long prev = atomicCAS(&h.key[s], kEmptyKey, (unsigned long long)k);
        if (prev == kEmptyKey) { *slot = s; return true; }
        if (prev == k) return false;
    }
    return false;  // the table is sized at least twice the keys it can receive: not reached
}

__global__ void hash_build_kernel(const uint64_t* __restrict__ keys, int64_t E, KeyHash h) {
    const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (e >= E) return;
    uint64_t s;
    if (hinsert(h, keys[e], &s)) h.val[s] = int32_t(e);
}

__global__ void keys_to_order_kernel(const uint64_t* __restrict__ keys, int64_t E, KeyShape ks, int32_t* __restrict__ order) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= E * ks.dim) return;
    const int64_t e = i / ks.dim;
    order[i] = ks.field(keys[e], int(i - e * ks.dim));
}

// ---- indicators ----------------------------------------------------------------
// sqrt of the block's sum of squares in block order (as element_norm_kernel), plus the second
// vector's when given, added in that order (DGAdapt::indicator_norm, DGAdapt.cpp:1018-1030)
__global__ void norms_kernel(const double* __restrict__ u, const double* __restrict__ u2, int B, int64_t E,
                             double* __restrict__ out, AdaptStats* st) {
    const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (e >= E) return;
    const double* x = u + e * B;
    double s = 0.0;
    for (int q = 0; q < B; ++q) s = __dadd_rn(s, __dmul_rn(x[q], x[q]));
    double v = sqrt(s);
    if (u2) {
        const double* y = u2 + e * B;
        double s2 = 0.0;
        for (int q = 0; q < B; ++q) s2 = __dadd_rn(s2, __dmul_rn(y[q], y[q]));
        v = __dadd_rn(v, sqrt(s2));
    }
    out[e] = v;
    if (!isfinite(v)) st->nonfinite = 1;
}

// ---- refinement ------------------------------------------------------------------
// Leaves (fewer present children than possible, DGAdapt::update_leaf) that want refinement get
// every missing child in every dimension (DGAdapt::refine), appended once to newk.
__global__ void refine_mark_kernel(const uint64_t* __restrict__ keys, int64_t E, KeyShape ks,
                                   const double* __restrict__ norms, double eps, const uint8_t* __restrict__ force,
                                   KeyHash h, uint64_t* __restrict__ newk, AdaptStats* st, int64_t cap,
                                   uint8_t* __restrict__ refined) {
    const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (e >= E) return;
    const bool want = force ? force[e] != 0 : (norms[e] > eps);
    refined[e] = 0;
    if (!want) return;
    const uint64_t key = keys[e];
    int existing = 0, total = 0, ch[2];
    for (int d = 0; d < ks.dim; ++d) {
        const int nc = children_of(ks.field(key, d), ks.nmax, ch);
        total += nc;
        for (int c = 0; c < nc; ++c) existing += hfind(h, ks.with(key, d, ch[c])) >= 0 ? 1 : 0;
    }
    if (existing >= total) return;
    refined[e] = 1;
    for (int d = 0; d < ks.dim; ++d) {
        const int nc = children_of(ks.field(key, d), ks.nmax, ch);
        for (int c = 0; c < nc; ++c) {
            const uint64_t ck = ks.with(key, d, ch[c]);
            if (hfind(h, ck) >= 0) continue;
            uint64_t slot;
            if (!hinsert(h, ck, &slot)) continue;
            const long long i = (long long)atomicAdd(&st->count, 1ull);
            if (i < cap) newk[i] = ck;
            else atomicOr(&st->err, 1);
        }
    }
}

// Hole filling (DGAdapt::check_hole) in one CTA: every parent of a new key must be present;
// rounds over the keys the previous round added, until a round adds none.  Then the level
// statistics of the added keys.
__global__ void __launch_bounds__(1024) hole_fill_kernel(KeyShape ks, KeyHash h, uint64_t* __restrict__ newk,
                                                         AdaptStats* st, int64_t cap) {
    __shared__ long long s_hi;
    long long lo = 0;
    int round = 0;
    for (;; ++round) {
        __syncthreads();
        if (threadIdx.x == 0) s_hi = (long long)*(volatile unsigned long long*)&st->count;
        __syncthreads();
        const long long hi = s_hi < cap ? s_hi : cap;
        if (lo >= hi) break;
        if (round >= 4 * kMaxDim * kMaxLevels) {  // a hole-free closure needs at most dim * nmax rounds
            if (threadIdx.x == 0) atomicOr(&st->err, 2);
            break;
        }
        for (long long i = lo + threadIdx.x; i < hi; i += blockDim.x) {
            const uint64_t key = newk[i];
            for (int d = 0; d < ks.dim; ++d) {
                const int o = ks.field(key, d);
                if (o == 0) continue;
                const uint64_t p = ks.with(key, d, parent_of(o));
                if (hcontains(h, p)) continue;
                uint64_t slot;
                if (!hinsert(h, p, &slot)) continue;
                const long long j = (long long)atomicAdd(&st->count, 1ull);
                if (j < cap) newk[j] = p;
                else atomicOr(&st->err, 1);
            }
        }
        lo = hi;
    }
    __syncthreads();
    const long long n = s_hi < cap ? s_hi : cap;
    for (long long i = threadIdx.x; i < n; i += blockDim.x) {
        const uint64_t key = newk[i];
        int sum = 0;
        for (int d = 0; d < ks.dim; ++d) {
            const int l = level_of(ks.field(key, d));
            sum += l;
            atomicAdd(&st->lev_sum[d], (unsigned long long)l);
            atomicMax(&st->lev_max[d], l);
        }
        atomicMax(&st->levsum_max, sum);
    }
}

__global__ void concat_keys_kernel(const uint64_t* __restrict__ a, int64_t na, const uint64_t* __restrict__ b, int64_t nb,
                                   uint64_t* __restrict__ out) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < na) out[i] = a[i];
    else if (i < na + nb) out[i] = b[i - na];
}

// new element -> old element (-1: added) through the old set's hash, and the new orders
__global__ void map_from_hash_kernel(const uint64_t* __restrict__ keys, int64_t E, KeyShape ks, KeyHash h,
                                     int32_t* __restrict__ map, int32_t* __restrict__ order) {
    const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (e >= E) return;
    const uint64_t key = keys[e];
    map[e] = hfind(h, key);
    for (int d = 0; d < ks.dim; ++d) order[e * ks.dim + d] = ks.field(key, d);
}

// ---- coarsening ------------------------------------------------------------------
// Elements of level sum L: removed when the indicator is below eta, some level is above 0, and
// every present child (level sum L + 1, decided by the previous pass) is removed -- the fixed
// point of DGAdapt::coarsen's repeated sweeps over childless elements.
__global__ void coarsen_pass_kernel(const uint64_t* __restrict__ keys, int64_t E, KeyShape ks,
                                    const double* __restrict__ norms, double eta, int L, KeyHash h,
                                    uint8_t* __restrict__ removed) {
    const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (e >= E) return;
    const uint64_t key = keys[e];
    int sum = 0, mx = 0;
    for (int d = 0; d < ks.dim; ++d) {
        const int l = level_of(ks.field(key, d));
        sum += l;
        mx = l > mx ? l : mx;
    }
    if (sum != L || mx == 0 || !(norms[e] < eta)) return;
    int ch[2];
    for (int d = 0; d < ks.dim; ++d) {
        const int nc = children_of(ks.field(key, d), ks.nmax, ch);
        for (int c = 0; c < nc; ++c) {
            const int32_t i = hfind(h, ks.with(key, d, ch[c]));
            if (i >= 0 && !removed[i]) return;
        }
    }
    removed[e] = 1;
}

__global__ void keep_flags_kernel(const uint8_t* __restrict__ removed, int64_t E, int32_t* __restrict__ keep) {
    const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (e < E) keep[e] = removed[e] ? 0 : 1;
    else if (e == E) keep[e] = 0;
}

// statistics of the kept set; with missed_eps > 0 the kept leaves (leaf in the kept set) whose
// indicator exceeds missed_eps are appended to `missed`
__global__ void coarsen_stats_kernel(const uint64_t* __restrict__ keys, int64_t E, KeyShape ks,
                                     const uint8_t* __restrict__ removed, const int32_t* __restrict__ pos,
                                     const double* __restrict__ norms, double missed_eps, KeyHash h,
                                     uint64_t* __restrict__ missed, int64_t missed_cap, AdaptStats* st) {
    const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (e == 0) st->count = pos[E];
    if (e >= E || removed[e]) return;
    const uint64_t key = keys[e];
    int sum = 0;
    for (int d = 0; d < ks.dim; ++d) {
        const int l = level_of(ks.field(key, d));
        sum += l;
        atomicAdd(&st->lev_sum[d], (unsigned long long)l);
        atomicMax(&st->lev_max[d], l);
    }
    atomicMax(&st->levsum_max, sum);
    if (missed_eps > 0.0 && norms[e] > missed_eps) {
        int existing = 0, total = 0, ch[2];
        for (int d = 0; d < ks.dim; ++d) {
            const int nc = children_of(ks.field(key, d), ks.nmax, ch);
            total += nc;
            for (int c = 0; c < nc; ++c) {
                const int32_t i = hfind(h, ks.with(key, d, ch[c]));
                existing += (i >= 0 && !removed[i]) ? 1 : 0;
            }
        }
        if (existing < total) {
            const long long j = (long long)atomicAdd(&st->missed, 1ull);
            if (j < missed_cap) missed[j] = key;
        }
    }
}

// The whole coarsening of a small element set in one CTA: the level-sum passes (finest first,
// separated by barriers), the keep flags and their exclusive scan (a block scan over
// kSmallCoarsenItems elements per thread), and the statistics of the kept set -- the same flags,
// positions and statistics as coarsen_pass_kernel + keep_flags_kernel + the device scan +
// coarsen_stats_kernel, without their launches.
constexpr int kSmallCoarsenThreads = 1024, kSmallCoarsenItems = 8;
constexpr int64_t kSmallCoarsenMax = int64_t(kSmallCoarsenThreads) * kSmallCoarsenItems;
__global__ void __launch_bounds__(kSmallCoarsenThreads)
    coarsen_small_kernel(const uint64_t* __restrict__ keys, int64_t E, KeyShape ks, const double* __restrict__ norms,
                         double eta, int levsum_max, KeyHash h, uint8_t* __restrict__ removed,
                         int32_t* __restrict__ pos, double missed_eps, uint64_t* __restrict__ missed,
                         int64_t missed_cap, AdaptStats* st) {
    const int tid = threadIdx.x;
    for (int64_t e = tid; e < E; e += kSmallCoarsenThreads) removed[e] = 0;
    __syncthreads();
    for (int L = levsum_max; L >= 1; --L) {
        for (int64_t e = tid; e < E; e += kSmallCoarsenThreads) {
            const uint64_t key = keys[e];
            int sum = 0, mx = 0;
            for (int d = 0; d < ks.dim; ++d) {
                const int l = level_of(ks.field(key, d));
                sum += l;
                mx = l > mx ? l : mx;
            }
            if (sum != L || mx == 0 || !(norms[e] < eta)) continue;
            bool keep_it = false;
            int ch[2];
            for (int d = 0; d < ks.dim && !keep_it; ++d) {
                const int nc = children_of(ks.field(key, d), ks.nmax, ch);
                for (int c = 0; c < nc; ++c) {
                    const int32_t i = hfind(h, ks.with(key, d, ch[c]));
                    if (i >= 0 && !removed[i]) keep_it = true;
                }
            }
            if (!keep_it) removed[e] = 1;
        }
        __syncthreads();  // pass L - 1 reads the flags of pass L
    }
    using Scan = cub::BlockScan<int, kSmallCoarsenThreads>;
    __shared__ typename Scan::TempStorage scan_tmp;
    int v[kSmallCoarsenItems];
#pragma unroll
    for (int i = 0; i < kSmallCoarsenItems; ++i) {
        const int64_t e = int64_t(tid) * kSmallCoarsenItems + i;
        v[i] = (e < E && !removed[e]) ? 1 : 0;
    }
    int total = 0;
    Scan(scan_tmp).ExclusiveSum(v, v, total);
#pragma unroll
    for (int i = 0; i < kSmallCoarsenItems; ++i) {
        const int64_t e = int64_t(tid) * kSmallCoarsenItems + i;
        if (e < E) pos[e] = v[i];
    }
    if (tid == 0) {
        pos[E] = total;
        st->count = (unsigned long long)total;
    }
    for (int64_t e = tid; e < E; e += kSmallCoarsenThreads) {
        if (removed[e]) continue;
        const uint64_t key = keys[e];
        int sum = 0;
        for (int d = 0; d < ks.dim; ++d) {
            const int l = level_of(ks.field(key, d));
            sum += l;
            atomicAdd(&st->lev_sum[d], (unsigned long long)l);
            atomicMax(&st->lev_max[d], l);
        }
        atomicMax(&st->levsum_max, sum);
        if (missed_eps > 0.0 && norms[e] > missed_eps) {
            int existing = 0, tot = 0, ch[2];
            for (int d = 0; d < ks.dim; ++d) {
                const int nc = children_of(ks.field(key, d), ks.nmax, ch);
                tot += nc;
                for (int c = 0; c < nc; ++c) {
                    const int32_t i = hfind(h, ks.with(key, d, ch[c]));
                    existing += (i >= 0 && !removed[i]) ? 1 : 0;
                }
            }
            if (existing < tot) {
                const long long j = (long long)atomicAdd(&st->missed, 1ull);
                if (j < missed_cap) missed[j] = key;
            }
        }
    }
}

__global__ void compact_kernel(const uint64_t* __restrict__ keys, int64_t E, KeyShape ks, const uint8_t* __restrict__ removed,
                               const int32_t* __restrict__ pos, uint64_t* __restrict__ out_keys,
                               int32_t* __restrict__ map, int32_t* __restrict__ order) {
    const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (e >= E || removed[e]) return;
    const int32_t p = pos[e];
    const uint64_t key = keys[e];
    out_keys[p] = key;
    map[p] = int32_t(e);
    for (int d = 0; d < ks.dim; ++d) order[int64_t(p) * ks.dim + d] = ks.field(key, d);
}

__global__ void mark_keys_kernel(const uint64_t* __restrict__ list, int64_t n, KeyHash h, uint8_t* __restrict__ flag) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int32_t e = hfind(h, list[i]);
    if (e >= 0) flag[e] = 1;
}

// ---- neighbour lists of the fast transforms ----------------------------------------
// 1D support [a, b) of order o in units of 2^-nmax (levels 0 and 1 cover the domain)
__device__ __forceinline__ void support_of(int o, int nmax, int64_t* a, int64_t* b) {
    const int n = level_of(o);
    if (n <= 1) { *a = 0; *b = int64_t(1) << nmax; return; }
    const int64_t w = int64_t(1) << (nmax - n + 1);
    *a = int64_t(o - (1 << (n - 1))) * w;
    *b = *a + w;
}

// The candidates of level l >= 2 for element support [a0, b0) (Element.cpp:283-348 as index
// ranges): the intersecting intervals first..last (vol), widened to lo..hi where an interval
// ends or starts exactly at the boundary (flx), and the intervals across the periodic boundary.
struct LevelRange {
    int cnt, first, last, lo, hi;
    bool wrap_lo, wrap_hi;  // interval 0 (across x = 1) / interval cnt - 1 (across x = 0)
};
__device__ __forceinline__ LevelRange level_range(int l, int nmax, int64_t a0, int64_t b0) {
    LevelRange r;
    const int64_t one = int64_t(1) << nmax;
    r.cnt = 1 << (l - 1);
    const int64_t w = one >> (l - 1);
    r.first = int(a0 / w);
    r.last = int((b0 - 1) / w);
    r.lo = r.first;
    r.hi = r.last;
    if (a0 % w == 0 && r.first >= 1) --r.lo;
    if (b0 % w == 0 && r.last + 1 < r.cnt) ++r.hi;
    r.wrap_lo = b0 == one && r.lo > 0;
    r.wrap_hi = a0 == 0 && r.hi < r.cnt - 1;
    return r;
}

struct TopoArgs {
    const uint64_t* keys;
    int64_t E;
    KeyShape ks;
    KeyHash h;
};

// The candidate 1D orders of level l for a row (element, dimension t) with 1D support [a0, b0),
// in increasing order: levels 0 and 1 are the single order l (intersecting every support); at
// level l >= 2 the interval across x = 1 (when it touches the support from the periodic side),
// the intervals lo .. hi (first .. last intersect the support: vol; the ones beside them touch
// it: flx only), and the interval across x = 0.  This is the host builder's sequence
// (csrc/grid.cpp, fibre_neighbours), so the lists come out in the same order.
struct LevelCands {
    int n;                 // candidates at this level
    int base, lo, wl;      // order of candidate i: cnt if i < wl (wrap), else base + lo + i - wl, ...
    int vfirst, vlast;     // vol range (orders)
    int wrap_hi_order;     // last candidate when >= 0
};
__device__ __forceinline__ LevelCands level_cands(int l, int nmax, int64_t a0, int64_t b0) {
    LevelCands c;
    if (l <= 1) {
        c.n = 1;
        c.base = l;
        c.lo = 0;
        c.wl = 0;
        c.vfirst = c.vlast = l;
        c.wrap_hi_order = -1;
        return c;
    }
    const LevelRange r = level_range(l, nmax, a0, b0);
    c.wl = r.wrap_lo ? 1 : 0;
    c.base = r.cnt;
    c.lo = r.lo;
    c.n = c.wl + (r.hi - r.lo + 1) + (r.wrap_hi ? 1 : 0);
    c.vfirst = r.cnt + r.first;
    c.vlast = r.cnt + r.last;
    c.wrap_hi_order = r.wrap_hi ? 2 * r.cnt - 1 : -1;
    return c;
}
__device__ __forceinline__ int cand_order(const LevelCands& c, int i) {
    if (i < c.wl) return c.base;  // the interval across x = 1 (order cnt)
    if (c.wrap_hi_order >= 0 && i == c.n - 1) return c.wrap_hi_order;
    return c.base + c.lo + (i - c.wl);
}

// One warp per row (element, dimension): every level's candidates looked up 32 at a time, the
// present ones counted (fill == nullptr) or written in order (ballot prefix) -- no per-thread
// chains of dependent lookups.  Returns, on lane 0, the vol / flx counts and the counts at levels
// up to the element's own (the split between the "U" and "L" parts).
struct RowOut {
    int2* vol;
    int2* flx;
    int64_t vmax, fmax;  // entries the row may write (fill)
};
__device__ __forceinline__ void row_lists(const TopoArgs& A, int64_t e, int t, const RowOut* out, int* nv_out,
                                          int* nf_out, int* sv_out, int* sf_out) {
    const int lane = threadIdx.x & 31;
    const int nmax = A.ks.nmax;
    const uint64_t key = A.keys[e];
    const int oi = A.ks.field(key, t), own = level_of(oi);
    int64_t a0, b0;
    support_of(oi, nmax, &a0, &b0);
    int nv = 0, nf = 0, sv = 0, sf = 0;
    for (int l = 0; l <= nmax; ++l) {
        const LevelCands c = level_cands(l, nmax, a0, b0);
        for (int base = 0; base < c.n; base += 32) {
            const int i = base + lane;
            int s = -1, o = 0;
            if (i < c.n) {
                o = cand_order(c, i);
                s = hfind(A.h, A.ks.with(key, t, o));
            }
            const bool inv = s >= 0 && o >= c.vfirst && o <= c.vlast;
            const unsigned bf = __ballot_sync(0xffffffffu, s >= 0);
            const unsigned bv = __ballot_sync(0xffffffffu, inv);
            if (out) {
                const unsigned below = (1u << lane) - 1u;
                if (s >= 0) {
                    const int pf = nf + __popc(bf & below);
                    if (pf < out->fmax) out->flx[pf] = make_int2(s, o);
                }
                if (inv) {
                    const int pv = nv + __popc(bv & below);
                    if (pv < out->vmax) out->vol[pv] = make_int2(s, o);
                }
            }
            nf += __popc(bf);
            nv += __popc(bv);
        }
        if (l <= own) {
            sv = nv;
            sf = nf;
        }
    }
    *nv_out = nv;
    *nf_out = nf;
    *sv_out = sv;
    *sf_out = sf;
}

__global__ void topo_count_kernel(TopoArgs A, int32_t* __restrict__ vcnt, int32_t* __restrict__ fcnt) {
    const int64_t row = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int dim = A.ks.dim;
    if (row > A.E * dim) return;  // whole warps: the row test is uniform
    if (row == A.E * dim) {
        if ((threadIdx.x & 31) == 0) vcnt[row] = fcnt[row] = 0;
        return;
    }
    const int64_t e = row / dim;
    int nv, nf, sv, sf;
    row_lists(A, e, int(row - e * dim), nullptr, &nv, &nf, &sv, &sf);
    if ((threadIdx.x & 31) == 0) {
        vcnt[row] = nv;
        fcnt[row] = nf;
    }
}

__global__ void topo_fill_kernel(TopoArgs A, const int32_t* __restrict__ vol_ptr, const int32_t* __restrict__ flx_ptr,
                                 int2* __restrict__ vol_nbr, int2* __restrict__ flx_nbr, int32_t* __restrict__ vol_split,
                                 int32_t* __restrict__ flx_split, int64_t vol_cap, int64_t flx_cap, int* err) {
    const int64_t row = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int dim = A.ks.dim;
    if (row >= A.E * dim) return;
    const int64_t v0 = vol_ptr[row], f0 = flx_ptr[row];
    const int64_t v1 = vol_ptr[row + 1], f1 = flx_ptr[row + 1];
    if (v1 > vol_cap || f1 > flx_cap) {  // lists beyond the arrays: write nothing
        if ((threadIdx.x & 31) == 0) atomicOr(err, 1);
        return;
    }
    const RowOut out{vol_nbr + v0, flx_nbr + f0, v1 - v0, f1 - f0};
    const int64_t e = row / dim;
    int nv, nf, sv, sf;
    row_lists(A, e, int(row - e * dim), &out, &nv, &nf, &sv, &sf);
    if ((threadIdx.x & 31) == 0) {
        if (nv != v1 - v0 || nf != f1 - f0) atomicOr(err, 1);
        vol_split[row] = int32_t(v0 + sv);
        flx_split[row] = int32_t(f0 + sf);
    }
}

// surplus ancestors anc[e][d][ic]: the element owning surplus point ic of e along d
// (LagrInterpolation::eval_fp_to_coe_D_Lag, Interplation.cpp:1318-1376); -1 for level 0
__global__ void ancestors_kernel(TopoArgs A, const int32_t* __restrict__ anc_order, int p1, int32_t* __restrict__ anc,
                                 int* err) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const int dim = A.ks.dim;
    if (i >= A.E * dim) return;
    const int64_t e = i / dim;
    const int d = int(i - e * dim);
    const uint64_t key = A.keys[e];
    const int o = A.ks.field(key, d);
    int32_t* out = anc + i * p1;
    for (int ic = 0; ic < p1; ++ic) {
        if (o == 0) { out[ic] = -1; continue; }
        const int32_t s = hfind(A.h, A.ks.with(key, d, anc_order[o * p1 + ic]));
        if (s < 0) atomicOr(err, 2);
        out[ic] = s;
    }
}

__global__ void parent_table_kernel(TopoArgs A, int32_t* __restrict__ pg) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const int dim = A.ks.dim;
    if (i >= A.E * dim) return;
    const int64_t e = i / dim;
    const int d = int(i - e * dim);
    uint64_t k = A.keys[e];
    int32_t* out = pg + i * 2;
    out[0] = out[1] = -1;
    for (int gen = 0; gen < 2; ++gen) {
        const int o = A.ks.field(k, d);
        if (o == 0) break;
        k = A.ks.with(k, d, parent_of(o));
        out[gen] = hfind(A.h, k);
    }
}

inline unsigned blocks_for(int64_t n, int threads) { return unsigned((n + threads - 1) / threads); }

KeyHash hash_of(const amdg_grid* g) {
    KeyHash h;
    h.key = g->dev.hkey;
    h.val = g->dev.hval;
    h.mask = uint64_t(g->dev.hcap) - 1;
    h.bits = g->dev.hbits;
    return h;
}

amdg_status read_stats(amdg_grid* g, AdaptStats* out) {
    cudaStream_t st = stream_of(g);
    AMDG_CK(cudaMemcpyAsync(g->dev.host_stats, g->dev.stats, sizeof(AdaptStats), cudaMemcpyDeviceToHost, st));
    AMDG_CK(cudaStreamSynchronize(st));
    std::memcpy(out, g->dev.host_stats, sizeof(AdaptStats));
    if (out->topo_err) {  // reported once
        AMDG_CK(cudaMemsetAsync(&static_cast<AdaptStats*>(g->dev.stats)->topo_err, 0, sizeof(int), st));
        return fail(AMDG_ERR_STATE, out->topo_err & 2 ? "element set has a hole: a surplus ancestor is missing"
                                                      : "device neighbour list overflow");
    }
    return AMDG_OK;
}

// Learned pre-adaptation flags (amdg_burgers_adaptive_step_learned): the classifier's "refine"
// (class 0) where its largest probability is at least tau, the surplus criterion where it is
// unsure (or everywhere without a classifier).  counts[0] += refined by the network,
// counts[1] += unsure.
__global__ void learned_flags_kernel(const float* __restrict__ prob, int64_t E, float tau,
                                     const double* __restrict__ norms, double eps, uint8_t* __restrict__ force,
                                     unsigned long long* counts) {
    const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (e >= E) return;
    uint8_t f;
    if (!prob) {
        f = norms[e] > eps ? 1 : 0;
        atomicAdd(&counts[1], 1ull);
    } else {
        const float* p = prob + 3 * e;
        int arg = 0;
        for (int q = 1; q < 3; ++q)
            if (p[q] > p[arg]) arg = q;
        if (p[arg] < tau) {
            f = norms[e] > eps ? 1 : 0;
            atomicAdd(&counts[1], 1ull);
        } else if (arg == 0) {
            f = 1;
            atomicAdd(&counts[0], 1ull);
        } else {
            f = 0;
        }
    }
    force[e] = f;
}

amdg_status ensure_flags(amdg_grid* g, int64_t E) {
    GridDevice& d = g->dev;
    if (E + 1 <= d.flag_cap) return AMDG_OK;
    cudaFree(d.flag);
    cudaFree(d.force);
    cudaFree(d.pos);
    d.flag = d.force = nullptr;
    d.pos = nullptr;
    d.flag_cap = 0;
    const int64_t want = E + E / 2 + 64;
    if (amdg::device_malloc(&d.flag, size_t(want)) != cudaSuccess || amdg::device_malloc(&d.force, size_t(want)) != cudaSuccess ||
        amdg::device_malloc(&d.pos, size_t(want) * sizeof(int32_t)) != cudaSuccess)
        return fail(AMDG_ERR_NOMEM, "cudaMalloc failed (adaptivity flags)");
    d.flag_cap = want;
    return AMDG_OK;
}

}  // namespace

namespace amdg {

void grid_host_level_stats(amdg_grid* g) {
    const int dim = g->host.dim;
    for (int d = 0; d < kMaxDim; ++d) {
        g->lev_max[d] = 0;
        g->lev_sum[d] = 0;
    }
    g->levsum_max = 0;
    for (int64_t e = 0; e < g->host.num_elements; ++e) {
        int s = 0;
        for (int d = 0; d < dim; ++d) {
            const int l = level_of(g->host.order[size_t(e) * dim + d]);
            s += l;
            g->lev_sum[d] += l;
            g->lev_max[d] = std::max(g->lev_max[d], l);
        }
        g->levsum_max = std::max(g->levsum_max, s);
    }
}

// both key arrays hold at least E keys (the swaps keep them the same size); with `preserve` the
// current keys are carried over when they move
static amdg_status ensure_keys(amdg_grid* g, int64_t E, bool preserve) {
    GridDevice& d = g->dev;
    if (E <= d.key_cap && d.key && d.key_alt) return AMDG_OK;
    const int64_t want = std::max<int64_t>(E + E / 4 + 16, d.key_cap);
    uint64_t *k = nullptr, *a = nullptr;
    if (amdg::device_malloc(&k, size_t(want) * sizeof(uint64_t)) != cudaSuccess ||
        amdg::device_malloc(&a, size_t(want) * sizeof(uint64_t)) != cudaSuccess) {
        cudaFree(k);
        return fail(AMDG_ERR_NOMEM, "cudaMalloc failed (element keys)");
    }
    const int64_t n = g->host.num_elements;
    cudaStream_t st = stream_of(g);
    if (preserve && n > 0 && d.key) AMDG_CK(cudaMemcpyAsync(k, d.key, size_t(n) * sizeof(uint64_t), cudaMemcpyDeviceToDevice, st));
    AMDG_CK(cudaStreamSynchronize(st));
    cudaFree(d.key);
    cudaFree(d.key_alt);
    d.key = k;
    d.key_alt = a;
    d.key_cap = want;
    return AMDG_OK;
}

amdg_status grid_upload_keys(amdg_grid* g) {
    const int64_t E = g->host.num_elements;
    if (amdg_status s = ensure_keys(g, E, false); s != AMDG_OK) return s;
    if (E > 0)
        AMDG_CK(cudaMemcpyAsync(g->dev.key, g->host.key.data(), size_t(E) * sizeof(uint64_t), cudaMemcpyHostToDevice,
                                stream_of(g)));
    g->dev.hash_version = -1;
    g->host_stale = false;
    grid_host_level_stats(g);
    return AMDG_OK;
}

amdg_status grid_ensure_host(const amdg_grid* cg) {
    amdg_grid* g = const_cast<amdg_grid*>(cg);
    if (!g->host_stale) return AMDG_OK;
    const int64_t E = g->host.num_elements;
    std::vector<uint64_t> keys(static_cast<size_t>(E));
    cudaStream_t st = stream_of(g);
    if (E > 0) AMDG_CK(cudaMemcpyAsync(keys.data(), g->dev.key, size_t(E) * sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
    AMDG_CK(cudaStreamSynchronize(st));
    const int sparse = g->host.sparse;
    grid_from_keys(g->host.dim, g->host.nmax, g->host.k, std::move(keys), &g->host);
    g->host.sparse = sparse;
    g->host_stale = false;
    return AMDG_OK;
}

amdg_status grid_hash(amdg_grid* g) {
    GridDevice& d = g->dev;
    if (d.hash_version == g->version) return AMDG_OK;
    const int64_t E = g->host.num_elements;
    // room for the element set and everything one refinement can add (at most 2 dim children of
    // existing elements per element), at most half full
    const int64_t need = 2 * (1 + 2 * int64_t(g->host.dim)) * std::max<int64_t>(E, 1);
    if (need > d.hcap) {
        cudaFree(d.hkey);
        cudaFree(d.hval);
        d.hkey = nullptr;
        d.hval = nullptr;
        d.hcap = 0;
        int bits = 6;
        while ((int64_t(1) << bits) < need + need / 2) ++bits;
        const int64_t cap = int64_t(1) << bits;
        if (amdg::device_malloc(&d.hkey, size_t(cap) * sizeof(unsigned long long)) != cudaSuccess ||
            amdg::device_malloc(&d.hval, size_t(cap) * sizeof(int32_t)) != cudaSuccess)
            return fail(AMDG_ERR_NOMEM, "cudaMalloc failed (element hash)");
        d.hcap = cap;
        d.hbits = bits;
    }
    cudaStream_t st = stream_of(g);
    AMDG_CK(cudaMemsetAsync(d.hkey, 0xFF, size_t(d.hcap) * sizeof(unsigned long long), st));
    AMDG_CK(cudaMemsetAsync(d.hval, 0xFF, size_t(d.hcap) * sizeof(int32_t), st));
    if (E > 0) {
        hash_build_kernel<<<blocks_for(E, 256), 256, 0, st>>>(d.key, E, hash_of(g));
        AMDG_CK(cudaGetLastError());
        g->ctx->launches++;
    }
    d.hash_version = g->version;
    return AMDG_OK;
}

amdg_status grid_device_norms(amdg_grid* g, const double* d_u, const double* d_u2) {
    const int64_t E = g->host.num_elements;
    if (amdg_status s = ensure_stats(g->dev); s != AMDG_OK) return s;
    if (E > g->norms_capacity) {
        cudaFree(g->d_norms);
        g->d_norms = nullptr;
        g->norms_capacity = 0;
        const int64_t cap = E + E / 4 + 16;
        if (amdg::device_malloc(reinterpret_cast<void**>(&g->d_norms), size_t(cap) * sizeof(double)) != cudaSuccess)
            return fail(AMDG_ERR_NOMEM, "cudaMalloc failed (indicators)");
        g->norms_capacity = cap;
    }
    cudaStream_t st = stream_of(g);
    AMDG_CK(cudaMemsetAsync(g->dev.stats, 0, offsetof(AdaptStats, topo_err), st));
    if (E > 0) {
        norms_kernel<<<blocks_for(E, 128), 128, 0, st>>>(d_u, d_u2, g->block, E, g->d_norms,
                                                         static_cast<AdaptStats*>(g->dev.stats));
        AMDG_CK(cudaGetLastError());
        g->ctx->launches++;
    }
    return AMDG_OK;
}

amdg_status grid_reserve_remap(amdg_grid* g, int64_t E) {
    const int64_t grown = E + E / 4 + 16;
    auto regrow = [&](double** p, int64_t* cap) -> amdg_status {
        if (E <= *cap) return AMDG_OK;
        cudaFree(*p);
        *p = nullptr;
        *cap = 0;
        if (amdg::device_malloc(reinterpret_cast<void**>(p), size_t(grown) * g->block * sizeof(double)) != cudaSuccess)
            return fail(AMDG_ERR_NOMEM, "cudaMalloc failed (coefficient remap)");
        *cap = grown;
        return AMDG_OK;
    };
    amdg_status s;
    if ((s = regrow(&g->d_u_spare, &g->spare_capacity)) != AMDG_OK) return s;
    if (g->d_v && (s = regrow(&g->d_v_spare, &g->v_spare_capacity)) != AMDG_OK) return s;
    if (g->d_pred && (s = regrow(&g->d_pred_spare, &g->pred_spare_capacity)) != AMDG_OK) return s;
    if (g->d_pred_v && (s = regrow(&g->d_pred_v_spare, &g->pred_v_spare_capacity)) != AMDG_OK) return s;
    return AMDG_OK;
}

amdg_status grid_apply_remap(amdg_grid* g, int64_t E) {
    cudaStream_t st = stream_of(g);
    if (amdg_status s = grid_reserve_remap(g, E); s != AMDG_OK) return s;
    AMDG_CK(launch_remap(g->d_u, g->d_map, g->block, E, g->d_u_spare, st));
    g->ctx->launches++;
    if (g->d_v) {
        AMDG_CK(launch_remap(g->d_v, g->d_map, g->block, E, g->d_v_spare, st));
        g->ctx->launches++;
        std::swap(g->d_v, g->d_v_spare);
        std::swap(g->v_capacity, g->v_spare_capacity);
    }
    if (g->d_pred) {
        AMDG_CK(launch_remap(g->d_pred, g->d_map, g->block, E, g->d_pred_spare, st));
        g->ctx->launches++;
        std::swap(g->d_pred, g->d_pred_spare);
        std::swap(g->pred_capacity, g->pred_spare_capacity);
    }
    if (g->d_pred_v) {
        AMDG_CK(launch_remap(g->d_pred_v, g->d_map, g->block, E, g->d_pred_v_spare, st));
        g->ctx->launches++;
        std::swap(g->d_pred_v, g->d_pred_v_spare);
        std::swap(g->pred_v_capacity, g->pred_v_spare_capacity);
    }
    std::swap(g->d_u, g->d_u_spare);
    std::swap(g->capacity, g->spare_capacity);
    g->host.num_elements = E;
    g->dof = E * g->block;
    g->version++;
    return AMDG_OK;
}

// map, order and key arrays for E_new elements (grow-only)
static amdg_status ensure_set_arrays(amdg_grid* g, int64_t E) {
    const int64_t grown = E + E / 4 + 16;
    if (E > g->map_capacity) {
        cudaFree(g->d_map);
        g->d_map = nullptr;
        g->map_capacity = 0;
        if (amdg::device_malloc(reinterpret_cast<void**>(&g->d_map), size_t(grown) * sizeof(int32_t)) != cudaSuccess)
            return fail(AMDG_ERR_NOMEM, "cudaMalloc failed (element map)");
        g->map_capacity = grown;
    }
    if (E > g->order_capacity) {  // the current set's orders move along (a failure later leaves them intact)
        int32_t* p = nullptr;
        if (amdg::device_malloc(&p, size_t(grown) * g->host.dim * sizeof(int32_t)) != cudaSuccess)
            return fail(AMDG_ERR_NOMEM, "cudaMalloc failed (element orders)");
        const int64_t n = g->host.num_elements * g->host.dim;
        cudaStream_t st = stream_of(g);
        if (n > 0) AMDG_CK(cudaMemcpyAsync(p, g->d_order, size_t(n) * sizeof(int32_t), cudaMemcpyDeviceToDevice, st));
        AMDG_CK(cudaStreamSynchronize(st));
        cudaFree(g->d_order);
        g->d_order = p;
        g->order_capacity = grown;
    }
    return AMDG_OK;
}

amdg_status grid_device_refine(amdg_grid* g, double eps, const uint8_t* d_force, int8_t* refined, int64_t* added) {
    const KeyShape ks{g->host.dim, g->host.nmax};
    const int64_t E = g->host.num_elements;
    GridDevice& d = g->dev;
    amdg_status s;
    if ((s = ensure_stats(d)) != AMDG_OK || (s = grid_hash(g)) != AMDG_OK || (s = ensure_flags(g, E)) != AMDG_OK)
        return s;
    // added keys are children of existing elements: at most 2 dim per element
    const int64_t cap = 2 * int64_t(ks.dim) * E + 16;
    if ((s = grow(&d.newk, &d.new_cap, cap, cap + cap / 4)) != AMDG_OK) return s;
    cudaStream_t st = stream_of(g);
    AdaptStats* dst = static_cast<AdaptStats*>(d.stats);
    AMDG_CK(cudaMemsetAsync(dst, 0, kStatsReset, st));
    if (E > 0) {
        refine_mark_kernel<<<blocks_for(E, 128), 128, 0, st>>>(d.key, E, ks, d_force ? nullptr : g->d_norms, eps,
                                                               d_force, hash_of(g), d.newk, dst, d.new_cap, d.flag);
        AMDG_CK(cudaGetLastError());
        hole_fill_kernel<<<1, 1024, 0, st>>>(ks, hash_of(g), d.newk, dst, d.new_cap);
        AMDG_CK(cudaGetLastError());
        g->ctx->launches += 2;
    }
    AdaptStats hs;
    if ((s = read_stats(g, &hs)) != AMDG_OK) return s;
    if (hs.nonfinite) return fail(AMDG_ERR_NONFINITE, "element indicator is not finite");
    if (hs.err) return fail(AMDG_ERR_STATE, "device refinement: key list overflow or unfinished hole filling");
    if (refined && E > 0) {
        AMDG_CK(cudaMemcpyAsync(refined, d.flag, size_t(E), cudaMemcpyDeviceToHost, st));
        AMDG_CK(cudaStreamSynchronize(st));
    }
    const int64_t n_new = hs.count;
    if (added) *added = n_new;
    if (n_new == 0) return AMDG_OK;
    const int64_t En = E + n_new;
    if (En > (int64_t(1) << 31) - 1) return fail(AMDG_ERR_CAPACITY, "more than 2^31-1 elements");
    // every allocation before the first change, so a failure leaves the element set as it was
    if ((s = ensure_keys(g, En, true)) != AMDG_OK || (s = ensure_set_arrays(g, En)) != AMDG_OK ||
        (s = grid_reserve_remap(g, En)) != AMDG_OK)
        return s;
    size_t temp = 0;
    AMDG_CK(cub::DeviceRadixSort::SortKeys(nullptr, temp, d.key_alt, d.key, int(En), 0, ks.dim * ks.nmax, st));
    if ((s = grow_temp(d, temp)) != AMDG_OK) return s;
    // old and new keys side by side in key_alt, then sorted into key (keys use dim * nmax bits);
    // the old keys are not needed again: the map comes from the old set's hash
    concat_keys_kernel<<<blocks_for(En, 256), 256, 0, st>>>(d.key, E, d.newk, n_new, d.key_alt);
    AMDG_CK(cudaGetLastError());
    const int bits = ks.dim * ks.nmax;
    size_t tb = d.temp_bytes;
    AMDG_CK(cub::DeviceRadixSort::SortKeys(d.temp, tb, d.key_alt, d.key, int(En), 0, bits, st));
    map_from_hash_kernel<<<blocks_for(En, 256), 256, 0, st>>>(d.key, En, ks, hash_of(g), g->d_map, g->d_order);
    AMDG_CK(cudaGetLastError());
    g->ctx->launches += 3;
    if ((s = grid_apply_remap(g, En)) != AMDG_OK) return s;
    for (int k = 0; k < ks.dim; ++k) {
        g->lev_sum[k] += hs.lev_sum[k];
        g->lev_max[k] = std::max(g->lev_max[k], hs.lev_max[k]);
    }
    g->levsum_max = std::max(g->levsum_max, hs.levsum_max);
    g->host_stale = true;
    return AMDG_OK;
}

amdg_status grid_device_coarsen(amdg_grid* g, double eta, double missed_eps, int64_t* removed_out) {
    const KeyShape ks{g->host.dim, g->host.nmax};
    const int64_t E = g->host.num_elements;
    GridDevice& d = g->dev;
    amdg_status s;
    if ((s = ensure_stats(d)) != AMDG_OK || (s = grid_hash(g)) != AMDG_OK || (s = ensure_flags(g, E)) != AMDG_OK)
        return s;
    if (missed_eps > 0 && (s = grow(&d.missed, &d.missed_cap, E, E + E / 4 + 16)) != AMDG_OK) return s;
    cudaStream_t st = stream_of(g);
    AdaptStats* dst = static_cast<AdaptStats*>(d.stats);
    AMDG_CK(cudaMemsetAsync(dst, 0, kStatsReset, st));
    if (E == 0) {
        if (removed_out) *removed_out = 0;
        return AMDG_OK;
    }
    if (E <= kSmallCoarsenMax) {  // one CTA does it all
        coarsen_small_kernel<<<1, kSmallCoarsenThreads, 0, st>>>(d.key, E, ks, g->d_norms, eta, g->levsum_max,
                                                                  hash_of(g), d.flag, d.pos, missed_eps, d.missed,
                                                                  d.missed_cap, dst);
        AMDG_CK(cudaGetLastError());
        g->ctx->launches++;
    } else {
        AMDG_CK(cudaMemsetAsync(d.flag, 0, size_t(E), st));
        for (int L = g->levsum_max; L >= 1; --L) {
            coarsen_pass_kernel<<<blocks_for(E, 128), 128, 0, st>>>(d.key, E, ks, g->d_norms, eta, L, hash_of(g),
                                                                    d.flag);
            AMDG_CK(cudaGetLastError());
            g->ctx->launches++;
        }
        // kept positions: exclusive scan of keep flags (E + 1 entries, the last one 0 -> total)
        keep_flags_kernel<<<blocks_for(E + 1, 256), 256, 0, st>>>(d.flag, E, d.pos);
        AMDG_CK(cudaGetLastError());
        size_t temp = 0;
        AMDG_CK(cub::DeviceScan::ExclusiveSum(nullptr, temp, d.pos, d.pos, int(E + 1), st));
        if ((s = grow_temp(d, temp)) != AMDG_OK) return s;
        size_t tb = d.temp_bytes;
        AMDG_CK(cub::DeviceScan::ExclusiveSum(d.temp, tb, d.pos, d.pos, int(E + 1), st));
        coarsen_stats_kernel<<<blocks_for(E, 128), 128, 0, st>>>(d.key, E, ks, d.flag, d.pos, g->d_norms, missed_eps,
                                                                 hash_of(g), d.missed, d.missed_cap, dst);
        AMDG_CK(cudaGetLastError());
        g->ctx->launches += 3;
    }
    AdaptStats hs;
    if ((s = read_stats(g, &hs)) != AMDG_OK) return s;
    if (hs.nonfinite) return fail(AMDG_ERR_NONFINITE, "element indicator is not finite");
    const int64_t En = hs.count;
    if (missed_eps > 0) d.n_missed = std::min<int64_t>(hs.missed, d.missed_cap);
    if (removed_out) *removed_out = E - En;
    if (En == E) return AMDG_OK;
    if ((s = ensure_keys(g, En, true)) != AMDG_OK || (s = ensure_set_arrays(g, En)) != AMDG_OK ||
        (s = grid_reserve_remap(g, En)) != AMDG_OK)
        return s;
    compact_kernel<<<blocks_for(E, 256), 256, 0, st>>>(d.key, E, ks, d.flag, d.pos, d.key_alt, g->d_map, g->d_order);
    AMDG_CK(cudaGetLastError());
    g->ctx->launches++;
    std::swap(d.key, d.key_alt);
    if ((s = grid_apply_remap(g, En)) != AMDG_OK) return s;
    for (int k = 0; k < ks.dim; ++k) {
        g->lev_sum[k] = hs.lev_sum[k];
        g->lev_max[k] = hs.lev_max[k];
    }
    g->levsum_max = hs.levsum_max;
    g->host_stale = true;
    return AMDG_OK;
}

amdg_status grid_learned_flags(amdg_grid* g, const float* d_prob, double tau, double eps, uint8_t** d_force,
                               unsigned long long* d_counts) {
    const int64_t E = g->host.num_elements;
    if (amdg_status s = ensure_flags(g, E); s != AMDG_OK) return s;
    *d_force = g->dev.force;
    if (E == 0) return AMDG_OK;
    learned_flags_kernel<<<blocks_for(E, 128), 128, 0, stream_of(g)>>>(d_prob, E, float(tau), g->d_norms, eps,
                                                                      g->dev.force, d_counts);
    AMDG_CK(cudaGetLastError());
    g->ctx->launches++;
    return AMDG_OK;
}

int* grid_topology_error_flag(amdg_grid* g) {
    if (ensure_stats(g->dev) != AMDG_OK) return nullptr;
    return &static_cast<AdaptStats*>(g->dev.stats)->topo_err;
}

amdg_status grid_check_topology(amdg_grid* g) {
    if (amdg_status s = ensure_stats(g->dev); s != AMDG_OK) return s;
    AdaptStats hs;
    return read_stats(g, &hs);
}

amdg_status grid_mark_missed(amdg_grid* g, uint8_t* d_force) {
    if (g->dev.n_missed == 0) return AMDG_OK;
    if (amdg_status s = grid_hash(g); s != AMDG_OK) return s;
    mark_keys_kernel<<<blocks_for(g->dev.n_missed, 128), 128, 0, stream_of(g)>>>(g->dev.missed, g->dev.n_missed,
                                                                                hash_of(g), d_force);
    AMDG_CK(cudaGetLastError());
    g->ctx->launches++;
    return AMDG_OK;
}

void transform_topology_bounds(const amdg_grid* g, int64_t* vol_pairs, int64_t* flx_pairs) {
    // |vol(e, t)| = level_t(e) + 1 ancestors (itself included) + its present descendants; over a
    // hole-free set every ancestor relation is counted from both ends: E + 2 sum_e level_t(e).
    // flx adds at most 4 touching intervals per level >= 2.
    const int64_t E = g->host.num_elements;
    int64_t v = 0;
    for (int t = 0; t < g->host.dim; ++t) v += E + 2 * g->lev_sum[t];
    *vol_pairs = v;
    *flx_pairs = v + 4 * int64_t(std::max(g->host.nmax - 1, 0)) * E * g->host.dim;
}

// Exclusive scans of the vol and flx row counts (n entries each) in one CTA, for small element
// sets: the results of the two device-wide scans without their launches.
__global__ void __launch_bounds__(kSmallCoarsenThreads)
    scan_pair_small_kernel(const int32_t* __restrict__ a, const int32_t* __restrict__ b, int64_t n,
                           int32_t* __restrict__ sa, int32_t* __restrict__ sb) {
    using Scan = cub::BlockScan<int, kSmallCoarsenThreads>;
    __shared__ typename Scan::TempStorage tmp;
    const int tid = threadIdx.x;
    for (int which = 0; which < 2; ++which) {
        const int32_t* in = which ? b : a;
        int32_t* out = which ? sb : sa;
        int v[kSmallCoarsenItems];
#pragma unroll
        for (int i = 0; i < kSmallCoarsenItems; ++i) {
            const int64_t r = int64_t(tid) * kSmallCoarsenItems + i;
            v[i] = r < n ? in[r] : 0;
        }
        Scan(tmp).ExclusiveSum(v, v);
#pragma unroll
        for (int i = 0; i < kSmallCoarsenItems; ++i) {
            const int64_t r = int64_t(tid) * kSmallCoarsenItems + i;
            if (r < n) out[r] = v[i];
        }
        __syncthreads();  // the temp storage is reused
    }
}

amdg_status device_transform_topology(amdg_grid* g, const DeviceTopoOut& out, int32_t* d_cnt, void* stream) {
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (amdg_status s = grid_hash(g); s != AMDG_OK) return s;
    const int64_t E = g->host.num_elements;
    const int dim = g->host.dim;
    const int64_t rows = E * dim;
    TopoArgs A{g->dev.key, E, KeyShape{dim, g->host.nmax}, hash_of(g)};
    // counts of the vol rows in d_cnt[0 .. rows], of the flx rows in d_cnt[rows + 1 ..]
    int32_t* vcnt = d_cnt;
    int32_t* fcnt = d_cnt + rows + 1;
    topo_count_kernel<<<blocks_for(32 * (rows + 1), 256), 256, 0, st>>>(A, vcnt, fcnt);
    AMDG_CK(cudaGetLastError());
    if (rows + 1 <= kSmallCoarsenMax) {
        scan_pair_small_kernel<<<1, kSmallCoarsenThreads, 0, st>>>(vcnt, fcnt, rows + 1, out.vol_ptr, out.flx_ptr);
        AMDG_CK(cudaGetLastError());
    } else {
        size_t temp = 0;
        AMDG_CK(cub::DeviceScan::ExclusiveSum(nullptr, temp, vcnt, out.vol_ptr, int(rows + 1), st));
        if (amdg_status s = grow_temp(g->dev, temp); s != AMDG_OK) return s;
        size_t tb = g->dev.temp_bytes;
        AMDG_CK(cub::DeviceScan::ExclusiveSum(g->dev.temp, tb, vcnt, out.vol_ptr, int(rows + 1), st));
        tb = g->dev.temp_bytes;
        AMDG_CK(cub::DeviceScan::ExclusiveSum(g->dev.temp, tb, fcnt, out.flx_ptr, int(rows + 1), st));
    }
    topo_fill_kernel<<<blocks_for(32 * rows, 256), 256, 0, st>>>(
        A, out.vol_ptr, out.flx_ptr, reinterpret_cast<int2*>(out.vol_nbr), reinterpret_cast<int2*>(out.flx_nbr),
        out.vol_split, out.flx_split, out.vol_cap, out.flx_cap, out.err);
    AMDG_CK(cudaGetLastError());
    ancestors_kernel<<<blocks_for(rows, 128), 128, 0, st>>>(A, out.anc_order, out.p1, out.anc, out.err);
    AMDG_CK(cudaGetLastError());
    g->ctx->launches += 6;
    return AMDG_OK;
}

amdg_status device_parent_table(amdg_grid* g, int32_t* d_pg, void* stream) {
    if (amdg_status s = grid_hash(g); s != AMDG_OK) return s;
    const int64_t E = g->host.num_elements;
    const int dim = g->host.dim;
    if (E == 0) return AMDG_OK;
    TopoArgs A{g->dev.key, E, KeyShape{dim, g->host.nmax}, hash_of(g)};
    parent_table_kernel<<<blocks_for(E * dim, 128), 128, 0, static_cast<cudaStream_t>(stream)>>>(A, d_pg);
    AMDG_CK(cudaGetLastError());
    g->ctx->launches++;
    return AMDG_OK;
}

}  // namespace amdg
