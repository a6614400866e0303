// Flattened sparse-grid element table and the neighbour lists of the linear
// operator.  Replaces the reference's std::unordered_map<int,Element> with an
// int32 hash key (DGSolution.h:219, Hash.cpp:55-114) and its O(E^2) pointer
// discovery (DGSolution.cpp:675-728): elements are sorted packed 64-bit keys
// and neighbours are found by binary search.
#include <algorithm>
#include <cmath>
#include <unordered_map>

#include "amdg_internal.hpp"

namespace amdg {

static uint64_t pack(const int32_t* o, int dim, int nmax) {
    uint64_t key = 0;
    for (int d = 0; d < dim; ++d) key = (key << nmax) | uint64_t(o[d]);
    return key;
}

void build_grid(int dim, int nmax, int sparse, HostGrid* g, int level_init) {
    if (level_init < 0 || level_init > nmax) level_init = nmax;
    g->dim = dim;
    g->nmax = nmax;
    g->sparse = sparse;
    g->order.clear();
    g->key.clear();
    // Level vectors with sum <= nmax (sparse) or all of them (full),
    // DGSolution.cpp:17-27; within a level vector every support combination.
    // Keys are then sorted, which orders elements lexicographically by their
    // 1D orders.
    std::vector<int> lv(dim, 0);
    std::vector<int32_t> o(dim);
    for (;;) {
        int lsum = 0;
        for (int d = 0; d < dim; ++d) lsum += lv[d];
        if (!sparse || lsum <= level_init) {
            int64_t ne = 1;
            for (int d = 0; d < dim; ++d) ne *= lv[d] == 0 ? 1 : (int64_t(1) << (lv[d] - 1));
            for (int64_t i = 0; i < ne; ++i) {
                int64_t rem = i;
                for (int d = dim - 1; d >= 0; --d) {
                    const int64_t nd = lv[d] == 0 ? 1 : (int64_t(1) << (lv[d] - 1));
                    o[d] = lv[d] == 0 ? 0 : int32_t((int64_t(1) << (lv[d] - 1)) + rem % nd);
                    rem /= nd;
                }
                g->key.push_back(pack(o.data(), dim, nmax));
            }
        }
        int d = dim - 1;
        while (d >= 0) {
            if (++lv[d] <= level_init) break;
            lv[d] = 0;
            --d;
        }
        if (d < 0) break;
    }
    std::sort(g->key.begin(), g->key.end());
    g->num_elements = int64_t(g->key.size());
    g->order.resize(size_t(g->num_elements) * dim);
    const uint64_t mask = nmax == 0 ? 0 : ((uint64_t(1) << nmax) - 1);
    for (int64_t e = 0; e < g->num_elements; ++e)
        for (int d = 0; d < dim; ++d)
            g->order[size_t(e) * dim + d] = int32_t((g->key[e] >> (uint64_t(nmax) * (dim - 1 - d))) & mask);
    build_key_index(g);
}

void build_key_index(HostGrid* g) {
    const int64_t E = g->num_elements;
    int bits = 4;
    while ((int64_t(1) << bits) < 2 * E) ++bits;
    const uint64_t cap = uint64_t(1) << bits, mask = cap - 1;
    g->hbits = bits;
    g->hkey.assign(cap, 0);
    g->hval.assign(cap, -1);
    for (int64_t e = 0; e < E; ++e) {
        uint64_t h = (g->key[e] * 0x9E3779B97F4A7C15ull) >> (64 - bits);
        while (g->hval[h] >= 0) h = (h + 1) & mask;
        g->hkey[h] = g->key[e];
        g->hval[h] = int32_t(e);
    }
}

int64_t find_element(const HostGrid& g, const int32_t* orders) { return g.index_of(pack(orders, g.dim, g.nmax)); }

// 1D flux-neighbour predicate (Element.cpp:283-348): supports intersect, are
// adjacent, or are adjacent across the periodic boundary.
static bool flux_related(int64_t a, int64_t b, int64_t a2, int64_t b2, int64_t one) {
    const bool no_int = (a >= b2) || (b <= a2);
    const bool adj = (a == b2) || (b == a2);
    const bool per = (a == 0 && b2 == one) || (a2 == 0 && b == one);
    return !no_int || adj || per;
}

void build_linear_topology(const HostGrid& g, const Oper1D& op, const double* coef, LinearTopology* out) {
    const int dim = g.dim, nmax = g.nmax, np = g.k + 1, n1 = 1 << nmax;
    const int64_t one = int64_t(1) << nmax;
    const int nb = op.nb;
    // 1D block of (solution element oc -> test element o) in dimension t:
    // c_t*u_vx on intersecting supports plus c_t*flux, each entry dropped below
    // 1e-13 as in BilinearFormAlpt::assemble_matrix_alpt (BilinearForm.cpp:64-75).
    std::vector<std::vector<int>> rel1d(n1);  // solution orders related to test order o
    out->blocks.clear();
    // count blocks per dimension first: identical pair list for every dimension
    std::vector<std::vector<std::vector<double>>> tmp(dim);
    int nblocks = 0;
    for (int o = 0; o < n1; ++o) {
        int64_t a, b;
        support_units(o, nmax, &a, &b);
        for (int oc = 0; oc < n1; ++oc) {
            int64_t a2, b2;
            support_units(oc, nmax, &a2, &b2);
            if (!flux_related(a, b, a2, b2, one)) continue;
            const bool vol = !((a >= b2) || (b <= a2));
            bool any = false;
            std::vector<std::vector<double>> blk(dim, std::vector<double>(np * np, 0.0));
            for (int t = 0; t < dim; ++t) {
                const std::vector<double>& flux = coef[t] >= 0 ? op.ulft_vjp : op.urgt_vjp;
                for (int p = 0; p < np; ++p)
                    for (int q = 0; q < np; ++q) {
                        const size_t idx = size_t(oc * np + p) * nb + (o * np + q);
                        double v = 0.0;
                        const double mv = coef[t] * op.u_vx[idx];
                        const double mf = coef[t] * flux[idx];
                        if (vol && std::fabs(mv) >= kRoundOff) v += mv;
                        if (std::fabs(mf) >= kRoundOff) v += mf;
                        blk[t][p * np + q] = v;
                        any = any || (v != 0.0);
                    }
            }
            if (!any) continue;
            rel1d[o].push_back(oc);
            for (int t = 0; t < dim; ++t) tmp[t].push_back(blk[t]);
            ++nblocks;
        }
    }
    out->num_blocks = nblocks;
    out->blocks.assign(size_t(dim) * nblocks * np * np, 0.0);
    for (int t = 0; t < dim; ++t)
        for (int i = 0; i < nblocks; ++i)
            std::copy(tmp[t][i].begin(), tmp[t][i].end(), out->blocks.begin() + (size_t(t) * nblocks + i) * np * np);
    // block id of (o, idx-th related)
    std::vector<int> blk_base(n1 + 1, 0);
    for (int o = 0; o < n1; ++o) blk_base[o + 1] = blk_base[o] + int(rel1d[o].size());

    const int64_t E = g.num_elements;
    out->row_ptr.assign(size_t(E) * dim + 1, 0);
    out->src.clear();
    out->blk.clear();
    std::vector<int32_t> o2(dim);
    for (int64_t e = 0; e < E; ++e) {
        const int32_t* oe = &g.order[size_t(e) * dim];
        for (int t = 0; t < dim; ++t) {
            std::copy(oe, oe + dim, o2.begin());
            const int o = oe[t];
            for (size_t i = 0; i < rel1d[o].size(); ++i) {
                const int id = blk_base[o] + int(i);
                const double* bp = &out->blocks[(size_t(t) * nblocks + id) * np * np];
                bool nz = false;
                for (int m = 0; m < np * np; ++m) nz = nz || (bp[m] != 0.0);
                if (!nz) continue;  // zero in this dimension (e.g. c_t == 0)
                o2[t] = rel1d[o][i];
                const int64_t s = find_element(g, o2.data());
                if (s < 0) continue;
                out->src.push_back(int32_t(s));
                out->blk.push_back(int32_t(id));
            }
            out->row_ptr[size_t(e) * dim + t + 1] = int32_t(out->src.size());
        }
    }
}

}  // namespace amdg

namespace amdg {

// Element indices grouped into fibres along dimension t (equal orders in every
// other dimension), each fibre in increasing order along t; start holds the
// fibre boundaries.
static void fibres_along(const HostGrid& g, int t, std::vector<int32_t>* perm, std::vector<int64_t>* start) {
    const uint64_t shift = uint64_t(g.nmax) * (g.dim - 1 - t);
    const uint64_t field = (g.nmax == 0 ? 0 : ((uint64_t(1) << g.nmax) - 1));
    const int64_t E = g.num_elements;
    perm->resize(E);
    // sort key: the other dimensions' fields (fibre), then the field of t
    std::vector<std::pair<uint64_t, int32_t>> ck(E);
    for (int64_t e = 0; e < E; ++e) {
        const uint64_t k = g.key[e];
        const uint64_t high = shift + g.nmax >= 64 ? 0 : k >> (shift + g.nmax);
        const uint64_t low = k & ((uint64_t(1) << shift) - 1);
        ck[e] = {(((high << shift) | low) << g.nmax) | ((k >> shift) & field), int32_t(e)};
    }
    if (t != g.dim - 1) std::sort(ck.begin(), ck.end());  // sorted keys are already grouped along the last dimension
    start->clear();
    for (int64_t i = 0; i < E; ++i) {
        (*perm)[i] = ck[i].second;
        if (i == 0 || (ck[i].first >> g.nmax) != (ck[i - 1].first >> g.nmax)) start->push_back(i);
    }
    start->push_back(E);
}

namespace {

// One fibre along t: members perm[s0 .. s1) sorted by 1D order.  A long fibre also keeps
// cum[o] = the number of members whose 1D order is below o (o = 0 .. 2^nmax), so the members
// with orders in [lo, hi] are perm[s0 + cum[lo] .. s0 + cum[hi + 1]); a short one is scanned.
constexpr int64_t kScanFibre = 48;
struct Fibre {
    const HostGrid& g;
    const int32_t* perm;
    const int64_t* lo;  // 1D support [lo[o], hi[o]) of order o, in units of 2^-nmax
    const int64_t* hi;
    int t;
    int64_t s0, s1;
    bool indexed;
    std::vector<int32_t>& cum;
    Fibre(const HostGrid& g_, const int32_t* perm_, const int64_t* lo_, const int64_t* hi_, int t_, int64_t s0_,
          int64_t s1_, std::vector<int32_t>& cum_)
        : g(g_), perm(perm_), lo(lo_), hi(hi_), t(t_), s0(s0_), s1(s1_), indexed(s1_ - s0_ > kScanFibre), cum(cum_) {
        if (!indexed) return;
        const int n1 = 1 << g.nmax;
        cum.assign(size_t(n1) + 1, 0);
        for (int64_t j = s0; j < s1; ++j) ++cum[size_t(ord(j)) + 1];
        for (int o = 0; o < n1; ++o) cum[size_t(o) + 1] += cum[o];
    }
    int ord(int64_t j) const { return g.order[size_t(perm[j]) * g.dim + t]; }
    template <class Fn>
    void range(int64_t lo, int64_t hi, Fn&& fn) const {
        for (int64_t j = s0 + cum[size_t(lo)]; j < s0 + cum[size_t(hi) + 1]; ++j) fn(perm[j], ord(j));
    }
};

// The neighbours of fibre member i along t, in increasing 1D order: vol(s, o) for the members
// whose 1D supports intersect i's, flx(s, o) for those that intersect or touch it, also across
// the periodic boundary (Element.cpp:283-348).  Levels 0 and 1 cover the whole domain; at level
// l >= 2 the intervals meeting [a, b) are an index range, widened by one on a side where an
// interval ends (or starts) exactly at the boundary, plus the wrap-around neighbour.
template <class V, class F>
void fibre_neighbours(const Fibre& fb, int64_t i, V&& vol, F&& flx) {
    const int nmax = fb.g.nmax;
    const int64_t one = int64_t(1) << nmax;
    const int oi = fb.ord(i);
    const int64_t a0 = fb.lo[oi], b0 = fb.hi[oi];
    if (!fb.indexed) {  // short fibre: test every member
        for (int64_t j = fb.s0; j < fb.s1; ++j) {
            const int o = fb.ord(j);
            const int64_t a2 = fb.lo[o], b2 = fb.hi[o];
            const bool v = !((a0 >= b2) || (b0 <= a2));
            if (v) vol(fb.perm[j], o);
            if (v || flux_related(a0, b0, a2, b2, one)) flx(fb.perm[j], o);
        }
        return;
    }
    for (int l = 0; l <= nmax && l <= 1; ++l) {
        fb.range(l, l, vol);
        fb.range(l, l, flx);
    }
    for (int l = 2; l <= nmax; ++l) {
        const int64_t cnt = int64_t(1) << (l - 1), w = one >> (l - 1);
        const int64_t first = a0 / w, last = (b0 - 1) / w;
        fb.range(cnt + first, cnt + last, vol);
        int64_t lo = first, hi = last;
        if (a0 % w == 0 && first >= 1) --lo;
        if (b0 % w == 0 && last + 1 < cnt) ++hi;
        if (b0 == one && lo > 0) fb.range(cnt, cnt, flx);  // the first interval, across x = 1
        fb.range(cnt + lo, cnt + hi, flx);
        if (a0 == 0 && hi < cnt - 1) fb.range(2 * cnt - 1, 2 * cnt - 1, flx);  // the last, across x = 0
    }
}

}  // namespace

void build_transform_topology(const HostGrid& g, TransformTopology* out) {
    const int dim = g.dim, nmax = g.nmax, n1 = 1 << nmax;
    std::vector<int32_t> lev(n1);
    std::vector<int64_t> slo(n1), shi(n1);
    for (int o = 0; o < n1; ++o) {
        lev[o] = level_of_order(o);
        support_units(o, nmax, &slo[o], &shi[o]);
    }
    const int64_t E = g.num_elements;
    std::vector<std::vector<int32_t>> perm(dim);
    std::vector<std::vector<int64_t>> start(dim);
#pragma omp parallel for schedule(static) if (E >= 4096)
    for (int t = 0; t < dim; ++t) fibres_along(g, t, &perm[t], &start[t]);
    // pass 1: neighbour counts per (element, dimension); pass 2: the lists at their final place
    std::vector<int32_t> vcnt(size_t(E) * dim), fcnt(size_t(E) * dim);
    for (int t = 0; t < dim; ++t) {
        const int64_t nf = int64_t(start[t].size()) - 1;
#pragma omp parallel if (E >= 8192)
        {
            std::vector<int32_t> cum;
#pragma omp for schedule(dynamic, 8)
            for (int64_t f = 0; f < nf; ++f) {
                const Fibre fb(g, perm[t].data(), slo.data(), shi.data(), t, start[t][f], start[t][f + 1], cum);
                for (int64_t i = start[t][f]; i < start[t][f + 1]; ++i) {
                    int32_t nv = 0, nfx = 0;
                    fibre_neighbours(fb, i, [&](int32_t, int) { ++nv; }, [&](int32_t, int) { ++nfx; });
                    const size_t r = size_t(perm[t][i]) * dim + t;
                    vcnt[r] = nv;
                    fcnt[r] = nfx;
                }
            }
        }
    }
    out->vol_ptr.assign(size_t(E) * dim + 1, 0);
    out->flx_ptr.assign(size_t(E) * dim + 1, 0);
    for (size_t r = 0; r < size_t(E) * dim; ++r) {
        out->vol_ptr[r + 1] = out->vol_ptr[r] + vcnt[r];
        out->flx_ptr[r + 1] = out->flx_ptr[r] + fcnt[r];
    }
    out->vol_nbr.resize(size_t(2) * out->vol_ptr.back());
    out->flx_nbr.resize(size_t(2) * out->flx_ptr.back());
    out->vol_split.assign(size_t(E) * dim, 0);
    out->flx_split.assign(size_t(E) * dim, 0);
    for (int t = 0; t < dim; ++t) {
        const int64_t nf = int64_t(start[t].size()) - 1;
#pragma omp parallel if (E >= 8192)
        {
            std::vector<int32_t> cum;
#pragma omp for schedule(dynamic, 8)
            for (int64_t f = 0; f < nf; ++f) {
                const Fibre fb(g, perm[t].data(), slo.data(), shi.data(), t, start[t][f], start[t][f + 1], cum);
                for (int64_t i = start[t][f]; i < start[t][f + 1]; ++i) {
                    const size_t r = size_t(perm[t][i]) * dim + t;
                    const int own = lev[fb.ord(i)];
                    int32_t* vp = &out->vol_nbr[2 * size_t(out->vol_ptr[r])];
                    int32_t* fp = &out->flx_nbr[2 * size_t(out->flx_ptr[r])];
                    // the "U" part (level <= own) is a prefix, the "L" part (finer) the rest
                    int32_t nv = 0, nfx = 0, sv = 0, sf = 0;
                    fibre_neighbours(
                        fb, i,
                        [&](int32_t s, int o) {
                            vp[2 * nv] = s;
                            vp[2 * nv + 1] = o;
                            ++nv;
                            if (lev[o] <= own) sv = nv;
                        },
                        [&](int32_t s, int o) {
                            fp[2 * nfx] = s;
                            fp[2 * nfx + 1] = o;
                            ++nfx;
                            if (lev[o] <= own) sf = nfx;
                        });
                    out->vol_split[r] = out->vol_ptr[r] + sv;
                    out->flx_split[r] = out->flx_ptr[r] + sf;
                }
            }
        }
    }
}

bool build_surplus_ancestors(const HostGrid& g, const LagrTables& t, std::vector<int32_t>* anc) {
    const int dim = g.dim;
    const int64_t E = g.num_elements;
    const int P1 = t.p1;
    anc->assign(size_t(E) * dim * P1, -1);
    int holes = 0;
#pragma omp parallel for schedule(static) reduction(+ : holes) if (E >= 4096)
    for (int64_t e = 0; e < E; ++e) {
        int32_t o2[kMaxDim];
        const int32_t* oe = &g.order[size_t(e) * dim];
        for (int d = 0; d < dim; ++d) {
            if (oe[d] == 0) continue;
            for (int ic = 0; ic < P1; ++ic) {
                std::copy(oe, oe + dim, o2);
                o2[d] = t.anc_order[size_t(oe[d]) * P1 + ic];
                const int64_t s = find_element(g, o2);
                if (s < 0) ++holes;  // the element set has a hole
                (*anc)[(size_t(e) * dim + d) * P1 + ic] = int32_t(s);
            }
        }
    }
    return holes == 0;
}

}  // namespace amdg

namespace amdg {

void build_batch_tables(const Oper1D& op, int nmax, int np, BatchTables* out) {
    const int n1 = 1 << nmax;
    const int64_t one = int64_t(1) << nmax;
    const int nb = op.nb;
    // shared 1D blocks, one table per upwind side: u_vx on intersecting supports
    // plus ulft_vjp (c >= 0) or urgt_vjp (c < 0), entries below 1e-13 dropped;
    // a pair is listed when either side is nonzero
    out->rel1d.assign(n1, {});
    std::vector<double> t0, t1;
    for (int o = 0; o < n1; ++o) {
        int64_t a, b;
        support_units(o, nmax, &a, &b);
        for (int oc = 0; oc < n1; ++oc) {
            int64_t a2, b2;
            support_units(oc, nmax, &a2, &b2);
            if (!flux_related(a, b, a2, b2, one)) continue;
            const bool vol = !((a >= b2) || (b <= a2));
            double blk[2][16];
            bool any = false;
            for (int side = 0; side < 2; ++side) {
                const std::vector<double>& flux = side == 0 ? op.ulft_vjp : op.urgt_vjp;
                for (int p = 0; p < np; ++p)
                    for (int q = 0; q < np; ++q) {
                        const size_t idx = size_t(oc * np + p) * nb + (o * np + q);
                        double v = 0.0;
                        if (vol && std::fabs(op.u_vx[idx]) >= kRoundOff) v += op.u_vx[idx];
                        if (std::fabs(flux[idx]) >= kRoundOff) v += flux[idx];
                        blk[side][p * np + q] = v;
                        any = any || v != 0.0;
                    }
            }
            if (!any) continue;
            out->rel1d[o].push_back(oc);
            t0.insert(t0.end(), blk[0], blk[0] + np * np);
            t1.insert(t1.end(), blk[1], blk[1] + np * np);
        }
    }
    out->num_blocks = int(t0.size() / (np * np));
    out->blocks = t0;
    out->blocks.insert(out->blocks.end(), t1.begin(), t1.end());
    out->blk_base.assign(n1 + 1, 0);
    for (int o = 0; o < n1; ++o) out->blk_base[o + 1] = out->blk_base[o] + int(out->rel1d[o].size());
}

void build_batch_topology(const std::vector<const HostGrid*>& grids, const BatchTables& t, BatchTopology* out) {
    const int dim = grids[0]->dim;
    const int64_t n = int64_t(grids.size());
    out->num_blocks = t.num_blocks;
    out->blocks = t.blocks;
    out->elem_offset.assign(n + 1, 0);
    for (int64_t sv = 0; sv < n; ++sv) out->elem_offset[sv + 1] = out->elem_offset[sv] + grids[sv]->num_elements;
    const int64_t total = out->elem_offset[n];
    // per solve: row ends relative to the solve's first pair, sources relative to its first element
    std::vector<std::vector<int64_t>> rows(n);
    std::vector<std::vector<int32_t>> src(n), blk(n);
#pragma omp parallel for schedule(dynamic, 1) if (total >= 16384)
    for (int64_t sv = 0; sv < n; ++sv) {
        const HostGrid& g = *grids[sv];
        std::vector<int32_t> o2(dim);
        rows[sv].resize(size_t(g.num_elements) * dim);
        for (int64_t e = 0; e < g.num_elements; ++e) {
            const int32_t* oe = &g.order[size_t(e) * dim];
            for (int d = 0; d < dim; ++d) {
                std::copy(oe, oe + dim, o2.begin());
                const int o = oe[d];
                const std::vector<int>& rel = t.rel1d[o];
                for (size_t i = 0; i < rel.size(); ++i) {
                    o2[d] = rel[i];
                    const int64_t s = find_element(g, o2.data());
                    if (s < 0) continue;
                    src[sv].push_back(int32_t(s));
                    blk[sv].push_back(t.blk_base[o] + int32_t(i));
                }
                rows[sv][size_t(e) * dim + d] = int64_t(src[sv].size());
            }
        }
    }
    std::vector<int64_t> pair_offset(n + 1, 0);
    for (int64_t sv = 0; sv < n; ++sv) pair_offset[sv + 1] = pair_offset[sv] + int64_t(src[sv].size());
    out->row_ptr.assign(size_t(total) * dim + 1, 0);
    out->src.resize(pair_offset[n]);
    out->blk.resize(pair_offset[n]);
    out->solve_of.resize(total);
#pragma omp parallel for schedule(dynamic, 1) if (total >= 16384)
    for (int64_t sv = 0; sv < n; ++sv) {
        const int64_t e0 = out->elem_offset[sv], p0 = pair_offset[sv];
        for (size_t r = 0; r < rows[sv].size(); ++r) out->row_ptr[size_t(e0) * dim + r + 1] = p0 + rows[sv][r];
        for (size_t i = 0; i < src[sv].size(); ++i) {
            out->src[p0 + i] = e0 + src[sv][i];
            out->blk[p0 + i] = blk[sv][i];
        }
        std::fill(out->solve_of.begin() + e0, out->solve_of.begin() + e0 + grids[sv]->num_elements, int32_t(sv));
    }
}

}  // namespace amdg
