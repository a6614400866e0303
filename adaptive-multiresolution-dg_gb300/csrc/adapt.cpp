// Adaptivity on the flattened element table: refine, coarsen and hole
// filling on packed keys (DGAdapt::refine DGAdapt.cpp:371-404, coarsen
// :675-688,982-1016, check_hole :1351-1385, child/parent index rules
// :1250-1312), and the adaptive separable initialisation
// (DGAdapt::init_separable_scalar_sum, :120-147, 850-894).
//
// Keys pack the 1D orders of an element, nmax bits per dimension, first
// dimension most significant.  In 1D order space the children of o are
// {1} for o = 0, {2o, 2o+1} for 1 <= level < nmax and none at level nmax; the
// parent of o >= 1 is 0 for o = 1 and o/2 otherwise.
#include <algorithm>
#include <cmath>
#include <unordered_set>

#include "amdg_internal.hpp"

namespace amdg {
namespace {

inline int field(uint64_t key, int d, int dim, int nmax) {
    const uint64_t mask = nmax == 0 ? 0 : ((uint64_t(1) << nmax) - 1);
    return int((key >> (uint64_t(nmax) * (dim - 1 - d))) & mask);
}

inline uint64_t with_field(uint64_t key, int d, int dim, int nmax, int o) {
    const uint64_t shift = uint64_t(nmax) * (dim - 1 - d);
    const uint64_t mask = (nmax == 0 ? 0 : ((uint64_t(1) << nmax) - 1)) << shift;
    return (key & ~mask) | (uint64_t(o) << shift);
}

int children_1d(int o, int nmax, int* out) {
    const int n = level_of_order(o);
    if (n == 0) { out[0] = 1; return nmax >= 1 ? 1 : 0; }
    if (n == nmax) return 0;
    out[0] = 2 * o;
    out[1] = 2 * o + 1;
    return 2;
}

// Growable open-addressing set of keys (keys never have all bits set: they
// use at most 60 bits).
class KeySet {
public:
    bool insert(uint64_t k) {
        if (2 * (n_ + 1) > slot_.size()) grow();
        const uint64_t mask = slot_.size() - 1;
        for (uint64_t h = hash(k, mask); ; h = (h + 1) & mask) {
            if (slot_[h] == kEmpty) {
                slot_[h] = k;
                ++n_;
                return true;
            }
            if (slot_[h] == k) return false;
        }
    }
private:
    static constexpr uint64_t kEmpty = ~uint64_t(0);
    static uint64_t hash(uint64_t k, uint64_t mask) { return (k * 0x9E3779B97F4A7C15ull >> 17) & mask; }
    void grow() {
        std::vector<uint64_t> old;
        old.swap(slot_);
        slot_.assign(std::max<size_t>(64, old.size() * 2), kEmpty);
        n_ = 0;
        for (uint64_t k : old)
            if (k != kEmpty) insert(k);
    }
    std::vector<uint64_t> slot_;
    size_t n_ = 0;
};

// existing children of element e and the number it can have
void child_counts(const HostGrid& g, int64_t e, int* existing, int* total) {
    const int dim = g.dim, nmax = g.nmax;
    int ch[2];
    *existing = *total = 0;
    for (int d = 0; d < dim; ++d) {
        const int nc = children_1d(field(g.key[e], d, dim, nmax), nmax, ch);
        *total += nc;
        for (int c = 0; c < nc; ++c) *existing += g.index_of(with_field(g.key[e], d, dim, nmax, ch[c])) >= 0 ? 1 : 0;
    }
}

}  // namespace

std::vector<uint64_t> refine_keys(const HostGrid& g, const double* norms, double eps, std::vector<uint8_t>* refined,
                                  const uint8_t* force) {
    const int dim = g.dim, nmax = g.nmax;
    KeySet added;  // keys not in g
    std::vector<uint64_t> work, fresh;
    if (refined) refined->assign(g.num_elements, 0);
    int ch[2];
    for (int64_t e = 0; e < g.num_elements; ++e) {
        // a leaf has fewer existing children than possible (DGAdapt::update_leaf)
        const bool want = force ? force[e] != 0 : (norms[e] > eps);
        if (!want) continue;
        int existing, total;
        child_counts(g, e, &existing, &total);
        if (existing >= total) continue;
        if (refined) (*refined)[e] = 1;
        const uint64_t key = g.key[e];
        for (int d = 0; d < dim; ++d) {
            const int nc = children_1d(field(key, d, dim, nmax), nmax, ch);
            for (int c = 0; c < nc; ++c) {
                const uint64_t ck = with_field(key, d, dim, nmax, ch[c]);
                if (g.index_of(ck) < 0 && added.insert(ck)) work.push_back(ck);
            }
        }
    }
    // hole filling: every parent of a new element must exist (DGAdapt::check_hole)
    fresh = work;
    while (!work.empty()) {
        std::vector<uint64_t> next;
        for (uint64_t key : work)
            for (int d = 0; d < dim; ++d) {
                const int o = field(key, d, dim, nmax);
                if (o == 0) continue;
                const uint64_t p = with_field(key, d, dim, nmax, o == 1 ? 0 : o / 2);
                if (g.index_of(p) < 0 && added.insert(p)) {
                    next.push_back(p);
                    fresh.push_back(p);
                }
            }
        work.swap(next);
    }
    // the existing keys are ascending: sort the new ones and merge
    std::sort(fresh.begin(), fresh.end());
    std::vector<uint64_t> keys(g.key.size() + fresh.size());
    std::merge(g.key.begin(), g.key.end(), fresh.begin(), fresh.end(), keys.begin());
    return keys;
}

std::vector<uint64_t> coarsen_keys(const HostGrid& g, const double* norms, double eta) {
    const int dim = g.dim, nmax = g.nmax;
    const int64_t E = g.num_elements;
    std::vector<char> alive(E, 1);
    // existing-children counts, kept up to date as elements are removed
    std::vector<int> kids(E, 0);
    std::vector<int64_t> parent(size_t(E) * dim, -1);
    for (int64_t e = 0; e < E; ++e)
        for (int d = 0; d < dim; ++d) {
            const int o = field(g.key[e], d, dim, nmax);
            if (o == 0) continue;
            const int64_t p = g.index_of(with_field(g.key[e], d, dim, nmax, o == 1 ? 0 : o / 2));
            parent[size_t(e) * dim + d] = p;
            if (p >= 0) ++kids[p];
        }
    auto removable = [&](int64_t e) {
        if (!alive[e] || kids[e] != 0 || !(norms[e] < eta)) return false;
        int maxlev = 0;
        for (int d = 0; d < dim; ++d) maxlev = std::max(maxlev, level_of_order(field(g.key[e], d, dim, nmax)));
        return maxlev > 0;
    };
    // repeated sweeps over childless elements until nothing changes (DGAdapt::coarsen_no_leaf)
    std::vector<int64_t> work;
    for (int64_t e = 0; e < E; ++e) if (removable(e)) work.push_back(e);
    while (!work.empty()) {
        std::vector<int64_t> next;
        for (int64_t e : work) {
            if (!removable(e)) continue;
            alive[e] = 0;
            for (int d = 0; d < dim; ++d) {
                const int64_t p = parent[size_t(e) * dim + d];
                if (p >= 0 && --kids[p] == 0 && removable(p)) next.push_back(p);
            }
        }
        work.swap(next);
    }
    std::vector<uint64_t> keys;
    for (int64_t e = 0; e < E; ++e) if (alive[e]) keys.push_back(g.key[e]);
    return keys;
}

void leaf_flags(const HostGrid& g, std::vector<uint8_t>* leaf) {
    leaf->assign(g.num_elements, 0);
    for (int64_t e = 0; e < g.num_elements; ++e) {
        int existing, total;
        child_counts(g, e, &existing, &total);
        (*leaf)[e] = existing < total ? 1 : 0;
    }
}

void parent_table(const HostGrid& g, std::vector<int32_t>* pg) {
    const int dim = g.dim, nmax = g.nmax;
    pg->assign(size_t(g.num_elements) * dim * 2, -1);
    for (int64_t e = 0; e < g.num_elements; ++e)
        for (int d = 0; d < dim; ++d) {
            uint64_t k = g.key[e];
            for (int gen = 0; gen < 2; ++gen) {
                const int o = field(k, d, dim, nmax);
                if (o == 0) break;
                k = with_field(k, d, dim, nmax, o == 1 ? 0 : o / 2);
                (*pg)[(size_t(e) * dim + d) * 2 + gen] = int32_t(g.index_of(k));
            }
        }
}

void batch_parent_table(const std::vector<const HostGrid*>& grids, const std::vector<int64_t>& offset,
                        std::vector<int32_t>* pg) {
    const int64_t n = int64_t(grids.size());
    const int dim = n ? grids[0]->dim : 0;
    pg->assign(n ? size_t(offset[n]) * dim * 2 : 0, -1);
#pragma omp parallel for schedule(dynamic, 1) if (n > 1 && offset[n] >= 16384)
    for (int64_t i = 0; i < n; ++i) {
        std::vector<int32_t> local;
        parent_table(*grids[i], &local);
        int32_t* out = pg->data() + size_t(offset[i]) * dim * 2;
        for (size_t j = 0; j < local.size(); ++j) out[j] = local[j] < 0 ? -1 : int32_t(offset[i] + local[j]);
    }
}

void adapt_keys_between_steps(const HostGrid& g, const double* norms, const uint8_t* force, double eps, double eta,
                              std::vector<uint64_t>* keys, std::vector<uint8_t>* carry) {
    const int64_t E = g.num_elements;
    HostGrid kept;
    kept.sparse = g.sparse;
    grid_from_keys(g.dim, g.nmax, g.k, coarsen_keys(g, norms, eta), &kept);
    carry->assign(E, 0);
    std::vector<uint8_t> pick(kept.num_elements, 0);
    for (int64_t e = 0, j = 0; e < kept.num_elements; ++e) {
        while (g.key[j] < kept.key[e]) ++j;  // kept is a subset of the ascending old keys
        (*carry)[j] = 1;
        pick[e] = force ? force[j] : (norms[j] > eps ? 1 : 0);
    }
    *keys = refine_keys(kept, nullptr, eps, nullptr, pick.data());
}

void batch_adapt_keys(const std::vector<const HostGrid*>& grids, const std::vector<int64_t>& offset,
                      const double* norms, const uint8_t* force, double eps, double eta,
                      std::vector<std::vector<uint64_t>>* keys, std::vector<std::vector<uint8_t>>* carry) {
    const int64_t n = int64_t(grids.size());
    keys->assign(n, {});
    carry->assign(n, {});
#pragma omp parallel for schedule(dynamic, 1) if (n > 1 && offset[n] >= 16384)
    for (int64_t i = 0; i < n; ++i)
        adapt_keys_between_steps(*grids[i], norms + offset[i], force ? force + offset[i] : nullptr, eps, eta,
                                 &(*keys)[i], &(*carry)[i]);
}

void grid_from_keys(int dim, int nmax, int k, std::vector<uint64_t> keys, HostGrid* g) {
    if (!std::is_sorted(keys.begin(), keys.end())) std::sort(keys.begin(), keys.end());
    keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
    g->dim = dim;
    g->nmax = nmax;
    g->k = k;
    g->key = std::move(keys);
    g->num_elements = int64_t(g->key.size());
    g->order.resize(size_t(g->num_elements) * dim);
    for (int64_t e = 0; e < g->num_elements; ++e)
        for (int d = 0; d < dim; ++d) g->order[size_t(e) * dim + d] = field(g->key[e], d, dim, nmax);
    build_key_index(g);
}

void element_separable_norms(const HostGrid& g, const std::vector<double>& coef1d, int nterms, std::vector<double>* norms) {
    const int dim = g.dim, np = g.k + 1, nb1 = (1 << g.nmax) * np;
    int B = 1;
    for (int d = 0; d < dim; ++d) B *= np;
    norms->assign(g.num_elements, 0.0);
    for (int64_t e = 0; e < g.num_elements; ++e) {
        double s = 0.0;
        for (int q = 0; q < B; ++q) {
            int dig[kMaxDim];
            int rem = q;
            for (int d = dim - 1; d >= 0; --d) { dig[d] = rem % np; rem /= np; }
            double v = 0.0;
            for (int t = 0; t < nterms; ++t) {
                double p = 1.0;
                for (int d = 0; d < dim; ++d)
                    p *= coef1d[(size_t(t) * dim + d) * nb1 + g.order[size_t(e) * dim + d] * np + dig[d]];
                v += p;
            }
            s += v * v;
        }
        (*norms)[e] = std::sqrt(s);
    }
}

}  // namespace amdg
