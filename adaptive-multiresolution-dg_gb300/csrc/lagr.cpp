// Host set-up of the Lagrange-interpolation path for nonlinear fluxes:
// hierarchical Lagrange bases of degree 3 (node layout msh_case 1,
// LagrBasis.cpp:65-70, the Burgers examples) and degree 4 (msh_case 2,
// LagrBasis.cpp:92-97, the wave example), the Alpert-at-Lagrange-point table
// (Interplation.cpp:16-101), the Lagrange x Alpert 1D matrices
// (OperatorMatrix1D<LagrBasis,AlptBasis>, OperatorMatrix1D.h:166-199), the
// dimension-order / L-U schedule of the fast transforms
// (FastMultiplyLU.cpp:596-664) and the ancestor table of the hierarchical
// surplus (Interplation.cpp:775-888).
#include <algorithm>
#include <cmath>

#include "amdg_internal.hpp"

namespace amdg {
namespace {

// Degree 3, msh_case 1: level-0 nodes {-3/5,-1/5,1/5,3/5}; level-1 nodes
// {-4/5,-2/5} on the left half and {2/5,4/5} on the right half, each the cubic
// through the four nodes of its half (with the two level-0 nodes there).
const LagrSpec kDeg3 = {4,
                        {-0.6, -0.2, 0.2, 0.6},
                        {-0.8, -0.4, 0.4, 0.8},
                        {-0.6, -0.2, 0.2, 0.6},
                        {{-0.8, -0.6, -0.4, -0.2}, {0.2, 0.4, 0.6, 0.8}},
                        {0, 0, 1, 1},
                        {0, 2, 1, 3}};
// Degree 4, msh_case 2: level-0 nodes {-1,-1/2,0,1/2,1}, whose points sit
// 1e-13 inside the element (left of the node except at -1); level-1 nodes
// {-3/4,-1/4} on the left half and {0,1/4,3/4} on the right half (the point
// at 0 just right of it), each the quartic through the nodes of its half at
// spacing 1/4.
const LagrSpec kDeg4 = {5,
                        {-1 + kRoundOff, -0.5 - kRoundOff, 0 - kRoundOff, 0.5 - kRoundOff, 1 - kRoundOff},
                        {-0.75 - kRoundOff, -0.25 - kRoundOff, 0 + kRoundOff, 0.25 - kRoundOff, 0.75 - kRoundOff},
                        {-1, -0.5, 0, 0.5, 1},
                        {{-1, -0.75, -0.5, -0.25, 0}, {0, 0.25, 0.5, 0.75, 1}},
                        {0, 0, 1, 1, 1},
                        {1, 3, 0, 1, 3}};
// Degree 5, msh_case 1 (the node layout of the linear example's initial interpolation):
// level-0 nodes {-1,-3/5,-1/5,1/5,3/5,1}, the end points 1e-13 inside the element; level-1
// nodes {-4/5,-2/5,0} on the left half and {0,2/5,4/5} on the right half (0 just left / right
// of it), each the quintic through the level-0 nodes mapped onto its half.
const LagrSpec kDeg5 = {6,
                        {-1 + kRoundOff, -0.6, -0.2, 0.2, 0.6, 1 - kRoundOff},
                        {-0.8, -0.4, 0 - kRoundOff, 0 + kRoundOff, 0.4, 0.8},
                        {-1, -0.6, -0.2, 0.2, 0.6, 1},
                        {{-1, -0.8, -0.6, -0.4, -0.2, 0}, {0, 0.2, 0.4, 0.6, 0.8, 1}},
                        {0, 0, 0, 1, 1, 1},
                        {1, 3, 5, 0, 2, 4}};

double lagrange_poly(const double* nodes, int n, int i, double x) {
    double v = 1.0;
    for (int m = 0; m < n; ++m)
        if (m != i) v *= (x - nodes[m]) / (nodes[i] - nodes[m]);
    return v;
}

// level-0 / level-1 mother functions on [0,1]
double lagr_mother(const LagrSpec& s, double xt, int msh, int p) {
    const double x = 2.0 * xt - 1.0;
    if (x < -1.0 || x > 1.0) return 0.0;
    if (msh == 0) return lagrange_poly(s.node0, s.p1, p, x);
    if (s.side[p] == 0) {
        if (x > 0.0) return 0.0;
        return lagrange_poly(s.half[0], s.p1, s.node[p], x);
    }
    if (x < 0.0) return 0.0;
    return lagrange_poly(s.half[1], s.p1, s.node[p], x);
}

double supp_lo(int o) { int n, j; elem_of_order(o, &n, &j); return n <= 1 ? 0.0 : std::pow(2.0, 1.0 - n) * (j - 1.0) / 2.0; }
double supp_hi(int o) { int n, j; elem_of_order(o, &n, &j); return n <= 1 ? 1.0 : std::pow(2.0, 1.0 - n) * (j + 1.0) / 2.0; }

struct GL10 {
    double x[10], w[10];
    GL10() {
        for (int i = 0; i < 10; ++i) {
            double z = std::cos(M_PI * (i + 0.75) / 10.5), dp = 1.0;
            for (int it = 0; it < 100; ++it) {
                double p0 = 1.0, p1 = z;
                for (int m = 2; m <= 10; ++m) {
                    const double p2 = ((2.0 * m - 1.0) * z * p1 - (m - 1.0) * p0) / m;
                    p0 = p1;
                    p1 = p2;
                }
                dp = 10 * (z * p1 - p0) / (z * z - 1.0);
                const double dz = p1 / dp;
                z -= dz;
                if (std::fabs(dz) < 1e-16) break;
            }
            double p0 = 1.0, p1 = z;
            for (int m = 2; m <= 10; ++m) {
                const double p2 = ((2.0 * m - 1.0) * z * p1 - (m - 1.0) * p0) / m;
                p0 = p1;
                p1 = p2;
            }
            dp = 10 * (z * p1 - p0) / (z * z - 1.0);
            x[9 - i] = z;
            w[9 - i] = 2.0 / ((1.0 - z * z) * dp * dp);
        }
    }
    template <class F>
    double integrate(F&& f, double a, double b) const {
        double s = 0.0;
        for (int i = 0; i < 10; ++i) s += w[i] * f(a + (x[i] + 1.0) * 0.5 * (b - a));
        return s * (b - a) / 2.0;
    }
};

}  // namespace

const LagrSpec* lagr_spec(int degree) {
    if (degree == 3) return &kDeg3;
    if (degree == 4) return &kDeg4;
    if (degree == 5) return &kDeg5;
    return nullptr;
}

double lagr_eval(const LagrSpec& s, int order, double x, int sgn) {
    const int o = order / s.p1, p = order % s.p1;
    int n, j;
    elem_of_order(o, &n, &j);
    double xl = x;
    if (sgn == -1) {
        if (std::fabs(x) <= kRoundOff) return 0.0;
        xl -= kRoundOff;
    } else if (sgn == 1) {
        if (std::fabs(x - 1.0) <= kRoundOff) return 0.0;
        xl += kRoundOff;
    }
    if (n <= 1) return lagr_mother(s, xl, n, p);
    return lagr_mother(s, std::pow(2.0, n - 1) * xl - double((j - 1) / 2), 1, p);
}

double lagr_point(const LagrSpec& s, int o, int p) {
    int n, j;
    elem_of_order(o, &n, &j);
    if (n == 0) return (s.pt0[p] + 1.0) / 2.0;
    const double a = supp_lo(o), b = supp_hi(o);
    return a + (b - a) * (s.pt1[p] + 1.0) / 2.0;
}

void build_lagr_ancestors(const Basis1D& alpt, int degree, LagrTables* t) {
    const LagrSpec& S = *lagr_spec(degree);
    const int n1 = alpt.num_elem(), P1 = S.p1;
    t->spec = &S;
    t->p1 = P1;
    // surplus: ancestors (coarser-level points inside each element's support) and weights
    t->anc_order.assign(size_t(n1) * P1, -1);
    t->anc_point.assign(size_t(n1) * P1, 0);
    t->anc_rank.assign(size_t(n1) * P1, 0);
    for (int o = 1; o < n1; ++o) {
        const int l = level_of_order(o);
        const double xl = supp_lo(o), xr = supp_hi(o);
        int ic = 0;
        double pos[kMaxLagrPoints] = {0};
        for (int oa = 0; oa < n1 && ic < P1; ++oa) {
            if (level_of_order(oa) >= l) break;
            for (int q = 0; q < P1 && ic < P1; ++q) {
                const double x = lagr_point(S, oa, q);
                if (x > xl && x < xr) {
                    t->anc_order[size_t(o) * P1 + ic] = oa;
                    t->anc_point[size_t(o) * P1 + ic] = q;
                    pos[ic] = x;
                    ++ic;
                }
            }
        }
        for (int a = 0; a < P1; ++a) {
            int rk = 0;
            for (int b = 0; b < P1; ++b) rk += pos[b] < pos[a];
            t->anc_rank[size_t(o) * P1 + a] = rk;
        }
    }
}

void lagr_mass_diag(const LagrSpec& S, int nmax, std::vector<double>* out) {
    static const GL10 g;
    const int n1 = 1 << nmax, P1 = S.p1;
    out->assign(size_t(n1) * P1, 0.0);
    for (int o = 0; o < n1; ++o) {
        const double a = supp_lo(o), b = supp_hi(o), m = 0.5 * (a + b);
        for (int p = 0; p < P1; ++p) {
            const int r = o * P1 + p;
            auto sq = [&](double x) {
                const double v = lagr_eval(S, r, x, 0);
                return v * v;
            };
            (*out)[r] = g.integrate(sq, a, m) + g.integrate(sq, m, b);
        }
    }
}

// Interpolation basis (rows, 1D order * p1 + p) x Alpert basis (columns) products of
// OperatorMatrix1D<Interp, AlptBasis> (OperatorMatrix1D.h:166-199): u_v and u_vx by 10-point
// Gauss on the two halves of the finer support, ulft_vjp + urgt_vjp from the one-sided values at
// the Alpert function's discontinuities.  S selects the Lagrange basis; nullptr the cubic Hermite
// basis (herm_eval).
void build_interp_products(const Basis1D& alpt, const LagrSpec* S, int P1, LagrTables* t) {
    static const GL10 g;
    const int n1 = alpt.num_elem(), na = alpt.num_basis(), np = alpt.k + 1, nl = n1 * P1;
    auto ieval = [S](int r, double x, int sgn) { return S ? lagr_eval(*S, r, x, sgn) : herm_eval(r, 0, x, sgn); };
    t->lv.assign(size_t(nl) * na, 0.0);
    t->lvx.assign(size_t(nl) * na, 0.0);
    t->lflx.assign(size_t(nl) * na, 0.0);
#pragma omp parallel for schedule(dynamic)
    for (int r = 0; r < nl; ++r) {
        const int ou = r / P1;
        const int lu = level_of_order(ou);
        const double ua = supp_lo(ou), ub = supp_hi(ou);
        for (int c = 0; c < na; ++c) {
            const int ov = c / np;
            const double va = supp_lo(ov), vb = supp_hi(ov);
            const size_t idx = size_t(r) * na + c;
            if (!(va >= ub || vb <= ua)) {
                double xl = ua, xr = ub;
                if (lu <= level_of_order(ov)) { xl = va; xr = vb; }
                const double xm = 0.5 * (xl + xr);
                auto fv = [&](double x) { return ieval(r, x, 0) * alpt.eval(c, 0, x, 0); };
                auto fvx = [&](double x) { return ieval(r, x, 0) * alpt.eval(c, 1, x, 0); };
                t->lv[idx] = g.integrate(fv, xl, xm) + g.integrate(fv, xm, xr);
                t->lvx[idx] = g.integrate(fvx, xl, xm) + g.integrate(fvx, xm, xr);
            }
            const double pts[3] = {va, 0.5 * (va + vb), vb};
            const int npts = level_of_order(ov) <= 1 ? 2 : 3;
            auto edge = [&](int su, int sv) {
                double s = 0.0;
                for (int i = 0; i < npts; ++i) {
                    const double x = pts[i];
                    double fu = ieval(r, x, su), fw = alpt.eval(c, 0, x, sv);
                    if (std::fabs(x) < kRoundOff) {
                        if (su == -1) fu = ieval(r, 1.0, su);
                        if (sv == -1) fw = alpt.eval(c, 0, 1.0, sv);
                    } else if (std::fabs(x - 1.0) < kRoundOff) {
                        if (su == 1) fu = ieval(r, 0.0, su);
                        if (sv == 1) fw = alpt.eval(c, 0, 0.0, sv);
                    }
                    s += fu * fw;
                }
                return s;
            };
            // (ulft_vjp + urgt_vjp), HyperbolicLagrRHS::rhs_flx_intp_scalar (FastMultiplyLU.cpp:1166)
            t->lflx[idx] = (edge(-1, 1) - edge(-1, -1)) + (edge(1, 1) - edge(1, -1));
        }
    }
}

void build_lagr_tables(const Basis1D& alpt, int degree, LagrTables* t, bool diffusion) {
    static const GL10 g;
    const LagrSpec& S = *lagr_spec(degree);
    const int P1 = S.p1;
    const int n1 = alpt.num_elem(), na = alpt.num_basis(), np = alpt.k + 1, nl = n1 * P1;
    t->spec = &S;
    t->p1 = P1;
    t->n_lagr = nl;
    t->n_alpt = na;
    // Alpert basis at Lagrange points, row = Alpert basis, col = Lagrange point
    t->a2p.assign(size_t(na) * nl, 0.0);
    for (int c = 0; c < nl; ++c) {
        const double x = lagr_point(S, c / P1, c % P1);
        for (int r = 0; r < na; ++r) {
            const int o = r / np;
            if (x < supp_lo(o) || x > supp_hi(o)) continue;
            t->a2p[size_t(r) * nl + c] = alpt.eval(r, 0, x, 0);
        }
    }
    build_interp_products(alpt, &S, P1, t);
    if (diffusion) {
        // Alpert derivative at the Lagrange points (Lag_pt_Alpt_1D_d1, Interplation.cpp:16-101)
        // and the point coordinates
        t->a2pd.assign(size_t(na) * nl, 0.0);
        t->pts.assign(nl, 0.0);
        for (int c = 0; c < nl; ++c) {
            const double x = lagr_point(S, c / P1, c % P1);
            t->pts[c] = x;
            for (int r = 0; r < na; ++r) {
                const int o = r / np;
                if (x < supp_lo(o) || x > supp_hi(o)) continue;
                t->a2pd[size_t(r) * nl + c] = alpt.eval(r, 1, x, 0);
            }
        }
        // [u] times the one-sided v_x at u's discontinuities: ujp_vxlft + ujp_vxrgt
        // (OperatorMatrix1D.h:206-211, Basis::product_edge_dis_u, Basis.cpp:175-230)
        t->ljv.assign(size_t(nl) * na, 0.0);
#pragma omp parallel for schedule(dynamic)
        for (int r = 0; r < nl; ++r) {
            const int ou = r / P1;
            const double ua = supp_lo(ou), ub = supp_hi(ou);
            const double pts[3] = {ua, 0.5 * (ua + ub), ub};
            const int npts = level_of_order(ou) <= 1 ? 2 : 3;
            for (int c = 0; c < na; ++c) {
                auto edge = [&](int su, int sv) {
                    double s = 0.0;
                    for (int i = 0; i < npts; ++i) {
                        const double x = pts[i];
                        double fu = lagr_eval(S, r, x, su), fw = alpt.eval(c, 1, x, sv);
                        if (std::fabs(x) < kRoundOff) {
                            if (su == -1) fu = lagr_eval(S, r, 1.0, su);
                            if (sv == -1) fw = alpt.eval(c, 1, 1.0, sv);
                        } else if (std::fabs(x - 1.0) < kRoundOff) {
                            if (su == 1) fu = lagr_eval(S, r, 0.0, su);
                            if (sv == 1) fw = alpt.eval(c, 1, 0.0, sv);
                        }
                        s += fu * fw;
                    }
                    return s;
                };
                const double lft = edge(1, -1) - edge(-1, -1), rgt = edge(1, 1) - edge(-1, 1);
                t->ljv[size_t(r) * na + c] = lft + rgt;
            }
        }
    }
    // Alpert x Alpert jump-jump (ujp_vjp = urgt_vjp - ulft_vjp), LxF penalty
    Oper1D op;
    build_oper1d(alpt, &op, false);
    t->ajump.assign(size_t(na) * na, 0.0);
    for (size_t i = 0; i < t->ajump.size(); ++i) t->ajump[i] = op.urgt_vjp[i] - op.ulft_vjp[i];
    build_lagr_ancestors(alpt, degree, t);
    // weight[p0][rank] = -L0_rank(point p0 of the element, in its reference coordinates)
    for (int p0 = 0; p0 < P1; ++p0)
        for (int r = 0; r < P1; ++r) t->weight[p0 * P1 + r] = -lagr_mother(S, (S.pt1[p0] + 1.0) / 2.0, 0, r);
}

SweepTree build_sweep_tree(const std::vector<PartialSum>& terms, int first, int count, int dim,
                           std::vector<PartialSum>* nodes) {
    // A coefficient of a power of two commutes exactly with the linear sweeps (every rounding is
    // scale-invariant), so such a term may apply it in its last sweep and share earlier ones.
    auto pow2 = [](double c) {
        int e = 0;
        return c != 0.0 && std::frexp(std::fabs(c), &e) == 0.5;
    };
    SweepTree tree;
    std::vector<std::vector<PartialSum>> level(dim);
    std::vector<int> at(count, -1);  // node of each term at the current sweep
    for (int j = 0; j + 1 < dim; ++j) {
        for (int i = 0; i < count; ++i) {
            const PartialSum& t = terms[size_t(first + i)];
            if (t.kind != 0) continue;  // the penalty is a single (last) sweep
            const bool share = pow2(t.coef);
            PartialSum n = t;
            n.parent = j == 0 ? -1 : at[i];
            n.coef = (j == 0 && !share) ? t.coef : 1.0;
            int found = -1;
            for (size_t k = 0; share && k < level[j].size() && found < 0; ++k) {
                const PartialSum& o = level[j][k];
                bool same = o.parent == n.parent && o.coef == 1.0 && o.kind == 0 && (j > 0 || o.src == n.src);
                for (int q = 0; same && q <= j; ++q)
                    same = o.dims[q] == n.dims[q] && o.lu[q] == n.lu[q] && o.mat[q] == n.mat[q] && o.flx[q] == n.flx[q];
                if (same) found = int(k);
            }
            if (found < 0) {  // a new node (an unshared term's nodes are never matched: their
                found = int(level[j].size());  // first one carries a coefficient other than 1)
                level[j].push_back(n);
            }
            at[i] = found;
        }
    }
    for (int i = 0; i < count; ++i) {  // the last sweep: one node per term, in term order
        const PartialSum& t = terms[size_t(first + i)];
        PartialSum n = t;
        n.parent = (t.kind != 0 || dim == 1) ? -1 : at[i];
        n.coef = (t.kind != 0 || dim == 1 || pow2(t.coef)) ? t.coef : 1.0;
        level[dim - 1].push_back(n);
    }
    for (int j = 0; j < dim; ++j) {
        tree.offset[j] = int(nodes->size());
        tree.count[j] = int(level[j].size());
        nodes->insert(nodes->end(), level[j].begin(), level[j].end());
    }
    return tree;
}

void transform_schedule(int dim, std::vector<std::vector<int>>* dim_order, std::vector<std::vector<int>>* lu) {
    // 2^(dim-1) partial sums; sum s: dimension d gets tag 2*bit_d(s) for d < dim-1
    // and tag 1 for the last, then dimensions are ordered by tag
    // (0 = L, 1 = full, 2 = U); FastMultiplyLU.cpp:614-664
    dim_order->clear();
    lu->clear();
    if (dim == 1) {
        dim_order->push_back({0});
        lu->push_back({1});
        return;
    }
    const int nsum = 1 << (dim - 1);
    for (int s = 0; s < nsum; ++s) {
        std::vector<int> tag(dim);
        for (int d = 0; d < dim - 1; ++d) tag[d] = 2 * ((s >> (dim - 2 - d)) & 1);
        tag[dim - 1] = 1;
        std::vector<int> order(dim);
        for (int d = 0; d < dim; ++d) order[d] = d;
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return tag[a] < tag[b]; });
        std::vector<int> tags_sorted(dim);
        for (int d = 0; d < dim; ++d) tags_sorted[d] = tag[order[d]];
        dim_order->push_back(order);
        lu->push_back(tags_sorted);
    }
}

}  // namespace amdg
