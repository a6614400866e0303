// Host set-up of the cubic Hermite interpolation of the flux: HermBasis with PMAX 3 and
// msh_case 1 (HermBasis.cpp), as the 2D Burgers driver example/02_hyperbolic_05_burgers_adapt.cpp
// sets it, for HermInterpolation::nonlinear_Herm_2D_fast (Interplation.cpp:4609-4621) and
// HyperbolicSameFluxHermRHS (FastMultiplyLU.cpp:970-1016).  A 1D Hermite element carries four
// degrees of freedom p: the value (p / 2 = 0) or the slope (p / 2 = 1) at point p % 2.  Level 0
// interpolates at the two ends of [0, 1], every finer level at the two sides of its element's
// midpoint, the left pair supported on the left half and the right pair on the right half.
#include <cmath>

#include "amdg_internal.hpp"

namespace amdg {
namespace {

double lo_of(int o) { int n, j; elem_of_order(o, &n, &j); return n <= 1 ? 0.0 : std::ldexp(j - 1.0, -n); }
double hi_of(int o) { int n, j; elem_of_order(o, &n, &j); return n <= 1 ? 1.0 : std::ldexp(j + 1.0, -n); }

// Mother functions on [0, 1] (msh 0: level 0, msh 1: level 1) and their first derivatives
// (HermBasis::phi_P1_L1 and its derivative): cubic Hermite cardinal functions, written in the
// factored forms that vanish where they must.
double mother(double x, int msh, int pp, int deriv) {
    if (x < 0.0 || x > 1.0) return 0.0;
    const bool right = pp % 2 == 1, slope = pp / 2 == 1;
    if (msh == 0) {
        const double y = right ? 1.0 - x : x;  // distance from the interpolating end
        const double s = right ? -1.0 : 1.0;   // d/dx of y
        if (!slope) return deriv ? s * 6.0 * y * (y - 1.0) : (y - 1.0) * (y - 1.0) * (1.0 + 2.0 * y);
        // the slope function changes sign under the reflection
        return deriv ? (1.0 - y) * (1.0 - 3.0 * y) : s * (1.0 - y) * (1.0 - y) * y;
    }
    if (!right && x > 0.5) return 0.0;
    if (right && x < 0.5) return 0.0;
    // z: distance from the far end of the half, in units of the half width
    const double z = right ? 2.0 * (1.0 - x) : 2.0 * x;
    const double s = right ? -2.0 : 2.0;  // dz/dx
    if (!slope) return deriv ? s * 6.0 * z * (1.0 - z) : z * z * (3.0 - 2.0 * z);
    // slope 1 at the midpoint: (z^3 - z^2) / 2 per unit of x, the sign again by reflection
    const double r = right ? -1.0 : 1.0;
    return deriv ? r * 0.5 * s * z * (3.0 * z - 2.0) : r * 0.5 * (z * z * z - z * z);
}

}  // namespace

double herm_eval(int order, int deriv, double x, int sgn) {
    const int o = order / 4, p = order % 4;
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
    if (n <= 1) return mother(xl, n, p, deriv);
    // a level-n slope dof scales by the support width 2^-(n-1), each derivative by 2^(n-1)
    return mother(std::pow(2.0, n - 1) * xl - double((j - 1) / 2), 1, p, deriv) *
           std::pow(2.0, -(n - 1) * (p / 2 - deriv));
}

double herm_point(int o, int p) {
    // HermBasis::set_interp_msh01: level 0 at -1 + 1e-13 and 1 - 1e-13, finer levels at
    // -1e-13 and +1e-13, in [-1, 1] coordinates mapped by (x + 1) / 2
    if (o == 0) return ((p % 2 == 0 ? (-1.0 + kRoundOff) : (1.0 - kRoundOff)) + 1.0) / 2.0;
    const double m = ((p % 2 == 0 ? (0.0 - kRoundOff) : (0.0 + kRoundOff)) + 1.0) / 2.0;
    const double a = lo_of(o), b = hi_of(o);
    return a + (b - a) * m;
}

void build_herm_tables(const Basis1D& alpt, LagrTables* t) {
    const int P1 = 4;
    const int n1 = alpt.num_elem(), na = alpt.num_basis(), np = alpt.k + 1, nh = n1 * P1;
    t->spec = nullptr;
    t->p1 = P1;
    t->n_lagr = nh;
    t->n_alpt = na;
    t->herm = true;
    // Alpert basis (rows) at the Hermite dofs (columns): the value for a value dof, the slope for
    // a slope dof, zero off the support (eval_Her_pt_at_Alpt_1D, Interplation.cpp:1886-1975)
    t->a2p.assign(size_t(na) * nh, 0.0);
    for (int c = 0; c < nh; ++c) {
        const double x = herm_point(c / P1, c % P1);
        for (int r = 0; r < na; ++r) {
            const int o = r / np;
            if (x < lo_of(o) || x > hi_of(o)) continue;
            t->a2p[size_t(r) * nh + c] = alpt.eval(r, (c % P1) / 2, x, 0);
        }
    }
    build_interp_products(alpt, nullptr, P1, t);
    Oper1D op;
    build_oper1d(alpt, &op, false);
    t->ajump.assign(size_t(na) * na, 0.0);
    for (size_t i = 0; i < t->ajump.size(); ++i) t->ajump[i] = op.urgt_vjp[i] - op.ulft_vjp[i];
    // surplus ancestors (set_pts_wts_1d_ada_Her, Interplation.cpp:3166-3316): the four coarser
    // dofs inside an element's support, in the order of coarser orders and dofs; they sit at the
    // support's two ends, and the dof number ic0 counts 0, 2 at the left end and 1, 3 at the right
    t->anc_order.assign(size_t(n1) * P1, -1);
    t->anc_point.assign(size_t(n1) * P1, 0);
    t->anc_rank.assign(size_t(n1) * P1, 0);
    for (int o = 1; o < n1; ++o) {
        const int l = level_of_order(o);
        const double xl = lo_of(o), xr = hi_of(o);
        double pos[4] = {0, 0, 0, 0};
        int ic = 0;
        for (int oa = 0; oa < n1 && ic < P1; ++oa) {
            if (level_of_order(oa) >= l) break;
            for (int q = 0; q < P1 && ic < P1; ++q) {
                const double x = herm_point(oa, q);
                if (x > xl && x < xr) {
                    t->anc_order[size_t(o) * P1 + ic] = oa;
                    t->anc_point[size_t(o) * P1 + ic] = q;
                    pos[ic++] = x;
                }
            }
        }
        const double left = std::fmin(std::fmin(pos[0], pos[1]), std::fmin(pos[2], pos[3]));
        int next_left = 0, next_right = 1;
        for (int a = 0; a < P1; ++a) {
            int& n = std::fabs(pos[a] - left) < 1e-14 ? next_left : next_right;
            t->anc_rank[size_t(o) * P1 + a] = n;
            n += 2;
        }
    }
    // weight[p0][ic0] = -H0_ic0^(l1)(x_p0): the level-0 cardinal function of dof ic0 (derivative
    // order l1 = p0 / 2) at dof p0's point in the element's [0, 1] coordinates; the kernel scales
    // it by 2^((level - 1)(l1 - ic0 / 2)), exactly (a power of two)
    for (int p0 = 0; p0 < P1; ++p0) {
        const double xt = ((p0 % 2 == 0 ? (0.0 - kRoundOff) : (0.0 + kRoundOff)) + 1.0) / 2.0;
        for (int r = 0; r < P1; ++r) t->weight[p0 * P1 + r] = -mother(xt, 0, r, p0 / 2);
    }
}

}  // namespace amdg
