// 1D Alpert multiwavelet basis, Gauss-Legendre quadrature and the dense 1D
// operator matrices of the DG discretisation.  Host-side FP64 set-up, run once
// per grid; the device kernels only read the resulting 1D blocks.
//
// Follows AlptBasis.cpp:16-81,256-299 (basis and one-sided limits),
// Basis.cpp:38-173 (volume and edge products, periodic wrap) and
// OperatorMatrix1D.h:166-199 (which products form which matrix).
#include <cmath>
#include <cstring>
#include <stdexcept>

#include "amdg_internal.hpp"

namespace amdg {
namespace {

// Right-half (x in [0,1]) polynomial of Alpert's mother multiwavelet f_p of
// degree k on [-1,1], monomial coefficients times a normalisation; the left
// half follows from f_p(-x) = (-1)^(p+k+1) f_p(x) (Alpert 1993).
struct MotherPoly {
    double c[4];
    double norm;
};

MotherPoly mother_poly(int k, int p) {
    switch (k) {
        case 1: {
            static const MotherPoly t[2] = {{{-1, 2, 0, 0}, std::sqrt(1.5)}, {{-2, 3, 0, 0}, std::sqrt(0.5)}};
            return t[p];
        }
        case 2: {
            static const MotherPoly t[3] = {{{1, -24, 30, 0}, std::sqrt(0.5) / 3.0},
                                            {{3, -16, 15, 0}, std::sqrt(1.5) * 0.5},
                                            {{4, -15, 12, 0}, std::sqrt(2.5) / 3.0}};
            return t[p];
        }
        case 3: {
            static const MotherPoly t[4] = {{{1, 4, -30, 28}, std::sqrt(15.0 / 34.0)},
                                            {{-4, 105, -300, 210}, std::sqrt(1.0 / 42.0)},
                                            {{-5, 48, -105, 64}, std::sqrt(35.0 / 34.0) * 0.5},
                                            {{-16, 105, -192, 105}, std::sqrt(5.0 / 42.0) * 0.5}};
            return t[p];
        }
    }
    throw std::invalid_argument("Alpert degree must be 1..3");
}

// d-th derivative of sum_m c[m] x^m
double poly_deriv(const double* c, int deg, int d, double x) {
    double v = 0.0;
    for (int m = deg; m >= d; --m) {
        double f = 1.0;
        for (int r = 0; r < d; ++r) f *= double(m - r);
        v = v * x + c[m] * f;
    }
    return v;
}

double mother(int k, int p, int d, double x) {
    const MotherPoly mp = mother_poly(k, p);
    double s = 1.0;
    if (x < 0) {
        s = ((p + k + 1 + d) & 1) ? -1.0 : 1.0;
        x = -x;
    }
    return s * mp.norm * poly_deriv(mp.c, k, d, x);
}

// Legendre P_p on [-1,1] as monomial coefficients (p <= 3 needed for k <= 3)
void legendre_coeffs(int p, double* c) {
    double a[5] = {1, 0, 0, 0, 0}, b[5] = {0, 1, 0, 0, 0};
    if (p == 0) { std::memcpy(c, a, sizeof a); return; }
    for (int n = 1; n < p; ++n) {
        double nx[5] = {0, 0, 0, 0, 0};
        for (int m = 0; m < 4; ++m) nx[m + 1] += (2.0 * n + 1.0) * b[m] / (n + 1.0);
        for (int m = 0; m < 5; ++m) nx[m] -= n * a[m] / (n + 1.0);
        std::memcpy(a, b, sizeof a);
        std::memcpy(b, nx, sizeof b);
    }
    std::memcpy(c, b, sizeof b);
}

double basis_raw(int k, int n, int j, int p, int d, double x) {
    if (n == 0) {
        const double y = 2.0 * x - 1.0;
        if (std::fabs(y) > 1.0) return 0.0;
        double c[5];
        legendre_coeffs(p, c);
        return poly_deriv(c, 4, d, y) * std::pow(2.0, d) * std::sqrt(2.0 * p + 1.0);
    }
    double y = x;
    double scale = 1.0;
    if (n >= 2) {
        y = std::pow(2.0, n - 1) * x - double((j - 1) / 2);
        scale = std::pow(2.0, (n - 1) * (d + 0.5));
    }
    if (!(y >= 0.0 && y <= 1.0)) return 0.0;
    return scale * std::pow(2.0, d + 0.5) * mother(k, p, d, 2.0 * y - 1.0);
}

// Gauss-Legendre nodes/weights on [-1,1] by Newton's method on P_n
struct GaussRule {
    int n;
    double x[16], w[16];
    explicit GaussRule(int npts) : n(npts) {
        for (int i = 0; i < n; ++i) {
            double z = std::cos(M_PI * (i + 0.75) / (n + 0.5)), dp = 1.0;
            for (int it = 0; it < 100; ++it) {
                double p0 = 1.0, p1 = z;
                for (int m = 2; m <= n; ++m) {
                    const double p2 = ((2.0 * m - 1.0) * z * p1 - (m - 1.0) * p0) / m;
                    p0 = p1;
                    p1 = p2;
                }
                dp = n * (z * p1 - p0) / (z * z - 1.0);
                const double dz = p1 / dp;
                z -= dz;
                if (std::fabs(dz) < 1e-16) break;
            }
            double p0 = 1.0, p1 = z;
            for (int m = 2; m <= n; ++m) {
                const double p2 = ((2.0 * m - 1.0) * z * p1 - (m - 1.0) * p0) / m;
                p0 = p1;
                p1 = p2;
            }
            dp = n * (z * p1 - p0) / (z * z - 1.0);
            x[n - 1 - i] = z;
            w[n - 1 - i] = 2.0 / ((1.0 - z * z) * dp * dp);
        }
    }
    template <class F>
    double integrate(F&& f, double a, double b) const {
        double s = 0.0;
        for (int i = 0; i < n; ++i) s += w[i] * f(a + (x[i] + 1.0) * 0.5 * (b - a));
        return s * (b - a) / 2.0;
    }
};

const GaussRule& gauss10() {
    static const GaussRule g(10);
    return g;
}

double supp_lo(int o) { int n, j; elem_of_order(o, &n, &j); return n <= 1 ? 0.0 : std::pow(2.0, 1.0 - n) * (j - 1.0) / 2.0; }
double supp_hi(int o) { int n, j; elem_of_order(o, &n, &j); return n <= 1 ? 1.0 : std::pow(2.0, 1.0 - n) * (j + 1.0) / 2.0; }

}  // namespace

double Basis1D::eval(int order, int deriv, double x, int sgn) const {
    const int o = order / (k + 1), p = order % (k + 1);
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
    return basis_raw(k, n, j, p, deriv, xl);
}

void build_oper1d(const Basis1D& b, Oper1D* out, bool want_u_v) {
    const int nb = b.num_basis(), np = b.k + 1;
    out->nb = nb;
    out->u_vx.assign(size_t(nb) * nb, 0.0);
    out->ulft_vjp.assign(size_t(nb) * nb, 0.0);
    out->urgt_vjp.assign(size_t(nb) * nb, 0.0);
    if (want_u_v) out->u_v.assign(size_t(nb) * nb, 0.0);
    const GaussRule& g = gauss10();
#pragma omp parallel for schedule(dynamic)
    for (int r = 0; r < nb; ++r) {
        const int ou = r / np;
        const int lu = level_of_order(ou);
        const double ua = supp_lo(ou), ub = supp_hi(ou);
        for (int c = 0; c < nb; ++c) {
            const int ov = c / np;
            const double va = supp_lo(ov), vb = supp_hi(ov);
            const size_t idx = size_t(r) * nb + c;
            // volume products over the finer support, split at its midpoint
            if (!(va >= ub || vb <= ua)) {
                double xl = ua, xr = ub;
                if (lu <= level_of_order(ov)) { xl = va; xr = vb; }
                const double xm = 0.5 * (xl + xr);
                auto fvx = [&](double x) { return b.eval(r, 0, x, 0) * b.eval(c, 1, x, 0); };
                out->u_vx[idx] = g.integrate(fvx, xl, xm) + g.integrate(fvx, xm, xr);
                if (want_u_v) {
                    auto fv = [&](double x) { return b.eval(r, 0, x, 0) * b.eval(c, 0, x, 0); };
                    out->u_v[idx] = g.integrate(fv, xl, xm) + g.integrate(fv, xm, xr);
                }
            }
            // edge products at the discontinuity points of the test function,
            // periodic: u(0^-) = u(1^-), u(1^+) = u(0^+)
            const double pts[3] = {va, 0.5 * (va + vb), vb};
            const int npts = level_of_order(ov) <= 1 ? 2 : 3;
            auto edge = [&](int su, int sv) {
                double s = 0.0;
                for (int i = 0; i < npts; ++i) {
                    const double x = pts[i];
                    double fu = b.eval(r, 0, x, su), fv = b.eval(c, 0, x, sv);
                    if (std::fabs(x) < kRoundOff) {
                        if (su == -1) fu = b.eval(r, 0, 1.0, su);
                        if (sv == -1) fv = b.eval(c, 0, 1.0, sv);
                    } else if (std::fabs(x - 1.0) < kRoundOff) {
                        if (su == 1) fu = b.eval(r, 0, 0.0, su);
                        if (sv == 1) fv = b.eval(c, 0, 0.0, sv);
                    }
                    s += fu * fv;
                }
                return s;
            };
            out->ulft_vjp[idx] = edge(-1, 1) - edge(-1, -1);
            out->urgt_vjp[idx] = edge(1, 1) - edge(1, -1);
        }
    }
}

void project_1d(const Basis1D& b, const Fn1d& f, int d, int term, double* out) {
    const GaussRule& g = gauss10();
    const int nb = b.num_basis(), np = b.k + 1, nq = g.n, n1 = nb / np;
    auto qpt = [&](int q, double a, double c) { return a + (g.x[q] + 1.0) * 0.5 * (c - a); };
    // Gauss sum over [a, c] of basis r times f, with f given at the rule's points
    auto panel = [&](int r, const double* fv, double a, double c) {
        double s = 0.0;
        for (int q = 0; q < nq; ++q) s += g.w[q] * (b.eval(r, 0, qpt(q, a, c), 0) * fv[q]);
        return s * (c - a) / 2.0;
    };
    // f is evaluated once per quadrature point, all points in one call: the 16
    // uniform panels shared by every coarse order, then the two half-supports of
    // every finer order (shared by its k+1 functions)
    std::vector<double> x, v;
    for (int i = 0; i < 16; ++i)
        for (int q = 0; q < nq; ++q) x.push_back(qpt(q, i / 16.0, (i + 1) / 16.0));
    for (int o = 0; o < n1; ++o) {
        if (level_of_order(o) <= 4) continue;
        const double a = supp_lo(o), c = supp_hi(o), m = 0.5 * (a + c);
        for (int q = 0; q < nq; ++q) x.push_back(qpt(q, a, m));
        for (int q = 0; q < nq; ++q) x.push_back(qpt(q, m, c));
    }
    v.resize(x.size());
    f.eval(x.data(), int64_t(x.size()), d, term, v.data());
    const double* fc = v.data();
    const double* ff = v.data() + size_t(16) * nq;
    for (int o = 0; o < n1; ++o) {
        if (level_of_order(o) <= 4) {
            // coarse levels: 16 uniform panels over [0,1] (Basis.cpp:38-59)
            for (int p = 0; p < np; ++p) {
                double s = 0.0;
                for (int i = 0; i < 16; ++i) s += panel(o * np + p, fc + size_t(i) * nq, i / 16.0, (i + 1) / 16.0);
                out[o * np + p] = s;
            }
        } else {
            const double a = supp_lo(o), c = supp_hi(o), m = 0.5 * (a + c);
            for (int p = 0; p < np; ++p) out[o * np + p] = panel(o * np + p, ff, a, m) + panel(o * np + p, ff + nq, m, c);
            ff += size_t(2) * nq;
        }
    }
}

void gauss_legendre(int n, double* x, double* w) {
    const GaussRule g(n);
    for (int i = 0; i < n; ++i) {
        x[i] = g.x[i];
        w[i] = g.w[i];
    }
}

}  // namespace amdg
