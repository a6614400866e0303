/*
 * CPU oracle (test infrastructure only): plain C restatement of the AdaM-DG
 * reference algorithm for the linear constant-coefficient sparse-grid DG
 * right-hand side and its SSP-RK3 time stepping.  Pinned against the
 * reference library itself (oracle/ref_harness.cpp, fixtures in tests/golden/).
 * Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg use it.
 */
#include "amdg_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ROUND_OFF 1e-13 /* Const::ROUND_OFF, libs.h:28 */

/* ------------------------------------------------------------------------ */
/* 1D Alpert multiwavelets (AlptBasis.cpp:57-81, 256-299).                    */
/* Mother functions on [-1,1]: for x >= 0 a polynomial of degree k (monomial   */
/* coefficients below, Alpert 1993); for x < 0, f(-x) = (-1)^(p+k+1) f(x).     */
/* ------------------------------------------------------------------------ */
static const double* alpert_right_poly(int k, int p, double* scale) {
    /* returns monomial coefficients c[0..k] of the right-half polynomial */
    static const double k1[2][4] = {{-1, 2, 0, 0}, {-2, 3, 0, 0}};
    static const double k2[3][4] = {{1, -24, 30, 0}, {3, -16, 15, 0}, {4, -15, 12, 0}};
    static const double k3[4][4] = {{1, 4, -30, 28}, {-4, 105, -300, 210}, {-5, 48, -105, 64}, {-16, 105, -192, 105}};
    static const double k0[1][4] = {{1, 0, 0, 0}};
    switch (k) {
        case 0: *scale = sqrt(0.5); return k0[p];
        case 1: *scale = (p == 0) ? sqrt(1.5) : sqrt(0.5); return k1[p];
        case 2: *scale = (p == 0) ? sqrt(0.5) / 3.0 : (p == 1) ? sqrt(1.5) * 0.5 : sqrt(2.5) / 3.0; return k2[p];
        case 3:
            *scale = (p == 0) ? sqrt(15.0 / 34.0) : (p == 1) ? sqrt(1.0 / 42.0) : (p == 2) ? sqrt(35.0 / 34.0) * 0.5 : sqrt(5.0 / 42.0) * 0.5;
            return k3[p];
        default: *scale = 0; return NULL;
    }
}

/* l-th derivative of the mother function at x in [-1,1] */
static double alpert_mother(int k, int p, int l, double x) {
    double sgn = 1.0;
    if (x < 0) {
        /* parity of the l-th derivative flips with l */
        const int odd = (p + k + 1 + l) % 2;
        sgn = odd ? -1.0 : 1.0;
        x = -x;
    }
    double scale;
    const double* c = alpert_right_poly(k, p, &scale);
    if (!c) return 0.0;
    double v = 0.0;
    for (int m = k; m >= l; --m) {
        double fac = 1.0;
        for (int r = 0; r < l; ++r) fac *= (double)(m - r);
        v = v * x + c[m] * fac; /* Horner on the derivative polynomial */
    }
    /* Horner above accumulates c[m]*fac with powers x^(m-l) */
    return sgn * scale * v;
}

/* Legendre polynomial P_p and derivatives on [-1,1] by the three-term recurrence. */
static double legendre_deriv(int p, int l, double x) {
    if (fabs(x) > 1.0) return 0.0;
    /* values and derivatives up to order l via recurrences on coefficients */
    double c_prev[8] = {1, 0, 0, 0, 0, 0, 0, 0}; /* P_0 */
    double c_cur[8] = {0, 1, 0, 0, 0, 0, 0, 0};  /* P_1 */
    double c[8] = {0};
    if (p == 0) memcpy(c, c_prev, sizeof c);
    else if (p == 1) memcpy(c, c_cur, sizeof c);
    else {
        for (int n = 1; n < p; ++n) {
            double nx[8] = {0};
            /* (n+1) P_{n+1} = (2n+1) x P_n - n P_{n-1} */
            for (int m = 0; m < 7; ++m) nx[m + 1] += (2.0 * n + 1.0) * c_cur[m];
            for (int m = 0; m < 8; ++m) nx[m] -= n * c_prev[m];
            for (int m = 0; m < 8; ++m) nx[m] /= (n + 1.0);
            memcpy(c_prev, c_cur, sizeof c_prev);
            memcpy(c_cur, nx, sizeof c_cur);
        }
        memcpy(c, c_cur, sizeof c);
    }
    double v = 0.0;
    for (int m = 7; m >= l; --m) {
        double fac = 1.0;
        for (int r = 0; r < l; ++r) fac *= (double)(m - r);
        v = v * x + c[m] * fac;
    }
    return v;
}

static double alpert_raw(int k, int n, int j, int p, int l, double x) {
    if (n == 0) {
        /* normalized Legendre polynomial on [0,1] */
        return legendre_deriv(p, l, 2 * x - 1) * pow(2.0, l) * sqrt(2 * p + 1.0);
    } else if (n == 1) {
        if (x >= 0 && x <= 1) return pow(2.0, l + 0.5) * alpert_mother(k, p, l, 2 * x - 1);
        return 0.0;
    } else {
        const int jodd = (j - 1) / 2;
        const double sx = pow(2.0, n - 1) * x - jodd;
        return pow(2.0, (n - 1) * (l + 0.5)) * alpert_raw(k, 1, 1, p, l, sx);
    }
}

double amdg_oracle_alpert_val(int k, int level, int suppt, int p, int deriv, double x, int sgn) {
    /* one-sided limits by a 1e-13 shift, zero outside [0,1] (AlptBasis.cpp:16-30) */
    double xl = x;
    if (sgn == -1) {
        if (fabs(x) <= ROUND_OFF) return 0.0;
        xl -= ROUND_OFF;
    } else if (sgn == 1) {
        if (fabs(x - 1) <= ROUND_OFF) return 0.0;
        xl += ROUND_OFF;
    }
    return alpert_raw(k, level, suppt, p, deriv, xl);
}

/* ------------------------------------------------------------------------ */
/* Gauss-Legendre nodes by Newton iteration on P_n.                           */
/* ------------------------------------------------------------------------ */
int amdg_oracle_gauss_legendre(int n, double* x, double* w) {
    if (n < 1 || n > 16) return -1;
    const double pi = 3.14159265358979323846;
    for (int i = 0; i < n; ++i) {
        double z = cos(pi * (i + 0.75) / (n + 0.5));
        double dp = 1.0;
        for (int it = 0; it < 100; ++it) {
            double p0 = 1.0, p1 = z;
            for (int m = 2; m <= n; ++m) {
                double p2 = ((2.0 * m - 1.0) * z * p1 - (m - 1.0) * p0) / m;
                p0 = p1;
                p1 = p2;
            }
            if (n == 1) { p1 = z; p0 = 1.0; }
            dp = n * (z * p1 - p0) / (z * z - 1.0);
            double dz = p1 / dp;
            z -= dz;
            if (fabs(dz) < 1e-16) break;
        }
        {
            double p0 = 1.0, p1 = z;
            for (int m = 2; m <= n; ++m) {
                double p2 = ((2.0 * m - 1.0) * z * p1 - (m - 1.0) * p0) / m;
                p0 = p1;
                p1 = p2;
            }
            if (n == 1) { p1 = z; p0 = 1.0; }
            dp = n * (z * p1 - p0) / (z * z - 1.0);
        }
        /* ascending order */
        x[n - 1 - i] = z;
        w[n - 1 - i] = 2.0 / ((1.0 - z * z) * dp * dp);
    }
    if (n == 1) { x[0] = 0.0; w[0] = 2.0; }
    return 0;
}

static double gl_integrate(double (*f)(double, const void*), const void* ctx, double a, double b, int npts) {
    double gx[16], gw[16];
    amdg_oracle_gauss_legendre(npts, gx, gw);
    double s = 0.0;
    for (int i = 0; i < npts; ++i) s += gw[i] * f(a + (gx[i] + 1.0) * 0.5 * (b - a), ctx);
    return s * (b - a) / 2.0;
}

/* 1D element helpers ------------------------------------------------------ */
typedef struct { int n, j; } elem1d;

static elem1d elem_of_order(int o) {
    elem1d e;
    if (o == 0) { e.n = 0; e.j = 1; return e; }
    int n = 1;
    while ((1 << n) <= o) ++n;          /* 2^(n-1) <= o < 2^n */
    e.n = n;
    e.j = 2 * (o - (1 << (n - 1))) + 1;
    return e;
}

static int order_of_elem(int n, int j) { return n == 0 ? 0 : (1 << (n - 1)) + (j - 1) / 2; }

/* support in units of 2^-N */
static void support_units(int n, int j, int N, long* a, long* b) {
    if (n <= 1) { *a = 0; *b = 1L << N; return; }
    const long w = 1L << (N - n + 1);
    *a = (long)((j - 1) / 2) * w;
    *b = *a + w;
}

static double support_lo(int n, int j) { return n <= 1 ? 0.0 : pow(2.0, -n + 1.0) * (j - 1.0) / 2.0; }
static double support_hi(int n, int j) { return n <= 1 ? 1.0 : pow(2.0, -n + 1.0) * (j + 1.0) / 2.0; }

/* ------------------------------------------------------------------------ */
/* 1D operator matrices (OperatorMatrix1D.h:166-199, Basis.cpp:61-173)       */
/* ------------------------------------------------------------------------ */
typedef struct { int k; elem1d u, v; int pu, pv; int du, dv; } prod_ctx;

static double prod_integrand(double x, const void* c) {
    const prod_ctx* p = (const prod_ctx*)c;
    return amdg_oracle_alpert_val(p->k, p->u.n, p->u.j, p->pu, p->du, x, 0) *
           amdg_oracle_alpert_val(p->k, p->v.n, p->v.j, p->pv, p->dv, x, 0);
}

static double product_volume(int k, elem1d u, int pu, elem1d v, int pv, int du, int dv) {
    const double ua = support_lo(u.n, u.j), ub = support_hi(u.n, u.j);
    const double va = support_lo(v.n, v.j), vb = support_hi(v.n, v.j);
    if (va >= ub || vb <= ua) return 0.0;
    double xl = ua, xr = ub;
    if (u.n <= v.n) { xl = va; xr = vb; }
    const double xm = (xl + xr) / 2.0;
    prod_ctx c = {k, u, v, pu, pv, du, dv};
    return gl_integrate(prod_integrand, &c, xl, xm, 10) + gl_integrate(prod_integrand, &c, xm, xr, 10);
}

/* sum over the discontinuity points of v of u^(su) v^(sv), periodic boundary */
static double product_edge_dis_v(int k, elem1d u, int pu, elem1d v, int pv, int su, int sv) {
    const double pts[3] = {support_lo(v.n, v.j), 0.5 * (support_lo(v.n, v.j) + support_hi(v.n, v.j)), support_hi(v.n, v.j)};
    double s = 0.0;
    for (int i = 0; i < 3; ++i) {
        if (v.n <= 1 && i == 2) continue; /* 0 and 1 are the same point */
        const double x = pts[i];
        double vu = amdg_oracle_alpert_val(k, u.n, u.j, pu, 0, x, su);
        double vv = amdg_oracle_alpert_val(k, v.n, v.j, pv, 0, x, sv);
        if (fabs(x) < ROUND_OFF) {
            if (su == -1) vu = amdg_oracle_alpert_val(k, u.n, u.j, pu, 0, 1.0, su);
            if (sv == -1) vv = amdg_oracle_alpert_val(k, v.n, v.j, pv, 0, 1.0, sv);
        } else if (fabs(x - 1.0) < ROUND_OFF) {
            if (su == 1) vu = amdg_oracle_alpert_val(k, u.n, u.j, pu, 0, 0.0, su);
            if (sv == 1) vv = amdg_oracle_alpert_val(k, v.n, v.j, pv, 0, 0.0, sv);
        }
        s += vu * vv;
    }
    return s;
}

int amdg_oracle_oper1d(int N, int k, double* u_v, double* u_vx, double* ulft_vjp, double* urgt_vjp) {
    const int nb = (1 << N) * (k + 1);
#pragma omp parallel for schedule(dynamic)
    for (int r = 0; r < nb; ++r) {
        const elem1d u = elem_of_order(r / (k + 1));
        const int pu = r % (k + 1);
        for (int c = 0; c < nb; ++c) {
            const elem1d v = elem_of_order(c / (k + 1));
            const int pv = c % (k + 1);
            const size_t idx = (size_t)r * nb + c;
            if (u_v) u_v[idx] = product_volume(k, u, pu, v, pv, 0, 0);
            if (u_vx) u_vx[idx] = product_volume(k, u, pu, v, pv, 0, 1);
            if (ulft_vjp) ulft_vjp[idx] = product_edge_dis_v(k, u, pu, v, pv, -1, 1) - product_edge_dis_v(k, u, pu, v, pv, -1, -1);
            if (urgt_vjp) urgt_vjp[idx] = product_edge_dis_v(k, u, pu, v, pv, 1, 1) - product_edge_dis_v(k, u, pu, v, pv, 1, -1);
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Sparse / full grid (DGSolution.cpp:10-57)                                  */
/* ------------------------------------------------------------------------ */
/* Level vectors with sum <= N (sparse) or all of them (full); within a level
 * vector every support combination.  Elements are returned sorted by their
 * packed 1D orders (first dimension most significant). */
static int cmp_u64(const void* a, const void* b) {
    const uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
    return x < y ? -1 : (x > y);
}

static int64_t grid_walk(int dim, int N, int sparse, int32_t* level, int32_t* suppt) {
    int lv[16] = {0};
    int64_t count = 0;
    uint64_t* keys = NULL;
    int64_t cap = 0;
    for (;;) {
        int lsum = 0;
        for (int d = 0; d < dim; ++d) lsum += lv[d];
        if (!sparse || lsum <= N) {
            int64_t ne = 1;
            for (int d = 0; d < dim; ++d) ne *= (lv[d] == 0) ? 1 : (1L << (lv[d] - 1));
            if (level) {
                if (count + ne > cap) {
                    cap = 2 * (count + ne);
                    keys = (uint64_t*)realloc(keys, cap * sizeof(uint64_t));
                }
                for (int64_t i = 0; i < ne; ++i) {
                    int64_t rem = i;
                    uint64_t key = 0;
                    int o[16];
                    for (int d = dim - 1; d >= 0; --d) {
                        const int64_t nd = (lv[d] == 0) ? 1 : (1L << (lv[d] - 1));
                        const int s = (int)(rem % nd);
                        rem /= nd;
                        o[d] = (lv[d] == 0) ? 0 : (1 << (lv[d] - 1)) + s;
                    }
                    for (int d = 0; d < dim; ++d) key = (key << N) | (uint64_t)o[d];
                    keys[count + i] = key;
                }
            }
            count += ne;
        }
        int d = dim - 1;
        while (d >= 0) {
            if (++lv[d] <= N) break;
            lv[d] = 0;
            --d;
        }
        if (d < 0) break;
    }
    if (level) {
        qsort(keys, count, sizeof(uint64_t), cmp_u64);
        const uint64_t mask = (N == 0) ? 0 : ((1ULL << N) - 1);
        for (int64_t e = 0; e < count; ++e) {
            for (int d = 0; d < dim; ++d) {
                const int o = (int)((keys[e] >> (uint64_t)(N * (dim - 1 - d))) & mask);
                elem1d el = elem_of_order(o);
                level[e * dim + d] = el.n;
                suppt[e * dim + d] = el.j;
            }
        }
        free(keys);
    }
    return count;
}

int64_t amdg_oracle_grid_count(int dim, int N, int sparse) {
    if (dim < 1 || dim > 16 || N < 0 || N > 20) return -1;
    return grid_walk(dim, N, sparse, NULL, NULL);
}

int64_t amdg_oracle_grid(int dim, int N, int sparse, int32_t* level, int32_t* suppt) {
    if (dim < 1 || dim > 16 || N < 0 || N > 20) return -1;
    return grid_walk(dim, N, sparse, level, suppt);
}

/* ------------------------------------------------------------------------ */
/* Separable projection and initialisation (Basis.cpp:38-59, DGSolution.cpp:150-184) */
/* ------------------------------------------------------------------------ */
typedef struct { int k; elem1d e; int p; amdg_oracle_fn1d f; void* user; int d, term; } proj_ctx;

static double proj_integrand(double x, const void* c) {
    const proj_ctx* p = (const proj_ctx*)c;
    return amdg_oracle_alpert_val(p->k, p->e.n, p->e.j, p->p, 0, x, 0) * p->f(x, p->d, p->term, p->user);
}

int amdg_oracle_project_separable(int N, int k, int dim, int nterms, amdg_oracle_fn1d f, void* user, double* out) {
    const int nb = (1 << N) * (k + 1);
    for (int t = 0; t < nterms; ++t)
        for (int d = 0; d < dim; ++d)
            for (int b = 0; b < nb; ++b) {
                proj_ctx c = {k, elem_of_order(b / (k + 1)), b % (k + 1), f, user, d, t};
                double s = 0.0;
                if (c.e.n <= 4) {
                    for (int i = 0; i < 16; ++i) s += gl_integrate(proj_integrand, &c, i / 16.0, (i + 1) / 16.0, 10);
                } else {
                    const double a = support_lo(c.e.n, c.e.j), bb = support_hi(c.e.n, c.e.j), m = (a + bb) / 2.0;
                    s = gl_integrate(proj_integrand, &c, a, m, 10) + gl_integrate(proj_integrand, &c, m, bb, 10);
                }
                out[((size_t)t * dim + d) * nb + b] = s;
            }
    return 0;
}

static int ipow(int b, int e) { int r = 1; while (e-- > 0) r *= b; return r; }

int amdg_oracle_init_separable(int dim, int N, int k, int64_t E, const int32_t* level, const int32_t* suppt,
                               int nterms, const double* coef1d, double* u) {
    const int nb1 = (1 << N) * (k + 1);
    const int B = ipow(k + 1, dim);
#pragma omp parallel for
    for (int64_t e = 0; e < E; ++e) {
        int o[16];
        for (int d = 0; d < dim; ++d) o[d] = order_of_elem(level[e * dim + d], suppt[e * dim + d]);
        for (int q = 0; q < B; ++q) u[e * B + q] = 0.0;
        for (int t = 0; t < nterms; ++t)
            for (int q = 0; q < B; ++q) {
                int dig[16];
                int rem = q;
                for (int d = dim - 1; d >= 0; --d) { dig[d] = rem % (k + 1); rem /= (k + 1); }
                double v = 1.0;
                for (int d = 0; d < dim; ++d) v *= coef1d[((size_t)t * dim + d) * nb1 + o[d] * (k + 1) + dig[d]];
                u[e * B + q] += v;
            }
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Element lookup: open-addressing hash over packed 1D orders.                */
/* ------------------------------------------------------------------------ */
typedef struct { uint64_t* keys; int64_t* vals; uint64_t mask; } ehash;

static uint64_t pack_key(const int* o, int dim, int N) {
    uint64_t key = 0;
    for (int d = 0; d < dim; ++d) key = (key << N) | (uint64_t)o[d];
    return key;
}

static uint64_t mix64(uint64_t x) {
    x ^= x >> 33; x *= 0xff51afd7ed558ccdULL; x ^= x >> 33; x *= 0xc4ceb9fe1a85ec53ULL; x ^= x >> 33;
    return x;
}

static int ehash_build(ehash* h, int dim, int N, int64_t E, const int32_t* level, const int32_t* suppt) {
    uint64_t cap = 16;
    while (cap < (uint64_t)E * 2) cap <<= 1;
    h->keys = (uint64_t*)malloc(cap * sizeof(uint64_t));
    h->vals = (int64_t*)malloc(cap * sizeof(int64_t));
    if (!h->keys || !h->vals) return -1;
    h->mask = cap - 1;
    for (uint64_t i = 0; i < cap; ++i) h->vals[i] = -1;
    for (int64_t e = 0; e < E; ++e) {
        int o[16];
        for (int d = 0; d < dim; ++d) o[d] = order_of_elem(level[e * dim + d], suppt[e * dim + d]);
        const uint64_t key = pack_key(o, dim, N);
        uint64_t s = mix64(key) & h->mask;
        while (h->vals[s] >= 0 && h->keys[s] != key) s = (s + 1) & h->mask;
        h->keys[s] = key;
        h->vals[s] = e;
    }
    return 0;
}

static int64_t ehash_find(const ehash* h, uint64_t key) {
    uint64_t s = mix64(key) & h->mask;
    while (h->vals[s] >= 0) {
        if (h->keys[s] == key) return h->vals[s];
        s = (s + 1) & h->mask;
    }
    return -1;
}

static void ehash_free(ehash* h) { free(h->keys); free(h->vals); }

/* flux-neighbour predicate in one dimension (Element.cpp:283-348): supports
 * intersect, or are adjacent, or are adjacent across the periodic boundary */
static int intersect_or_adjacent(long a, long b, long a2, long b2, long one) {
    const int no_int = (a >= b2) || (b <= a2);
    const int adj = (a == b2) || (b == a2);
    const int per = (a == 0 && b2 == one) || (a2 == 0 && b == one);
    return !no_int || adj || per;
}

/* ------------------------------------------------------------------------ */
/* Linear operator (BilinearForm.cpp:25-87, 691-710)                          */
/* ------------------------------------------------------------------------ */
typedef struct {
    int dim, N, k, nb1;
    double* mvol; /* per dim: c_d * u_vx, dropped below ROUND_OFF */
    double* mflx; /* per dim: c_d * (ulft_vjp | urgt_vjp) */
} linop;

static int linop_build(linop* L, int dim, int N, int k, const double* c) {
    L->dim = dim; L->N = N; L->k = k;
    L->nb1 = (1 << N) * (k + 1);
    const size_t n2 = (size_t)L->nb1 * L->nb1;
    double* uvx = (double*)malloc(n2 * sizeof(double));
    double* ul = (double*)malloc(n2 * sizeof(double));
    double* ur = (double*)malloc(n2 * sizeof(double));
    L->mvol = (double*)malloc(n2 * dim * sizeof(double));
    L->mflx = (double*)malloc(n2 * dim * sizeof(double));
    if (!uvx || !ul || !ur || !L->mvol || !L->mflx) return -1;
    amdg_oracle_oper1d(N, k, NULL, uvx, ul, ur);
    for (int d = 0; d < dim; ++d) {
        const double* f = (c[d] >= 0) ? ul : ur;
        for (size_t i = 0; i < n2; ++i) {
            double a = c[d] * uvx[i];
            double b = c[d] * f[i];
            L->mvol[d * n2 + i] = (fabs(a) >= ROUND_OFF) ? a : 0.0;
            L->mflx[d * n2 + i] = (fabs(b) >= ROUND_OFF) ? b : 0.0;
        }
    }
    free(uvx); free(ul); free(ur);
    return 0;
}

static void linop_free(linop* L) { free(L->mvol); free(L->mflx); }

static void linear_rhs_range(const linop* L, const ehash* h, int64_t E, const int32_t* level, const int32_t* suppt,
                             const double* u, double* rhs, int64_t e0, int64_t e1, int nthreads) {
    const int dim = L->dim, N = L->N, k = L->k, np = k + 1, nb1 = L->nb1;
    const int B = ipow(np, dim);
    const size_t n2 = (size_t)nb1 * nb1;
    const long one = 1L << N;
    (void)E;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t e = e0; e < e1; ++e) {
        int o[16], lv[16], sp[16];
        for (int d = 0; d < dim; ++d) {
            lv[d] = level[e * dim + d];
            sp[d] = suppt[e * dim + d];
            o[d] = order_of_elem(lv[d], sp[d]);
        }
        double* y = rhs + (e - e0) * B;
        for (int q = 0; q < B; ++q) y[q] = 0.0;
        int stride[16];
        stride[dim - 1] = 1;
        for (int d = dim - 2; d >= 0; --d) stride[d] = stride[d + 1] * np;
        for (int t = 0; t < dim; ++t) {
            long a, b;
            support_units(lv[t], sp[t], N, &a, &b);
            int o2[16];
            memcpy(o2, o, sizeof(int) * dim);
            for (int oc = 0; oc < (1 << N); ++oc) {
                const elem1d ec = elem_of_order(oc);
                long a2, b2;
                support_units(ec.n, ec.j, N, &a2, &b2);
                if (!intersect_or_adjacent(a, b, a2, b2, one)) continue;
                o2[t] = oc;
                const int64_t es = ehash_find(h, pack_key(o2, dim, N));
                if (es < 0) continue;
                const int is_vol = !((a >= b2) || (b <= a2));
                const double* us = u + es * B;
                const double* mv = L->mvol + t * n2;
                const double* mf = L->mflx + t * n2;
                for (int q = 0; q < B; ++q) {
                    const int qt = (q / stride[t]) % np;
                    const int base = q - qt * stride[t];
                    const int col = o[t] * np + qt; /* test basis */
                    double acc = 0.0;
                    for (int p = 0; p < np; ++p) {
                        const int row = oc * np + p; /* solution basis */
                        const double m = (is_vol ? mv[(size_t)row * nb1 + col] : 0.0) + mf[(size_t)row * nb1 + col];
                        acc += m * us[base + p * stride[t]];
                    }
                    y[q] += acc;
                }
            }
        }
    }
}

int amdg_oracle_linear_rhs_range(int dim, int N, int k, int64_t E, const int32_t* level, const int32_t* suppt,
                                 const double* c, const double* u, double* rhs, int64_t e_begin, int64_t e_end,
                                 int nthreads) {
    if (dim < 1 || dim > 16 || dim * N > 64) return -1;
    linop L;
    ehash h;
    if (linop_build(&L, dim, N, k, c)) return -2;
    if (ehash_build(&h, dim, N, E, level, suppt)) return -2;
    linear_rhs_range(&L, &h, E, level, suppt, u, rhs, e_begin, e_end, nthreads);
    ehash_free(&h);
    linop_free(&L);
    return 0;
}

/* Prebuilt operator handle (1D matrices and element hash built once), so that
 * timing samples measure only the right-hand-side evaluation. */
typedef struct {
    linop L;
    ehash h;
    int64_t E;
    const int32_t* level;
    const int32_t* suppt;
} oracle_linop;

void* amdg_oracle_linop_create(int dim, int N, int k, int64_t E, const int32_t* level, const int32_t* suppt,
                               const double* c) {
    if (dim < 1 || dim > 16 || dim * N > 64) return NULL;
    oracle_linop* op = (oracle_linop*)calloc(1, sizeof(oracle_linop));
    if (!op) return NULL;
    if (linop_build(&op->L, dim, N, k, c) || ehash_build(&op->h, dim, N, E, level, suppt)) { free(op); return NULL; }
    op->E = E;
    op->level = level;
    op->suppt = suppt;
    return op;
}

int amdg_oracle_linop_apply_range(void* handle, const double* u, double* rhs, int64_t e_begin, int64_t e_end, int nthreads) {
    oracle_linop* op = (oracle_linop*)handle;
    if (!op) return -1;
    linear_rhs_range(&op->L, &op->h, op->E, op->level, op->suppt, u, rhs, e_begin, e_end, nthreads);
    return 0;
}

void amdg_oracle_linop_destroy(void* handle) {
    oracle_linop* op = (oracle_linop*)handle;
    if (!op) return;
    ehash_free(&op->h);
    linop_free(&op->L);
    free(op);
}

int amdg_oracle_linear_rhs(int dim, int N, int k, int64_t E, const int32_t* level, const int32_t* suppt,
                           const double* c, const double* u, double* rhs, int nthreads) {
    return amdg_oracle_linear_rhs_range(dim, N, k, E, level, suppt, c, u, rhs, 0, E, nthreads);
}

int amdg_oracle_linear_rk3(int dim, int N, int k, int64_t E, const int32_t* level, const int32_t* suppt,
                           const double* c, double dt, int steps, double* u, int nthreads) {
    if (dim < 1 || dim > 16 || dim * N > 64) return -1;
    const int B = ipow(k + 1, dim);
    const size_t n = (size_t)E * B;
    linop L;
    ehash h;
    if (linop_build(&L, dim, N, k, c)) return -2;
    if (ehash_build(&h, dim, N, E, level, suppt)) return -2;
    double* rhs = (double*)malloc(n * sizeof(double));
    double* u1 = (double*)malloc(n * sizeof(double));
    double* u2 = (double*)malloc(n * sizeof(double));
    if (!rhs || !u1 || !u2) return -2;
    /* RK3SSP::step_rk (ODESolver.cpp:261-271), element-wise in the written order */
    for (int s = 0; s < steps; ++s) {
        linear_rhs_range(&L, &h, E, level, suppt, u, rhs, 0, E, nthreads);
        for (size_t i = 0; i < n; ++i) u1[i] = u[i] + dt * rhs[i];
        linear_rhs_range(&L, &h, E, level, suppt, u1, rhs, 0, E, nthreads);
        for (size_t i = 0; i < n; ++i) u2[i] = 3. / 4. * u[i] + 1. / 4. * (u1[i] + dt * rhs[i]);
        linear_rhs_range(&L, &h, E, level, suppt, u2, rhs, 0, E, nthreads);
        for (size_t i = 0; i < n; ++i) u[i] = 1. / 3. * u[i] + 2. / 3. * (u2[i] + dt * rhs[i]);
    }
    free(rhs); free(u1); free(u2);
    ehash_free(&h);
    linop_free(&L);
    return 0;
}

double amdg_oracle_l2_error_split(int dim, int N, int k, int64_t E, const int32_t* level, const int32_t* suppt,
                                  const double* u, const double* coef1d_exact, double l2_norm_exact) {
    const int nb1 = (1 << N) * (k + 1);
    const int B = ipow(k + 1, dim);
    double err2 = l2_norm_exact * l2_norm_exact;
    for (int64_t e = 0; e < E; ++e) {
        int o[16];
        for (int d = 0; d < dim; ++d) o[d] = order_of_elem(level[e * dim + d], suppt[e * dim + d]);
        for (int q = 0; q < B; ++q) {
            const double v = u[e * B + q];
            err2 += v * v;
            int dig[16];
            int rem = q;
            for (int d = dim - 1; d >= 0; --d) { dig[d] = rem % (k + 1); rem /= (k + 1); }
            double coe = 1.0;
            for (int d = 0; d < dim; ++d) coe *= coef1d_exact[(size_t)d * nb1 + o[d] * (k + 1) + dig[d]];
            err2 -= 2.0 * v * coe;
        }
    }
    return sqrt(err2 > 0 ? err2 : 0.0);
}

/* ======================================================================== */
/* Lagrange interpolation path for nonlinear fluxes (config: 3D Burgers)     */
/* ======================================================================== */
/* Hierarchical Lagrange bases (node layouts LagrBasis.cpp:33-155, mother
 * functions LagrBasis.cpp:190-615), chosen by amdg_oracle_set_lagr_degree:
 *  - degree 3, msh_case 1 (the Burgers examples): level-0 nodes {-3/5,-1/5,1/5,3/5}
 *    on [-1,1]; level-1 nodes {-4/5,-2/5} on the left half and {2/5,4/5} on the
 *    right half, each interpolating on its half together with the two level-0
 *    nodes of that half;
 *  - degree 4, msh_case 2 (03_wave_06_var_coeff_adapt.cpp:53-54): level-0 nodes
 *    {-1,-1/2,0,1/2,1} whose points sit 1e-13 inside the element (left of the
 *    node, except at -1); level-1 nodes {-3/4,-1/4} on the left half and
 *    {0,1/4,3/4} on the right half (the one at 0 just right of it), each the
 *    degree-4 polynomial on the nodes of its half at spacing 1/4. */
typedef struct {
    int p1;                /* points per element and dimension: degree + 1 */
    double pt0[6], pt1[6]; /* interpolation points of level 0 / levels >= 1 on [-1, 1] */
    double node0[6];       /* level-0 polynomial nodes */
    double half[2][6];     /* level-1 polynomial nodes of the left / right half */
    int side[6], node[6];  /* level-1 function p: its half and its node there */
} lagr_spec;

static const lagr_spec LAGR_DEG3 = {4,
                                    {-0.6, -0.2, 0.2, 0.6},
                                    {-0.8, -0.4, 0.4, 0.8},
                                    {-0.6, -0.2, 0.2, 0.6},
                                    {{-0.8, -0.6, -0.4, -0.2}, {0.2, 0.4, 0.6, 0.8}},
                                    {0, 0, 1, 1},
                                    {0, 2, 1, 3}};
static const lagr_spec LAGR_DEG4 = {5,
                                    {-1 + ROUND_OFF, -0.5 - ROUND_OFF, 0 - ROUND_OFF, 0.5 - ROUND_OFF, 1 - ROUND_OFF},
                                    {-0.75 - ROUND_OFF, -0.25 - ROUND_OFF, 0 + ROUND_OFF, 0.25 - ROUND_OFF, 0.75 - ROUND_OFF},
                                    {-1, -0.5, 0, 0.5, 1},
                                    {{-1, -0.75, -0.5, -0.25, 0}, {0, 0.25, 0.5, 0.75, 1}},
                                    {0, 0, 1, 1, 1},
                                    {1, 3, 0, 1, 3}};
/* degree 5, msh_case 1 (02_hyperbolic_01_scalar_const_coefficient.cpp:44-45): level-0 nodes
 * {-1,-3/5,-1/5,1/5,3/5,1}, the end points 1e-13 inside; level-1 nodes {-4/5,-2/5,0} on the
 * left half and {0,2/5,4/5} on the right half (0 just left / right of it), each the quintic on
 * the nodes of its half at spacing 1/5 (the level-0 nodes mapped onto the half) */
static const lagr_spec LAGR_DEG5 = {6,
                                    {-1 + ROUND_OFF, -0.6, -0.2, 0.2, 0.6, 1 - ROUND_OFF},
                                    {-0.8, -0.4, 0 - ROUND_OFF, 0 + ROUND_OFF, 0.4, 0.8},
                                    {-1, -0.6, -0.2, 0.2, 0.6, 1},
                                    {{-1, -0.8, -0.6, -0.4, -0.2, 0}, {0, 0.2, 0.4, 0.6, 0.8, 1}},
                                    {0, 0, 0, 1, 1, 1},
                                    {1, 3, 5, 0, 2, 4}};
static const lagr_spec* LS = &LAGR_DEG3;

int amdg_oracle_set_lagr_degree(int degree) {
    if (degree == 3) LS = &LAGR_DEG3;
    else if (degree == 4) LS = &LAGR_DEG4;
    else if (degree == 5) LS = &LAGR_DEG5;
    else return -1;
    return 0;
}

int amdg_oracle_lagr_points_per_dim(void) { return LS->p1; }

static double lagr_poly(const double* nodes, int i, double x) {
    double v = 1.0;
    for (int m = 0; m < LS->p1; ++m)
        if (m != i) v *= (x - nodes[m]) / (nodes[i] - nodes[m]);
    return v;
}

static double lagr_phi(double xt, int msh, int p) {
    const double x = 2.0 * xt - 1.0;
    if (x < -1.0 || x > 1.0) return 0.0;
    if (msh == 0) return lagr_poly(LS->node0, p, x);
    if (LS->side[p] == 0) {
        if (x > 0) return 0.0;
        return lagr_poly(LS->half[0], LS->node[p], x);
    }
    if (x < 0) return 0.0;
    return lagr_poly(LS->half[1], LS->node[p], x);
}

double amdg_oracle_lagr_val(int level, int suppt, int p, double x, int sgn) {
    double xl = x;
    if (sgn == -1) {
        if (fabs(x) <= ROUND_OFF) return 0.0;
        xl -= ROUND_OFF;
    } else if (sgn == 1) {
        if (fabs(x - 1) <= ROUND_OFF) return 0.0;
        xl += ROUND_OFF;
    }
    if (level <= 1) return lagr_phi(xl, level, p);
    const double xt = pow(2.0, level - 1) * xl - (suppt - 1) / 2;
    return lagr_phi(xt, 1, p);
}

/* interpolation point p of 1D element (n, j) (LagrBasis.cpp:18-27) */
double amdg_oracle_lagr_point(int level, int suppt, int p) {
    if (level == 0) return (LS->pt0[p] + 1.0) / 2.0;
    const double a = support_lo(level, suppt), b = support_hi(level, suppt);
    return a + (b - a) * (LS->pt1[p] + 1.0) / 2.0;
}

/* generic 1D basis evaluation: type 0 = Alpert (degree k), 1 = Lagrange (the chosen degree),
 * 2 = cubic Hermite */
static double basis_val(int type, int k, int n, int j, int p, int deriv, double x, int sgn) {
    if (type == 0) return amdg_oracle_alpert_val(k, n, j, p, deriv, x, sgn);
    if (type == 2) return amdg_oracle_herm_val(n, j, p, deriv, x, sgn);
    return amdg_oracle_lagr_val(n, j, p, x, sgn);
}

typedef struct { int tu, tv, k; elem1d u, v; int pu, pv, du, dv; } gprod_ctx;

static double gprod_integrand(double x, const void* c) {
    const gprod_ctx* p = (const gprod_ctx*)c;
    return basis_val(p->tu, p->k, p->u.n, p->u.j, p->pu, p->du, x, 0) * basis_val(p->tv, p->k, p->v.n, p->v.j, p->pv, p->dv, x, 0);
}

static double gproduct_volume(int tu, int tv, int k, elem1d u, int pu, elem1d v, int pv, int du, int dv) {
    const double ua = support_lo(u.n, u.j), ub = support_hi(u.n, u.j);
    const double va = support_lo(v.n, v.j), vb = support_hi(v.n, v.j);
    if (va >= ub || vb <= ua) return 0.0;
    double xl = ua, xr = ub;
    if (u.n <= v.n) { xl = va; xr = vb; }
    const double xm = (xl + xr) / 2.0;
    gprod_ctx c = {tu, tv, k, u, v, pu, pv, du, dv};
    return gl_integrate(gprod_integrand, &c, xl, xm, 10) + gl_integrate(gprod_integrand, &c, xm, xr, 10);
}

static double gproduct_edge(int tu, int tv, int k, elem1d u, int pu, elem1d v, int pv, int su, int sv) {
    const double pts[3] = {support_lo(v.n, v.j), 0.5 * (support_lo(v.n, v.j) + support_hi(v.n, v.j)), support_hi(v.n, v.j)};
    double s = 0.0;
    for (int i = 0; i < 3; ++i) {
        if (v.n <= 1 && i == 2) continue;
        const double x = pts[i];
        double fu = basis_val(tu, k, u.n, u.j, pu, 0, x, su), fv = basis_val(tv, k, v.n, v.j, pv, 0, x, sv);
        if (fabs(x) < ROUND_OFF) {
            if (su == -1) fu = basis_val(tu, k, u.n, u.j, pu, 0, 1.0, su);
            if (sv == -1) fv = basis_val(tv, k, v.n, v.j, pv, 0, 1.0, sv);
        } else if (fabs(x - 1.0) < ROUND_OFF) {
            if (su == 1) fu = basis_val(tu, k, u.n, u.j, pu, 0, 0.0, su);
            if (sv == 1) fv = basis_val(tv, k, v.n, v.j, pv, 0, 0.0, sv);
        }
        s += fu * fv;
    }
    return s;
}

/* Lagrange (rows) x Alpert (cols, degree k) 1D matrices, each
 * (2^N*p1) x (2^N*(k+1)): u_v, u_vx and (ulft_vjp + urgt_vjp). */
int amdg_oracle_oper1d_lagr(int N, int k, double* u_v, double* u_vx, double* uave2_vjp) {
    const int nr = (1 << N) * LS->p1, nc = (1 << N) * (k + 1);
#pragma omp parallel for schedule(dynamic)
    for (int r = 0; r < nr; ++r) {
        const elem1d u = elem_of_order(r / LS->p1);
        const int pu = r % LS->p1;
        for (int c = 0; c < nc; ++c) {
            const elem1d v = elem_of_order(c / (k + 1));
            const int pv = c % (k + 1);
            const size_t idx = (size_t)r * nc + c;
            if (u_v) u_v[idx] = gproduct_volume(1, 0, k, u, pu, v, pv, 0, 0);
            if (u_vx) u_vx[idx] = gproduct_volume(1, 0, k, u, pu, v, pv, 0, 1);
            if (uave2_vjp) {
                const double l = gproduct_edge(1, 0, k, u, pu, v, pv, -1, 1) - gproduct_edge(1, 0, k, u, pu, v, pv, -1, -1);
                const double rr = gproduct_edge(1, 0, k, u, pu, v, pv, 1, 1) - gproduct_edge(1, 0, k, u, pu, v, pv, 1, -1);
                uave2_vjp[idx] = l + rr;
            }
        }
    }
    return 0;
}

/* 1D element order containing x at level n (x never on a cell boundary) */
static int order_containing(int n, double x) {
    if (n == 0) return 0;
    if (n == 1) return 1;
    int s = (int)floor(x * (double)(1 << (n - 1)));
    if (s >= (1 << (n - 1))) s = (1 << (n - 1)) - 1;
    return (1 << (n - 1)) + s;
}

/* u_h at every interpolation point of every element, summed directly over
 * all elements whose support contains the point:  up[e][p], (m+1)^dim per
 * element.  Same quantity as FastLagrIntp::eval_up_Lagr (FastMultiplyLU.cpp:1362). */
int amdg_oracle_lagr_point_values(int dim, int N, int k, int64_t E, const int32_t* level, const int32_t* suppt,
                                  const double* u, double* up) {
    ehash h;
    if (ehash_build(&h, dim, N, E, level, suppt)) return -2;
    const int np = k + 1, B = ipow(np, dim), P = ipow(LS->p1, dim);
#pragma omp parallel for schedule(dynamic, 8)
    for (int64_t e = 0; e < E; ++e) {
        for (int p = 0; p < P; ++p) {
            double x[16];
            int rem = p;
            int pd[16];
            for (int d = dim - 1; d >= 0; --d) { pd[d] = rem % LS->p1; rem /= LS->p1; }
            for (int d = 0; d < dim; ++d) x[d] = amdg_oracle_lagr_point(level[e * dim + d], suppt[e * dim + d], pd[d]);
            double val = 0.0;
            int lv[16] = {0};
            for (;;) {
                int o[16];
                for (int d = 0; d < dim; ++d) o[d] = order_containing(lv[d], x[d]);
                const int64_t s = ehash_find(&h, pack_key(o, dim, N));
                if (s >= 0) {
                    double phi[16][4];
                    for (int d = 0; d < dim; ++d) {
                        const elem1d ed = elem_of_order(o[d]);
                        for (int q = 0; q < np; ++q) phi[d][q] = amdg_oracle_alpert_val(k, ed.n, ed.j, q, 0, x[d], 0);
                    }
                    for (int q = 0; q < B; ++q) {
                        int r2 = q;
                        double w = 1.0;
                        int qd[16];
                        for (int d = dim - 1; d >= 0; --d) { qd[d] = r2 % np; r2 /= np; }
                        for (int d = 0; d < dim; ++d) w *= phi[d][qd[d]];
                        val += w * u[s * B + q];
                    }
                }
                int d = dim - 1;
                while (d >= 0) {
                    if (++lv[d] <= N) break;
                    lv[d] = 0;
                    --d;
                }
                if (d < 0) break;
            }
            up[e * P + p] = val;
        }
    }
    ehash_free(&h);
    return 0;
}

/* Hierarchical surplus of point values, dimension by dimension
 * (LagrInterpolation::eval_fp_to_coe_D_Lag, Interplation.cpp:1222-1434, with
 * the weights of set_pts_wts_1d_ada_Lag, :775-888): in pass d every element
 * with level_d > 0 subtracts the interpolant, through the p1 coarser-level
 * points inside its dimension-d support, of the values left by pass d-1.  fp
 * and out are E x p1^dim; fp may equal out. */
int amdg_oracle_lagr_surplus(int dim, int N, int64_t E, const int32_t* level, const int32_t* suppt, const double* fp,
                             double* out) {
    ehash h;
    if (ehash_build(&h, dim, N, E, level, suppt)) return -2;
    const int P = ipow(LS->p1, dim);
    double* cur = (double*)malloc((size_t)E * P * sizeof(double));
    double* nxt = (double*)malloc((size_t)E * P * sizeof(double));
    if (!cur || !nxt) return -2;
    memcpy(cur, fp, (size_t)E * P * sizeof(double));
    for (int d = 0; d < dim; ++d) {
        int stride = 1;
        for (int s = d + 1; s < dim; ++s) stride *= LS->p1;
#pragma omp parallel for schedule(dynamic, 8)
        for (int64_t e = 0; e < E; ++e) {
            const int l = level[e * dim + d], j = suppt[e * dim + d];
            if (l == 0) {
                memcpy(nxt + e * P, cur + e * P, P * sizeof(double));
                continue;
            }
            /* the p1 coarser points inside this element's dimension-d support */
            const int P1 = LS->p1;
            const double xl = support_lo(l, j), xr = support_hi(l, j);
            int anc_o[6], anc_q[6];
            double anc_x[6];
            int ic = 0;
            for (int o = 0; o < (1 << l) && ic < P1; ++o) {
                const elem1d ea = elem_of_order(o);
                if (ea.n >= l) break;
                for (int q = 0; q < P1; ++q) {
                    const double pos = amdg_oracle_lagr_point(ea.n, ea.j, q);
                    if (pos > xl && pos < xr && ic < P1) {
                        anc_o[ic] = o;
                        anc_q[ic] = q;
                        anc_x[ic] = pos;
                        ++ic;
                    }
                }
            }
            /* weight: minus the level-0 Lagrange basis of the ancestor's rank among the
             * sorted ancestor positions, at this element's own node */
            int rank[6];
            for (int a = 0; a < P1; ++a) {
                rank[a] = 0;
                for (int b = 0; b < P1; ++b) if (anc_x[b] < anc_x[a]) ++rank[a];
            }
            int64_t anc_e[6];
            int missing = ic != P1;
            for (int a = 0; a < P1 && !missing; ++a) {
                int o[16];
                for (int s = 0; s < dim; ++s) o[s] = order_of_elem(level[e * dim + s], suppt[e * dim + s]);
                o[d] = anc_o[a];
                anc_e[a] = ehash_find(&h, pack_key(o, dim, N));
                missing |= anc_e[a] < 0;
            }
            if (missing) continue; /* hole: checked below */
            for (int p = 0; p < P; ++p) {
                const int pd = (p / stride) % P1;
                const int base = p - pd * stride;
                double c = cur[e * P + p];
                const double xt = (LS->pt1[pd] + 1.0) / 2.0;
                for (int a = 0; a < P1; ++a) {
                    const double wt = -lagr_phi(xt, 0, rank[a]);
                    c += wt * cur[anc_e[a] * P + base + anc_q[a] * stride];
                }
                nxt[e * P + p] = c;
            }
        }
        double* t = cur; cur = nxt; nxt = t;
    }
    memcpy(out, cur, (size_t)E * P * sizeof(double));
    free(cur); free(nxt);
    ehash_free(&h);
    return 0;
}

/* contract a p1^dim block with per-dimension 1D matrices M_s (rows: p1 source
 * Lagrange indices of the source element, cols: np target Alpert indices)
 * into a np^dim block, accumulating scale * result into y */
static void contract_block(int dim, int np, const double* x, const double* const* M, int nc, const int* row0,
                           const int* col0, double scale, double* y) {
    double bufA[4096], bufB[4096];
    const double* src = x;
    int shape[16];
    const int P1 = LS->p1;
    for (int s = 0; s < dim; ++s) shape[s] = P1;
    double* dst = bufA;
    for (int s = 0; s < dim; ++s) {
        /* contract dimension s: size p1 -> np */
        int outer = 1, inner = 1;
        for (int r = 0; r < s; ++r) outer *= shape[r];
        for (int r = s + 1; r < dim; ++r) inner *= shape[r];
        for (int a = 0; a < outer; ++a)
            for (int q = 0; q < np; ++q)
                for (int b = 0; b < inner; ++b) {
                    double acc = 0.0;
                    for (int p = 0; p < P1; ++p)
                        acc += src[(a * P1 + p) * inner + b] * M[s][(size_t)(row0[s] + p) * nc + col0[s] + q];
                    dst[(a * np + q) * inner + b] = acc;
                }
        shape[s] = np;
        src = dst;
        dst = (dst == bufA) ? bufB : bufA;
    }
    const int B = ipow(np, dim);
    for (int i = 0; i < B; ++i) y[i] += scale * src[i];
}

/* Right-hand side of the Lagrange-interpolated Burgers operator with global
 * Lax-Friedrichs flux, summed directly over element pairs:
 *   volume   sum_d  <F_d, (u_vx in d, u_v elsewhere)>            (HyperbolicLagrRHS::rhs_vol_scalar)
 *   interface 0.5 sum_d <F_d, ((ulft+urgt)_vjp in d, u_v elsewhere)> (rhs_flx_intp_scalar)
 *   penalty  -alpha/2 sum_d ujp_vjp(Alpert) in d                   (HyperbolicAlptRHS::rhs_flx_penalty_scalar)
 * fucoe: dim x E x p1^dim interpolation coefficients of the flux per dimension. */
int amdg_oracle_burgers_rhs(int dim, int N, int k, int64_t E, const int32_t* level, const int32_t* suppt,
                            const double* fucoe, const double* u, double alpha, double* rhs) {
    const int np = k + 1, B = ipow(np, dim), P = ipow(LS->p1, dim), n1 = 1 << N;
    const int nr = n1 * LS->p1, nc = n1 * np;
    const long one = 1L << N;
    double* Lv = (double*)malloc((size_t)nr * nc * sizeof(double));
    double* Lvx = (double*)malloc((size_t)nr * nc * sizeof(double));
    double* Lf = (double*)malloc((size_t)nr * nc * sizeof(double));
    double* ul = (double*)malloc((size_t)nc * nc * sizeof(double));
    double* ur = (double*)malloc((size_t)nc * nc * sizeof(double));
    ehash h;
    if (!Lv || !Lvx || !Lf || !ul || !ur || ehash_build(&h, dim, N, E, level, suppt)) return -2;
    amdg_oracle_oper1d_lagr(N, k, Lv, Lvx, Lf);
    amdg_oracle_oper1d(N, k, NULL, NULL, ul, ur);
    /* 1D relations: vol (supports intersect), flx (intersect, adjacent or periodic-adjacent) */
    int* volc = (int*)calloc(n1, sizeof(int));
    int* flxc = (int*)calloc(n1, sizeof(int));
    int* vol = (int*)malloc((size_t)n1 * n1 * sizeof(int));
    int* flx = (int*)malloc((size_t)n1 * n1 * sizeof(int));
    for (int o = 0; o < n1; ++o) {
        const elem1d eo = elem_of_order(o);
        long a, b;
        support_units(eo.n, eo.j, N, &a, &b);
        for (int oc = 0; oc < n1; ++oc) {
            const elem1d ec = elem_of_order(oc);
            long a2, b2;
            support_units(ec.n, ec.j, N, &a2, &b2);
            if (!((a >= b2) || (b <= a2))) vol[o * n1 + volc[o]++] = oc;
            if (intersect_or_adjacent(a, b, a2, b2, one)) flx[o * n1 + flxc[o]++] = oc;
        }
    }
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t e = 0; e < E; ++e) {
        int o[16];
        for (int s = 0; s < dim; ++s) o[s] = order_of_elem(level[e * dim + s], suppt[e * dim + s]);
        double* y = rhs + e * B;
        for (int q = 0; q < B; ++q) y[q] = 0.0;
        for (int d = 0; d < dim; ++d) {
            for (int term = 0; term < 2; ++term) {
                /* term 0: volume, vol sets everywhere; term 1: interface, flx set in d */
                const double* M[16];
                for (int s = 0; s < dim; ++s) M[s] = (s == d) ? (term == 0 ? Lvx : Lf) : Lv;
                const double scale = term == 0 ? 1.0 : 0.5;
                int idx[16] = {0};
                for (;;) {
                    int oc[16], row0[16], col0[16];
                    for (int s = 0; s < dim; ++s) {
                        const int use_flx = (term == 1 && s == d);
                        oc[s] = use_flx ? flx[o[s] * n1 + idx[s]] : vol[o[s] * n1 + idx[s]];
                        row0[s] = oc[s] * LS->p1;
                        col0[s] = o[s] * np;
                    }
                    const int64_t es = ehash_find(&h, pack_key(oc, dim, N));
                    if (es >= 0) contract_block(dim, np, fucoe + ((size_t)d * E + es) * P, M, nc, row0, col0, scale, y);
                    int s = dim - 1;
                    while (s >= 0) {
                        const int cnt = (term == 1 && s == d) ? flxc[o[s]] : volc[o[s]];
                        if (++idx[s] < cnt) break;
                        idx[s] = 0;
                        --s;
                    }
                    if (s < 0) break;
                }
            }
            /* penalty on Alpert coefficients, same indices in the other dimensions */
            int stride = 1;
            for (int s = d + 1; s < dim; ++s) stride *= np;
            int o2[16];
            memcpy(o2, o, sizeof(int) * dim);
            for (int i = 0; i < flxc[o[d]]; ++i) {
                o2[d] = flx[o[d] * n1 + i];
                const int64_t es = ehash_find(&h, pack_key(o2, dim, N));
                if (es < 0) continue;
                for (int q = 0; q < B; ++q) {
                    const int qd = (q / stride) % np, base = q - qd * stride;
                    double acc = 0.0;
                    for (int p = 0; p < np; ++p) {
                        const size_t mi = (size_t)(o2[d] * np + p) * nc + o[d] * np + qd;
                        acc += (ur[mi] - ul[mi]) * u[es * B + base + p * stride];
                    }
                    y[q] += -alpha / 2.0 * acc;
                }
            }
        }
    }
    free(Lv); free(Lvx); free(Lf); free(ul); free(ur);
    free(volc); free(flxc); free(vol); free(flx);
    ehash_free(&h);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* The reference's fast transforms, restated (FastMultiplyLU.cpp:436-512,   */
/* 596-664): on adaptive grids the L/U partial sums only see intermediate   */
/* elements that exist, so they are the reference's operator there; on      */
/* sparse grids they equal the direct pair sums above.                      */
/* ------------------------------------------------------------------------ */
typedef struct {
    int dim, N, n1;
    int64_t E;
    const int32_t* level;
    const int32_t* suppt;
    int* order;    /* E x dim */
    ehash h;
    int* volc; int* vol;  /* 1D relations */
    int* flxc; int* flx;
} fast_ctx;

static int fast_ctx_init(fast_ctx* c, int dim, int N, int64_t E, const int32_t* level, const int32_t* suppt) {
    c->dim = dim; c->N = N; c->n1 = 1 << N; c->E = E; c->level = level; c->suppt = suppt;
    c->order = (int*)malloc((size_t)E * dim * sizeof(int));
    if (!c->order || ehash_build(&c->h, dim, N, E, level, suppt)) return -2;
    for (int64_t e = 0; e < E * dim; ++e) c->order[e] = order_of_elem(level[e], suppt[e]);
    const int n1 = c->n1;
    const long one = 1L << N;
    c->volc = (int*)calloc(n1, sizeof(int)); c->flxc = (int*)calloc(n1, sizeof(int));
    c->vol = (int*)malloc((size_t)n1 * n1 * sizeof(int)); c->flx = (int*)malloc((size_t)n1 * n1 * sizeof(int));
    for (int o = 0; o < n1; ++o) {
        const elem1d eo = elem_of_order(o);
        long a, b;
        support_units(eo.n, eo.j, N, &a, &b);
        for (int oc = 0; oc < n1; ++oc) {
            const elem1d ec = elem_of_order(oc);
            long a2, b2;
            support_units(ec.n, ec.j, N, &a2, &b2);
            if (!((a >= b2) || (b <= a2))) c->vol[o * n1 + c->volc[o]++] = oc;
            if (intersect_or_adjacent(a, b, a2, b2, one)) c->flx[o * n1 + c->flxc[o]++] = oc;
        }
    }
    return 0;
}

static void fast_ctx_free(fast_ctx* c) {
    free(c->order); free(c->volc); free(c->flxc); free(c->vol); free(c->flx);
    ehash_free(&c->h);
}

/* one 1D transform in dimension t (lu: 0 = "L", 1 = full, 2 = "U"; flx: neighbour set) */
static void fast_transform_1d(const fast_ctx* c, const double* in, const int* from, double* out, const int* to, int t,
                              const double* M, int ncols, int lu, int flx, double coef, int accumulate) {
    const int dim = c->dim, n1 = c->n1;
    int in_block = 1, out_block = 1, stride = 1;
    for (int s = 0; s < dim; ++s) { in_block *= from[s]; out_block *= to[s]; }
    for (int s = t + 1; s < dim; ++s) stride *= from[s];
    const int nf = from[t], nt = to[t];
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t e = 0; e < c->E; ++e) {
        const int* oe = c->order + e * dim;
        const int le = c->level[e * dim + t];
        int o2[16];
        memcpy(o2, oe, sizeof(int) * dim);
        const int cnt = flx ? c->flxc[oe[t]] : c->volc[oe[t]];
        const int* lst = (flx ? c->flx : c->vol) + (size_t)oe[t] * n1;
        double* y = out + e * out_block;
        for (int idx = 0; idx < out_block; ++idx) {
            const int inner = idx % stride, qt = (idx / stride) % nt, outer = idx / (stride * nt);
            double acc = 0.0;
            for (int i = 0; i < cnt; ++i) {
                const int oc = lst[i];
                const int ls = elem_of_order(oc).n;
                if (lu == 0 && le >= ls) continue;
                if (lu == 2 && le < ls) continue;
                o2[t] = oc;
                const int64_t s = ehash_find(&c->h, pack_key(o2, dim, c->N));
                if (s < 0) continue;
                const double* x = in + s * in_block + outer * nf * stride + inner;
                for (int k = 0; k < nf; ++k) acc += x[k * stride] * M[(size_t)(oc * nf + k) * ncols + oe[t] * nt + qt];
            }
            acc *= coef;
            if (accumulate) y[idx] += acc; else y[idx] = acc;
        }
    }
}

/* partial-sum schedule (generate_transform_order): nsum x dim dims and L/full/U tags */
static int fast_schedule(int dim, int dims[][16], int tags[][16]) {
    if (dim == 1) { dims[0][0] = 0; tags[0][0] = 1; return 1; }
    const int nsum = 1 << (dim - 1);
    for (int s = 0; s < nsum; ++s) {
        int tag[16];
        for (int d = 0; d < dim - 1; ++d) tag[d] = 2 * ((s >> (dim - 2 - d)) & 1);
        tag[dim - 1] = 1;
        int n = 0;
        for (int v = 0; v <= 2; ++v)
            for (int d = 0; d < dim; ++d)
                if (tag[d] == v) { dims[s][n] = d; tags[s][n] = v; ++n; }
    }
    return nsum;
}

/* sum over the partial sums of dim successive transforms n_in -> n_out, added into out */
static int fast_partial_sums(const fast_ctx* c, const double* in, int n_in, int n_out, const double* const* M, const int* flx,
                             double coef, double* out) {
    const int dim = c->dim;
    int dims[64][16], tags[64][16];
    const int nsum = fast_schedule(dim, dims, tags);
    int maxb = 1;
    for (int s = 0; s < dim; ++s) maxb *= (n_in > n_out ? n_in : n_out);
    double* ta = (double*)malloc((size_t)c->E * maxb * sizeof(double));
    double* tb = (double*)malloc((size_t)c->E * maxb * sizeof(double));
    if (!ta || !tb) return -2;
    for (int s = 0; s < nsum; ++s) {
        int from[16], to[16];
        for (int d = 0; d < dim; ++d) from[d] = n_in;
        const double* cur = in;
        for (int i = 0; i < dim; ++i) {
            const int t = dims[s][i];
            memcpy(to, from, sizeof(int) * dim);
            to[t] = n_out;
            const int last = (i == dim - 1);
            double* dst = last ? out : (cur == ta ? tb : ta);
            fast_transform_1d(c, cur, from, dst, to, t, M[t], c->n1 * n_out, tags[s][i], flx[t], i == 0 ? coef : 1.0, last);
            cur = dst;
            memcpy(from, to, sizeof(int) * dim);
        }
    }
    free(ta); free(tb);
    return 0;
}

/* Alpert basis (deriv = 0) or its derivative (deriv = 1) at Lagrange points, rows = Alpert basis,
 * cols = Lagrange point (Lag_pt_Alpt_1D / Lag_pt_Alpt_1D_d1, Interplation.cpp:16-101) */
static double* alpt_at_lagr_points_d(int N, int k, int deriv);
static double* alpt_at_lagr_points(int N, int k) { return alpt_at_lagr_points_d(N, k, 0); }
static double* alpt_at_lagr_points_d(int N, int k, int deriv) {
    const int np = k + 1, n1 = 1 << N, na = n1 * np, nl = n1 * LS->p1;
    double* m = (double*)calloc((size_t)na * nl, sizeof(double));
    for (int c = 0; c < nl; ++c) {
        const elem1d el = elem_of_order(c / LS->p1);
        const double x = amdg_oracle_lagr_point(el.n, el.j, c % LS->p1);
        for (int r = 0; r < na; ++r) {
            const elem1d ea = elem_of_order(r / np);
            if (x < support_lo(ea.n, ea.j) || x > support_hi(ea.n, ea.j)) continue;
            m[(size_t)r * nl + c] = amdg_oracle_alpert_val(k, ea.n, ea.j, r % np, deriv, x, 0);
        }
    }
    return m;
}

int amdg_oracle_lagr_point_values_fast(int dim, int N, int k, int64_t E, const int32_t* level, const int32_t* suppt,
                                       const double* u, double* up) {
    fast_ctx c;
    if (fast_ctx_init(&c, dim, N, E, level, suppt)) return -2;
    double* a2p = alpt_at_lagr_points(N, k);
    const double* M[16];
    int flx[16];
    for (int d = 0; d < dim; ++d) { M[d] = a2p; flx[d] = 0; }
    memset(up, 0, (size_t)E * ipow(LS->p1, dim) * sizeof(double));
    int rc = fast_partial_sums(&c, u, k + 1, LS->p1, M, flx, 1.0, up);
    free(a2p);
    fast_ctx_free(&c);
    return rc;
}

/* Lagrange interpolation coefficients to Alpert coefficients: the partial sums of the transform
 * schedule with u_v (Lagrange x Alpert) along every dimension, summed into zeroed coefficients
 * (FastLagrInit::eval_ucoe_Alpt_Lagr, FastMultiplyLU.cpp:1617-1620, and
 * FastInitial::transform_ucoeintp_to_ucoealpt, FastMultiplyLU.cpp:1418-1436) */
int amdg_oracle_lagr_to_alpert_fast(int dim, int N, int k, int64_t E, const int32_t* level, const int32_t* suppt,
                                    const double* coe, double* out) {
    const int np = k + 1, n1 = 1 << N, nr = n1 * LS->p1, nc = n1 * np;
    fast_ctx c;
    if (fast_ctx_init(&c, dim, N, E, level, suppt)) return -2;
    double* Lv = (double*)malloc((size_t)nr * nc * sizeof(double));
    double* Lvx = (double*)malloc((size_t)nr * nc * sizeof(double));
    double* Lf = (double*)malloc((size_t)nr * nc * sizeof(double));
    if (!Lv || !Lvx || !Lf) return -2;
    amdg_oracle_oper1d_lagr(N, k, Lv, Lvx, Lf);
    memset(out, 0, (size_t)E * ipow(np, dim) * sizeof(double));
    const double* M[16];
    int flx[16];
    for (int s = 0; s < dim; ++s) {
        M[s] = Lv;
        flx[s] = 0;
    }
    const int rc = fast_partial_sums(&c, coe, LS->p1, np, M, flx, 1.0, out);
    free(Lv); free(Lvx); free(Lf);
    fast_ctx_free(&c);
    return rc;
}

/* Burgers RHS by the reference's fast transforms (HyperbolicLagrRHS::rhs_vol_scalar,
 * rhs_flx_intp_scalar, HyperbolicAlptRHS::rhs_flx_penalty_scalar) */
int amdg_oracle_burgers_rhs_fast(int dim, int N, int k, int64_t E, const int32_t* level, const int32_t* suppt,
                                 const double* fucoe, const double* u, double alpha, double* rhs) {
    const int np = k + 1, n1 = 1 << N, nr = n1 * LS->p1, nc = n1 * np;
    const int B = ipow(np, dim), P = ipow(LS->p1, dim);
    fast_ctx c;
    if (fast_ctx_init(&c, dim, N, E, level, suppt)) return -2;
    double* Lv = (double*)malloc((size_t)nr * nc * sizeof(double));
    double* Lvx = (double*)malloc((size_t)nr * nc * sizeof(double));
    double* Lf = (double*)malloc((size_t)nr * nc * sizeof(double));
    double* ul = (double*)malloc((size_t)nc * nc * sizeof(double));
    double* ur = (double*)malloc((size_t)nc * nc * sizeof(double));
    if (!Lv || !Lvx || !Lf || !ul || !ur) return -2;
    amdg_oracle_oper1d_lagr(N, k, Lv, Lvx, Lf);
    amdg_oracle_oper1d(N, k, NULL, NULL, ul, ur);
    for (size_t i = 0; i < (size_t)nc * nc; ++i) ur[i] = ur[i] - ul[i]; /* ujp_vjp */
    memset(rhs, 0, (size_t)E * B * sizeof(double));
    int rc = 0;
    for (int d = 0; d < dim && !rc; ++d) {
        for (int term = 0; term < 2 && !rc; ++term) {
            const double* M[16];
            int flx[16];
            for (int s = 0; s < dim; ++s) {
                M[s] = (s == d) ? (term == 0 ? Lvx : Lf) : Lv;
                flx[s] = (term == 1 && s == d);
            }
            rc = fast_partial_sums(&c, fucoe + (size_t)d * E * P, LS->p1, np, M, flx, term == 0 ? 1.0 : 0.5, rhs);
        }
        int from[16];
        for (int s = 0; s < dim; ++s) from[s] = np;
        fast_transform_1d(&c, u, from, rhs, from, d, ur, nc, 1, 1, -alpha / 2.0, 1);
    }
    free(Lv); free(Lvx); free(Lf); free(ul); free(ur);
    fast_ctx_free(&c);
    return rc;
}

/* ------------------------------------------------------------------------ */
/* Point values and quadrature errors against the Burgers exact solution.    */
/* ------------------------------------------------------------------------ */
static void elem_support(int level, int suppt, double* lo, double* hi) {
    if (level <= 1) { *lo = 0.0; *hi = 1.0; return; }
    const double h = ldexp(1.0, 1 - level);
    *lo = h * (suppt - 1) / 2.0;
    *hi = h * (suppt + 1) / 2.0;
}

static double eval_one(int dim, int k, int64_t E, const int32_t* level, const int32_t* suppt, const double* u,
                       const double* x) {
    const int np = k + 1;
    int B = 1;
    for (int d = 0; d < dim; ++d) B *= np;
    double v = 0.0;
    for (int64_t e = 0; e < E; ++e) {
        int inside = 1;
        for (int d = 0; d < dim && inside; ++d) {
            double lo, hi;
            elem_support(level[e * dim + d], suppt[e * dim + d], &lo, &hi);
            if (x[d] < lo || x[d] > hi) inside = 0;
        }
        if (!inside) continue;
        double phi[8][4];
        for (int d = 0; d < dim; ++d)
            for (int p = 0; p < np; ++p) phi[d][p] = amdg_oracle_alpert_val(k, level[e * dim + d], suppt[e * dim + d], p, 0, x[d], 0);
        double ve = 0.0;
        for (int idx = 0; idx < B; ++idx) {
            int pd[8], r = idx;
            for (int d = dim - 1; d >= 0; --d) { pd[d] = r % np; r /= np; }
            double t = u[e * B + idx];
            for (int d = 0; d < dim; ++d) t *= phi[d][pd[d]];
            ve += t;
        }
        v += ve;
    }
    return v;
}

int amdg_oracle_eval_points(int dim, int N, int k, int64_t E, const int32_t* level, const int32_t* suppt,
                            const double* u, int64_t npts, const double* x, double* out) {
    (void)N;
    if (dim < 1 || dim > 8 || k < 0 || k > 3) return -1;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < npts; ++i) out[i] = eval_one(dim, k, E, level, suppt, u, x + i * dim);
    return 0;
}

double amdg_oracle_burgers_wave(double x, double t) {
    const double pi = 3.14159265358979323846;
    double xp = fmod(x, 1.0);
    if (xp < 0) xp = fmod(xp + 1.0, 1.0);
    if (fabs(xp) < ROUND_OFF || fabs(1 - xp) < ROUND_OFF || fabs(xp - 0.5) < ROUND_OFF) return 0.0;
    /* odd symmetry v(x) = -v(1 - x) */
    if (xp < 0.5) return -amdg_oracle_burgers_wave(1 - xp, t);
    /* initial guess: the first characteristic x0 + sin(2 pi x0) t (x0 from 1 down to 0.5) left of xp */
    const int n = 100;
    const double xl = 0.5, xr = 1.0, h = (xr - xl) / n;
    double u = 0.0;
    for (int i = 0; i < n; ++i) {
        const double x0 = xr - i * h;
        const double xT = x0 + sin(2 * pi * x0) * t;
        if (xp > xT) { u = sin(2 * pi * x0); break; }
    }
    /* Newton on f(u) = u - sin(2 pi (xp - u t)) */
    double err = 1.0;
    int iter = 0;
    while (err > ROUND_OFF) {
        const double un = u - (u + sin(2 * pi * (u * t - xp))) / (1 + 2 * pi * t * cos(2 * pi * (u * t - xp)));
        err = fabs(un - u);
        u = un;
        if (++iter > 10) return NAN;
    }
    return u;
}

double amdg_oracle_burgers_exact(int dim, const double* x, double a, double b, double c, double t) {
    double s = 0.0;
    for (int d = 0; d < dim; ++d) s += x[d];
    const double T = dim * t;
    return a + b * amdg_oracle_burgers_wave(s - a * T + c, b * T);
}

int amdg_oracle_error_burgers(int dim, int N, int k, int64_t E, const int32_t* level, const int32_t* suppt,
                              const double* u, int gauss, double a, double b, double c, double t, double* err3) {
    (void)N;
    if (dim < 1 || dim > 8 || gauss < 1 || gauss > 10) return -1;
    int qlev = 0;
    for (int64_t i = 0; i < E * dim; ++i) qlev = level[i] > qlev ? level[i] : qlev;
    const int64_t n = (int64_t)1 << qlev;
    const double h = 1.0 / n;
    double gx[16], gw[16];
    amdg_oracle_gauss_legendre(gauss, gx, gw);
    int64_t cells = 1, qn = 1;
    for (int d = 0; d < dim; ++d) { cells *= n; qn *= gauss; }
    double l1 = 0.0, l2 = 0.0, linf = 0.0;
    int bad = 0;
#pragma omp parallel for schedule(static) reduction(+ : l1, l2, bad) reduction(max : linf)
    for (int64_t cell = 0; cell < cells; ++cell) {
        int64_t ci[8], r = cell;
        for (int d = dim - 1; d >= 0; --d) { ci[d] = r % n; r /= n; }
        for (int64_t q = 0; q < qn; ++q) {
            double x[8], w = 1.0;
            int64_t rq = q;
            for (int d = dim - 1; d >= 0; --d) {
                const int qd = (int)(rq % gauss);
                rq /= gauss;
                const double tl = ci[d] * h, tr = (ci[d] + 1) * h;
                x[d] = tl + (gx[qd] + 1.0) * 0.5 * (tr - tl);
                w *= gw[qd];
            }
            const double ex = amdg_oracle_burgers_exact(dim, x, a, b, c, t);
            if (isnan(ex)) bad += 1;
            const double f = fabs(eval_one(dim, k, E, level, suppt, u, x) - ex);
            l1 += w * f;
            l2 += w * f * f;
            if (f > linf) linf = f;
        }
    }
    if (bad) return -2;
    const double s = pow(h / 2.0, dim);
    err3[0] = l1 * s;
    err3[1] = sqrt(l2 * s);
    err3[2] = linf;
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Wave equation u_tt = div(K(x) grad u), K = (1 + a prod_d sin(2 pi x_d))^2,    */
/* periodic: DiffusionRHS with Lagrange-interpolated K u_x and K u            */
/* (03_wave_06_var_coeff_adapt.cpp:154-245; Interplation.cpp:527-577,         */
/* 648-698, 4159-4212; FastMultiplyLU.cpp:1691-1765) plus the IPDG jump        */
/* penalty -sigma/dx [u][v] (BilinearForm.cpp:920-929).                       */
/* ------------------------------------------------------------------------ */

/* sum over the discontinuity points of u (lo, mid, hi of u's support; 0 and 1/2 at levels
 * 0 and 1, periodic) of u(x^su) v'(x^sv) (Basis::product_edge_dis_u, Basis.cpp:175-230) */
static double gproduct_edge_dis_u(int tu, int tv, int k, elem1d u, int pu, elem1d v, int pv, int su, int sv, int dv) {
    const double pts[3] = {support_lo(u.n, u.j), 0.5 * (support_lo(u.n, u.j) + support_hi(u.n, u.j)), support_hi(u.n, u.j)};
    double s = 0.0;
    for (int i = 0; i < 3; ++i) {
        if (u.n <= 1 && i == 2) continue;
        const double x = pts[i];
        double fu = basis_val(tu, k, u.n, u.j, pu, 0, x, su), fv = basis_val(tv, k, v.n, v.j, pv, dv, x, sv);
        if (fabs(x) < ROUND_OFF) {
            if (su == -1) fu = basis_val(tu, k, u.n, u.j, pu, 0, 1.0, su);
            if (sv == -1) fv = basis_val(tv, k, v.n, v.j, pv, dv, 1.0, sv);
        } else if (fabs(x - 1.0) < ROUND_OFF) {
            if (su == 1) fu = basis_val(tu, k, u.n, u.j, pu, 0, 0.0, su);
            if (sv == 1) fv = basis_val(tv, k, v.n, v.j, pv, dv, 0.0, sv);
        }
        s += fu * fv;
    }
    return s;
}

/* Lagrange (rows) x Alpert (cols): ujp_vxlft + ujp_vxrgt, [u] times the one-sided v_x
 * (OperatorMatrix1D.h:206-211) */
int amdg_oracle_oper1d_lagr_ujp_vx(int N, int k, double* ujp_vxave) {
    const int nr = (1 << N) * LS->p1, nc = (1 << N) * (k + 1);
#pragma omp parallel for schedule(dynamic)
    for (int r = 0; r < nr; ++r) {
        const elem1d u = elem_of_order(r / LS->p1);
        const int pu = r % LS->p1;
        for (int c = 0; c < nc; ++c) {
            const elem1d v = elem_of_order(c / (k + 1));
            const int pv = c % (k + 1);
            const double ur_vxr = gproduct_edge_dis_u(1, 0, k, u, pu, v, pv, 1, 1, 1);
            const double ul_vxr = gproduct_edge_dis_u(1, 0, k, u, pu, v, pv, -1, 1, 1);
            const double ur_vxl = gproduct_edge_dis_u(1, 0, k, u, pu, v, pv, 1, -1, 1);
            const double ul_vxl = gproduct_edge_dis_u(1, 0, k, u, pu, v, pv, -1, -1, 1);
            const double lft = ur_vxl - ul_vxl, rgt = ur_vxr - ul_vxr;
            ujp_vxave[(size_t)r * nc + c] = lft + rgt;
        }
    }
    return 0;
}

double amdg_oracle_wave_coef(int dim, const double* x, double amp) {
    const double pi = 3.14159265358979323846;
    double s = 1.0;
    for (int d = 0; d < dim; ++d) s *= sin(2 * pi * x[d]);
    const double c = 1.0 + amp * s;
    return c * c;
}

/* K at every interpolation point times the given point values, then the surplus */
static int wave_coef_surplus(int dim, int N, int64_t E, const int32_t* level, const int32_t* suppt, double amp, double* up,
                             double* fucoe) {
    const int P = ipow(LS->p1, dim);
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < E; ++e)
        for (int p = 0; p < P; ++p) {
            double x[16];
            int r = p;
            for (int d = dim - 1; d >= 0; --d) {
                x[d] = amdg_oracle_lagr_point(level[e * dim + d], suppt[e * dim + d], r % LS->p1);
                r /= LS->p1;
            }
            up[e * P + p] = amdg_oracle_wave_coef(dim, x, amp) * up[e * P + p];
        }
    return amdg_oracle_lagr_surplus(dim, N, E, level, suppt, up, fucoe);
}

int amdg_oracle_wave_rhs_fast(int dim, int N, int k, int64_t E, const int32_t* level, const int32_t* suppt,
                              const double* u, double sigma, double amp, double* rhs) {
    const int np = k + 1, n1 = 1 << N, nr = n1 * LS->p1, nc = n1 * np;
    const int B = ipow(np, dim), P = ipow(LS->p1, dim);
    fast_ctx c;
    if (fast_ctx_init(&c, dim, N, E, level, suppt)) return -2;
    double* a2p = alpt_at_lagr_points_d(N, k, 0);
    double* a2pd = alpt_at_lagr_points_d(N, k, 1);
    double* Lv = (double*)malloc((size_t)nr * nc * sizeof(double));
    double* Lvx = (double*)malloc((size_t)nr * nc * sizeof(double));
    double* Lf = (double*)malloc((size_t)nr * nc * sizeof(double));
    double* Lj = (double*)malloc((size_t)nr * nc * sizeof(double));
    double* ul = (double*)malloc((size_t)nc * nc * sizeof(double));
    double* ur = (double*)malloc((size_t)nc * nc * sizeof(double));
    double* up = (double*)malloc((size_t)E * P * sizeof(double));
    double* fg = (double*)malloc((size_t)dim * E * P * sizeof(double));
    double* fu = (double*)malloc((size_t)E * P * sizeof(double));
    if (!a2p || !a2pd || !Lv || !Lvx || !Lf || !Lj || !ul || !ur || !up || !fg || !fu) return -2;
    amdg_oracle_oper1d_lagr(N, k, Lv, Lvx, Lf);
    amdg_oracle_oper1d_lagr_ujp_vx(N, k, Lj);
    amdg_oracle_oper1d(N, k, NULL, NULL, ul, ur);
    for (size_t i = 0; i < (size_t)nc * nc; ++i) ur[i] = ur[i] - ul[i]; /* ujp_vjp */
    int rc = 0;
    const double* M[16] = {0};
    int flx[16] = {0};
    /* K u_{x_d} at the points and its interpolation coefficients, per d */
    for (int d = 0; d < dim && !rc; ++d) {
        for (int s = 0; s < dim; ++s) { M[s] = (s == d) ? a2pd : a2p; flx[s] = 0; }
        memset(up, 0, (size_t)E * P * sizeof(double));
        rc = fast_partial_sums(&c, u, np, LS->p1, M, flx, 1.0, up);
        if (!rc) rc = wave_coef_surplus(dim, N, E, level, suppt, amp, up, fg + (size_t)d * E * P);
    }
    /* K u at the points */
    if (!rc) {
        for (int s = 0; s < dim; ++s) { M[s] = a2p; flx[s] = 0; }
        memset(up, 0, (size_t)E * P * sizeof(double));
        rc = fast_partial_sums(&c, u, np, LS->p1, M, flx, 1.0, up);
        if (!rc) rc = wave_coef_surplus(dim, N, E, level, suppt, amp, up, fu);
    }
    memset(rhs, 0, (size_t)E * B * sizeof(double));
    /* rhs_flx_gradu: -{K u_x}[v] (uave_vjp = (ulft + urgt)_vjp / 2) */
    for (int d = 0; d < dim && !rc; ++d) {
        for (int s = 0; s < dim; ++s) { M[s] = (s == d) ? Lf : Lv; flx[s] = (s == d); }
        rc = fast_partial_sums(&c, fg + (size_t)d * E * P, LS->p1, np, M, flx, -0.5, rhs);
    }
    /* rhs_vol: -K u_x v_x */
    for (int d = 0; d < dim && !rc; ++d) {
        for (int s = 0; s < dim; ++s) { M[s] = (s == d) ? Lvx : Lv; flx[s] = 0; }
        rc = fast_partial_sums(&c, fg + (size_t)d * E * P, LS->p1, np, M, flx, -1.0, rhs);
    }
    /* rhs_flx_u: -1/2 [K u] (v_x^- + v_x^+) */
    for (int d = 0; d < dim && !rc; ++d) {
        for (int s = 0; s < dim; ++s) { M[s] = (s == d) ? Lj : Lv; flx[s] = (s == d); }
        rc = fast_partial_sums(&c, fu, LS->p1, np, M, flx, -0.5, rhs);
    }
    /* IPDG: -sigma/dx [u][v], dx the finest element size */
    int maxl = 0;
    for (int64_t i = 0; i < E * dim; ++i) maxl = level[i] > maxl ? level[i] : maxl;
    const double dx = 1.0 / pow(2.0, maxl);
    for (int d = 0; d < dim && !rc; ++d) {
        int from[16];
        for (int s = 0; s < dim; ++s) from[s] = np;
        fast_transform_1d(&c, u, from, rhs, from, d, ur, nc, 1, 1, -sigma / dx, 1);
    }
    free(a2p); free(a2pd); free(Lv); free(Lvx); free(Lf); free(Lj); free(ul); free(ur); free(up); free(fg); free(fu);
    fast_ctx_free(&c);
    return rc;
}

/* The IPDG term alone, rhs = -sigma/dx sum_d [u][v]: what EulerODE2nd::step_rk_source uses as
 * the predictor's right-hand side (it recomputes rhs as the operator matrix times u,
 * ODESolver.cpp:402-407, BilinearForm.h:23). */
int amdg_oracle_wave_penalty(int dim, int N, int k, int64_t E, const int32_t* level, const int32_t* suppt,
                             const double* u, double sigma, double* rhs) {
    const int np = k + 1, nc = (1 << N) * np, B = ipow(np, dim);
    fast_ctx c;
    if (fast_ctx_init(&c, dim, N, E, level, suppt)) return -2;
    double* ul = (double*)malloc((size_t)nc * nc * sizeof(double));
    double* ur = (double*)malloc((size_t)nc * nc * sizeof(double));
    if (!ul || !ur) return -2;
    amdg_oracle_oper1d(N, k, NULL, NULL, ul, ur);
    for (size_t i = 0; i < (size_t)nc * nc; ++i) ur[i] = ur[i] - ul[i]; /* ujp_vjp */
    int maxl = 0;
    for (int64_t i = 0; i < E * dim; ++i) maxl = level[i] > maxl ? level[i] : maxl;
    const double dx = 1.0 / pow(2.0, maxl);
    memset(rhs, 0, (size_t)E * B * sizeof(double));
    for (int d = 0; d < dim; ++d) {
        int from[16];
        for (int s = 0; s < dim; ++s) from[s] = np;
        fast_transform_1d(&c, u, from, rhs, from, d, ur, nc, 1, 1, -sigma / dx, 1);
    }
    free(ul); free(ur);
    fast_ctx_free(&c);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Cubic Hermite interpolation of the flux (HermBasis with PMAX 3 and        */
/* msh_case 1, HermInterpolation::nonlinear_Herm_2D_fast,                    */
/* Interplation.cpp:4609-4621; the 2D Burgers driver                         */
/* example/02_hyperbolic_05_burgers_adapt.cpp).  A 1D element carries four   */
/* degrees of freedom pp: point pp % 2 and derivative order pp / 2           */
/* (HermBasis::deg_pt_deri_1d, HermBasis.cpp).                               */
/* ------------------------------------------------------------------------ */

/* Mother functions on [0, 1] and their first derivatives (HermBasis::phi_P1_L1 and its
 * derivative).  Level 0 interpolates value and slope at x = 0 (point 0) and x = 1 (point 1);
 * level 1 at the midpoint, the point-0 pair supported on [0, 1/2] and the point-1 pair on
 * [1/2, 1], both vanishing with their slope at the far end. */
static double herm_mother(double x, int msh, int pp, int deriv) {
    if (x < 0.0 || x > 1.0) return 0.0;
    const int pt = pp % 2, l = pp / 2;
    if (msh == 0) {
        if (pt == 0) {
            if (l == 0) return deriv ? 6.0 * x * (x - 1.0) : (x - 1.0) * (x - 1.0) * (1.0 + 2.0 * x);
            return deriv ? (1.0 - x) * (1.0 - 3.0 * x) : (1.0 - x) * (1.0 - x) * x;
        }
        if (l == 0) return deriv ? 6.0 * x * (1.0 - x) : x * x * (3.0 - 2.0 * x);
        return deriv ? x * (3.0 * x - 2.0) : (x - 1.0) * x * x;
    }
    if (pt == 0) {
        if (x > 0.5) return 0.0;
        if (l == 0) return deriv ? 24.0 * x * (1.0 - 2.0 * x) : 4.0 * x * x * (3.0 - 4.0 * x);
        return deriv ? 4.0 * x * (3.0 * x - 1.0) : 2.0 * x * x * (2.0 * x - 1.0);
    }
    if (x < 0.5) return 0.0;
    if (l == 0) return deriv ? 24.0 * (x - 1.0) * (2.0 * x - 1.0) : 4.0 * (x - 1.0) * (x - 1.0) * (4.0 * x - 1.0);
    return deriv ? 4.0 * (x - 1.0) * (3.0 * x - 2.0) : 2.0 * (x - 1.0) * (x - 1.0) * (2.0 * x - 1.0);
}

/* HermBasis::val (HermBasis.cpp): levels >= 2 are the level-1 pair mapped onto the support, a
 * slope dof scaled by the support width (2^-(n-1) per derivative order of the dof, 2^(n-1) per
 * derivative taken); the one-sided limits of Basis::val. */
double amdg_oracle_herm_val(int level, int suppt, int p, int deriv, double x, int sgn) {
    double xl = x;
    if (sgn == -1) {
        if (fabs(x) <= ROUND_OFF) return 0.0;
        xl -= ROUND_OFF;
    } else if (sgn == 1) {
        if (fabs(x - 1.0) <= ROUND_OFF) return 0.0;
        xl += ROUND_OFF;
    }
    if (level <= 1) return herm_mother(xl, level, p, deriv);
    const double xt = pow(2.0, level - 1) * xl - (suppt - 1) / 2;
    return herm_mother(xt, 1, p, deriv) * pow(2.0, -(level - 1) * (p / 2 - deriv));
}

/* interpolation point of dof p of 1D element (n, j) (HermBasis::set_interp_msh01 and the
 * HermBasis constructor): level 0 the two end points moved 1e-13 inside, in [-1, 1] coordinates
 * mapped by (x + 1) / 2; level >= 1 the two sides of the midpoint */
double amdg_oracle_herm_point(int level, int suppt, int p) {
    if (level == 0) return ((p % 2 == 0 ? (-1.0 + ROUND_OFF) : (1.0 - ROUND_OFF)) + 1.0) / 2.0;
    const double m = ((p % 2 == 0 ? (0.0 - ROUND_OFF) : (0.0 + ROUND_OFF)) + 1.0) / 2.0;
    const double a = support_lo(level, suppt), b = support_hi(level, suppt);
    return a + (b - a) * m;
}

/* Hermite (rows, 2^N x 4) x Alpert (cols, 2^N x (k+1)) 1D matrices of
 * OperatorMatrix1D<HermBasis, AlptBasis> (OperatorMatrix1D.h:166-199): u_v, u_vx and
 * (ulft_vjp + urgt_vjp) */
int amdg_oracle_oper1d_herm(int N, int k, double* u_v, double* u_vx, double* uave2_vjp) {
    const int nr = (1 << N) * 4, nc = (1 << N) * (k + 1);
#pragma omp parallel for schedule(dynamic)
    for (int r = 0; r < nr; ++r) {
        const elem1d u = elem_of_order(r / 4);
        const int pu = r % 4;
        for (int c = 0; c < nc; ++c) {
            const elem1d v = elem_of_order(c / (k + 1));
            const int pv = c % (k + 1);
            const size_t idx = (size_t)r * nc + c;
            if (u_v) u_v[idx] = gproduct_volume(2, 0, k, u, pu, v, pv, 0, 0);
            if (u_vx) u_vx[idx] = gproduct_volume(2, 0, k, u, pu, v, pv, 0, 1);
            if (uave2_vjp) {
                const double l = gproduct_edge(2, 0, k, u, pu, v, pv, -1, 1) - gproduct_edge(2, 0, k, u, pu, v, pv, -1, -1);
                const double rr = gproduct_edge(2, 0, k, u, pu, v, pv, 1, 1) - gproduct_edge(2, 0, k, u, pu, v, pv, 1, -1);
                uave2_vjp[idx] = l + rr;
            }
        }
    }
    return 0;
}

/* Alpert basis at the Hermite points, rows = Alpert basis, cols = Hermite dof: the value for a
 * value dof, the first derivative for a slope dof, zero where the point lies outside the
 * support (HermInterpolation::eval_Her_pt_at_Alpt_1D, Interplation.cpp:1886-1975, transposed as
 * FastHermIntp's alpt_basis_herm_pt, FastMultiplyLU.cpp:1316-1331) */
static double* alpt_at_herm_points(int N, int k) {
    const int np = k + 1, n1 = 1 << N, na = n1 * np, nh = n1 * 4;
    double* m = (double*)calloc((size_t)na * nh, sizeof(double));
    if (!m) return NULL;
    for (int c = 0; c < nh; ++c) {
        const elem1d eh = elem_of_order(c / 4);
        const double x = amdg_oracle_herm_point(eh.n, eh.j, c % 4);
        for (int r = 0; r < na; ++r) {
            const elem1d ea = elem_of_order(r / np);
            if (x < support_lo(ea.n, ea.j) || x > support_hi(ea.n, ea.j)) continue;
            m[(size_t)r * nh + c] = amdg_oracle_alpert_val(k, ea.n, ea.j, r % np, (c % 4) / 2, x, 0);
        }
    }
    return m;
}

/* u_h and its derivatives at the Hermite points of every element, summed directly over all
 * elements whose support holds the point: up[e][p], 4^dim per element, entry p the mixed
 * derivative of u_h given by the slope dofs of p (FastHermIntp::eval_up_Herm's quantity) */
int amdg_oracle_herm_point_values(int dim, int N, int k, int64_t E, const int32_t* level, const int32_t* suppt,
                                  const double* u, double* up) {
    ehash h;
    if (ehash_build(&h, dim, N, E, level, suppt)) return -2;
    const int np = k + 1, B = ipow(np, dim), P = ipow(4, dim);
#pragma omp parallel for schedule(dynamic, 8)
    for (int64_t e = 0; e < E; ++e) {
        for (int p = 0; p < P; ++p) {
            double x[16];
            int pd[16], rem = p;
            for (int d = dim - 1; d >= 0; --d) { pd[d] = rem % 4; rem /= 4; }
            for (int d = 0; d < dim; ++d) x[d] = amdg_oracle_herm_point(level[e * dim + d], suppt[e * dim + d], pd[d]);
            double val = 0.0;
            int lv[16] = {0};
            for (;;) {
                int o[16];
                for (int d = 0; d < dim; ++d) o[d] = order_containing(lv[d], x[d]);
                const int64_t s = ehash_find(&h, pack_key(o, dim, N));
                if (s >= 0) {
                    double phi[16][4];
                    for (int d = 0; d < dim; ++d) {
                        const elem1d ed = elem_of_order(o[d]);
                        for (int q = 0; q < np; ++q) phi[d][q] = amdg_oracle_alpert_val(k, ed.n, ed.j, q, pd[d] / 2, x[d], 0);
                    }
                    for (int q = 0; q < B; ++q) {
                        int r2 = q, qd[16];
                        double w = 1.0;
                        for (int d = dim - 1; d >= 0; --d) { qd[d] = r2 % np; r2 /= np; }
                        for (int d = 0; d < dim; ++d) w *= phi[d][qd[d]];
                        val += w * u[s * B + q];
                    }
                }
                int d = dim - 1;
                while (d >= 0) {
                    if (++lv[d] <= N) break;
                    lv[d] = 0;
                    --d;
                }
                if (d < 0) break;
            }
            up[e * P + p] = val;
        }
    }
    ehash_free(&h);
    return 0;
}

/* the same quantity by the reference's fast transforms (FastHermIntp::eval_up_Herm ->
 * transform_ucoealpt_to_upintp, FastMultiplyLU.cpp:1333-1336) */
int amdg_oracle_herm_point_values_fast(int dim, int N, int k, int64_t E, const int32_t* level, const int32_t* suppt,
                                       const double* u, double* up) {
    fast_ctx c;
    if (fast_ctx_init(&c, dim, N, E, level, suppt)) return -2;
    double* a2h = alpt_at_herm_points(N, k);
    if (!a2h) return -2;
    const double* M[16];
    int flx[16];
    for (int d = 0; d < dim; ++d) { M[d] = a2h; flx[d] = 0; }
    memset(up, 0, (size_t)E * ipow(4, dim) * sizeof(double));
    const int rc = fast_partial_sums(&c, u, k + 1, 4, M, flx, 1.0, up);
    free(a2h);
    fast_ctx_free(&c);
    return rc;
}

/* The Burgers flux f = u^2/2 and its derivatives at the 2D Hermite points, from u_h and its
 * derivatives there (HermInterpolation::eval_fp_Her_2D, Interplation.cpp:2045-2300, with
 * f' = u and f'' = 1, FluxFunction::burgers_flux_*, Interplation.cpp:5070-5083): f for a value
 * dof pair, f' u_x or f' u_y for one slope dof, f'' u_x u_y + f' u_xy for two; the same operation
 * order. */
int amdg_oracle_herm_flux_burgers2d(int64_t E, const double* up, double* fp) {
    for (int64_t e = 0; e < E; ++e) {
        const double* v = up + e * 16;
        double* f = fp + e * 16;
        for (int p0 = 0; p0 < 4; ++p0)
            for (int p1 = 0; p1 < 4; ++p1) {
                const int kx = p0 / 2, ky = p1 / 2, i = p0 * 4 + p1;
                if (!kx && !ky) {
                    f[i] = v[i] * v[i] * 0.5;
                } else if (kx && !ky) {
                    f[i] = 0.0 + v[(p0 - 2) * 4 + p1] * v[i];
                } else if (!kx && ky) {
                    f[i] = 0.0 + v[p0 * 4 + p1 - 2] * v[i];
                } else {
                    const double uu = v[(p0 - 2) * 4 + p1 - 2], ux = v[p0 * 4 + p1 - 2], uy = v[(p0 - 2) * 4 + p1];
                    double a = 0.0;
                    a += 1.0 * ux * uy;
                    a += uu * v[i];
                    f[i] = a;
                }
            }
    }
    return 0;
}

/* Hierarchical Hermite surplus, dimension by dimension (HermInterpolation::eval_fp_to_coe_D_Her,
 * Interplation.cpp:3651-3849, weights of set_pts_wts_1d_ada_Her, :3166-3316): in pass d every
 * element with level_d = l > 0 subtracts the cubic Hermite interpolant through the four coarser
 * dofs inside its dimension-d support (the two end points, value and slope each): ancestor ic
 * (found in the order of coarser levels, elements, dofs) is numbered ic0 = 0, 2 at the smaller
 * position and 1, 3 at the larger one, and dof p0 = (point, order l1) of the element adds
 * -2^((l-1)(l1 - l2)) H0_ic0^(l1)(x_p0) times the ancestor's value, l2 = ic0 / 2, H0 the level-0
 * Hermite functions on [0, 1] and x_p0 the dof's point in the element's [0, 1] coordinates. */
int amdg_oracle_herm_surplus(int dim, int N, int64_t E, const int32_t* level, const int32_t* suppt, const double* fp,
                             double* out) {
    ehash h;
    if (ehash_build(&h, dim, N, E, level, suppt)) return -2;
    const int P = ipow(4, dim);
    double* cur = (double*)malloc((size_t)E * P * sizeof(double));
    double* nxt = (double*)malloc((size_t)E * P * sizeof(double));
    if (!cur || !nxt) return -2;
    memcpy(cur, fp, (size_t)E * P * sizeof(double));
    for (int d = 0; d < dim; ++d) {
        int stride = 1;
        for (int s = d + 1; s < dim; ++s) stride *= 4;
#pragma omp parallel for schedule(dynamic, 8)
        for (int64_t e = 0; e < E; ++e) {
            const int l = level[e * dim + d], j = suppt[e * dim + d];
            if (l == 0) {
                memcpy(nxt + e * P, cur + e * P, P * sizeof(double));
                continue;
            }
            const double xl = support_lo(l, j), xr = support_hi(l, j);
            int anc_o[4], anc_q[4], ic = 0;
            double anc_x[4];
            for (int o = 0; o < (1 << l) && ic < 4; ++o) {
                const elem1d ea = elem_of_order(o);
                if (ea.n >= l) break;
                for (int q = 0; q < 4; ++q) {
                    const double pos = amdg_oracle_herm_point(ea.n, ea.j, q);
                    if (pos > xl && pos < xr && ic < 4) {
                        anc_o[ic] = o;
                        anc_q[ic] = q;
                        anc_x[ic] = pos;
                        ++ic;
                    }
                }
            }
            if (ic != 4) continue;
            double pl = anc_x[0];
            for (int a = 1; a < 4; ++a) pl = anc_x[a] < pl ? anc_x[a] : pl;
            int ic0[4], nl = 0, nr = 1;
            for (int a = 0; a < 4; ++a) {
                if (fabs(anc_x[a] - pl) < 1.0e-14) { ic0[a] = nl; nl += 2; }
                else { ic0[a] = nr; nr += 2; }
            }
            int64_t anc_e[4];
            int missing = 0;
            for (int a = 0; a < 4 && !missing; ++a) {
                int o[16];
                for (int s = 0; s < dim; ++s) o[s] = order_of_elem(level[e * dim + s], suppt[e * dim + s]);
                o[d] = anc_o[a];
                anc_e[a] = ehash_find(&h, pack_key(o, dim, N));
                missing |= anc_e[a] < 0;
            }
            if (missing) continue;
            double wt[4][4];
            for (int p0 = 0; p0 < 4; ++p0) {
                const int l1 = p0 / 2;
                const double xt = ((p0 % 2 == 0 ? (0.0 - ROUND_OFF) : (0.0 + ROUND_OFF)) + 1.0) / 2.0;
                for (int a = 0; a < 4; ++a) {
                    const int l2 = ic0[a] / 2;
                    wt[p0][a] = -1.0 * pow(2.0, (l - 1) * (l1 - l2)) * herm_mother(xt, 0, ic0[a], l1);
                }
            }
            for (int p = 0; p < P; ++p) {
                const int pd = (p / stride) % 4, base = p - pd * stride;
                double c = cur[e * P + p];
                for (int a = 0; a < 4; ++a) c += wt[pd][a] * cur[anc_e[a] * P + base + anc_q[a] * stride];
                nxt[e * P + p] = c;
            }
        }
        double* t = cur; cur = nxt; nxt = t;
    }
    memcpy(out, cur, (size_t)E * P * sizeof(double));
    free(cur); free(nxt);
    ehash_free(&h);
    return 0;
}

/* Burgers right-hand side from the Hermite coefficients of the flux (E x 4^dim, the same flux
 * in every dimension) by the fast transforms, in the reference's order:
 * HyperbolicSameFluxHermRHS::rhs_vol_scalar (u_vx along d, u_v elsewhere, every d), then
 * rhs_flx_intp_scalar (1/2 (ulft + urgt)_vjp along d on the flux sets, every d)
 * (FastMultiplyLU.cpp:970-1016), then the LxF penalty -alpha/2 ujp_vjp along every d (the
 * driver's assembled HyperbolicAlpt::assemble_matrix_flx_scalar(d, -1, alpha/2) and
 * (d, 1, -alpha/2), BilinearForm.cpp:759-769) */
int amdg_oracle_burgers_herm_rhs_fast(int dim, int N, int k, int64_t E, const int32_t* level, const int32_t* suppt,
                                      const double* fucoe, const double* u, double alpha, double* rhs) {
    const int np = k + 1, n1 = 1 << N, nr = n1 * 4, nc = n1 * np;
    fast_ctx c;
    if (fast_ctx_init(&c, dim, N, E, level, suppt)) return -2;
    double* Hv = (double*)malloc((size_t)nr * nc * sizeof(double));
    double* Hvx = (double*)malloc((size_t)nr * nc * sizeof(double));
    double* Hf = (double*)malloc((size_t)nr * nc * sizeof(double));
    double* ul = (double*)malloc((size_t)nc * nc * sizeof(double));
    double* ur = (double*)malloc((size_t)nc * nc * sizeof(double));
    if (!Hv || !Hvx || !Hf || !ul || !ur) return -2;
    amdg_oracle_oper1d_herm(N, k, Hv, Hvx, Hf);
    amdg_oracle_oper1d(N, k, NULL, NULL, ul, ur);
    for (size_t i = 0; i < (size_t)nc * nc; ++i) ur[i] = ur[i] - ul[i]; /* ujp_vjp */
    memset(rhs, 0, (size_t)E * ipow(np, dim) * sizeof(double));
    int rc = 0;
    for (int term = 0; term < 2 && !rc; ++term)
        for (int d = 0; d < dim && !rc; ++d) {
            const double* M[16];
            int flx[16];
            for (int s = 0; s < dim; ++s) {
                M[s] = (s == d) ? (term == 0 ? Hvx : Hf) : Hv;
                flx[s] = (term == 1 && s == d);
            }
            rc = fast_partial_sums(&c, fucoe, 4, np, M, flx, term == 0 ? 1.0 : 0.5, rhs);
        }
    for (int d = 0; d < dim && !rc; ++d) {
        int from[16];
        for (int s = 0; s < dim; ++s) from[s] = np;
        fast_transform_1d(&c, u, from, rhs, from, d, ur, nc, 1, 1, -alpha / 2.0, 1);
    }
    free(Hv); free(Hvx); free(Hf); free(ul); free(ur);
    fast_ctx_free(&c);
    return rc;
}
