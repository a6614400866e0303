"""ctypes front end of the CPU oracle (oracle/amdg_oracle.c).

Test infrastructure only: imported by tests/, __graft_entry__.smoke() and
bench.py's cpu_baseline leg as the checker, never by the product path.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "libamdg_oracle.so")

_FN1D = C.CFUNCTYPE(C.c_double, C.c_double, C.c_int, C.c_int, C.c_void_p)
_lib = None


def build() -> str:
    """Compile the C restatement into oracle/_ref/libamdg_oracle.so."""
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
        f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
        L.amdg_oracle_alpert_val.restype = C.c_double
        L.amdg_oracle_alpert_val.argtypes = [C.c_int] * 6 + [C.c_double, C.c_int]
        L.amdg_oracle_alpert_val.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int]
        L.amdg_oracle_gauss_legendre.argtypes = [C.c_int, f64p, f64p]
        L.amdg_oracle_oper1d.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.amdg_oracle_grid_count.restype = C.c_int64
        L.amdg_oracle_grid_count.argtypes = [C.c_int, C.c_int, C.c_int]
        L.amdg_oracle_grid.restype = C.c_int64
        L.amdg_oracle_grid.argtypes = [C.c_int, C.c_int, C.c_int, i32p, i32p]
        L.amdg_oracle_project_separable.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _FN1D, C.c_void_p, f64p]
        L.amdg_oracle_init_separable.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int64, i32p, i32p, C.c_int, f64p, f64p]
        L.amdg_oracle_linear_rhs.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int64, i32p, i32p, f64p, f64p, f64p, C.c_int]
        L.amdg_oracle_linear_rhs_range.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int64, i32p, i32p, f64p, f64p, f64p,
                                                   C.c_int64, C.c_int64, C.c_int]
        L.amdg_oracle_linear_rk3.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int64, i32p, i32p, f64p, C.c_double, C.c_int,
                                             f64p, C.c_int]
        L.amdg_oracle_linop_create.restype = C.c_void_p
        L.amdg_oracle_linop_create.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int64, i32p, i32p, f64p]
        L.amdg_oracle_linop_apply_range.argtypes = [C.c_void_p, f64p, f64p, C.c_int64, C.c_int64, C.c_int]
        L.amdg_oracle_linop_destroy.argtypes = [C.c_void_p]
        L.amdg_oracle_l2_error_split.restype = C.c_double
        L.amdg_oracle_l2_error_split.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int64, i32p, i32p, f64p, f64p, C.c_double]
        L.amdg_oracle_set_lagr_degree.argtypes = [C.c_int]
        L.amdg_oracle_lagr_val.restype = C.c_double
        L.amdg_oracle_lagr_val.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_int]
        L.amdg_oracle_lagr_point.restype = C.c_double
        L.amdg_oracle_lagr_point.argtypes = [C.c_int, C.c_int, C.c_int]
        L.amdg_oracle_oper1d_lagr.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        L.amdg_oracle_lagr_point_values.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int64, i32p, i32p, f64p, f64p]
        L.amdg_oracle_lagr_surplus.argtypes = [C.c_int, C.c_int, C.c_int64, i32p, i32p, f64p, f64p]
        L.amdg_oracle_lagr_to_alpert_fast.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int64, i32p, i32p, f64p, f64p]
        L.amdg_oracle_burgers_rhs.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int64, i32p, i32p, f64p, f64p, C.c_double,
                                              f64p]
        L.amdg_oracle_lagr_point_values_fast.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int64, i32p, i32p, f64p, f64p]
        L.amdg_oracle_burgers_rhs_fast.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int64, i32p, i32p, f64p, f64p,
                                                   C.c_double, f64p]
        L.amdg_oracle_eval_points.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int64, i32p, i32p, f64p, C.c_int64, f64p,
                                              f64p]
        L.amdg_oracle_burgers_wave.restype = C.c_double
        L.amdg_oracle_burgers_wave.argtypes = [C.c_double, C.c_double]
        L.amdg_oracle_burgers_exact.restype = C.c_double
        L.amdg_oracle_burgers_exact.argtypes = [C.c_int, f64p, C.c_double, C.c_double, C.c_double, C.c_double]
        L.amdg_oracle_error_burgers.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int64, i32p, i32p, f64p, C.c_int,
                                                C.c_double, C.c_double, C.c_double, C.c_double, f64p]
        L.amdg_oracle_wave_rhs_fast.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int64, i32p, i32p, f64p, C.c_double,
                                                C.c_double, f64p]
        L.amdg_oracle_wave_penalty.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int64, i32p, i32p, f64p, C.c_double, f64p]
        L.amdg_oracle_wave_coef.restype = C.c_double
        L.amdg_oracle_wave_coef.argtypes = [C.c_int, f64p, C.c_double]
        L.amdg_oracle_herm_val.restype = C.c_double
        L.amdg_oracle_herm_val.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int]
        L.amdg_oracle_herm_point.restype = C.c_double
        L.amdg_oracle_herm_point.argtypes = [C.c_int, C.c_int, C.c_int]
        L.amdg_oracle_oper1d_herm.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        for fn in ("amdg_oracle_herm_point_values", "amdg_oracle_herm_point_values_fast"):
            getattr(L, fn).argtypes = [C.c_int, C.c_int, C.c_int, C.c_int64, i32p, i32p, f64p, f64p]
        L.amdg_oracle_herm_flux_burgers2d.argtypes = [C.c_int64, f64p, f64p]
        L.amdg_oracle_herm_surplus.argtypes = [C.c_int, C.c_int, C.c_int64, i32p, i32p, f64p, f64p]
        L.amdg_oracle_burgers_herm_rhs_fast.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int64, i32p, i32p, f64p, f64p,
                                                        C.c_double, f64p]
        _lib = L
    return _lib


def _check(rc):
    if rc != 0:
        raise RuntimeError(f"oracle call failed: {rc}")


def alpert_val(k, level, suppt, p, deriv, x, sgn=0):
    return lib().amdg_oracle_alpert_val(k, level, suppt, p, deriv, float(x), sgn)


def gauss_legendre(n):
    x = np.zeros(n)
    w = np.zeros(n)
    _check(lib().amdg_oracle_gauss_legendre(n, x, w))
    return x, w


def oper1d(N, k):
    nb = (1 << N) * (k + 1)
    mats = {name: np.zeros((nb, nb)) for name in ("u_v", "u_vx", "ulft_vjp", "urgt_vjp")}
    _check(lib().amdg_oracle_oper1d(N, k, *(m.ctypes.data_as(C.c_void_p) for m in mats.values())))
    return mats


def grid(dim, N, sparse=True):
    E = lib().amdg_oracle_grid_count(dim, N, int(sparse))
    level = np.zeros((E, dim), np.int32)
    suppt = np.zeros((E, dim), np.int32)
    lib().amdg_oracle_grid(dim, N, int(sparse), level, suppt)
    return level, suppt


def project_separable(N, k, dim, funcs):
    """funcs: list (terms) of callables f(x, d) -> float."""
    nb = (1 << N) * (k + 1)
    out = np.zeros((len(funcs), dim, nb))

    def cb(x, d, term, _user):
        return float(funcs[term](x, d))

    fn = _FN1D(cb)
    _check(lib().amdg_oracle_project_separable(N, k, dim, len(funcs), fn, None, out))
    return out


def init_separable(dim, N, k, level, suppt, coef1d):
    E = level.shape[0]
    u = np.zeros((E, (k + 1) ** dim))
    _check(lib().amdg_oracle_init_separable(dim, N, k, E, level, suppt, coef1d.shape[0],
                                            np.ascontiguousarray(coef1d), u))
    return u


def linear_rhs(dim, N, k, level, suppt, c, u, nthreads=0):
    rhs = np.zeros_like(u)
    _check(lib().amdg_oracle_linear_rhs(dim, N, k, level.shape[0], level, suppt, np.asarray(c, np.float64),
                                        np.ascontiguousarray(u), rhs, nthreads))
    return rhs


def linear_rhs_range(dim, N, k, level, suppt, c, u, e0, e1, nthreads=0):
    B = (k + 1) ** dim
    rhs = np.zeros((e1 - e0, B))
    _check(lib().amdg_oracle_linear_rhs_range(dim, N, k, level.shape[0], level, suppt, np.asarray(c, np.float64),
                                              np.ascontiguousarray(u), rhs, e0, e1, nthreads))
    return rhs


class LinearOp:
    """Prebuilt oracle operator: apply_range() times only the RHS evaluation."""

    def __init__(self, dim, N, k, level, suppt, c):
        self.level = np.ascontiguousarray(level, np.int32)
        self.suppt = np.ascontiguousarray(suppt, np.int32)
        self.B = (k + 1) ** dim
        self.h = lib().amdg_oracle_linop_create(dim, N, k, self.level.shape[0], self.level, self.suppt,
                                                np.asarray(c, np.float64))
        if not self.h:
            raise RuntimeError("oracle operator build failed")

    def apply_range(self, u, e0, e1, nthreads=0, out=None):
        rhs = out if out is not None else np.zeros((e1 - e0, self.B))
        _check(lib().amdg_oracle_linop_apply_range(self.h, np.ascontiguousarray(u), rhs, e0, e1, nthreads))
        return rhs

    def close(self):
        if self.h:
            lib().amdg_oracle_linop_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()


def linear_rk3(dim, N, k, level, suppt, c, u, dt, steps, nthreads=0):
    u = np.array(u, np.float64, copy=True, order="C")
    _check(lib().amdg_oracle_linear_rk3(dim, N, k, level.shape[0], level, suppt, np.asarray(c, np.float64),
                                        float(dt), int(steps), u, nthreads))
    return u


def l2_error_split(dim, N, k, level, suppt, u, coef1d_exact, l2_norm_exact):
    return lib().amdg_oracle_l2_error_split(dim, N, k, level.shape[0], level, suppt, np.ascontiguousarray(u),
                                            np.ascontiguousarray(coef1d_exact), float(l2_norm_exact))


def eval_points(dim, N, k, level, suppt, u, x):
    """DGSolution::val at the rows of x (npts x dim)."""
    x = np.ascontiguousarray(x, np.float64).reshape(-1, dim)
    out = np.zeros(len(x))
    _check(lib().amdg_oracle_eval_points(dim, N, k, len(level), np.ascontiguousarray(level, np.int32),
                                         np.ascontiguousarray(suppt, np.int32), np.ascontiguousarray(u, np.float64),
                                         len(x), x, out))
    return out


def burgers_exact(dim, x, a=0.5, b=0.25, c=0.0, t=0.0):
    """Exact Burgers solution a + b v(sum x - dim a t + c, dim b t) at the rows of x."""
    x = np.ascontiguousarray(x, np.float64).reshape(-1, dim)
    f = lib().amdg_oracle_burgers_exact
    return np.array([f(dim, np.ascontiguousarray(xi), a, b, c, t) for xi in x])


def error_burgers(dim, N, k, level, suppt, u, gauss, a=0.5, b=0.25, c=0.0, t=0.0):
    """(L1, L2, Linf) error against the exact Burgers solution by uniform-mesh Gauss quadrature."""
    out = np.zeros(3)
    _check(lib().amdg_oracle_error_burgers(dim, N, k, len(level), np.ascontiguousarray(level, np.int32),
                                           np.ascontiguousarray(suppt, np.int32), np.ascontiguousarray(u, np.float64),
                                           gauss, a, b, c, t, out))
    return out


def lagr_degree(degree):
    """Select the Lagrange interpolation degree of the oracle calls that follow: 3 (node
    layout msh_case 1, the Burgers examples) or 4 (msh_case 2, the wave example)."""
    _check(lib().amdg_oracle_set_lagr_degree(degree))


# Lagrange degree of each problem, as its example program sets it
BURGERS_LAGR_DEGREE = 3
WAVE_LAGR_DEGREE = 4


def wave_rhs(dim, N, k, level, suppt, u, sigma, amp=0.5):
    """Right-hand side of u_tt = div(K grad u), K = (1 + amp prod sin(2 pi x_d))^2, with the IPDG
    penalty -sigma/dx [u][v] (fast transforms, the reference's operator on adaptive grids;
    degree-4 Lagrange interpolation, node layout msh_case 2)."""
    lagr_degree(WAVE_LAGR_DEGREE)
    B = (k + 1) ** dim
    rhs = np.zeros((len(level), B))
    _check(lib().amdg_oracle_wave_rhs_fast(dim, N, k, len(level), np.ascontiguousarray(level, np.int32),
                                           np.ascontiguousarray(suppt, np.int32),
                                           np.ascontiguousarray(u, np.float64).reshape(-1), sigma, amp, rhs))
    return rhs


def wave_penalty(dim, N, k, level, suppt, u, sigma):
    """The IPDG term alone, -sigma/dx [u][v]: the adaptive loop's predictor right-hand side
    (EulerODE2nd::step_rk_source recomputes rhs as the operator matrix times u)."""
    rhs = np.zeros((len(level), (k + 1) ** dim))
    _check(lib().amdg_oracle_wave_penalty(dim, N, k, len(level), np.ascontiguousarray(level, np.int32),
                                          np.ascontiguousarray(suppt, np.int32),
                                          np.ascontiguousarray(u, np.float64).reshape(-1), sigma, rhs))
    return rhs


def wave_rk4(dim, N, k, level, suppt, u, v, sigma, dt, steps, amp=0.5):
    """RK4ODE2nd steps of u' = v, v' = L u (ODESolver.cpp:579-615, same combination order)."""
    u = np.array(u, np.float64)
    v = np.array(v, np.float64)
    for _ in range(steps):
        un, vn = u.copy(), v.copy()
        ku, kv = [], []
        for stage in range(4):
            rhs = wave_rhs(dim, N, k, level, suppt, u, sigma, amp)
            ku.append(dt * v)
            kv.append(dt * rhs)
            if stage < 2:
                u, v = un + ku[-1] / 2.0, vn + kv[-1] / 2.0
            elif stage == 2:
                u, v = un + ku[-1], vn + kv[-1]
            else:
                u = un + 1.0 / 6.0 * (ku[0] + 2 * ku[1] + 2 * ku[2] + ku[3])
                v = vn + 1.0 / 6.0 * (kv[0] + 2 * kv[1] + 2 * kv[2] + kv[3])
    return u, v


def wave_ic_terms(dim, centre=(0.3, 0.4, 0.5), width=200.0):
    """Gaussian bump exp(-width |x - centre|^2) as one separable term."""
    return [lambda x, d: math.exp(-width * (x - centre[d]) ** 2)]


def sin_sum_terms(dim, shift=0.0):
    """sin(2 pi (sum_d x_d - shift)) as separable products of sin/cos."""
    terms = []
    for mask in range(1, 1 << dim):
        nsin = bin(mask).count("1")
        if nsin % 2 == 0:
            continue
        sign = 1.0 if ((nsin - 1) // 2) % 2 == 0 else -1.0

        def f(x, d, mask=mask, sign=sign):
            a = 2 * math.pi * (x - (shift if d == 0 else 0.0))
            v = math.sin(a) if (mask >> d) & 1 else math.cos(a)
            return sign * v if d == 0 else v

        terms.append(f)
    return terms


def lagr_point_values(dim, N, k, level, suppt, u, degree=BURGERS_LAGR_DEGREE):
    lagr_degree(degree)
    up = np.zeros((level.shape[0], (degree + 1) ** dim))
    _check(lib().amdg_oracle_lagr_point_values(dim, N, k, level.shape[0], level, suppt, np.ascontiguousarray(u), up))
    return up


def lagr_surplus(dim, N, level, suppt, fp, degree=BURGERS_LAGR_DEGREE):
    lagr_degree(degree)
    out = np.zeros_like(fp)
    _check(lib().amdg_oracle_lagr_surplus(dim, N, level.shape[0], level, suppt, np.ascontiguousarray(fp), out))
    return out


def lagr_to_alpert_fast(dim, N, k, level, suppt, coe, degree=BURGERS_LAGR_DEGREE):
    lagr_degree(degree)
    out = np.zeros((level.shape[0], (k + 1) ** dim))
    _check(lib().amdg_oracle_lagr_to_alpert_fast(dim, N, k, level.shape[0], level, suppt, np.ascontiguousarray(coe), out))
    return out


def lagr_points_1d(N, degree):
    """Interpolation point coordinates of every 1D element order (2^N x (degree + 1))."""
    lagr_degree(degree)
    P1 = degree + 1
    out = np.zeros((1 << N, P1))
    for o in range(1 << N):
        lev, sp = _elem_of_order(o)
        for p in range(P1):
            out[o, p] = lib().amdg_oracle_lagr_point(lev, sp, p)
    return out


def lagr_mass_diag_1d(N, degree):
    """Integral of the square of every 1D Lagrange interpolation basis function over its support
    (the diagonal of OperatorMatrix1D<LagrBasis, LagrBasis>::u_v), 10-point Gauss on each half."""
    lagr_degree(degree)
    P1 = degree + 1
    x, w = gauss_legendre(10)
    out = np.zeros((1 << N, P1))
    for o in range(1 << N):
        lev, sp = _elem_of_order(o)
        h = 1.0 if lev <= 1 else 2.0 ** (1 - lev)
        lo = 0.0 if lev <= 1 else (sp - 1) / 2 * h
        for p in range(P1):
            s = 0.0
            for a, b in ((lo, lo + h / 2), (lo + h / 2, lo + h)):
                for xi, wi in zip(x, w):
                    xx = 0.5 * (a + b) + 0.5 * (b - a) * xi
                    s += 0.5 * (b - a) * wi * lib().amdg_oracle_lagr_val(lev, sp, p, xx, 0) ** 2
            out[o, p] = s
    return out


def init_adaptive_intp(dim, n_init, nmax, k, func, eps, degree):
    """DGAdaptIntp::init_adaptive_intp (DGAdaptIntp.cpp:35-46, 184-235, 236-270): interpolate
    func (x: (n, dim) array -> (n,) values) at the Lagrange points of the sparse grid of level
    n_init, take the hierarchical surplus, refine every leaf whose indicator
    sqrt(sum_points prod_d M_d * surplus^2) (M the 1D Lagrange mass diagonal) exceeds eps, fill
    holes, repeat until nothing changes; then the Alpert coefficients by the fast transforms.
    Returns (keys, u, rounds)."""
    P1 = degree + 1
    pts1d = lagr_points_1d(nmax, degree)
    diag1d = lagr_mass_diag_1d(nmax, degree)
    pidx = np.indices((P1,) * dim).reshape(dim, -1).T  # point q -> (p_0, ..., p_{dim-1})
    lv, sp = grid(dim, n_init)
    keys = arrays_to_keys(lv, sp)
    rounds = 0
    while True:
        lv, sp = keys_to_arrays(keys, dim)
        o = np.where(lv == 0, 0, (1 << np.maximum(lv - 1, 0)) + (sp - 1) // 2)
        x = np.stack([pts1d[o[:, d][:, None], pidx[None, :, d]] for d in range(dim)], axis=-1)
        fp = np.asarray(func(x.reshape(-1, dim)), dtype=np.float64).reshape(len(keys), -1)
        coe = lagr_surplus(dim, nmax, lv, sp, fp, degree)
        wgt = np.ones((len(keys), P1 ** dim))
        for d in range(dim):
            wgt = wgt * diag1d[o[:, d][:, None], pidx[None, :, d]]
        norms = np.sqrt(np.sum(wgt * coe * coe, axis=1))
        new = refine_keys(keys, norms, eps, nmax)
        if len(new) == len(keys):
            return keys, lagr_to_alpert_fast(dim, nmax, k, lv, sp, coe, degree), rounds
        keys = new
        rounds += 1


def l2_error_split_grids(keys, u, keys_exact, u_exact):
    """DGAdaptIntp::get_L2_error_split_adaptive_intp_scalar (DGAdaptIntp.cpp:57-102): with the
    orthonormal Alpert basis, err^2 = |u_exact|^2 + |u|^2 - 2 sum over the shared elements of
    u . u_exact; a negative err^2 is returned as it is, else its square root."""
    err2 = float(np.sum(np.asarray(u_exact) ** 2)) + float(np.sum(np.asarray(u) ** 2))
    pos = {k: i for i, k in enumerate(keys_exact)}
    for i, k in enumerate(keys):
        j = pos.get(k)
        if j is not None:
            err2 -= 2.0 * float(np.dot(u[i], u_exact[j]))
    return err2 if err2 < 0 else math.sqrt(err2)


def lagr_point_values_fast(dim, N, k, level, suppt, u, degree=BURGERS_LAGR_DEGREE):
    lagr_degree(degree)
    up = np.zeros((level.shape[0], (degree + 1) ** dim))
    _check(lib().amdg_oracle_lagr_point_values_fast(dim, N, k, level.shape[0], level, suppt, np.ascontiguousarray(u),
                                                    up))
    return up


def burgers_rhs(dim, N, k, level, suppt, u, alpha, direct=False):
    """Full Burgers RHS: point values -> flux u^2/2 -> surplus -> volume/interface/penalty terms.
    direct=False follows the reference's fast L/U transforms (its operator on any
    hole-free grid); direct=True sums element pairs directly (equal on sparse grids)."""
    level = np.ascontiguousarray(level, np.int32)
    suppt = np.ascontiguousarray(suppt, np.int32)
    if direct:
        up = lagr_point_values(dim, N, k, level, suppt, u)
    else:
        up = lagr_point_values_fast(dim, N, k, level, suppt, u)
    fp = 0.5 * up * up
    fu = lagr_surplus(dim, N, level, suppt, fp)
    fucoe = np.ascontiguousarray(np.broadcast_to(fu, (dim,) + fu.shape))
    rhs = np.zeros_like(u)
    fn = lib().amdg_oracle_burgers_rhs if direct else lib().amdg_oracle_burgers_rhs_fast
    _check(fn(dim, N, k, level.shape[0], level, suppt, fucoe, np.ascontiguousarray(u), float(alpha), rhs))
    return rhs, up, fu


def burgers_rk3(dim, N, k, level, suppt, u, alpha, dt, steps):
    """SSP-RK3 stages with step_stage semantics (ODESolver.cpp:285-301)."""
    un = np.array(u, np.float64, copy=True)
    for _ in range(steps):
        cur = un.copy()
        for stage in range(3):
            rhs = burgers_rhs(dim, N, k, level, suppt, cur, alpha)[0]
            if stage == 0:
                cur = un + dt * rhs
            elif stage == 1:
                cur = 3. / 4. * un + 1. / 4. * (cur + dt * rhs)
            else:
                cur = 1. / 3. * un + 2. / 3. * (cur + dt * rhs)
        un = cur
    return un


def burgers_ic_terms(dim):
    """0.5 + 0.25 sin(2 pi sum x) as separable terms."""
    terms = [lambda x, d: 0.5 if d == 0 else 1.0]
    for f in sin_sum_terms(dim):
        terms.append(lambda x, d, f=f: (0.25 if d == 0 else 1.0) * f(x, d))
    return terms


# ---------------------------------------------------------------------------
# Adaptivity (DGAdapt::refine / coarsen / check_hole, DGAdapt.cpp:371-404,
# 675-688, 982-1063, 1250-1385; adaptive separable initialisation,
# DGAdapt.cpp:120-147, 850-894).  Elements are tuples of 1D orders.
# ---------------------------------------------------------------------------

def _level(o):
    return int(o).bit_length()


def _elem_of_order(o):
    o = int(o)
    if o == 0:
        return 0, 1
    n = o.bit_length()
    return n, 2 * (o - (1 << (n - 1))) + 1


def keys_to_arrays(keys, dim):
    level = np.zeros((len(keys), dim), np.int32)
    suppt = np.zeros((len(keys), dim), np.int32)
    for i, key in enumerate(keys):
        for d, o in enumerate(key):
            level[i, d], suppt[i, d] = _elem_of_order(o)
    return level, suppt


def arrays_to_keys(level, suppt):
    keys = []
    for lv, sp in zip(level, suppt):
        keys.append(tuple(0 if n == 0 else (1 << (int(n) - 1)) + (int(j) - 1) // 2 for n, j in zip(lv, sp)))
    return keys


def children_of(key, nmax):
    out = []
    for d, o in enumerate(key):
        n = _level(o)
        if n == 0:
            cs = [1]
        elif n == nmax:
            cs = []
        else:
            cs = [2 * o, 2 * o + 1]
        for c in cs:
            out.append(key[:d] + (c,) + key[d + 1:])
    return out


def parents_of(key):
    out = []
    for d, o in enumerate(key):
        if o == 0:
            continue
        p = 0 if o == 1 else o // 2
        out.append(key[:d] + (p,) + key[d + 1:])
    return out


def fill_holes(keyset):
    work = list(keyset)
    while work:
        nxt = []
        for key in work:
            for p in parents_of(key):
                if p not in keyset:
                    keyset.add(p)
                    nxt.append(p)
        work = nxt
    return keyset


def refine_keys(keys, norms, eps, nmax):
    """One refine pass: leaves (fewer existing children than possible) whose
    indicator exceeds eps get all their children, then holes are filled."""
    keyset = set(keys)
    new = set(keyset)
    for key, nrm in zip(keys, norms):
        ch = children_of(key, nmax)
        if sum(c in keyset for c in ch) < len(ch) and nrm > eps:
            new.update(ch)
    return sorted(fill_holes(new))


def coarsen_keys(keys, norms, eta):
    """Repeatedly delete childless elements with indicator < eta and max level > 0."""
    keyset = set(keys)
    norm = dict(zip(keys, norms))
    nmax = 64
    changed = True
    while changed:
        changed = False
        kids = {k: 0 for k in keyset}
        for k in keyset:
            for p in parents_of(k):
                if p in kids:
                    kids[p] += 1
        for k in list(keyset):
            if kids[k] == 0 and norm[k] < eta and max(_level(o) for o in k) > 0:
                keyset.discard(k)
                changed = True
    del nmax
    return sorted(keyset)


def element_norms(u):
    return np.sqrt(np.sum(np.asarray(u) ** 2, axis=1))


def init_adaptive_separable(dim, n_init, nmax, k, terms, eps):
    """Adaptive initialisation: start from the sparse grid of level n_init,
    refine every leaf whose projected coefficients exceed eps, fill holes,
    repeat until nothing changes."""
    coef = project_separable(nmax, k, dim, terms)
    lv, sp = grid(dim, n_init)
    keys = arrays_to_keys(lv, sp)
    while True:
        lv, sp = keys_to_arrays(keys, dim)
        u = init_separable(dim, nmax, k, lv, sp, coef)
        nrm = element_norms(u)
        new = refine_keys(keys, nrm, eps, nmax)
        if len(new) == len(keys):
            return keys, u
        keys = new


def remap(old_keys, u_old, new_keys):
    pos = {k: i for i, k in enumerate(old_keys)}
    out = np.zeros((len(new_keys), u_old.shape[1]))
    for i, k in enumerate(new_keys):
        j = pos.get(k)
        if j is not None:
            out[i] = u_old[j]
    return out


def burgers_adaptive_run(dim, n_init, nmax, eps, eta, alpha, cfl, umax, steps, k=2):
    """The adaptive Burgers time loop: predictor, refine, RK3, coarsen."""
    keys, u = init_adaptive_separable(dim, n_init, nmax, k, burgers_ic_terms(dim), eps)
    history = [(list(keys), u.copy(), None)]
    for _ in range(steps):
        lv, sp = keys_to_arrays(keys, dim)
        maxlev = lv.max(axis=0)
        dt = cfl / sum(umax * 2.0 ** int(m) for m in maxlev)
        rhs = burgers_rhs(dim, nmax, k, lv, sp, u, alpha)[0]
        pred = u + dt * rhs
        new_keys = refine_keys(keys, element_norms(pred), eps, nmax)
        u = remap(keys, u, new_keys)
        keys = new_keys
        lv, sp = keys_to_arrays(keys, dim)
        u = burgers_rk3(dim, nmax, k, lv, sp, u, alpha, dt, 1)
        new_keys = coarsen_keys(keys, element_norms(u), eta)
        u = remap(keys, u, new_keys)
        keys = new_keys
        history.append((list(keys), u.copy(), dt))
    return history


def wave_adaptive_run(dim, n_init, nmax, eps, eta, sigma, cfl, speed, steps, k=2, amp=0.5, centre=(0.3, 0.4, 0.5),
                      width=200.0):
    """The adaptive wave loop of 03_wave_06_var_coeff_adapt.cpp without source: EulerODE2nd
    predictor (u + dt v, v + dt (IPDG u): step_rk_source replaces the assembled right-hand side
    by the operator matrix times u), refine on the predicted ||u|| + ||u_t|| (the indicator of
    prob "wave", DGAdapt.cpp:1018-1030), RK4ODE2nd step, coarsen on ||u|| + ||u_t||; u0 the
    Gaussian bump, v0 = 0."""
    keys, u = init_adaptive_separable(dim, n_init, nmax, k, wave_ic_terms(dim, centre, width), eps)
    v = np.zeros_like(u)
    history = [(list(keys), u.copy(), v.copy(), None)]
    for _ in range(steps):
        lv, sp = keys_to_arrays(keys, dim)
        maxlev = lv.max(axis=0)
        dt = cfl / sum(speed * 2.0 ** int(m) for m in maxlev)
        pred_u = u + dt * v
        pred_v = v + dt * wave_penalty(dim, nmax, k, lv, sp, u, sigma)
        new_keys = refine_keys(keys, element_norms(pred_u) + element_norms(pred_v), eps, nmax)
        u, v = remap(keys, u, new_keys), remap(keys, v, new_keys)
        keys = new_keys
        lv, sp = keys_to_arrays(keys, dim)
        u, v = wave_rk4(dim, nmax, k, lv, sp, u, v, sigma, dt, 1, amp)
        new_keys = coarsen_keys(keys, element_norms(u) + element_norms(v), eta)
        u, v = remap(keys, u, new_keys), remap(keys, v, new_keys)
        keys = new_keys
        history.append((list(keys), u.copy(), v.copy(), dt))
    return history


# ---------------------------------------------------------------------------
# Batched-serving workload: sums of periodic Gaussian bumps (separable terms)
# ---------------------------------------------------------------------------

def gaussian_bump_terms(centers, widths, amplitudes, shift=None, vectorized=False):
    """Separable terms of sum_g a_g prod_d G(x_d; c_gd, w_g), G(x) = sum_{m=-1,0,1} exp(-((x - c + m)/w)^2);
    shift (dim,) translates every centre (periodic).  vectorized: the factors take numpy arrays."""
    terms = []
    dim = len(centers[0])
    for c, w, a in zip(centers, widths, amplitudes):
        cc = [(c[d] + (shift[d] if shift is not None else 0.0)) % 1.0 for d in range(dim)]

        if vectorized:
            def f(x, d, cc=cc, w=w, a=a):
                v = sum(np.exp(-((x - cc[d] + m) / w) ** 2) for m in (-1.0, 0.0, 1.0))
                return a * v if d == 0 else v
        else:
            def f(x, d, cc=cc, w=w, a=a):
                v = sum(math.exp(-((x - cc[d] + m) / w) ** 2) for m in (-1.0, 0.0, 1.0))
                return a * v if d == 0 else v

        terms.append(f)
    return terms


def gaussian_bump_norm(centers, widths, amplitudes, n=4000):
    """Exact L2 norm over [0,1]^dim of the bump sum (1D integrals by the midpoint rule on n cells)."""
    x = (np.arange(n) + 0.5) / n
    dim = len(centers[0])

    def g1(c, w):
        return sum(np.exp(-((x - c + m) / w) ** 2) for m in (-1.0, 0.0, 1.0))

    tot = 0.0
    for i in range(len(centers)):
        for j in range(len(centers)):
            p = amplitudes[i] * amplitudes[j]
            for d in range(dim):
                p *= float(np.mean(g1(centers[i][d], widths[i]) * g1(centers[j][d], widths[j])))
            tot += p
    return math.sqrt(tot)


def batched_workload(nsolves, seed=0, dim=3):
    """Seeded config: velocity U[-1,1]^dim, 1..4 bumps, centres U[0.2,0.8]^dim, widths U[0.03,0.15]."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(nsolves):
        vel = rng.uniform(-1.0, 1.0, dim)
        nb = int(rng.integers(1, 5))
        centers = rng.uniform(0.2, 0.8, (nb, dim)).tolist()
        widths = rng.uniform(0.03, 0.15, nb).tolist()
        out.append(dict(velocity=vel.tolist(), centers=centers, widths=widths, amplitudes=[1.0] * nb))
    return out


# ---------------------------------------------------------------------------
# CPU reference of the refine/keep/coarsen classifier (float64): forward pass,
# analytic backward pass, and finite differences, for checking the device
# kernels' gradients.  Parameter layout: per layer W[out][in] then b[out].
# ---------------------------------------------------------------------------

def mlp_unpack(params, dims):
    out, off = [], 0
    for i in range(len(dims) - 1):
        n_in, n_out = dims[i], dims[i + 1]
        W = np.asarray(params[off:off + n_in * n_out], np.float64).reshape(n_out, n_in)
        off += n_in * n_out
        b = np.asarray(params[off:off + n_out], np.float64)
        off += n_out
        out.append((W, b))
    return out


def mlp_loss_grad(params, dims, x, labels):
    layers = mlp_unpack(params, dims)
    acts = [np.asarray(x, np.float64)]
    for i, (W, b) in enumerate(layers):
        z = acts[-1] @ W.T + b
        acts.append(np.maximum(z, 0.0) if i + 1 < len(layers) else z)
    z = acts[-1]
    z = z - z.max(axis=1, keepdims=True)
    p = np.exp(z) / np.exp(z).sum(axis=1, keepdims=True)
    n = x.shape[0]
    loss = float(-np.mean(np.log(p[np.arange(n), labels])))
    delta = p.copy()
    delta[np.arange(n), labels] -= 1.0
    delta /= n
    grads = []
    for i in range(len(layers) - 1, -1, -1):
        W, _b = layers[i]
        xin = acts[i]
        grads.append((delta.T @ xin, delta.sum(axis=0)))
        if i > 0:
            delta = (delta @ W) * (xin > 0)
    grads.reverse()
    flat = np.concatenate([np.concatenate([gW.ravel(), gb]) for gW, gb in grads])
    return loss, flat


def mlp_loss(params, dims, x, labels):
    return mlp_loss_grad(params, dims, x, labels)[0]


# ---------------------------------------------------------------------------
# Cubic Hermite interpolation of the flux (2D Burgers driver
# example/02_hyperbolic_05_burgers_adapt.cpp): HermInterpolation::nonlinear_Herm_2D_fast
# (Interplation.cpp:4609-4621) + HyperbolicSameFluxHermRHS (FastMultiplyLU.cpp:970-1016) + the
# assembled LxF matrix
# ---------------------------------------------------------------------------

def oper1d_herm(N, k):
    """Hermite x Alpert 1D matrices (u_v, u_vx, ulft_vjp + urgt_vjp), (2^N 4) x (2^N (k+1))."""
    shape = ((1 << N) * 4, (1 << N) * (k + 1))
    mats = [np.zeros(shape) for _ in range(3)]
    _check(lib().amdg_oracle_oper1d_herm(N, k, *[m.ctypes.data for m in mats]))
    return mats


def herm_points_1d(N):
    """Hermite dof point coordinates of every 1D element order (2^N x 4)."""
    out = np.zeros((1 << N, 4))
    for o in range(1 << N):
        lev, sp = _elem_of_order(o)
        for p in range(4):
            out[o, p] = lib().amdg_oracle_herm_point(lev, sp, p)
    return out


def herm_point_values(dim, N, k, level, suppt, u, direct=False):
    level = np.ascontiguousarray(level, np.int32)
    suppt = np.ascontiguousarray(suppt, np.int32)
    up = np.zeros((level.shape[0], 4 ** dim))
    fn = lib().amdg_oracle_herm_point_values if direct else lib().amdg_oracle_herm_point_values_fast
    _check(fn(dim, N, k, level.shape[0], level, suppt, np.ascontiguousarray(u), up))
    return up


def herm_flux_burgers2d(up):
    fp = np.zeros_like(up)
    _check(lib().amdg_oracle_herm_flux_burgers2d(up.shape[0], np.ascontiguousarray(up), fp))
    return fp


def herm_surplus(dim, N, level, suppt, fp):
    level = np.ascontiguousarray(level, np.int32)
    suppt = np.ascontiguousarray(suppt, np.int32)
    out = np.zeros_like(fp)
    _check(lib().amdg_oracle_herm_surplus(dim, N, level.shape[0], level, suppt, np.ascontiguousarray(fp), out))
    return out


def burgers_herm_rhs(N, k, level, suppt, u, alpha, direct=False):
    """2D Burgers right-hand side with the Hermite-interpolated flux: point values and slopes ->
    f, f' u_x, f' u_y, f'' u_x u_y + f' u_xy -> Hermite surplus -> volume, interface and LxF
    penalty terms.  Returns (rhs, up, fu)."""
    level = np.ascontiguousarray(level, np.int32)
    suppt = np.ascontiguousarray(suppt, np.int32)
    up = herm_point_values(2, N, k, level, suppt, u, direct)
    fu = herm_surplus(2, N, level, suppt, herm_flux_burgers2d(up))
    rhs = np.zeros_like(u)
    _check(lib().amdg_oracle_burgers_herm_rhs_fast(2, N, k, level.shape[0], level, suppt, fu,
                                                   np.ascontiguousarray(u), float(alpha), rhs))
    return rhs, up, fu


def burgers_herm_rk3(N, k, level, suppt, u, alpha, dt, steps):
    un = np.array(u, np.float64, copy=True)
    for _ in range(steps):
        cur = un.copy()
        for stage in range(3):
            rhs = burgers_herm_rhs(N, k, level, suppt, cur, alpha)[0]
            if stage == 0:
                cur = un + dt * rhs
            elif stage == 1:
                cur = 3. / 4. * un + 1. / 4. * (cur + dt * rhs)
            else:
                cur = 1. / 3. * un + 2. / 3. * (cur + dt * rhs)
        un = cur
    return un


def burgers_herm_adaptive_run(n_init, nmax, eps, eta, alpha, cfl, steps, k=2):
    """The adaptive loop of 02_hyperbolic_05_burgers_adapt.cpp (no artificial viscosity):
    u0 = sin(2 pi (x+y)), dt = cfl / sum_d 2^maxlevel_d, predictor, refine, SSP-RK3, coarsen."""
    keys, u = init_adaptive_separable(2, n_init, nmax, k, sin_sum_terms(2), eps)
    history = [(list(keys), u.copy(), None)]
    for _ in range(steps):
        lv, sp = keys_to_arrays(keys, 2)
        dt = cfl / sum(2.0 ** int(m) for m in lv.max(axis=0))
        pred = u + dt * burgers_herm_rhs(nmax, k, lv, sp, u, alpha)[0]
        new_keys = refine_keys(keys, element_norms(pred), eps, nmax)
        u = remap(keys, u, new_keys)
        keys = new_keys
        lv, sp = keys_to_arrays(keys, 2)
        u = burgers_herm_rk3(nmax, k, lv, sp, u, alpha, dt, 1)
        new_keys = coarsen_keys(keys, element_norms(u), eta)
        u = remap(keys, u, new_keys)
        keys = new_keys
        history.append((list(keys), u.copy(), dt))
    return history
