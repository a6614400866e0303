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
        L.amdg_oracle_lagr_val.restype = C.c_double
        L.amdg_oracle_lagr_val.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_int]
        L.amdg_oracle_lagr_point.restype = C.c_double
        L.amdg_oracle_lagr_point.argtypes = [C.c_int, C.c_int, C.c_int]
        L.amdg_oracle_oper1d_lagr.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        L.amdg_oracle_lagr_point_values.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int64, i32p, i32p, f64p, f64p]
        L.amdg_oracle_lagr_surplus.argtypes = [C.c_int, C.c_int, C.c_int64, i32p, i32p, f64p, f64p]
        L.amdg_oracle_burgers_rhs.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int64, i32p, i32p, f64p, f64p, C.c_double,
                                              f64p]
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


def lagr_point_values(dim, N, k, level, suppt, u):
    up = np.zeros((level.shape[0], 4 ** dim))
    _check(lib().amdg_oracle_lagr_point_values(dim, N, k, level.shape[0], level, suppt, np.ascontiguousarray(u), up))
    return up


def lagr_surplus(dim, N, level, suppt, fp):
    out = np.zeros_like(fp)
    _check(lib().amdg_oracle_lagr_surplus(dim, N, level.shape[0], level, suppt, np.ascontiguousarray(fp), out))
    return out


def burgers_rhs(dim, N, k, level, suppt, u, alpha):
    """Full Burgers RHS: point values -> flux u^2/2 -> surplus -> volume/interface/penalty terms."""
    up = lagr_point_values(dim, N, k, level, suppt, u)
    fp = 0.5 * up * up
    fu = lagr_surplus(dim, N, level, suppt, fp)
    fucoe = np.ascontiguousarray(np.broadcast_to(fu, (dim,) + fu.shape))
    rhs = np.zeros_like(u)
    _check(lib().amdg_oracle_burgers_rhs(dim, N, k, level.shape[0], level, suppt, fucoe, np.ascontiguousarray(u),
                                         float(alpha), rhs))
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
