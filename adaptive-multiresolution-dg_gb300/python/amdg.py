"""ctypes binding of libamdg_gb300 (include/amdg.h).

Thin Python mirror of the reference's C++ interface for the sparse-grid DG
right-hand side: Grid ~ DGSolution/DGAdapt, LinearOperator ~ HyperbolicAlpt +
RK3SSP.  Every compute call goes to the CUDA library; if the shared library
is missing this module raises instead of computing anything on the CPU.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG, "lib", "libamdg_gb300.so")
HEADER = os.path.join(os.path.dirname(PKG), "include", "amdg.h")

FP64 = 0
MIXED = 1

STATUS = {0: "ok", 1: "invalid argument", 2: "capacity exceeded", 3: "non-finite value", 4: "device wait timed out",
          5: "CUDA error", 6: "invalid state", 7: "out of memory", 8: "I/O error", 9: "bad checkpoint"}

FN1D = C.CFUNCTYPE(C.c_double, C.c_double, C.c_int, C.c_int, C.c_void_p)
FN1D_BATCH = C.CFUNCTYPE(None, C.POINTER(C.c_double), C.c_int64, C.c_int, C.c_int, C.POINTER(C.c_double), C.c_void_p)
FN_POINTS = C.CFUNCTYPE(None, C.POINTER(C.c_double), C.c_int64, C.c_int, C.POINTER(C.c_double), C.c_void_p)


class AmdgError(RuntimeError):
    def __init__(self, status: int, where: str, msg: str):
        super().__init__(f"{where}: {STATUS.get(status, status)}: {msg}")
        self.status = status


_lib = None


def load():
    """Load libamdg_gb300.so (build it first with __graft_entry__.build())."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} not found: the CUDA library must be built (no CPU fallback exists)")
    L = C.CDLL(LIB_PATH)
    vp, i32, i64, dbl = C.c_void_p, C.c_int, C.c_int64, C.c_double
    pp = C.POINTER(C.c_void_p)
    sig = {
        "amdg_abi_version": ([], i32),
        "amdg_status_string": ([i32], C.c_char_p),
        "amdg_last_error": ([], C.c_char_p),
        "amdg_context_create": ([i32, pp], i32),
        "amdg_context_destroy": ([vp], i32),
        "amdg_context_set_stream": ([vp, vp], i32),
        "amdg_context_get_stream": ([vp, pp], i32),
        "amdg_context_synchronize": ([vp], i32),
        "amdg_context_launch_count": ([vp, C.POINTER(i64)], i32),
        "amdg_oper1d_build": ([i32, i32, vp, vp, vp, vp], i32),
        "amdg_grid_enumerate": ([i32, i32, i32, C.POINTER(i64), vp, vp], i32),
        "amdg_grid_create": ([vp, i32, i32, i32, i32, pp], i32),
        "amdg_grid_destroy": ([vp], i32),
        "amdg_grid_size": ([vp, C.POINTER(i64), C.POINTER(i64)], i32),
        "amdg_grid_elements": ([vp, vp, vp], i32),
        "amdg_grid_max_mesh_level": ([vp, vp], i32),
        "amdg_grid_set_coefficients": ([vp, vp, i64], i32),
        "amdg_grid_get_coefficients": ([vp, vp, i64], i32),
        "amdg_grid_coefficients_device": ([vp, pp], i32),
        "amdg_grid_init_separable": ([vp, i32, FN1D, vp], i32),
        "amdg_grid_l2_norm": ([vp, C.POINTER(dbl)], i32),
        "amdg_grid_l2_error_separable": ([vp, FN1D, vp, dbl, C.POINTER(dbl)], i32),
        "amdg_linear_create": ([vp, vp, pp], i32),
        "amdg_linear_destroy": ([vp], i32),
        "amdg_linear_stats": ([vp, C.POINTER(i64), C.POINTER(dbl)], i32),
        "amdg_linear_apply": ([vp, vp, vp, i32], i32),
        "amdg_linear_tuning": ([vp, vp, vp], i32),
        "amdg_linear_set_variant": ([vp, i32, i32], i32),
        "amdg_linear_copy_config": ([vp, vp, vp], i32),
        "amdg_linear_set_copy_config": ([vp, i32], i32),
        "amdg_rk3ssp_steps": ([vp, dbl, i32, i32], i32),
        "amdg_rk3ssp_steps_host": ([vp, dbl, i32, vp, i32], i32),
        "amdg_rk3ssp_serve_host": ([vp, dbl, i32, i32, i32, vp, vp], i32),
        "amdg_rk3_stage_update": ([vp, i32, dbl, vp, vp, vp, i64], i32),
        "amdg_rk3ssp_steps_noalloc": ([vp, vp, dbl, i32, i32], i32),
        "amdg_burgers_create": ([vp, vp, pp], i32),
        "amdg_burgers_create_herm": ([vp, vp, pp], i32),
        "amdg_burgers_adaptive_step": ([vp, dbl, dbl, dbl, dbl, i32, C.POINTER(dbl)], i32),
        "amdg_burgers_adaptive_step_ex": ([vp, dbl, dbl, dbl, dbl, i32, C.POINTER(dbl), vp], i32),
        "amdg_burgers_features": ([vp, vp, vp], i32),
        "amdg_burgers_adaptive_step_learned": ([vp, vp, dbl, dbl, dbl, dbl, dbl, i32, C.POINTER(dbl), vp], i32),
        "amdg_burgers_adaptive_steps_learned": ([vp, vp, dbl, dbl, dbl, dbl, dbl, i32, i32, dbl, vp, vp, vp], i32),
        "amdg_mlp_create": ([vp, i32, i32, i32, i32, C.c_uint64, pp], i32),
        "amdg_mlp_destroy": ([vp], i32),
        "amdg_mlp_num_params": ([vp, C.POINTER(i64)], i32),
        "amdg_mlp_get_params": ([vp, vp, i64], i32),
        "amdg_mlp_set_params": ([vp, vp, i64], i32),
        "amdg_mlp_predict": ([vp, vp, i64, vp], i32),
        "amdg_mlp_loss_grad": ([vp, vp, vp, i64, C.POINTER(dbl), vp], i32),
        "amdg_mlp_train": ([vp, vp, vp, i64, i32, i32, C.c_float, C.c_uint64, C.POINTER(dbl)], i32),
        "amdg_grid_create_ex": ([vp, i32, i32, i32, i32, i32, pp], i32),
        "amdg_grid_init_separable_adaptive": ([vp, i32, FN1D, vp, dbl], i32),
        "amdg_grid_init_separable_batch": ([vp, i32, FN1D_BATCH, vp], i32),
        "amdg_grid_init_separable_adaptive_batch": ([vp, i32, FN1D_BATCH, vp, dbl], i32),
        "amdg_grid_l2_error_separable_sum_batch": ([vp, i32, FN1D_BATCH, vp, dbl, C.POINTER(dbl)], i32),
        "amdg_grid_init_adaptive_intp": ([vp, i32, FN_POINTS, vp, dbl, C.POINTER(i32)], i32),
        "amdg_grid_l2_error_split_grid": ([vp, vp, C.POINTER(dbl)], i32),
        "amdg_grid_refine": ([vp, vp, dbl, C.POINTER(i64)], i32),
        "amdg_grid_coarsen": ([vp, dbl, C.POINTER(i64)], i32),
        "amdg_grid_version": ([vp, C.POINTER(i64)], i32),
        "amdg_grid_l2_error_separable_sum": ([vp, i32, FN1D, vp, dbl, C.POINTER(dbl)], i32),
        "amdg_grid_eval_tensor": ([vp, i32, vp, vp], i32),
        "amdg_grid_set_velocity": ([vp, vp, i64], i32),
        "amdg_grid_get_velocity": ([vp, vp, i64], i32),
        "amdg_grid_save": ([vp, C.c_char_p, dbl], i32),
        "amdg_grid_load": ([vp, C.c_char_p, pp, vp], i32),
        "amdg_grid_write_level_support": ([vp, C.c_char_p], i32),
        "amdg_grid_config": ([vp, vp, vp, vp, vp], i32),
        "amdg_wave_create": ([vp, dbl, dbl, pp], i32),
        "amdg_wave_destroy": ([vp], i32),
        "amdg_wave_rhs": ([vp, vp, vp, i32], i32),
        "amdg_wave_rk4_steps": ([vp, dbl, i32, i32], i32),
        "amdg_wave_adaptive_step": ([vp, dbl, dbl, dbl, dbl, i32, C.POINTER(dbl)], i32),
        "amdg_wave_counters": ([vp, C.POINTER(i64), C.POINTER(i64)], i32),
        "amdg_wave_adaptive_step_ex": ([vp, dbl, dbl, dbl, dbl, i32, C.POINTER(dbl), vp], i32),
        "amdg_wave_features": ([vp, vp, vp], i32),
        "amdg_wave_adaptive_step_learned": ([vp, vp, dbl, dbl, dbl, dbl, dbl, i32, C.POINTER(dbl), vp], i32),
        "amdg_wave_adaptive_steps_learned": ([vp, vp, dbl, dbl, dbl, dbl, dbl, i32, i32, dbl, vp, vp, vp], i32),
        "amdg_context_profile": ([vp, i32], i32),
        "amdg_context_set_adapt_mode": ([vp, i32], i32),
        "amdg_debug_fail_device_allocations": ([i64], i32),
        "amdg_linear_set_wait_limit": ([vp, C.c_uint32], i32),
        "amdg_grid_set_rhs_zero": ([vp], i32),
        "amdg_grid_rhs_device": ([vp, pp], i32),
        "amdg_grid_get_rhs": ([vp, vp, i64], i32),
        "amdg_grid_copy_ucoe_to_predict": ([vp], i32),
        "amdg_grid_copy_predict_to_ucoe": ([vp], i32),
        "amdg_grid_copy_ucoe_ut_to_predict": ([vp], i32),
        "amdg_grid_copy_predict_to_ucoe_ut": ([vp], i32),
        "amdg_grid_set_indicator": ([vp, i32], i32),
        "amdg_wave_set_sigma": ([vp, dbl], i32),
        "amdg_wave_interpolate": ([vp, i32, i32], i32),
        "amdg_wave_rhs_add": ([vp, i32, i32], i32),
        "amdg_ode_add_wave_penalty": ([vp, vp], i32),
        "amdg_vector_axpy": ([vp, dbl, vp, vp, i64], i32),
        "amdg_ode_create": ([vp, i32, dbl, pp], i32),
        "amdg_ode_destroy": ([vp], i32),
        "amdg_ode_set_rhs_zero": ([vp], i32),
        "amdg_ode_add_rhs_to_eigenvec": ([vp], i32),
        "amdg_ode_step_stage": ([vp, i32], i32),
        "amdg_ode_final": ([vp], i32),
        "amdg_lagr_interpolate": ([vp, i32], i32),
        "amdg_burgers_work": ([vp, C.POINTER(dbl), C.POINTER(dbl)], i32),
        "amdg_burgers_set_sweep_variant": ([vp, i32], i32),
        "amdg_wave_set_sweep_variant": ([vp, i32], i32),
        "amdg_lagr_rhs_add": ([vp, i32, vp, i32], i32),
        "amdg_context_profile_read": ([vp, vp, vp], i32),
        "amdg_burgers_counters": ([vp, C.POINTER(i64), C.POINTER(i64)], i32),
        "amdg_grid_error_burgers": ([vp, dbl, dbl, dbl, dbl, i32, vp], i32),
        "amdg_batch_create": ([vp, i32, vp, vp, pp], i32),
        "amdg_batch_destroy": ([vp], i32),
        "amdg_batch_size": ([vp, C.POINTER(i64), C.POINTER(i64), C.POINTER(i64)], i32),
        "amdg_batch_set_dt": ([vp, vp], i32),
        "amdg_batch_rk3_steps": ([vp, i32, i32, i32], i32),
        "amdg_batch_store": ([vp, i32], i32),
        "amdg_batch_coefficients_device": ([vp, pp, vp], i32),
        "amdg_batch_tuning": ([vp, vp, vp], i32),
        "amdg_batch_adapt": ([vp, vp, dbl, dbl, dbl, vp], i32),
        "amdg_batch_set_kernel": ([vp, i32, i32], i32),
        "amdg_batch_set_tile": ([vp, i32, i32], i32),
        "amdg_burgers_destroy": ([vp], i32),
        "amdg_burgers_rhs": ([vp, vp, vp, i32], i32),
        "amdg_burgers_point_values": ([vp, vp, vp, i32], i32),
        "amdg_burgers_flux_coefficients": ([vp, vp, vp, i32], i32),
        "amdg_burgers_rk3_steps": ([vp, dbl, i32, i32], i32),
    }
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _lib = L
    return L


def _ck(status: int, where: str):
    if status != 0:
        raise AmdgError(status, where, load().amdg_last_error().decode())


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def declared_functions() -> list[str]:
    """Names of every entry point declared in include/amdg.h."""
    import re
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:amdg_status|int|const char\*)\s+(amdg_\w+)\s*\(", text, re.M)))


def oper1d(nmax: int, k: int) -> dict:
    """OperatorMatrix1D equivalent (host): u_v, u_vx, ulft_vjp, urgt_vjp."""
    nb = (1 << nmax) * (k + 1)
    mats = {n: np.zeros((nb, nb)) for n in ("u_v", "u_vx", "ulft_vjp", "urgt_vjp")}
    _ck(load().amdg_oper1d_build(nmax, k, *(_ptr(m) for m in mats.values())), "oper1d_build")
    return mats


def enumerate_grid(dim: int, nmax: int, sparse: bool = True):
    n = C.c_int64()
    _ck(load().amdg_grid_enumerate(dim, nmax, int(sparse), C.byref(n), None, None), "grid_enumerate")
    level = np.zeros((n.value, dim), np.int32)
    suppt = np.zeros((n.value, dim), np.int32)
    _ck(load().amdg_grid_enumerate(dim, nmax, int(sparse), C.byref(n), _ptr(level), _ptr(suppt)), "grid_enumerate")
    return level, suppt


def _fn1d(funcs):
    def cb(x, d, term, _user):
        return float(funcs[term](x, d))
    return FN1D(cb)


def _fn1d_batch(funcs):
    """Callback for factors that take a numpy array of points: one call per dimension and term."""
    def cb(x, n, d, term, out, _user):
        xs = np.ctypeslib.as_array(x, shape=(n,))
        np.ctypeslib.as_array(out, shape=(n,))[:] = funcs[term](xs, d)
    return FN1D_BATCH(cb)


class Context:
    def __init__(self, device: int = 0):
        self._h = C.c_void_p()
        _ck(load().amdg_context_create(device, C.byref(self._h)), "context_create")

    @property
    def handle(self):
        return self._h

    def set_stream(self, stream_handle: int | None):
        _ck(load().amdg_context_set_stream(self._h, C.c_void_p(stream_handle or 0)), "context_set_stream")

    def synchronize(self):
        _ck(load().amdg_context_synchronize(self._h), "context_synchronize")

    def launch_count(self) -> int:
        n = C.c_int64()
        _ck(load().amdg_context_launch_count(self._h, C.byref(n)), "context_launch_count")
        return n.value

    PHASES = ("topology", "set_keys", "norms", "adapt_host", "rhs", "rk3", "classifier", "adapt_step", "adapt_device")
    ADAPT_DEVICE, ADAPT_HOST = 0, 1

    def set_adapt_mode(self, mode: int):
        """ADAPT_DEVICE (default): element-set changes and neighbour lists on the device;
        ADAPT_HOST: on the host key set."""
        _ck(load().amdg_context_set_adapt_mode(self._h, mode), "context_set_adapt_mode")

    def profile(self, enable: bool = True):
        """Start (and reset) or stop the host phase profile."""
        _ck(load().amdg_context_profile(self._h, 1 if enable else 0), "context_profile")

    def profile_read(self) -> dict:
        """{phase: (wall seconds, calls)} of the host phase profile."""
        sec = np.zeros(len(self.PHASES))
        calls = np.zeros(len(self.PHASES), np.int64)
        _ck(load().amdg_context_profile_read(self._h, _ptr(sec), _ptr(calls)), "context_profile_read")
        return {p: (float(s), int(c)) for p, s, c in zip(self.PHASES, sec, calls)}

    def stage_update(self, stage: int, dt: float, d_un: int, d_u: int, d_rhs: int, n: int):
        _ck(load().amdg_rk3_stage_update(self._h, stage, dt, C.c_void_p(d_un), C.c_void_p(d_u), C.c_void_p(d_rhs), n),
            "rk3_stage_update")

    def close(self):
        if self._h:
            load().amdg_context_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Grid:
    """DGSolution/DGAdapt on the device (sparse or full grid, Alpert degree k)."""

    def __init__(self, ctx: Context, dim: int, nmax: int, k: int = 2, sparse: bool = True, level_init: int | None = None):
        self.ctx, self.dim, self.nmax, self.k, self.sparse = ctx, dim, nmax, k, sparse
        self._h = C.c_void_p()
        li = nmax if level_init is None else level_init
        _ck(load().amdg_grid_create_ex(ctx.handle, dim, li, nmax, k, int(sparse), C.byref(self._h)), "grid_create")
        self.block = (k + 1) ** dim
        self._refresh()

    def _refresh(self):
        ne, dof = C.c_int64(), C.c_int64()
        _ck(load().amdg_grid_size(self._h, C.byref(ne), C.byref(dof)), "grid_size")
        self.num_elements, self.dof = ne.value, dof.value

    def save(self, path: str, time: float = 0.0):
        """Binary checkpoint: element keys, coefficients, u_t when present, and time."""
        _ck(load().amdg_grid_save(self._h, os.fsencode(path), time), "grid_save")

    @classmethod
    def load(cls, ctx: Context, path: str):
        """(grid, time) restored from a checkpoint written by save."""
        h, t = C.c_void_p(), C.c_double()
        _ck(load().amdg_grid_load(ctx.handle, os.fsencode(path), C.byref(h), C.byref(t)), "grid_load")
        dim, nmax, k, sparse = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        _ck(load().amdg_grid_config(h, C.byref(dim), C.byref(nmax), C.byref(k), C.byref(sparse)), "grid_config")
        g = cls.__new__(cls)
        g.ctx, g.dim, g.nmax, g.k, g.sparse = ctx, dim.value, nmax.value, k.value, bool(sparse.value)
        g._h = h
        g.block = (g.k + 1) ** g.dim
        g._refresh()
        return g, t.value

    def write_level_support(self, path: str):
        """IO::output_element_level_support: "level xl xr " per dimension, one element per line."""
        _ck(load().amdg_grid_write_level_support(self._h, os.fsencode(path)), "grid_write_level_support")

    def init_separable_adaptive(self, funcs, eps: float, vectorized: bool = False):
        """vectorized: the factors take a numpy array of points (one callback per dimension and term)."""
        if vectorized:
            cb = _fn1d_batch(funcs)
            _ck(load().amdg_grid_init_separable_adaptive_batch(self._h, len(funcs), cb, None, eps),
                "grid_init_separable_adaptive_batch")
        else:
            cb = _fn1d(funcs)
            _ck(load().amdg_grid_init_separable_adaptive(self._h, len(funcs), cb, None, eps),
                "grid_init_separable_adaptive")
        self._refresh()

    def init_adaptive_intp(self, func, eps: float, degree: int = 3) -> int:
        """DGAdaptIntp::init_adaptive_intp: adaptive Lagrange interpolation (degree 3, 4 or 5) of
        func, which maps an (n, dim) array of points to n values, from the current element set;
        returns the refinement rounds."""
        def cb(x, n, dim, out, _user):
            xs = np.ctypeslib.as_array(x, shape=(n, dim))
            np.ctypeslib.as_array(out, shape=(n,))[:] = func(xs)

        fn = FN_POINTS(cb)
        rounds = C.c_int()
        _ck(load().amdg_grid_init_adaptive_intp(self._h, degree, fn, None, eps, C.byref(rounds)),
            "grid_init_adaptive_intp")
        self._refresh()
        return rounds.value

    def l2_error_split_grid(self, exact) -> float:
        """DGAdaptIntp::get_L2_error_split_adaptive_intp_scalar against the solution on `exact`."""
        out = C.c_double()
        _ck(load().amdg_grid_l2_error_split_grid(self._h, exact.handle, C.byref(out)), "grid_l2_error_split_grid")
        return out.value

    def refine(self, eps: float, d_indicator: int | None = None):
        n = C.c_int64()
        _ck(load().amdg_grid_refine(self._h, C.c_void_p(d_indicator or 0), eps, C.byref(n)), "grid_refine")
        self._refresh()
        return n.value

    def coarsen(self, eta: float):
        n = C.c_int64()
        _ck(load().amdg_grid_coarsen(self._h, eta, C.byref(n)), "grid_coarsen")
        self._refresh()
        return n.value

    def version(self) -> int:
        v = C.c_int64()
        _ck(load().amdg_grid_version(self._h, C.byref(v)), "grid_version")
        return v.value

    @property
    def handle(self):
        return self._h

    def elements(self):
        level = np.zeros((self.num_elements, self.dim), np.int32)
        suppt = np.zeros((self.num_elements, self.dim), np.int32)
        _ck(load().amdg_grid_elements(self._h, _ptr(level), _ptr(suppt)), "grid_elements")
        return level, suppt

    def max_mesh_level(self):
        out = np.zeros(self.dim, np.int32)
        _ck(load().amdg_grid_max_mesh_level(self._h, _ptr(out)), "grid_max_mesh_level")
        return out

    def set_coefficients(self, u: np.ndarray):
        u = np.ascontiguousarray(u, np.float64).reshape(-1)
        _ck(load().amdg_grid_set_coefficients(self._h, _ptr(u), u.size), "grid_set_coefficients")

    def coefficients(self, out: np.ndarray | None = None) -> np.ndarray:
        """The coefficients as (num_elements, block); into `out` (dof float64 entries, e.g. pinned
        host memory) when given."""
        u = np.zeros(self.dof) if out is None else out.reshape(-1)[:self.dof]
        _ck(load().amdg_grid_get_coefficients(self._h, _ptr(u), self.dof), "grid_get_coefficients")
        return u.reshape(self.num_elements, self.block)

    def device_ptr(self) -> int:
        p = C.c_void_p()
        _ck(load().amdg_grid_coefficients_device(self._h, C.byref(p)), "grid_coefficients_device")
        return p.value

    def set_rhs_zero(self):
        """DGSolution::set_rhs_zero: the grid's Element::rhs vector = 0."""
        _ck(load().amdg_grid_set_rhs_zero(self._h), "grid_set_rhs_zero")

    def rhs_device_ptr(self) -> int:
        p = C.c_void_p()
        _ck(load().amdg_grid_rhs_device(self._h, C.byref(p)), "grid_rhs_device")
        return p.value

    def rhs(self) -> np.ndarray:
        """The grid's Element::rhs vector, as (num_elements, block)."""
        out = np.zeros(self.dof)
        _ck(load().amdg_grid_get_rhs(self._h, _ptr(out), self.dof), "grid_get_rhs")
        return out.reshape(self.num_elements, self.block)

    def copy_ucoe_to_predict(self):
        _ck(load().amdg_grid_copy_ucoe_to_predict(self._h), "grid_copy_ucoe_to_predict")

    def copy_predict_to_ucoe(self):
        _ck(load().amdg_grid_copy_predict_to_ucoe(self._h), "grid_copy_predict_to_ucoe")

    INDICATOR_U, INDICATOR_U_UT = 0, 1

    def set_indicator(self, mode: int):
        _ck(load().amdg_grid_set_indicator(self._h, mode), "grid_set_indicator")

    def copy_ucoe_ut_to_predict(self):
        _ck(load().amdg_grid_copy_ucoe_ut_to_predict(self._h), "grid_copy_ucoe_ut_to_predict")

    def copy_predict_to_ucoe_ut(self):
        _ck(load().amdg_grid_copy_predict_to_ucoe_ut(self._h), "grid_copy_predict_to_ucoe_ut")

    def init_separable(self, funcs, vectorized: bool = False):
        if vectorized:
            cb = _fn1d_batch(funcs)
            _ck(load().amdg_grid_init_separable_batch(self._h, len(funcs), cb, None), "grid_init_separable_batch")
        else:
            cb = _fn1d(funcs)
            _ck(load().amdg_grid_init_separable(self._h, len(funcs), cb, None), "grid_init_separable")

    def l2_norm_sq(self) -> float:
        r = C.c_double()
        _ck(load().amdg_grid_l2_norm(self._h, C.byref(r)), "grid_l2_norm")
        return r.value

    def l2_error_separable_sum(self, funcs, l2_norm_exact: float, vectorized: bool = False) -> float:
        r = C.c_double()
        if vectorized:
            cb = _fn1d_batch(funcs)
            _ck(load().amdg_grid_l2_error_separable_sum_batch(self._h, len(funcs), cb, None, l2_norm_exact,
                                                              C.byref(r)), "grid_l2_error_separable_sum_batch")
        else:
            cb = _fn1d(funcs)
            _ck(load().amdg_grid_l2_error_separable_sum(self._h, len(funcs), cb, None, l2_norm_exact, C.byref(r)),
                "grid_l2_error_separable_sum")
        return r.value

    def set_velocity(self, v: np.ndarray):
        v = np.ascontiguousarray(v, np.float64).reshape(-1)
        _ck(load().amdg_grid_set_velocity(self._h, _ptr(v), v.size), "grid_set_velocity")

    def velocity(self) -> np.ndarray:
        out = np.zeros((self.num_elements, self.block))
        _ck(load().amdg_grid_get_velocity(self._h, _ptr(out), out.size), "grid_get_velocity")
        return out

    def eval_tensor_device(self, x1d, d_out: int):
        """u_h on the tensor mesh x1d^dim into d_out (device, len(x1d)^dim doubles, last index fastest)."""
        x = np.ascontiguousarray(x1d, np.float64).reshape(-1)
        _ck(load().amdg_grid_eval_tensor(self._h, x.size, _ptr(x), C.c_void_p(d_out)), "grid_eval_tensor")

    def error_burgers(self, t: float, a: float = 0.5, b: float = 0.25, c: float = 0.0, gauss_points: int = 1):
        """(L1, L2, Linf) of u_h - u against the exact Burgers solution from a + b sin(2 pi (sum x + c))."""
        out = np.zeros(3)
        _ck(load().amdg_grid_error_burgers(self._h, a, b, c, t, gauss_points, _ptr(out)), "grid_error_burgers")
        return out

    def l2_error_separable(self, func, l2_norm_exact: float) -> float:
        cb = _fn1d([func])
        r = C.c_double()
        _ck(load().amdg_grid_l2_error_separable(self._h, cb, None, l2_norm_exact, C.byref(r)), "grid_l2_error_separable")
        return r.value

    def close(self):
        if self._h:
            load().amdg_grid_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class LinearOperator:
    """HyperbolicAlpt (upwind, constant coefficients) + RK3SSP on the device."""

    def __init__(self, grid: Grid, coef):
        self.grid = grid
        c = np.ascontiguousarray(coef, np.float64)
        assert c.size == grid.dim
        self._h = C.c_void_p()
        _ck(load().amdg_linear_create(grid.handle, _ptr(c), C.byref(self._h)), "linear_create")
        pairs, flops = C.c_int64(), C.c_double()
        _ck(load().amdg_linear_stats(self._h, C.byref(pairs), C.byref(flops)), "linear_stats")
        self.pairs, self.flops_per_apply = pairs.value, flops.value

    def tuning(self):
        """(variants[fp64, mixed], stage_ms[[fp64 v0 .. v3], [mixed v0 .. v3]]) chosen by the autotuner."""
        v = np.zeros(2, np.int32)
        ms = np.zeros(8, np.float32)
        _ck(load().amdg_linear_tuning(self._h, _ptr(v), _ptr(ms)), "linear_tuning")
        return v.tolist(), ms.reshape(2, 4).tolist()

    def set_variant(self, prec: int, variant: int):
        _ck(load().amdg_linear_set_variant(self._h, prec, variant), "linear_set_variant")

    def copy_config(self):
        """(configuration of the bulk-copy variant, stage ms per configuration)."""
        c = C.c_int()
        ms = np.zeros(8, np.float32)
        _ck(load().amdg_linear_copy_config(self._h, C.byref(c), _ptr(ms)), "linear_copy_config")
        return c.value, ms.tolist()

    def set_copy_config(self, config: int):
        _ck(load().amdg_linear_set_copy_config(self._h, config), "linear_set_copy_config")

    def set_wait_limit(self, polls: int):
        """Polls of the bulk-copy variant's waits (default 2**22; 0: give up at once, for tests)."""
        _ck(load().amdg_linear_set_wait_limit(self._h, polls), "linear_set_wait_limit")

    def apply_device(self, d_u: int, d_rhs: int, prec: int = FP64):
        _ck(load().amdg_linear_apply(self._h, C.c_void_p(d_u), C.c_void_p(d_rhs), prec), "linear_apply")

    def rk3_steps(self, dt: float, nsteps: int, prec: int = FP64):
        _ck(load().amdg_rk3ssp_steps(self._h, dt, nsteps, prec), "rk3ssp_steps")

    def rk3_steps_noalloc(self, d_u: int, dt: float, nsteps: int, prec: int = FP64):
        """RK3 steps on the caller's device vector without any device allocation."""
        _ck(load().amdg_rk3ssp_steps_noalloc(self._h, C.c_void_p(d_u), dt, nsteps, prec), "rk3ssp_steps_noalloc")

    def rk3_steps_host(self, u: np.ndarray, dt: float, nsteps: int, prec: int = FP64):
        assert u.dtype == np.float64 and u.flags.c_contiguous and u.size == self.grid.dof
        _ck(load().amdg_rk3ssp_steps_host(self._h, dt, nsteps, _ptr(u), prec), "rk3ssp_steps_host")

    def serve_host(self, inputs, outputs, dt: float, nsteps: int, prec: int = FP64):
        """Independent requests: inputs[r] (host, dof doubles) stepped into outputs[r], copies of
        neighbouring requests overlapped with the steps (pin the buffers for overlap)."""
        assert len(inputs) == len(outputs)
        for a in list(inputs) + list(outputs):
            assert a.dtype == np.float64 and a.flags.c_contiguous and a.size == self.grid.dof
        n = len(inputs)
        pin = (C.c_void_p * n)(*[a.ctypes.data for a in inputs])
        pout = (C.c_void_p * n)(*[a.ctypes.data for a in outputs])
        _ck(load().amdg_rk3ssp_serve_host(self._h, dt, nsteps, prec, n, pin, pout), "rk3ssp_serve_host")

    def close(self):
        if self._h:
            load().amdg_linear_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class BurgersOperator:
    """LagrInterpolation + HyperbolicLagrRHS + HyperbolicAlptRHS for the Burgers
    flux u^2/2 with global Lax-Friedrichs penalty alpha, on the device."""

    def __init__(self, grid: Grid, alpha, hermite: bool = False):
        """hermite=True: the flux interpolated by cubic Hermite interpolation (2D;
        HermInterpolation + HyperbolicSameFluxHermRHS, amdg_burgers_create_herm)."""
        self.grid = grid
        a = np.ascontiguousarray(np.broadcast_to(np.asarray(alpha, np.float64), (grid.dim,)))
        self._h = C.c_void_p()
        fn = load().amdg_burgers_create_herm if hermite else load().amdg_burgers_create
        _ck(fn(grid.handle, _ptr(a), C.byref(self._h)), "burgers_create_herm" if hermite else "burgers_create")
        self.points = 4 ** grid.dim

    def rhs_device(self, d_u: int, d_rhs: int, prec: int = FP64):
        _ck(load().amdg_burgers_rhs(self._h, C.c_void_p(d_u), C.c_void_p(d_rhs), prec), "burgers_rhs")

    RHS_VOL, RHS_FLX, RHS_PENALTY = 0, 1, 2

    def set_sweep_variant(self, variant: int):
        _ck(load().amdg_burgers_set_sweep_variant(self._h, variant), "burgers_set_sweep_variant")

    def work(self):
        """(flops, neighbour pairs) of one right-hand side on the current element set."""
        f, p = C.c_double(), C.c_double()
        _ck(load().amdg_burgers_work(self._h, C.byref(f), C.byref(p)), "burgers_work")
        return f.value, p.value

    def interpolate(self, prec: int = FP64):
        """LagrInterpolation::nonlinear_Lagr_fast for u^2/2 on the grid's coefficients."""
        _ck(load().amdg_lagr_interpolate(self._h, prec), "lagr_interpolate")

    def rhs_add(self, group: int, alpha=None, prec: int = FP64):
        """Add one term group (RHS_VOL / RHS_FLX / RHS_PENALTY) into the grid's Element::rhs."""
        a = None if alpha is None else np.ascontiguousarray(
            np.broadcast_to(np.asarray(alpha, np.float64), (self.grid.dim,)))
        _ck(load().amdg_lagr_rhs_add(self._h, group, None if a is None else _ptr(a), prec), "lagr_rhs_add")

    def point_values_device(self, d_u: int, d_up: int, prec: int = FP64):
        _ck(load().amdg_burgers_point_values(self._h, C.c_void_p(d_u), C.c_void_p(d_up), prec), "burgers_point_values")

    def flux_coefficients_device(self, d_u: int, d_fu: int, prec: int = FP64):
        _ck(load().amdg_burgers_flux_coefficients(self._h, C.c_void_p(d_u), C.c_void_p(d_fu), prec),
            "burgers_flux_coefficients")

    def rk3_steps(self, dt: float, nsteps: int, prec: int = FP64):
        _ck(load().amdg_burgers_rk3_steps(self._h, dt, nsteps, prec), "burgers_rk3_steps")

    def adaptive_step_ex(self, cfl: float, wave_speed: float, eps: float, eta: float, prec: int = FP64):
        """Adaptive step that also returns the surplus criterion's decision per old element (0 keep, 1 refine, 2 coarsen)."""
        dec = np.zeros(self.grid.num_elements, np.int8)
        dt = C.c_double()
        _ck(load().amdg_burgers_adaptive_step_ex(self._h, cfl, wave_speed, eps, eta, prec, C.byref(dt), _ptr(dec)),
            "burgers_adaptive_step_ex")
        self.grid._refresh()
        return dt.value, dec

    def features_device(self, d_u: int, d_feat: int):
        _ck(load().amdg_burgers_features(self._h, C.c_void_p(d_u), C.c_void_p(d_feat)), "burgers_features")

    def adaptive_step_learned(self, mlp, cfl: float, wave_speed: float, eps: float, eta: float, tau: float,
                              prec: int = FP64):
        stats = np.zeros(4, np.int64)
        dt = C.c_double()
        _ck(load().amdg_burgers_adaptive_step_learned(self._h, mlp.handle if mlp is not None else None, cfl, wave_speed, eps, eta, tau, prec,
                                                      C.byref(dt), _ptr(stats)), "burgers_adaptive_step_learned")
        self.grid._refresh()
        return dt.value, stats

    def adaptive_steps_learned(self, mlp, cfl: float, wave_speed: float, eps: float, eta: float, tau: float,
                               horizon: int, t_left: float = 0.0, prec: int = FP64):
        """(time advanced, steps taken, stats) of one learned pre-adaptation and `horizon` steps."""
        stats = np.zeros(4, np.int64)
        ta, n = C.c_double(), C.c_int()
        _ck(load().amdg_burgers_adaptive_steps_learned(self._h, mlp.handle if mlp is not None else None, cfl, wave_speed, eps, eta, tau, prec,
                                                       horizon, t_left, C.byref(ta), C.byref(n), _ptr(stats)),
            "burgers_adaptive_steps_learned")
        self.grid._refresh()
        return ta.value, n.value, stats

    def counters(self):
        """(RK-stage DOF updates, right-hand-side evaluations) since creation."""
        a, b = C.c_int64(), C.c_int64()
        _ck(load().amdg_burgers_counters(self._h, C.byref(a), C.byref(b)), "burgers_counters")
        return a.value, b.value

    def adaptive_step(self, cfl: float, wave_speed: float, eps: float, eta: float, prec: int = FP64) -> float:
        dt = C.c_double()
        _ck(load().amdg_burgers_adaptive_step(self._h, cfl, wave_speed, eps, eta, prec, C.byref(dt)),
            "burgers_adaptive_step")
        self.grid._refresh()
        return dt.value

    def close(self):
        if self._h:
            load().amdg_burgers_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class WaveOperator:
    """u_tt = div(K grad u), K = (1 + amplitude prod sin(2 pi x_d))^2, interpolated K grad u and K u,
    DiffusionRHS terms and the IPDG penalty (sigma), on the device."""

    def __init__(self, grid: Grid, sigma: float, amplitude: float = 0.5):
        self.grid = grid
        self._h = C.c_void_p()
        _ck(load().amdg_wave_create(grid.handle, sigma, amplitude, C.byref(self._h)), "wave_create")

    def rhs_device(self, d_u: int, d_rhs: int, prec: int = FP64):
        _ck(load().amdg_wave_rhs(self._h, C.c_void_p(d_u), C.c_void_p(d_rhs), prec), "wave_rhs")

    def set_sweep_variant(self, variant: int):
        _ck(load().amdg_wave_set_sweep_variant(self._h, variant), "wave_set_sweep_variant")

    INTERP_GRADU, INTERP_U = 0, 1
    RHS_FLX_GRADU, RHS_VOL, RHS_FLX_U, RHS_IPDG = 0, 1, 2, 3

    def set_sigma(self, sigma: float):
        _ck(load().amdg_wave_set_sigma(self._h, sigma), "wave_set_sigma")

    def interpolate(self, which: int, prec: int = FP64):
        """LagrInterpolation::var_coeff_gradu_Lagr_fast (INTERP_GRADU) / var_coeff_u_Lagr_fast (INTERP_U)."""
        _ck(load().amdg_wave_interpolate(self._h, which, prec), "wave_interpolate")

    def rhs_add(self, group: int, prec: int = FP64):
        """DiffusionRHS::rhs_flx_gradu / rhs_vol / rhs_flx_u or the IPDG term, added into the grid's rhs."""
        _ck(load().amdg_wave_rhs_add(self._h, group, prec), "wave_rhs_add")

    def rk4_steps(self, dt: float, nsteps: int, prec: int = FP64):
        _ck(load().amdg_wave_rk4_steps(self._h, dt, nsteps, prec), "wave_rk4_steps")

    def adaptive_step(self, cfl: float, wave_speed: float, eps: float, eta: float, prec: int = FP64) -> float:
        dt = C.c_double()
        _ck(load().amdg_wave_adaptive_step(self._h, cfl, wave_speed, eps, eta, prec, C.byref(dt)),
            "wave_adaptive_step")
        self.grid._refresh()
        return dt.value

    def counters(self):
        a, b = C.c_int64(), C.c_int64()
        _ck(load().amdg_wave_counters(self._h, C.byref(a), C.byref(b)), "wave_counters")
        return a.value, b.value

    def adaptive_step_ex(self, cfl: float, wave_speed: float, eps: float, eta: float, prec: int = FP64):
        """Adaptive step that also returns the criterion's decision per old element (0 keep, 1 refine, 2 coarsen)."""
        dec = np.zeros(self.grid.num_elements, np.int8)
        dt = C.c_double()
        _ck(load().amdg_wave_adaptive_step_ex(self._h, cfl, wave_speed, eps, eta, prec, C.byref(dt), _ptr(dec)),
            "wave_adaptive_step_ex")
        self.grid._refresh()
        return dt.value, dec

    @property
    def num_features(self) -> int:
        """Classifier inputs per element: the features of u followed by those of u_t."""
        return 2 * self.grid.block * (1 + 2 * self.grid.dim)

    def features_device(self, d_u: int, d_feat: int):
        _ck(load().amdg_wave_features(self._h, C.c_void_p(d_u), C.c_void_p(d_feat)), "wave_features")

    def adaptive_step_learned(self, mlp, cfl: float, wave_speed: float, eps: float, eta: float, tau: float,
                              prec: int = FP64):
        stats = np.zeros(4, np.int64)
        dt = C.c_double()
        _ck(load().amdg_wave_adaptive_step_learned(self._h, mlp.handle if mlp is not None else None, cfl, wave_speed, eps, eta, tau, prec,
                                                   C.byref(dt), _ptr(stats)), "wave_adaptive_step_learned")
        self.grid._refresh()
        return dt.value, stats

    def adaptive_steps_learned(self, mlp, cfl: float, wave_speed: float, eps: float, eta: float, tau: float,
                               horizon: int, t_left: float = 0.0, prec: int = FP64):
        stats = np.zeros(4, np.int64)
        ta, n = C.c_double(), C.c_int()
        _ck(load().amdg_wave_adaptive_steps_learned(self._h, mlp.handle if mlp is not None else None, cfl, wave_speed, eps, eta, tau, prec,
                                                    horizon, t_left, C.byref(ta), C.byref(n), _ptr(stats)),
            "wave_adaptive_steps_learned")
        self.grid._refresh()
        return ta.value, n.value, stats

    def close(self):
        if self._h:
            load().amdg_wave_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class ODE:
    """ForwardEuler / RK3SSP / EulerODE2nd / RK4ODE2nd (ODESolver) on a grid's device state, stage by stage."""
    FORWARD_EULER, RK3SSP, EULER_ODE2ND, RK4ODE2ND = 0, 1, 2, 3

    def __init__(self, grid: Grid, scheme: int, dt: float):
        self._h = C.c_void_p()
        _ck(load().amdg_ode_create(grid.handle, scheme, dt, C.byref(self._h)), "ode_create")

    def set_rhs_zero(self):
        _ck(load().amdg_ode_set_rhs_zero(self._h), "ode_set_rhs_zero")

    def add_rhs_to_eigenvec(self):
        _ck(load().amdg_ode_add_rhs_to_eigenvec(self._h), "ode_add_rhs_to_eigenvec")

    def step_stage(self, stage: int):
        _ck(load().amdg_ode_step_stage(self._h, stage), "ode_step_stage")

    def final(self):
        _ck(load().amdg_ode_final(self._h), "ode_final")

    def add_wave_penalty(self, op):
        """RKODE2nd::add_rhs_matrix: the solver's rhs += the IPDG term of the grid's current u."""
        _ck(load().amdg_ode_add_wave_penalty(self._h, op._h), "ode_add_wave_penalty")

    def close(self):
        if self._h:
            load().amdg_ode_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Independent constant-coefficient solves advanced together (one launch per RK stage)."""

    def __init__(self, ctx: Context, grids, coef):
        self.ctx, self.grids = ctx, list(grids)
        arr = (C.c_void_p * len(self.grids))(*[g.handle.value for g in self.grids])
        c = np.ascontiguousarray(coef, np.float64).reshape(len(self.grids), -1)
        self._h = C.c_void_p()
        _ck(load().amdg_batch_create(ctx.handle, len(self.grids), arr, _ptr(c), C.byref(self._h)), "batch_create")
        ne, dof, pairs = C.c_int64(), C.c_int64(), C.c_int64()
        _ck(load().amdg_batch_size(self._h, C.byref(ne), C.byref(dof), C.byref(pairs)), "batch_size")
        self.num_elements, self.dof, self.pairs = ne.value, dof.value, pairs.value

    def set_dt(self, dt):
        a = np.ascontiguousarray(dt, np.float64)
        _ck(load().amdg_batch_set_dt(self._h, _ptr(a)), "batch_set_dt")

    def rk3_steps(self, nsteps: int, prec: int = FP64, use_graph: bool = True):
        _ck(load().amdg_batch_rk3_steps(self._h, nsteps, prec, int(use_graph)), "batch_rk3_steps")

    def store(self, solve: int):
        _ck(load().amdg_batch_store(self._h, solve), "batch_store")

    def adapt(self, eps: float, eta: float, mlp=None, tau: float = 0.8):
        """Refine (criterion, or classifier + criterion) and coarsen every solve's grid, then rebuild
        the batch; returns [refined by the classifier, uncertain, elements after]."""
        stats = np.zeros(3, np.int64)
        _ck(load().amdg_batch_adapt(self._h, mlp.handle if mlp is not None else None, eps, eta, tau, _ptr(stats)),
            "batch_adapt")
        ne, dof, pairs = C.c_int64(), C.c_int64(), C.c_int64()
        _ck(load().amdg_batch_size(self._h, C.byref(ne), C.byref(dof), C.byref(pairs)), "batch_size")
        self.num_elements, self.dof, self.pairs = ne.value, dof.value, pairs.value
        for g in self.grids:
            g._refresh()
        return stats

    # stage-kernel candidates: the column kernel at these CTA sizes, then the bulk-copy ring kernel
    # (mixed only) in these (ring slots, elements per CTA) configurations, then the warp-per-element
    # kernel (mixed only) in these (warps per CTA, schedule) configurations
    TILES = (64, 128, 256, 512, 1024)
    RING_CONFIGS = ((1, 1), (1, 2), (1, 4), (2, 1), (2, 2), (2, 4))
    PERSIST_CONFIGS = ((64, "static tile order"), (128, "static tile order"), (64, "tiles from a counter"))
    WARP_CONFIGS = ((8, "one CTA per 8 elements"),)
    DF_COLUMN_FIRST = len(TILES)       # the column kernel on the FP32-pair state (mixed)
    RING_FIRST = 2 * len(TILES)        # the bulk-copy ring kernel (mixed)
    PERSIST_FIRST = RING_FIRST + len(RING_CONFIGS)  # the column kernel, persistent (mixed)
    WARP_FIRST = PERSIST_FIRST + len(PERSIST_CONFIGS)  # the warp-per-element kernel (mixed)
    KERNELS = WARP_FIRST + len(WARP_CONFIGS)

    @classmethod
    def kernel_name(cls, c: int) -> str:
        if c < cls.DF_COLUMN_FIRST:
            return f"column {cls.TILES[c]} threads"
        if c < cls.RING_FIRST:
            return f"column {cls.TILES[c - cls.DF_COLUMN_FIRST]} threads, FP32-pair state"
        if c < cls.PERSIST_FIRST:
            r, w = cls.RING_CONFIGS[c - cls.RING_FIRST]
            return f"bulk-copy ring {r} slot{'s' if r > 1 else ''}, {w} element{'s' if w > 1 else ''} per CTA"
        if c < cls.WARP_FIRST:
            t, sched = cls.PERSIST_CONFIGS[c - cls.PERSIST_FIRST]
            return f"column {t} threads, FP32-pair state, persistent, {sched}"
        w, sched = cls.WARP_CONFIGS[c - cls.WARP_FIRST]
        return f"warp per element, {w} warps per CTA, {sched}"

    def tuning(self):
        """(stage-kernel candidate per precision [FP64, mixed], stage ms per candidate [2][KERNELS])."""
        k = np.zeros(2, np.int32)
        ms = np.zeros(2 * self.KERNELS, np.float32)
        _ck(load().amdg_batch_tuning(self._h, _ptr(k), _ptr(ms)), "batch_tuning")
        return k.tolist(), ms.reshape(2, self.KERNELS).tolist()

    def set_kernel(self, prec: int, kernel: int):
        _ck(load().amdg_batch_set_kernel(self._h, prec, kernel), "batch_set_kernel")

    def set_tile(self, prec: int, threads: int):
        _ck(load().amdg_batch_set_tile(self._h, prec, threads), "batch_set_tile")

    def close(self):
        if self._h:
            load().amdg_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class MLP:
    """Per-element refine/keep/coarsen classifier trained and run by the library's own kernels."""

    def __init__(self, ctx: Context, n_in: int, hidden: int = 64, n_hidden_layers: int = 3, n_out: int = 3, seed: int = 0):
        self.ctx = ctx
        self.dims = [n_in] + [hidden] * n_hidden_layers + [n_out]
        self._h = C.c_void_p()
        _ck(load().amdg_mlp_create(ctx.handle, n_in, hidden, n_hidden_layers, n_out, seed, C.byref(self._h)), "mlp_create")
        n = C.c_int64()
        _ck(load().amdg_mlp_num_params(self._h, C.byref(n)), "mlp_num_params")
        self.num_params = n.value

    @property
    def handle(self):
        return self._h

    def params(self) -> np.ndarray:
        p = np.zeros(self.num_params, np.float32)
        _ck(load().amdg_mlp_get_params(self._h, _ptr(p), p.size), "mlp_get_params")
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        _ck(load().amdg_mlp_set_params(self._h, _ptr(p), p.size), "mlp_set_params")

    def predict_device(self, d_x: int, n: int, d_probs: int):
        _ck(load().amdg_mlp_predict(self._h, C.c_void_p(d_x), n, C.c_void_p(d_probs)), "mlp_predict")

    def loss_grad_device(self, d_x: int, d_labels: int, n: int):
        g = np.zeros(self.num_params, np.float32)
        loss = C.c_double()
        _ck(load().amdg_mlp_loss_grad(self._h, C.c_void_p(d_x), C.c_void_p(d_labels), n, C.byref(loss), _ptr(g)),
            "mlp_loss_grad")
        return loss.value, g

    def train_device(self, d_x: int, d_labels: int, n: int, epochs: int, batch: int, lr: float, seed: int = 0) -> float:
        loss = C.c_double()
        _ck(load().amdg_mlp_train(self._h, C.c_void_p(d_x), C.c_void_p(d_labels), n, epochs, batch, lr, seed,
                                  C.byref(loss)), "mlp_train")
        return loss.value

    def close(self):
        if self._h:
            load().amdg_mlp_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
