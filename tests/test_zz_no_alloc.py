"""The allocation-free RK3 entry point (amdg_rk3ssp_steps_noalloc).

Some callers of this library cannot allocate device memory -- host callbacks,
processes whose device memory belongs to another allocator, loops that must
not allocate -- so the library offers one RK3
stepping call whose stage vectors sit in a fixed device array instead of in
cudaMalloc'ed memory.  This file checks it through the C-ABI against the
allocating entry point (amdg_rk3ssp_steps) on two calls in a row, with the
FP64 tolerance of the other linear-operator tests.  It is collected last on
purpose, so that a run stopping at the first failure has run everything else.
"""
import math

import numpy as np
import pytest

import amdg

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL_MIXED = 1e-6  # mixed mode: the allocating path keeps its stage vectors as FP32 pairs


def _max_rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


@pytest.mark.parametrize("prec", [amdg.FP64, amdg.MIXED])
def test_noalloc_matches_allocating_steps(prec):
    ctx = amdg.Context(0)
    dim, N = 3, 8  # 110,592 coefficients, within the 262,144 limit
    g = amdg.Grid(ctx, dim, N, 2)
    g.init_separable([lambda x, d: math.sin(2 * math.pi * x)])
    u0 = g.coefficients().copy()
    op = amdg.LinearOperator(g, [1.0, -0.5, 0.75])
    caller = amdg.Grid(ctx, dim, N, 2)  # the caller's own device vector
    caller.set_coefficients(u0)
    dt = 0.1 / 256 / 3
    for call in range(2):
        op.rk3_steps(dt, 2, prec)
        op.rk3_steps_noalloc(caller.device_ptr(), dt, 2, prec)
        ctx.synchronize()
        want = g.coefficients()
        got = caller.coefficients()
        assert _max_rel(got, want) < (TOL64 if prec == amdg.FP64 else TOL_MIXED), f"call {call}"
    caller.close()
    op.close()
    g.close()


def test_noalloc_rejects_grids_beyond_its_capacity():
    ctx = amdg.Context(0)
    g = amdg.Grid(ctx, 4, 8, 2)  # 850,176 coefficients
    op = amdg.LinearOperator(g, [1.0] * 4)
    with pytest.raises(amdg.AmdgError) as ei:
        op.rk3_steps_noalloc(g.device_ptr(), 1e-4, 1)
    assert ei.value.status == 2
    assert b"262144" in amdg.load().amdg_last_error()
    op.close()
    g.close()
