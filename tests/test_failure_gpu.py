"""Failure detection without a GPU fault: a bounded device-side wait made to give up at once must
come back as AMDG_ERR_TIMEOUT with the state left as it was, and device allocations made to fail
must come back as AMDG_ERR_NOMEM, with the library usable afterwards."""
import numpy as np
import pytest

import amdg
import amdg_oracle as O

pytestmark = pytest.mark.gpu

TIMEOUT, NOMEM = 4, 7


def test_bulk_copy_wait_timeout_reports_and_leaves_the_state(ctx):
    """The bulk-copy linear kernel with a wait limit of 0 polls: every warp's first wait gives up,
    the kernel drains the copies it issued (their own bound) and returns without writing; the call
    fails with AMDG_ERR_TIMEOUT and the coefficients are bitwise unchanged.  With the default
    limit restored the same step succeeds and equals a step of a fresh operator."""
    g = amdg.Grid(ctx, 3, 6, 2)
    g.init_separable(O.sin_sum_terms(3))
    u0 = g.coefficients().copy()
    op = amdg.LinearOperator(g, [1.0, -0.5, 0.25])
    op.set_variant(amdg.MIXED, 2)
    op.set_wait_limit(0)
    with pytest.raises(amdg.AmdgError) as ei:
        op.rk3_steps(1e-3, 1, amdg.MIXED)
    assert ei.value.status == TIMEOUT
    ctx.synchronize()
    assert np.array_equal(g.coefficients(), u0)
    op.set_wait_limit(1 << 22)
    op.rk3_steps(1e-3, 1, amdg.MIXED)
    ctx.synchronize()
    stepped = g.coefficients().copy()
    g.set_coefficients(u0)
    op2 = amdg.LinearOperator(g, [1.0, -0.5, 0.25])
    op2.set_variant(amdg.MIXED, 2)
    op2.rk3_steps(1e-3, 1, amdg.MIXED)
    ctx.synchronize()
    assert np.array_equal(g.coefficients(), stepped)
    op.close()
    op2.close()
    g.close()


def test_device_allocation_failure_reports_nomem(ctx):
    """Every device allocation made to fail: grid, operator and classifier creation report
    AMDG_ERR_NOMEM (not a CUDA error, not a crash); after some successful allocations the failure
    surfaces from a later call the same way; with the hook off the library works again."""
    lib = amdg.load()
    try:
        lib.amdg_debug_fail_device_allocations(0)
        with pytest.raises(amdg.AmdgError) as ei:
            amdg.Grid(ctx, 2, 5, 2)
        assert ei.value.status == NOMEM
        with pytest.raises(amdg.AmdgError) as ei:
            amdg.MLP(ctx, 45, 64, 3, 3, seed=1)
        assert ei.value.status == NOMEM
        lib.amdg_debug_fail_device_allocations(-1)
        g = amdg.Grid(ctx, 2, 5, 2, level_init=3)
        g.init_separable_adaptive(O.burgers_ic_terms(2), 1e-4)
        # the operator's own allocations fail part-way
        for after in (0, 3, 9):
            lib.amdg_debug_fail_device_allocations(after)
            with pytest.raises(amdg.AmdgError) as ei:
                amdg.BurgersOperator(g, 0.825)
            assert ei.value.status == NOMEM, after
        lib.amdg_debug_fail_device_allocations(-1)
        op = amdg.BurgersOperator(g, 0.825)
        op.adaptive_step(0.1, 0.75, 1e-4, 1e-5)
        ctx.synchronize()
        assert np.all(np.isfinite(g.coefficients()))
        op.close()
        g.close()
    finally:
        lib.amdg_debug_fail_device_allocations(-1)
