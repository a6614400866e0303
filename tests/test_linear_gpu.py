"""Parity of the CUDA linear sparse-grid DG operator (C-ABI) with the oracle
and the reference fixtures.  Tolerances: FP64 path 1e-12 relative (max-norm
relative to the field's max), mixed path (FP32 operator apply, FP64 state)
2e-6 relative for one apply and 1e-6 for RK3 steps."""
import math

import numpy as np
import pytest

import amdg
import amdg_oracle as O
from helpers import align, golden, ic_terms, manifest, rel_err

pytestmark = pytest.mark.gpu

LINEAR = [n for n, m in manifest().items() if m["kind"] == "linear"]
TOL64 = 1e-12
TOL_MIXED_APPLY = 2e-6
TOL_MIXED_STEP = 1e-6


def _device_apply(ctx, op, grid, u, prec):
    """rhs = L u through the C-ABI, using the grid's state buffer as input."""
    grid.set_coefficients(u)
    keep = grid.coefficients().copy()
    # second device buffer: a scratch grid of the same shape holds the rhs
    out = amdg.Grid(ctx, grid.dim, grid.nmax, grid.k, grid.sparse)
    op.apply_device(grid.device_ptr(), out.device_ptr(), prec)
    ctx.synchronize()
    rhs = out.coefficients().copy()
    out.close()
    assert np.array_equal(keep, grid.coefficients())
    return rhs


@pytest.mark.parametrize("name", LINEAR)
def test_linear_matches_reference(ctx, name):
    m = manifest()[name]
    z = golden(name)
    dim, N, k = m["dim"], m["N"], m["k"]
    g = amdg.Grid(ctx, dim, N, k)
    lv, sp = g.elements()
    perm = align(z["level"], z["suppt"], lv, sp)
    g.init_separable(ic_terms(m["ic"], dim))
    assert rel_err(g.coefficients(), z["u0"][perm]) < 1e-13
    op = amdg.LinearOperator(g, m["c"])
    u0 = np.ascontiguousarray(z["u0"][perm])
    rhs = _device_apply(ctx, op, g, u0, amdg.FP64)
    assert rel_err(rhs, z["rhs0"][perm]) < TOL64
    rhs32 = _device_apply(ctx, op, g, u0, amdg.MIXED)
    assert rel_err(rhs32, z["rhs0"][perm]) < TOL_MIXED_APPLY
    g.set_coefficients(u0)
    op.rk3_steps(m["dt"], m["steps"], amdg.FP64)
    ctx.synchronize()
    assert rel_err(g.coefficients(), z["uT"][perm]) < TOL64
    g.set_coefficients(u0)
    op.rk3_steps(m["dt"], m["steps"], amdg.MIXED)
    ctx.synchronize()
    assert rel_err(g.coefficients(), z["uT"][perm]) < TOL_MIXED_STEP
    op.close()
    g.close()


LONG = [n for n, m in manifest().items() if m["kind"] == "linear_long"]


@pytest.mark.parametrize("name", LONG)
def test_linear_full_length_matches_reference(ctx, name):
    """The 2D linear advection case over its whole length (full sparse grid N = 7, 2561 SSP-RK3
    steps of 1/2561 to T = 1) against the reference run: FP64 coefficients to 1e-12 relative, the
    L1/L2/Linf errors against the exact translated solution (2 Gauss points) to 1e-9 relative; the
    mixed path's coefficients to 1e-6 and its L2 error within 1 % of the reference's."""
    m = manifest()[name]
    z = golden(name)
    dim, N, k = m["dim"], m["N"], m["k"]
    g = amdg.Grid(ctx, dim, N, k)
    lv, sp = g.elements()
    perm = align(z["level"], z["suppt"], lv, sp)
    g.init_separable(ic_terms(m["ic"], dim))
    u0 = g.coefficients().copy()
    assert rel_err(u0, z["u0"][perm]) < 1e-13
    op = amdg.LinearOperator(g, m["c"])
    T = m["steps"] * m["dt"]
    shift = -sum(m["c"]) * T
    for prec, tol, etol in ((amdg.FP64, TOL64, 1e-9), (amdg.MIXED, TOL_MIXED_STEP, 1e-2)):
        g.set_coefficients(u0)
        op.rk3_steps(m["dt"], m["steps"], prec)
        ctx.synchronize()
        assert rel_err(g.coefficients(), z["uT"][perm]) < tol
        err = g.error_burgers(0.0, a=0.0, b=1.0, c=shift, gauss_points=2)
        ref = z["normerr_g2"]
        assert np.all(np.abs(err - ref) <= etol * np.abs(ref)), (prec, err, ref)
    op.close()
    g.close()


@pytest.mark.parametrize("dim,N,k,c", [(1, 6, 2, [1.0]), (2, 5, 2, [0.0, 1.0]), (3, 5, 3, [-1.0, 0.5, 2.0]),
                                       (5, 4, 1, [1.0, -1.0, 1.0, -1.0, 1.0]), (2, 4, 2, [1.0, 1.0])])
def test_random_state_matches_oracle(ctx, dim, N, k, c):
    g = amdg.Grid(ctx, dim, N, k)
    lv, sp = g.elements()
    rng = np.random.default_rng(dim * 100 + N)
    u = rng.standard_normal((g.num_elements, g.block))
    op = amdg.LinearOperator(g, c)
    rhs = _device_apply(ctx, op, g, u, amdg.FP64)
    ref = O.linear_rhs(dim, N, k, lv, sp, c, u)
    assert rel_err(rhs, ref) < TOL64
    g.set_coefficients(u)
    op.rk3_steps(1e-3, 2, amdg.FP64)
    ctx.synchronize()
    ref2 = O.linear_rk3(dim, N, k, lv, sp, c, u, 1e-3, 2)
    assert rel_err(g.coefficients(), ref2) < TOL64


def test_full_grid(ctx):
    g = amdg.Grid(ctx, 2, 4, 2, sparse=False)
    lv, sp = g.elements()
    assert g.num_elements == 256
    u = np.random.default_rng(5).standard_normal((g.num_elements, g.block))
    op = amdg.LinearOperator(g, [1.0, -1.0])
    rhs = _device_apply(ctx, op, g, u, amdg.FP64)
    assert rel_err(rhs, O.linear_rhs(2, 4, 2, lv, sp, [1.0, -1.0], u)) < TOL64


def test_4d_n8_one_step_full_compare(ctx):
    dim, N, k, c = 4, 8, 2, [1.0] * 4
    g = amdg.Grid(ctx, dim, N, k)
    lv, sp = g.elements()
    assert g.num_elements == 10496 and g.dof == 850176
    g.init_separable([lambda x, d: math.sin(2 * math.pi * x)])
    u0 = g.coefficients().copy()
    op = amdg.LinearOperator(g, c)
    dt = 0.1 / 256 / 4
    op.rk3_steps(dt, 1, amdg.FP64)
    ctx.synchronize()
    ref = O.linear_rk3(dim, N, k, lv, sp, c, u0, dt, 1)
    assert rel_err(g.coefficients(), ref) < TOL64


def test_6d_n8_sampled_parity_and_properties(ctx):
    """Config-2 size (34,455,456 DOF): rhs parity on sampled element ranges,
    linearity, determinism and host/device step equivalence."""
    dim, N, k, c = 6, 8, 2, [1.0] * 6
    g = amdg.Grid(ctx, dim, N, k)
    assert g.num_elements == 47264 and g.dof == 34455456
    lv, sp = g.elements()
    g.init_separable([lambda x, d: math.sin(2 * math.pi * x)])
    u0 = g.coefficients().copy()
    op = amdg.LinearOperator(g, c)
    out = amdg.Grid(ctx, dim, N, k)
    op.apply_device(g.device_ptr(), out.device_ptr(), amdg.FP64)
    ctx.synchronize()
    rhs = out.coefficients().copy()
    oop = O.LinearOp(dim, N, k, lv, sp, c)
    scale = np.abs(rhs).max()  # relative to the field's max norm, as for the smaller cases
    for e0 in (0, 1000, 23000, 47000):
        e1 = min(e0 + 264, g.num_elements)
        ref = oop.apply_range(u0, e0, e1)
        assert np.abs(rhs[e0:e1] - ref).max() < TOL64 * scale
    # determinism: a second apply is bitwise identical
    op.apply_device(g.device_ptr(), out.device_ptr(), amdg.FP64)
    ctx.synchronize()
    assert np.array_equal(out.coefficients(), rhs)
    # linearity: L(2u) = 2 L(u) exactly in binary floating point
    g.set_coefficients(2.0 * u0)
    op.apply_device(g.device_ptr(), out.device_ptr(), amdg.FP64)
    ctx.synchronize()
    assert np.array_equal(out.coefficients(), 2.0 * rhs)
    # host-buffer step equals device step
    dt = 0.1 * (1.0 / 256) / 6
    g.set_coefficients(u0)
    op.rk3_steps(dt, 1, amdg.FP64)
    ctx.synchronize()
    dev = g.coefficients().copy()
    host = np.ascontiguousarray(u0.reshape(-1))
    op.rk3_steps_host(host, dt, 1, amdg.FP64)
    assert np.array_equal(host.reshape(dev.shape), dev)
    # L2 error vs the exact translated solution stays at the discretisation level
    T = dt
    err = g.l2_error_separable(lambda x, d: math.sin(2 * math.pi * (x - T)), 0.5 ** 3)
    err0_ex = O.project_separable(N, k, dim, [lambda x, d: math.sin(2 * math.pi * (x - T))])[0]
    ref_err = O.l2_error_split(dim, N, k, lv, sp, dev, err0_ex, 0.5 ** 3)
    # the split formula sqrt(|u|^2 + sum(u_h^2 - 2 u_h c)) cancels ~0.125 down to err^2 ~ 4e-9,
    # so summation order alone moves err by ~1e-7 relative
    assert abs(err - ref_err) <= 1e-6 * ref_err
    oop.close()
    out.close()
    op.close()
    g.close()


def test_stage_update_matches_formula(ctx):
    g = amdg.Grid(ctx, 2, 3, 2)
    rng = np.random.default_rng(3)
    n = g.dof
    un, u, rhs = (rng.standard_normal(n) for _ in range(3))
    bufs = [amdg.Grid(ctx, 2, 3, 2) for _ in range(3)]
    for b, v in zip(bufs, (un, u, rhs)):
        b.set_coefficients(v)
    dt = 0.01
    ctx.stage_update(1, dt, bufs[0].device_ptr(), bufs[1].device_ptr(), bufs[2].device_ptr(), n)
    ctx.synchronize()
    got = bufs[1].coefficients().reshape(-1)
    want = 3. / 4. * un + 1. / 4. * (u + dt * rhs)
    assert np.array_equal(got, want)


def test_l2_norm_and_launch_count(ctx):
    g = amdg.Grid(ctx, 3, 4, 2)
    u = np.random.default_rng(9).standard_normal(g.dof)
    g.set_coefficients(u)
    before = ctx.launch_count()
    s = g.l2_norm_sq()
    assert ctx.launch_count() == before + 2
    assert abs(s - float(np.dot(u, u))) <= 1e-12 * s


def test_nonfinite_norm_reports_status(ctx):
    g = amdg.Grid(ctx, 2, 3, 2)
    u = np.zeros(g.dof)
    u[7] = np.nan
    g.set_coefficients(u)
    with pytest.raises(amdg.AmdgError) as ei:
        g.l2_norm_sq()
    assert ei.value.status == 3


def test_kernel_variants_agree_on_mixed_steps(ctx):
    """The three mixed-precision kernels (thread per output, column, column fed
    by bulk asynchronous copies) sum in the same order per output, so two SSP-RK3
    steps agree to rounding of the stage update (1e-14 relative)."""
    dim, N, k = 4, 6, 2
    g = amdg.Grid(ctx, dim, N, k)
    g.init_separable([lambda x, d: math.sin(2 * math.pi * x) + 0.3 * math.cos(6 * math.pi * x)])
    u0 = g.coefficients().copy()
    op = amdg.LinearOperator(g, [1.0, -0.5, 0.25, 0.75])
    out = {}
    for v in (0, 1, 2):
        g.set_coefficients(u0)
        op.rk3_steps(1e-3, 1, amdg.MIXED)  # builds the operator (the autotuner may pick any variant)
        g.set_coefficients(u0)
        op.set_variant(amdg.MIXED, v)
        op.rk3_steps(1e-3, 2, amdg.MIXED)
        ctx.synchronize()
        out[v] = g.coefficients().copy()
    ref = np.abs(out[1]).max()
    assert np.abs(out[2] - out[1]).max() <= 1e-14 * ref
    assert np.abs(out[0] - out[1]).max() <= 1e-6 * ref
    # the bulk-copy variant's configurations (ring depth, operator-block source) agree bitwise
    op.set_variant(amdg.MIXED, 2)
    for cfg in range(8):
        g.set_coefficients(u0)
        op.set_copy_config(cfg)
        op.rk3_steps(1e-3, 2, amdg.MIXED)
        ctx.synchronize()
        assert np.array_equal(g.coefficients(), out[2]), f"copy configuration {cfg}"
    with pytest.raises(amdg.AmdgError):
        op.set_copy_config(8)
    with pytest.raises(amdg.AmdgError):
        op.set_variant(amdg.FP64, 2)
    op.close()
    g.close()


@pytest.mark.parametrize("dim,N,k,c", [(3, 6, 2, [1.0, -0.5, 0.25]), (4, 6, 2, [1.0, -0.5, 0.25, 0.75]),
                                       (2, 7, 1, [0.7, -1.3]), (3, 5, 3, [-1.0, 0.5, 2.0])])
def test_tensor_core_variant_matches_oracle(ctx, dim, N, k, c):
    """Variant 3 (the bulk-copy ring with the contraction as 3xTF32 mma.sync, FP32 accumulation)
    against the oracle: two mixed SSP-RK3 steps of a random state to 1e-6 relative, and to 1e-6 of
    the FP32 column variant, whose sums run in another order (k = 1, 2, 3: 4, 2 and 2 neighbours
    per k8 step)."""
    g = amdg.Grid(ctx, dim, N, k)
    lv, sp = g.elements()
    rng = np.random.default_rng(dim * 10 + N)
    u0 = rng.standard_normal((g.num_elements, g.block))
    op = amdg.LinearOperator(g, c)
    dt = 1e-3
    ref = O.linear_rk3(dim, N, k, lv, sp, c, u0, dt, 2)
    g.set_coefficients(u0)
    op.rk3_steps(dt, 1, amdg.MIXED)  # builds the operator
    out = {}
    for v in (1, 3):
        op.set_variant(amdg.MIXED, v)
        g.set_coefficients(u0)
        op.rk3_steps(dt, 2, amdg.MIXED)
        ctx.synchronize()
        out[v] = g.coefficients().copy()
    assert rel_err(out[3], ref) < TOL_MIXED_STEP
    assert rel_err(out[3], out[1]) < TOL_MIXED_STEP
    op.close()
    g.close()


def test_tensor_core_variant_timeout_leaves_the_state(ctx):
    """The tensor-core variant's bounded waits: with a wait limit of 0 the step fails with
    AMDG_ERR_TIMEOUT and leaves the coefficients bitwise unchanged; with the limit restored it
    steps."""
    g = amdg.Grid(ctx, 3, 6, 2)
    g.init_separable(O.sin_sum_terms(3))
    u0 = g.coefficients().copy()
    op = amdg.LinearOperator(g, [1.0, -0.5, 0.25])
    op.set_variant(amdg.MIXED, 3)
    op.set_wait_limit(0)
    with pytest.raises(amdg.AmdgError) as ei:
        op.rk3_steps(1e-3, 1, amdg.MIXED)
    assert ei.value.status == 4
    ctx.synchronize()
    assert np.array_equal(g.coefficients(), u0)
    op.set_wait_limit(1 << 22)
    op.rk3_steps(1e-3, 1, amdg.MIXED)
    ctx.synchronize()
    assert not np.array_equal(g.coefficients(), u0)
    with pytest.raises(amdg.AmdgError):
        op.set_variant(amdg.FP64, 3)
    op.close()
    g.close()


@pytest.mark.parametrize("prec", [amdg.FP64, amdg.MIXED])
def test_serve_host_matches_device_steps(ctx, prec):
    """Pipelined host requests: every result bitwise equal to the same steps on the device state,
    the grid's own state untouched, and an in-place request (output = input) allowed."""
    g = amdg.Grid(ctx, 4, 6, 2)
    op = amdg.LinearOperator(g, [1.0, -0.5, 0.25, 0.75])
    rng = np.random.default_rng(9)
    base = rng.standard_normal(g.dof)
    g.set_coefficients(base)
    inputs = [rng.standard_normal(g.dof) for _ in range(5)]
    outputs = [np.zeros(g.dof) for _ in range(4)]
    inplace = inputs[4].copy()
    dt = 1e-3
    op.serve_host(inputs[:4] + [inplace], outputs + [inplace], dt, 2, prec)
    assert np.array_equal(g.coefficients().reshape(-1), base)
    for r in range(5):
        g.set_coefficients(inputs[r])
        op.rk3_steps(dt, 2, prec)
        ctx.synchronize()
        want = g.coefficients().reshape(-1)
        got = outputs[r] if r < 4 else inplace
        assert np.array_equal(got, want), f"request {r}"
    op.close()
    g.close()
