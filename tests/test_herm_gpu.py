"""Parity of the CUDA cubic-Hermite path (2D Burgers flux interpolated by Hermite interpolation,
HermInterpolation::nonlinear_Herm_2D_fast + HyperbolicSameFluxHermRHS + the LxF penalty) with the
reference fixtures (oracle/ref_harness burgers_herm and burgers_herm_adapt) and the oracle.
Tolerances: FP64 1e-12 relative to the field's max norm for point values and slopes, flux
coefficients and RK3 steps, 5e-12 for one right-hand side; element sets of the adaptive loop
identical, coefficients 1e-12; mixed mode (double-float point values, FP64 surplus, FP32 back
transforms) 1e-4 relative in the L2 norm for one right-hand side and 1e-6 for RK3 steps."""
import numpy as np
import pytest

import amdg
import amdg_oracle as O
from helpers import align, golden, manifest, rel_err
from test_burgers_gpu import run_on

pytestmark = pytest.mark.gpu

HERM = [n for n, m in manifest().items() if m["kind"] == "burgers_herm"]
HERM_ADAPT = [n for n, m in manifest().items() if m["kind"] == "burgers_herm_adapt"]


@pytest.mark.parametrize("name", HERM)
def test_hermite_burgers_matches_reference(ctx, name):
    m = manifest()[name]
    z = golden(name)
    N, k = m["N"], m["k"]
    g = amdg.Grid(ctx, 2, N, k)
    lv, sp = g.elements()
    perm = align(z["level"], z["suppt"], lv, sp)
    g.init_separable(O.burgers_ic_terms(2))
    assert rel_err(g.coefficients(), z["u0"][perm]) < 1e-13
    u0 = np.ascontiguousarray(z["u0"][perm])
    op = amdg.BurgersOperator(g, m["alpha"], hermite=True)
    up = run_on(ctx, op.point_values_device, u0, g.num_elements * 16).reshape(-1, 16)
    assert rel_err(up, z["up0"][perm]) < 1e-12
    fu = run_on(ctx, op.flux_coefficients_device, u0, g.num_elements * 16).reshape(-1, 16)
    assert rel_err(fu, z["fu0"][perm]) < 1e-12
    rhs = run_on(ctx, op.rhs_device, u0, g.dof).reshape(-1, g.block)
    assert rel_err(rhs, z["rhs0"][perm]) < 5e-12
    rhs32 = run_on(ctx, lambda a, b: op.rhs_device(a, b, amdg.MIXED), u0, g.dof).reshape(-1, g.block)
    ref = z["rhs0"][perm]
    assert np.linalg.norm(rhs32 - ref) / np.linalg.norm(ref) < 1e-4
    g.set_coefficients(u0)
    op.rk3_steps(m["dt"], m["steps"], amdg.FP64)
    ctx.synchronize()
    assert rel_err(g.coefficients(), z["uT"][perm]) < 1e-12
    g.set_coefficients(u0)
    op.rk3_steps(m["dt"], m["steps"], amdg.MIXED)
    ctx.synchronize()
    assert rel_err(g.coefficients(), z["uT"][perm]) < 1e-6
    op.close()
    g.close()


def test_hermite_burgers_matches_oracle_at_level_7(ctx):
    """A finer full sparse grid than the fixtures (N = 7, 640 elements) against the oracle."""
    N, k, alpha = 7, 2, 1.2
    g = amdg.Grid(ctx, 2, N, k)
    lv, sp = g.elements()
    g.init_separable(O.burgers_ic_terms(2))
    u0 = g.coefficients().copy()
    op = amdg.BurgersOperator(g, alpha, hermite=True)
    rhs = run_on(ctx, op.rhs_device, u0, g.dof).reshape(-1, g.block)
    ref, up_ref, fu_ref = O.burgers_herm_rhs(N, k, lv, sp, u0, alpha)
    assert rel_err(rhs, ref) < 5e-12
    fu = run_on(ctx, op.flux_coefficients_device, u0, g.num_elements * 16).reshape(-1, 16)
    assert rel_err(fu, fu_ref) < 1e-12
    op.close()
    g.close()


def _check(g, z, i, full=True):
    from golden.make_golden import checksums
    lv, sp = g.elements()
    keys = O.arrays_to_keys(lv, sp)
    ref_keys = O.arrays_to_keys(z[f"level_{i}"], z[f"suppt_{i}"])
    assert set(keys) == set(ref_keys), f"element set differs at step {i}"
    u = g.coefficients()
    cs, ref_cs = checksums(lv, sp, u), z["checksums"][i]
    assert abs(cs[0] - ref_cs[0]) <= 1e-12 * ref_cs[0], f"checksum differs at step {i}"
    assert abs(cs[2] - ref_cs[2]) <= 1e-12 * ref_cs[3], f"checksum differs at step {i}"
    if f"u_{i}" in z:
        pos = {kk: j for j, kk in enumerate(ref_keys)}
        perm = np.array([pos[kk] for kk in keys])
        assert rel_err(u, z[f"u_{i}"][perm]) < 1e-12, f"coefficients differ at step {i}"


@pytest.mark.parametrize("name", HERM_ADAPT)
def test_adaptive_hermite_burgers_matches_reference(ctx, name):
    """The loop of example/02_hyperbolic_05_burgers_adapt.cpp with the Hermite flux (wave speed 1
    in the CFL rule), FP64: element sets bit-exact after the adaptive initialisation and every
    step, checksums after every step and coefficients at the fixture's snapshots to 1e-12."""
    m = manifest()[name]
    z = golden(name)
    g = amdg.Grid(ctx, 2, m["nmax"], 2, level_init=m["n_init"])
    g.init_separable_adaptive(O.sin_sum_terms(2), m["eps"])
    _check(g, z, 0)
    op = amdg.BurgersOperator(g, m["alpha"], hermite=True)
    for i in range(m["steps"]):
        dt = op.adaptive_step(m["cfl"], 1.0, m["eps"], m["eta"], amdg.FP64)
        ctx.synchronize()
        assert dt == z["dt"][i]
        _check(g, z, i + 1)
    op.close()
    g.close()


def test_adaptive_hermite_host_and_device_modes_agree():
    """Element-set changes on the host and on the device give identical element sets and bitwise
    identical coefficients for the Hermite operator."""
    out = []
    for mode in (amdg.Context.ADAPT_HOST, amdg.Context.ADAPT_DEVICE):
        ctx = amdg.Context(0)
        ctx.set_adapt_mode(mode)
        g = amdg.Grid(ctx, 2, 7, 2, level_init=3)
        g.init_separable_adaptive(O.sin_sum_terms(2), 1e-4)
        op = amdg.BurgersOperator(g, 1.2, hermite=True)
        for _ in range(4):
            op.adaptive_step(0.2, 1.0, 1e-4, 1e-5, amdg.FP64)
        ctx.synchronize()
        out.append((g.elements(), g.coefficients().copy()))
        op.close()
        g.close()
    (lv0, sp0), u0 = out[0]
    (lv1, sp1), u1 = out[1]
    assert (lv0 == lv1).all() and (sp0 == sp1).all()
    assert (u0 == u1).all()


def test_hermite_operator_is_two_dimensional(ctx):
    g = amdg.Grid(ctx, 3, 3, 2)
    with pytest.raises(RuntimeError):
        amdg.BurgersOperator(g, 1.2, hermite=True)
    g.close()
