"""Adaptivity on the device against the reference's adaptive Burgers runs
(fixtures from oracle/ref_harness burgers_adapt): adaptive separable
initialisation, then per step the forward-Euler prediction, refine, one
SSP-RK3 step and coarsen.  Element sets must match exactly; coefficients to
1e-12 relative (max norm over the field), FP64."""
import numpy as np
import pytest

import amdg
import amdg_oracle as O
from helpers import golden, manifest, rel_err

pytestmark = pytest.mark.gpu

ADAPT = [n for n, m in manifest().items() if m["kind"] == "burgers_adapt"]


def _check(g, z, i):
    lv, sp = g.elements()
    keys = O.arrays_to_keys(lv, sp)
    ref_keys = O.arrays_to_keys(z[f"level_{i}"], z[f"suppt_{i}"])
    assert set(keys) == set(ref_keys), f"element set differs at step {i}"
    pos = {k: j for j, k in enumerate(ref_keys)}
    perm = np.array([pos[k] for k in keys])
    assert rel_err(g.coefficients(), z[f"u_{i}"][perm]) < 1e-12, f"coefficients differ at step {i}"


@pytest.mark.parametrize("name", ADAPT)
def test_adaptive_burgers_matches_reference(ctx, name):
    m = manifest()[name]
    z = golden(name)
    g = amdg.Grid(ctx, m["dim"], m["nmax"], 2, level_init=m["n_init"])
    g.init_separable_adaptive(O.burgers_ic_terms(m["dim"]), m["eps"])
    _check(g, z, 0)
    op = amdg.BurgersOperator(g, m["alpha"])
    for i in range(m["steps"]):
        op.adaptive_step(m["cfl"], m["umax"], m["eps"], m["eta"], amdg.FP64)
        ctx.synchronize()
        _check(g, z, i + 1)
    op.close()
    g.close()


LONG = [n for n, m in manifest().items() if m["kind"] == "burgers_adapt_long"]


@pytest.mark.parametrize("name", LONG)
def test_adaptive_burgers_full_run_matches_reference(ctx, name):
    """The benchmark's 3D configuration over its whole length (36 steps to T = 0.05): after the
    adaptive initialisation and after every step the element set equals the reference's; the
    coefficients agree to 1e-12 relative at the snapshot steps, and every step's checksums (sum of
    squares, max |u|, a position-weighted sum) agree to 1e-12 relative."""
    from golden.make_golden import checksums
    m = manifest()[name]
    z = golden(name)
    dim = m["dim"]
    g = amdg.Grid(ctx, dim, m["nmax"], 2, level_init=m["n_init"])
    g.init_separable_adaptive(O.burgers_ic_terms(dim), m["eps"])
    op = amdg.BurgersOperator(g, m["alpha"])
    for i in range(m["steps"] + 1):
        if i > 0:
            dt = op.adaptive_step(m["cfl"], m["umax"], m["eps"], m["eta"], amdg.FP64)
            assert dt == z["dt"][i - 1]
            ctx.synchronize()
        lv, sp = g.elements()
        keys = O.arrays_to_keys(lv, sp)
        ref_keys = O.arrays_to_keys(z[f"level_{i}"], z[f"suppt_{i}"])
        assert set(keys) == set(ref_keys), f"element set differs at step {i}"
        u = g.coefficients().reshape(len(keys), -1)
        cs, ref_cs = checksums(lv, sp, u), z["checksums"][i]
        assert abs(cs[0] - ref_cs[0]) <= 1e-12 * ref_cs[0], f"sum of squares differs at step {i}"
        assert abs(cs[1] - ref_cs[1]) <= 1e-12 * ref_cs[1], f"max |u| differs at step {i}"
        assert abs(cs[2] - ref_cs[2]) <= 1e-12 * ref_cs[3], f"weighted sum differs at step {i}"
        if f"u_{i}" in z:
            pos = {k: j for j, k in enumerate(ref_keys)}
            perm = np.array([pos[k] for k in keys])
            assert rel_err(u, z[f"u_{i}"][perm]) < 1e-12, f"coefficients differ at step {i}"
    op.close()
    g.close()


def test_refine_coarsen_round_trip_and_version(ctx):
    g = amdg.Grid(ctx, 2, 6, 2, level_init=3)
    g.init_separable(O.burgers_ic_terms(2))
    v0, e0 = g.version(), g.num_elements
    u0 = g.coefficients().copy()
    n = g.refine(-1.0)          # every leaf refines by one level
    assert n > e0 and g.version() == v0 + 1
    # old coefficients carried over, new elements zero
    lv0, sp0 = O.grid(2, 3)
    keys0 = O.arrays_to_keys(lv0, sp0)
    lv, sp = g.elements()
    keys = O.arrays_to_keys(lv, sp)
    u = g.coefficients()
    pos0 = {k: i for i, k in enumerate(keys0)}
    for i, k in enumerate(keys):
        if k in pos0:
            assert np.array_equal(u[i], u0[pos0[k]])
        else:
            assert not u[i].any()
    # zero-coefficient children are coarsened away again
    g.coarsen(1e-300)
    assert g.num_elements == e0
    assert np.array_equal(g.coefficients(), u0)
    g.close()


def test_host_phase_profile_counts_adaptive_work(ctx):
    """Two plain adaptive steps: every step evaluates four right-hand sides
    (predictor and three stages), changes the element set twice on the device
    (refine and coarsen, no norms read back to the host), and rebuilds the
    neighbour lists whenever the element set changed; the profile stops when
    disabled."""
    g = amdg.Grid(ctx, 2, 6, 2, level_init=3)
    g.init_separable_adaptive(O.burgers_ic_terms(2), 1e-4)
    op = amdg.BurgersOperator(g, 0.825)
    ctx.synchronize()
    ctx.profile(True)
    for _ in range(2):
        op.adaptive_step(0.1, 0.75, 1e-4, 1e-5)
    ctx.synchronize()
    prof = ctx.profile_read()
    assert prof["adapt_step"][1] == 2
    assert prof["rhs"][1] == 8
    assert prof["rk3"][1] == 2
    assert prof["adapt_device"][1] == 4
    assert prof["norms"][1] == 0 and prof["adapt_host"][1] == 0
    assert prof["topology"][1] >= 1
    assert all(v[0] >= 0.0 for v in prof.values())
    assert prof["adapt_step"][0] >= prof["rk3"][0]
    ctx.profile(False)
    op.adaptive_step(0.1, 0.75, 1e-4, 1e-5)
    assert ctx.profile_read() == {k: (0.0, 0) for k in amdg.Context.PHASES}
    op.close()
    g.close()
