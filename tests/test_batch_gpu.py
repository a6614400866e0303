"""Batched independent solves (one launch per RK stage for all grids) against
the oracle's SSP-RK3 per solve (its own grid, velocity and time step) and
against the same solves stepped one by one with the single-grid operator.  The
batch multiplies the velocity after the 1D contraction instead of into the 1D
blocks, so the FP64 results agree to 1e-12 relative, not bitwise."""
import numpy as np
import pytest

import amdg
import amdg_oracle as O

pytestmark = pytest.mark.gpu


def _grids(ctx, work, nmax, eps):
    grids = []
    for w in work:
        g = amdg.Grid(ctx, 3, nmax, 2, level_init=2)
        g.init_separable_adaptive(O.gaussian_bump_terms(w["centers"], w["widths"], w["amplitudes"]), eps)
        grids.append(g)
    return grids


def _keys(g):
    """One int per element: its per-dimension (level, support index) pairs packed together."""
    lv, sp = g.elements()
    return (lv.astype(np.int64) * 1024 + sp).dot(1 << (20 * np.arange(lv.shape[1], dtype=np.int64)))


@pytest.mark.parametrize("use_graph", [False, True])
def test_batch_matches_individual_solves(ctx, use_graph):
    work = O.batched_workload(5, seed=3)
    grids = _grids(ctx, work, 5, 1e-3)
    sizes = [g.num_elements for g in grids]
    assert len(set(sizes)) > 1, "grids should be uneven"
    u0 = [g.coefficients().copy() for g in grids]
    dts = [0.1 / (sum(abs(v) for v in w["velocity"]) * 32) for w in work]
    batch = amdg.Batch(ctx, grids, [w["velocity"] for w in work])
    assert batch.num_elements == sum(sizes)
    batch.set_dt(dts)
    batch.rk3_steps(3, amdg.FP64, use_graph=use_graph)
    ctx.synchronize()
    for i, (g, w) in enumerate(zip(grids, work)):
        batch.store(i)
        got = g.coefficients().copy()
        g.set_coefficients(u0[i])
        op = amdg.LinearOperator(g, w["velocity"])
        op.rk3_steps(dts[i], 3, amdg.FP64)
        ctx.synchronize()
        want = g.coefficients()
        assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max(), f"solve {i}"
        op.close()
    batch.close()
    for g in grids:
        g.close()


@pytest.mark.parametrize("prec,tol", [(amdg.FP64, 1e-12), (amdg.MIXED, 1e-6)])
def test_batch_matches_oracle_per_solve(ctx, prec, tol):
    """Every solve of the batch against the oracle's SSP-RK3 (the reference's linear operator
    restated on the CPU) at that solve's own velocity and time step, on its own adaptive grid:
    FP64 to 1e-12 and mixed to 1e-6 relative (max norm over the solve's field)."""
    work = O.batched_workload(6, seed=11)
    grids = _grids(ctx, work, 5, 1e-3)
    u0 = [g.coefficients().copy() for g in grids]
    dts = [0.1 / (sum(abs(v) for v in w["velocity"]) * 32) for w in work]
    batch = amdg.Batch(ctx, grids, [w["velocity"] for w in work])
    batch.set_dt(dts)
    nsteps = 3
    batch.rk3_steps(nsteps, prec, use_graph=True)
    ctx.synchronize()
    for i, (g, w) in enumerate(zip(grids, work)):
        batch.store(i)
        got = g.coefficients()
        lv, sp = g.elements()
        want = O.linear_rk3(3, g.nmax, 2, lv, sp, w["velocity"], u0[i], dts[i], nsteps)
        assert np.abs(got - want).max() <= tol * np.abs(want).max(), f"solve {i}"
    batch.close()
    for g in grids:
        g.close()


def test_batch_mixed_and_l2_error(ctx):
    """Mixed-precision batch steps agree with FP64 batch steps; their L2 errors
    against the exact translated bumps (split formula) agree to 1e-3."""
    work = O.batched_workload(3, seed=7)
    errs = {}
    for prec in (amdg.FP64, amdg.MIXED):
        grids = _grids(ctx, work, 5, 1e-3)
        batch = amdg.Batch(ctx, grids, [w["velocity"] for w in work])
        dts = [0.1 / (sum(abs(v) for v in w["velocity"]) * 32) for w in work]
        batch.set_dt(dts)
        nsteps = 4
        batch.rk3_steps(nsteps, prec, use_graph=True)
        ctx.synchronize()
        for i, (g, w) in enumerate(zip(grids, work)):
            batch.store(i)
            shift = [v * dts[i] * nsteps for v in w["velocity"]]
            exact = O.gaussian_bump_terms(w["centers"], w["widths"], w["amplitudes"], shift=shift)
            norm = O.gaussian_bump_norm(w["centers"], w["widths"], w["amplitudes"])
            errs[(prec, i)] = g.l2_error_separable_sum(exact, norm)
            assert errs[(prec, i)] < norm
        batch.close()
        for g in grids:
            g.close()
    for i in range(len(work)):
        assert abs(errs[(amdg.MIXED, i)] - errs[(amdg.FP64, i)]) <= 1e-3 * errs[(amdg.FP64, i)]


def test_batch_kernels_agree_and_autotuner_picks_one(ctx):
    """Every CTA size of the column kernel sums each output in the same order (bitwise the same
    steps); on the FP32-pair stage state the column tiles and the bulk-copy ring configurations
    agree bitwise with each other and, their stage vectors being FP32 pairs instead of FP64, with
    the mixed column kernel on the FP64 state to 1e-6.  A batch over 100,000 DOF is timed with every
    candidate and keeps the fastest."""
    work = O.batched_workload(8, seed=11)
    grids = _grids(ctx, work, 6, 1e-4)
    dts = [0.1 / (sum(abs(v) for v in w["velocity"]) * 64) for w in work]
    K = amdg.Batch.KERNELS
    results = {}
    for prec in (amdg.FP64, amdg.MIXED):
        pi = 0 if prec == amdg.FP64 else 1
        cands = range(K) if prec == amdg.MIXED else range(len(amdg.Batch.TILES))
        for c in cands:
            batch = amdg.Batch(ctx, grids, [w["velocity"] for w in work])
            assert batch.dof > 100000
            kernel, ms = batch.tuning()
            row = ms[pi]
            timed = [i for i in range(K) if row[i] > 0]
            assert set(timed) == set(cands)
            assert kernel[pi] == min(timed, key=lambda i: row[i])
            batch.set_kernel(prec, c)
            batch.set_dt(dts)
            batch.rk3_steps(2, prec, use_graph=True)
            ctx.synchronize()
            batch.store(3)
            results[(prec, c)] = grids[3].coefficients().copy()
            batch.close()
            for g, w in zip(grids, work):  # restore the initial state for the next batch
                g.init_separable(O.gaussian_bump_terms(w["centers"], w["widths"], w["amplitudes"]))
        for c in range(1, len(amdg.Batch.TILES)):
            assert np.array_equal(results[(prec, c)], results[(prec, 0)])
    ring0, df0 = amdg.Batch.RING_FIRST, amdg.Batch.DF_COLUMN_FIRST
    # FP32-pair state: the column tiles and the ring configurations sum in the same order
    for c in range(df0 + 1, K):
        assert np.array_equal(results[(amdg.MIXED, c)], results[(amdg.MIXED, df0)]), amdg.Batch.kernel_name(c)
    ref = results[(amdg.MIXED, 2)]
    assert np.abs(results[(amdg.MIXED, df0)] - ref).max() <= 1e-6 * np.abs(ref).max()
    with pytest.raises(amdg.AmdgError):
        batch = amdg.Batch(ctx, grids, [w["velocity"] for w in work])
        try:
            batch.set_kernel(amdg.FP64, ring0)
        finally:
            batch.close()
    for g in grids:
        g.close()


@pytest.mark.parametrize("seed,which", [(3, "ring"), (8, "ring"), (3, "column")])
def test_batch_ring_kernel_matches_oracle(ctx, seed, which):
    """The FP32-pair stage state (FP32 contraction) with the bulk-copy ring kernel or the column
    kernel against the oracle's SSP-RK3 per solve, each at its own velocity and step: 1e-6
    relative after 3 steps."""
    work = O.batched_workload(5, seed=seed)
    grids = _grids(ctx, work, 5, 1e-3)
    u0 = [g.coefficients().copy() for g in grids]
    dts = [0.1 / (sum(abs(v) for v in w["velocity"]) * 32) for w in work]
    batch = amdg.Batch(ctx, grids, [w["velocity"] for w in work])
    batch.set_kernel(amdg.MIXED, amdg.Batch.RING_FIRST if which == "ring" else amdg.Batch.DF_COLUMN_FIRST + 2)
    batch.set_dt(dts)
    batch.rk3_steps(3, amdg.MIXED, use_graph=False)
    ctx.synchronize()
    for i, (g, w) in enumerate(zip(grids, work)):
        batch.store(i)
        lv, sp = g.elements()
        want = O.linear_rk3(3, g.nmax, 2, lv, sp, w["velocity"], u0[i], dts[i], 3)
        assert np.abs(g.coefficients() - want).max() <= 1e-6 * np.abs(want).max(), f"solve {i}"
    batch.close()
    for g in grids:
        g.close()


def test_bulk_factor_callbacks_match_pointwise(ctx):
    """The bulk-callback entry points evaluate the same points in the same order: the adaptive
    initialisation gives the same element set and coefficients as the pointwise one (numpy's and
    the C library's exp may differ in the last bit, hence 1e-13), and the split L2 errors agree."""
    work = O.batched_workload(2, seed=5)
    for w in work:
        a = amdg.Grid(ctx, 3, 5, 2, level_init=2)
        b = amdg.Grid(ctx, 3, 5, 2, level_init=2)
        a.init_separable_adaptive(O.gaussian_bump_terms(w["centers"], w["widths"], w["amplitudes"]), 1e-3)
        b.init_separable_adaptive(O.gaussian_bump_terms(w["centers"], w["widths"], w["amplitudes"], vectorized=True),
                                  1e-3, vectorized=True)
        for x, y in zip(a.elements(), b.elements()):
            assert np.array_equal(x, y)
        ua, ub = a.coefficients(), b.coefficients()
        assert np.abs(ua - ub).max() <= 1e-13 * np.abs(ua).max()
        norm = O.gaussian_bump_norm(w["centers"], w["widths"], w["amplitudes"])
        ea = a.l2_error_separable_sum(O.gaussian_bump_terms(w["centers"], w["widths"], w["amplitudes"]), norm)
        eb = b.l2_error_separable_sum(O.gaussian_bump_terms(w["centers"], w["widths"], w["amplitudes"],
                                                            vectorized=True), norm, vectorized=True)
        assert abs(ea - eb) <= 1e-9 * norm
        a.close()
        b.close()


def test_batch_adapt_matches_per_grid_adaptivity(ctx):
    """amdg_batch_adapt with the surplus criterion coarsens and refines every solve's grid as
    amdg_grid_coarsen + amdg_grid_refine do on its own (the between-steps part of the reference's
    refine -> step -> coarsen loop: the new children survive the call), and the rebuilt batch
    still steps every solve as the single-grid operator does; a classifier that is never sure
    (tau above 1) falls back to the criterion everywhere and gives the same grids."""
    work = O.batched_workload(4, seed=13)
    eps, eta = 3e-4, 3e-5
    dts = [0.1 / (sum(abs(v) for v in w["velocity"]) * 32) for w in work]

    def fresh():
        return _grids(ctx, work, 5, 1e-3)

    ga, gb, gc = fresh(), fresh(), fresh()
    batch = amdg.Batch(ctx, ga, [w["velocity"] for w in work])
    batch.set_dt(dts)
    batch.rk3_steps(2, amdg.FP64, use_graph=True)
    for i in range(len(work)):  # the same two steps on the reference copies
        batch.store(i)
    u_after = [g.coefficients().copy() for g in ga]
    for g, u in zip(gb, u_after):
        g.set_coefficients(u)
    for g, u in zip(gc, u_after):
        g.set_coefficients(u)
    keys_before = [_keys(g) for g in ga]
    stats = batch.adapt(eps, eta)
    assert stats[2] == batch.num_elements
    # new children start at zero; coarsened leaves whose parent is refined come straight back,
    # also at zero (as in the reference loop, where the next refine re-adds what coarsen removed);
    # every other element keeps its coefficients
    fresh_total = zeroed_total = 0
    for g, kb, ub in zip(ga, keys_before, u_after):
        ka, ua = _keys(g), g.coefficients()
        new = ~np.isin(ka, kb)
        fresh_total += int(new.sum())
        assert not ua[new].any()
        srt = np.argsort(kb)
        pos = srt[np.searchsorted(kb[srt], ka[~new])]
        same = np.all(ua[~new] == ub[pos], axis=1)
        zero = ~ua[~new].any(axis=1)
        assert np.all(same | zero)
        zeroed_total += int((zero & ~same).sum())
    assert fresh_total > 0 and zeroed_total > 0
    for g in gb:
        g.coarsen(eta)
        g.refine(eps)
    for a, b in zip(ga, gb):
        for x, y in zip(a.elements(), b.elements()):
            assert np.array_equal(x, y)
        assert np.array_equal(a.coefficients(), b.coefficients())
    assert batch.num_elements == sum(g.num_elements for g in gb)
    # the rebuilt batch steps each solve as the single-grid operator
    batch.set_dt(dts)
    batch.rk3_steps(2, amdg.FP64, use_graph=True)
    for i, (g, w) in enumerate(zip(gb, work)):
        batch.store(i)
        op = amdg.LinearOperator(g, w["velocity"])
        op.rk3_steps(dts[i], 2, amdg.FP64)
        ctx.synchronize()
        want = g.coefficients()
        assert np.abs(ga[i].coefficients() - want).max() <= 1e-12 * np.abs(want).max()
        op.close()
    batch.close()
    # a classifier that is never sure: the criterion decides everywhere
    F = 27 * (1 + 2 * 3)
    mlp = amdg.MLP(ctx, F, 64, 3, 3, seed=5)
    batch2 = amdg.Batch(ctx, gc, [w["velocity"] for w in work])
    st = batch2.adapt(eps, eta, mlp=mlp, tau=1.5)
    assert st[0] == 0 and st[1] > 0
    gd = fresh()
    for g, u in zip(gd, u_after):
        g.set_coefficients(u)
    for g in gd:
        g.coarsen(eta)
        g.refine(eps)
    for a, b in zip(gc, gd):
        for x, y in zip(a.elements(), b.elements()):
            assert np.array_equal(x, y)
    batch2.close()
    mlp.close()
    for g in ga + gb + gc + gd:
        g.close()
