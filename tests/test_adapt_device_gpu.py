"""Element-set changes on the device (refine, coarsen, hole filling, the fast
transforms' neighbour lists and surplus ancestors built from the sorted keys)
against the host implementation of the same steps: for adaptive Burgers, the
adaptive wave equation, the learned and criterion-only horizon steps and the
grid-level refine / coarsen calls, both modes must give identical element sets
and bitwise identical coefficients after every step."""
import numpy as np
import pytest

import amdg
import amdg_oracle as O

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def contexts():
    dev = amdg.Context(0)
    host = amdg.Context(0)
    host.set_adapt_mode(amdg.Context.ADAPT_HOST)
    yield dev, host


def _same(ga, gb, what):
    la, sa = ga.elements()
    lb, sb = gb.elements()
    assert np.array_equal(la, lb) and np.array_equal(sa, sb), f"element sets differ ({what})"
    assert np.array_equal(ga.coefficients(), gb.coefficients()), f"coefficients differ ({what})"


@pytest.mark.parametrize("dim,nmax,eps,eta,prec", [(2, 7, 1e-4, 1e-5, amdg.FP64), (3, 6, 3e-5, 3e-6, amdg.FP64),
                                                   (3, 6, 3e-5, 3e-6, amdg.MIXED)])
def test_adaptive_burgers_device_matches_host(contexts, dim, nmax, eps, eta, prec):
    runs = []
    for ctx in contexts:
        g = amdg.Grid(ctx, dim, nmax, 2, level_init=3)
        g.init_separable_adaptive(O.burgers_ic_terms(dim), eps)
        runs.append((g, amdg.BurgersOperator(g, 0.825)))
    for step in range(5):
        dts = [op.adaptive_step(0.1, 0.75, eps, eta, prec) for _, op in runs]
        assert dts[0] == dts[1]
        for ctx in contexts:
            ctx.synchronize()
        _same(runs[0][0], runs[1][0], f"step {step}")
    for g, op in runs:
        op.close()
        g.close()


def test_adaptive_step_decisions_device_matches_host(contexts):
    runs = []
    for ctx in contexts:
        g = amdg.Grid(ctx, 2, 7, 2, level_init=3)
        g.init_separable_adaptive(O.burgers_ic_terms(2), 1e-4)
        runs.append((g, amdg.BurgersOperator(g, 0.825)))
    for step in range(4):
        out = [op.adaptive_step_ex(0.1, 0.75, 1e-4, 1e-5) for _, op in runs]
        assert out[0][0] == out[1][0]
        assert np.array_equal(out[0][1], out[1][1]), f"decisions differ at step {step}"
        _same(runs[0][0], runs[1][0], f"step {step}")
    for g, op in runs:
        op.close()
        g.close()


def test_adaptive_wave_device_matches_host(contexts):
    runs = []
    for ctx in contexts:
        g = amdg.Grid(ctx, 2, 6, 2, level_init=3)
        g.init_separable_adaptive(O.wave_ic_terms(2), 1e-5)
        runs.append((g, amdg.WaveOperator(g, 10.0)))
    for step in range(4):
        dts = [op.adaptive_step(0.1, 1.0, 1e-5, 1e-6) for _, op in runs]
        assert dts[0] == dts[1]
        _same(runs[0][0], runs[1][0], f"step {step}")
        assert np.array_equal(runs[0][0].velocity(), runs[1][0].velocity()), f"u_t differs at step {step}"
    for g, op in runs:
        op.close()
        g.close()


@pytest.mark.parametrize("learned", [True, False])
def test_horizon_steps_device_matches_host(contexts, learned):
    """Pre-adaptation by a (seeded, untrained) classifier or by the criterion alone, horizon 3:
    refinements, unsure counts, missed refinements and the solution agree between the modes."""
    dim = 3
    F = 27 * (1 + 2 * dim)
    runs = []
    for ctx in contexts:
        g = amdg.Grid(ctx, dim, 6, 2, level_init=3)
        g.init_separable_adaptive(O.burgers_ic_terms(dim), 3e-5)
        mlp = amdg.MLP(ctx, F, 64, 3, 3, seed=7) if learned else None
        runs.append((g, amdg.BurgersOperator(g, 0.825), mlp))
    for rnd in range(3):
        res = [op.adaptive_steps_learned(mlp, 0.1, 0.75, 3e-5, 3e-6, 0.6, 3, 0.0) for _, op, mlp in runs]
        assert res[0][0] == res[1][0] and res[0][1] == res[1][1]
        assert np.array_equal(res[0][2], res[1][2]), f"stats differ in round {rnd}: {res[0][2]} {res[1][2]}"
        _same(runs[0][0], runs[1][0], f"round {rnd}")
    for g, op, mlp in runs:
        op.close()
        g.close()
        if mlp is not None:
            mlp.close()


def test_grid_refine_coarsen_device_matches_host(contexts):
    """amdg_grid_refine / amdg_grid_coarsen on a random indicator field: same element sets, the
    coefficients carried over and zero on new elements, in both modes; then the Burgers
    right-hand side on the device-built neighbour lists equals the one on the host-built lists."""
    rng = np.random.default_rng(4)
    grids = []
    for ctx in contexts:
        g = amdg.Grid(ctx, 3, 6, 2, level_init=3)
        g.init_separable(O.burgers_ic_terms(3))
        grids.append(g)
    for rnd in range(3):
        ind = rng.standard_normal(grids[0].dof) * np.repeat(rng.uniform(0, 2e-3, grids[0].num_elements), 27)
        for g in grids:
            d = torch.from_numpy(ind).cuda()
            torch.cuda.synchronize()
            g.refine(1e-3, d.data_ptr())
            g.ctx.synchronize()
            del d
        _same(grids[0], grids[1], f"refine {rnd}")
        u = grids[0].coefficients() + 1e-4 * rng.standard_normal((grids[0].num_elements, 27))
        for g in grids:
            g.set_coefficients(u)
        for g in grids:
            g.coarsen(2e-4)
        _same(grids[0], grids[1], f"coarsen {rnd}")
    outs = []
    for g in grids:
        op = amdg.BurgersOperator(g, 0.825)
        du = torch.from_numpy(g.coefficients().reshape(-1).copy()).cuda()
        out = torch.zeros_like(du)
        torch.cuda.synchronize()
        op.rhs_device(du.data_ptr(), out.data_ptr())
        g.ctx.synchronize()
        outs.append(out.cpu().numpy())
        op.close()
    assert np.array_equal(outs[0], outs[1])
    lv, sp = grids[0].elements()
    ref = O.burgers_rhs(3, 6, 2, lv, sp, grids[0].coefficients(), 0.825)[0]
    assert np.abs(outs[0].reshape(ref.shape) - ref).max() <= 5e-12 * np.abs(ref).max()
    for g in grids:
        g.close()


def test_device_adaptivity_keeps_host_views_current(contexts):
    """After device-side steps the host-facing calls (elements, finest levels, checkpoint, point
    values) see the new element set."""
    ctx = contexts[0]
    g = amdg.Grid(ctx, 2, 7, 2, level_init=3)
    g.init_separable_adaptive(O.burgers_ic_terms(2), 1e-4)
    op = amdg.BurgersOperator(g, 0.825)
    for _ in range(3):
        op.adaptive_step(0.1, 0.75, 1e-4, 1e-5)
    lv, sp = g.elements()
    assert lv.shape == (g.num_elements, 2)
    assert np.array_equal(g.max_mesh_level(), lv.max(axis=0))
    keys = O.arrays_to_keys(lv, sp)
    assert len(set(keys)) == len(keys)
    u = g.coefficients()
    x = np.array([0.11, 0.37, 0.73])
    vals = torch.zeros(9, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    g.eval_tensor_device(x, vals.data_ptr())
    ctx.synchronize()
    pts = np.array([[a, b] for a in x for b in x])
    ref = O.eval_points(2, 7, 2, lv, sp, u, pts)
    assert np.abs(vals.cpu().numpy() - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max())
    op.close()
    g.close()
