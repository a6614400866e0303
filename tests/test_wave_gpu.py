"""The second-order wave path (u_tt = div(K grad u): interpolated K grad u and K u,
DiffusionRHS terms, IPDG penalty, RK4ODE2nd) on the GPU against the reference fixtures and
the oracle.  FP64: 1e-12 relative (max norm) for the right-hand side and RK4 steps;
mixed (FP64 point values and surplus, FP32 back transforms): 1e-4 relative in L2 for one
right-hand side (the IPDG penalty makes it a difference of large terms) and 1e-6 for steps."""
import numpy as np
import pytest

import amdg
import amdg_oracle as O
from helpers import align, golden, manifest, rel_err

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

WAVE = [n for n, m in manifest().items() if m["kind"] == "wave"]
WAVE_ADAPT = [n for n, m in manifest().items() if m["kind"] == "wave_adapt"]


def _on_device(u):
    torch.cuda.synchronize()
    return torch.from_numpy(np.ascontiguousarray(u).reshape(-1)).cuda()


@pytest.mark.parametrize("name", WAVE)
def test_wave_matches_reference(ctx, name):
    m = manifest()[name]
    z = golden(name)
    dim, N = m["dim"], m["N"]
    g = amdg.Grid(ctx, dim, N, 2)
    lv, sp = g.elements()
    perm = align(z["level"], z["suppt"], lv, sp)
    u0 = np.ascontiguousarray(z["u0"][perm])
    op = amdg.WaveOperator(g, m["sigma"])
    du = _on_device(u0)
    out = torch.zeros_like(du)
    torch.cuda.synchronize()
    op.rhs_device(du.data_ptr(), out.data_ptr())
    ctx.synchronize()
    ref = z["rhs0"][perm]
    assert rel_err(out.cpu().numpy().reshape(ref.shape), ref) < 1e-12
    op.rhs_device(du.data_ptr(), out.data_ptr(), amdg.MIXED)
    ctx.synchronize()
    r32 = out.cpu().numpy().reshape(ref.shape)
    assert np.linalg.norm(r32 - ref) / np.linalg.norm(ref) < 1e-4
    for prec, tol in ((amdg.FP64, 1e-12), (amdg.MIXED, 1e-6)):
        g.set_coefficients(u0)
        g.set_velocity(np.zeros_like(u0))
        op.rk4_steps(m["dt"], m["steps"], prec)
        ctx.synchronize()
        assert rel_err(g.coefficients(), z["uT"][perm]) < tol
        assert rel_err(g.velocity(), z["vT"][perm]) < tol * 10
    op.close()
    g.close()


def test_wave_rhs_matches_oracle_on_random_state(ctx):
    dim, N = 2, 6
    g = amdg.Grid(ctx, dim, N, 2)
    rng = np.random.default_rng(4)
    u = rng.standard_normal((g.num_elements, g.block))
    op = amdg.WaveOperator(g, 10.0)
    du = _on_device(u)
    out = torch.zeros_like(du)
    torch.cuda.synchronize()
    op.rhs_device(du.data_ptr(), out.data_ptr())
    ctx.synchronize()
    lv, sp = g.elements()
    ref = O.wave_rhs(dim, N, 2, lv, sp, u, 10.0)
    assert rel_err(out.cpu().numpy().reshape(ref.shape), ref) < 1e-12
    op.close()
    g.close()


def test_adaptive_wave_matches_oracle(ctx):
    """Element sets identical to the oracle's adaptive loop after every step, (u, v) to 1e-12."""
    dim, nmax, eps, eta, sigma, cfl = 2, 6, 1e-4, 1e-5, 10.0, 0.1
    steps = 3
    hist = O.wave_adaptive_run(dim, 3, nmax, eps, eta, sigma, cfl, 1.0, steps)
    g = amdg.Grid(ctx, dim, nmax, 2, level_init=3)
    g.init_separable_adaptive(O.wave_ic_terms(dim), eps)
    op = amdg.WaveOperator(g, sigma)
    def check(keys, u, v):
        lv, sp = g.elements()
        mine = O.arrays_to_keys(lv, sp)
        assert set(mine) == set(keys)
        pos = {k: j for j, k in enumerate(keys)}
        perm = np.array([pos[k] for k in mine])
        assert rel_err(g.coefficients(), u[perm]) < 1e-12
        if np.abs(v).max() > 0:
            assert rel_err(g.velocity(), v[perm]) < 1e-11

    check(hist[0][0], hist[0][1], hist[0][2])
    for s in range(steps):
        dt = op.adaptive_step(cfl, 1.0, eps, eta)
        keys, u, v, dt_ref = hist[s + 1]
        assert dt == dt_ref
        check(keys, u, v)
    stage_dof, rhs = op.counters()
    assert rhs == 4 * steps  # the predictor evaluates the IPDG term alone
    op.close()
    g.close()


@pytest.mark.parametrize("name", WAVE_ADAPT)
def test_adaptive_wave_matches_reference(ctx, name):
    """The adaptive loop of 03_wave_06_var_coeff_adapt.cpp on the GPU against the reference run:
    element sets bit-exact after the adaptive initialisation and every step, u and u_t to 1e-12
    of their largest entry."""
    m = manifest()[name]
    z = golden(name)
    dim = m["dim"]
    g = amdg.Grid(ctx, dim, m["nmax"], 2, level_init=m["n_init"])
    g.init_separable_adaptive(O.wave_ic_terms(dim), m["eps"])
    op = amdg.WaveOperator(g, m["sigma"])
    for i in range(m["steps"] + 1):
        if i > 0:
            op.adaptive_step(m["cfl"], 1.0, m["eps"], m["eta"])
        lv, sp = g.elements()
        mine = O.arrays_to_keys(lv, sp)
        ref = O.arrays_to_keys(z[f"level_{i}"], z[f"suppt_{i}"])
        assert sorted(mine) == sorted(ref), f"element set differs after step {i}"
        pos = {k: j for j, k in enumerate(ref)}
        perm = np.array([pos[k] for k in mine])
        u_ref, v_ref = z[f"u_{i}"][perm], z[f"ut_{i}"][perm]
        assert np.abs(g.coefficients() - u_ref).max() <= 1e-12 * np.abs(u_ref).max()
        if i > 0:
            assert np.abs(g.velocity() - v_ref).max() <= 1e-12 * np.abs(v_ref).max()
    op.close()
    g.close()


WAVE_LONG = [n for n, m in manifest().items() if m["kind"] == "wave_adapt_long"]


@pytest.mark.parametrize("name", WAVE_LONG)
def test_adaptive_wave_long_run_matches_reference(ctx, name):
    """The adaptive wave loop at max level 7 over 24 steps against the reference run: element sets
    bit-exact after the initialisation and every step; every step's checksums of u and u_t (sum of
    squares, max, position-weighted sum) to 1e-12 relative; u at the snapshot steps to 1e-12 and u_t
    to 1e-11 of their largest entry."""
    from golden.make_golden import checksums
    m = manifest()[name]
    z = golden(name)
    dim = m["dim"]
    g = amdg.Grid(ctx, dim, m["nmax"], 2, level_init=m["n_init"])
    g.init_separable_adaptive(O.wave_ic_terms(dim), m["eps"])
    op = amdg.WaveOperator(g, m["sigma"])
    for i in range(m["steps"] + 1):
        if i > 0:
            op.adaptive_step(m["cfl"], 1.0, m["eps"], m["eta"])
        lv, sp = g.elements()
        mine = O.arrays_to_keys(lv, sp)
        ref = O.arrays_to_keys(z[f"level_{i}"], z[f"suppt_{i}"])
        assert sorted(mine) == sorted(ref), f"element set differs after step {i}"
        u = g.coefficients()
        v = g.velocity() if i > 0 else np.zeros_like(u)  # u_t exists from the first step on (zero before)
        cs = np.concatenate([checksums(lv, sp, u), checksums(lv, sp, v)])
        rc = z["checksums"][i]
        for j, what in ((0, "u sum of squares"), (1, "u max"), (4, "u_t sum of squares"), (5, "u_t max")):
            assert abs(cs[j] - rc[j]) <= 1e-12 * max(rc[j], 1e-300) + 1e-300, f"{what} differs after step {i}"
        for j, jn, what in ((2, 3, "u weighted sum"), (6, 7, "u_t weighted sum")):
            assert abs(cs[j] - rc[j]) <= 1e-12 * max(rc[jn], 1e-300), f"{what} differs after step {i}"
        if f"u_{i}" in z:
            pos = {k: j for j, k in enumerate(ref)}
            perm = np.array([pos[k] for k in mine])
            u_ref, v_ref = z[f"u_{i}"][perm], z[f"ut_{i}"][perm]
            assert np.abs(u - u_ref).max() <= 1e-12 * np.abs(u_ref).max()
            if i > 0:  # u_t carries the IPDG term sigma/dx [u] (dx = 2^-7): rounding amplified
                assert np.abs(v - v_ref).max() <= 1e-11 * np.abs(v_ref).max()
    op.close()
    g.close()


@pytest.mark.parametrize("prec", [amdg.FP64, amdg.MIXED])
def test_wave_terms_compose_the_fused_rhs(ctx, prec):
    """The right-hand side composed term by term as the reference's driver does (K grad u
    interpolation, DiffusionRHS::rhs_flx_gradu, rhs_vol, K u interpolation, rhs_flx_u, the IPDG
    term) into the grid's rhs vector equals the fused amdg_wave_rhs bitwise (same terms, same
    order); a group read before its interpolation is refused."""
    g = amdg.Grid(ctx, 2, 6, 2, level_init=3)
    g.init_separable_adaptive(O.wave_ic_terms(2), 1e-5)
    op = amdg.WaveOperator(g, 10.0)
    u = g.coefficients().copy()
    du = _on_device(u)
    out = torch.zeros_like(du)
    torch.cuda.synchronize()
    op.rhs_device(du.data_ptr(), out.data_ptr(), prec)
    ctx.synchronize()
    fused = out.cpu().numpy().reshape(u.shape)
    g.set_rhs_zero()
    with pytest.raises(amdg.AmdgError) as ei:
        op.rhs_add(op.RHS_FLX_U, prec)
    assert ei.value.status == 6
    op.interpolate(op.INTERP_GRADU, prec)
    op.rhs_add(op.RHS_FLX_GRADU, prec)
    op.rhs_add(op.RHS_VOL, prec)
    op.interpolate(op.INTERP_U, prec)
    op.rhs_add(op.RHS_FLX_U, prec)
    op.rhs_add(op.RHS_IPDG, prec)
    ctx.synchronize()
    assert np.array_equal(g.rhs(), fused)
    op.close()
    g.close()


def test_wave_rk4ode2nd_stages_match_the_fused_step(ctx):
    """RK4ODE2nd stage by stage (the integrator object, rhs_to_eigenvec + add_rhs_matrix per
    stage) equals amdg_wave_rk4_steps bitwise; EulerODE2nd's step_rk (rhs = the IPDG term alone)
    gives u + dt u_t and u_t + dt IPDG(u)."""
    g = amdg.Grid(ctx, 2, 5, 2)
    g.init_separable(O.wave_ic_terms(2))
    u0 = g.coefficients().copy()
    rng = np.random.default_rng(2)
    v0 = 1e-3 * rng.standard_normal(u0.shape)
    op = amdg.WaveOperator(g, 10.0)
    dt = 1e-4
    g.set_coefficients(u0)
    g.set_velocity(v0)
    op.rk4_steps(dt, 1)
    ctx.synchronize()
    want_u, want_v = g.coefficients().copy(), g.velocity().copy()
    g.set_coefficients(u0)
    g.set_velocity(v0)
    ode = amdg.ODE(g, amdg.ODE.RK4ODE2ND, dt)
    for stage in range(4):
        g.set_rhs_zero()
        op.interpolate(op.INTERP_GRADU)
        op.rhs_add(op.RHS_FLX_GRADU)
        op.rhs_add(op.RHS_VOL)
        op.interpolate(op.INTERP_U)
        op.rhs_add(op.RHS_FLX_U)
        ode.set_rhs_zero()
        ode.add_rhs_to_eigenvec()
        ode.add_wave_penalty(op)
        ode.step_stage(stage)
        ode.final()
    ctx.synchronize()
    assert np.array_equal(g.coefficients(), want_u)
    assert np.array_equal(g.velocity(), want_v)
    ode.close()
    # EulerODE2nd: u + dt v, v + dt IPDG(u)
    g.set_coefficients(u0)
    g.set_velocity(v0)
    pen = torch.zeros(g.dof, dtype=torch.float64, device="cuda")
    g.set_rhs_zero()
    op.rhs_add(op.RHS_IPDG)
    ctx.synchronize()
    ipdg = g.rhs().copy()
    ode = amdg.ODE(g, amdg.ODE.EULER_ODE2ND, dt)
    ode.set_rhs_zero()
    ode.add_wave_penalty(op)
    ode.step_stage(0)
    ode.final()
    ctx.synchronize()
    assert np.array_equal(g.coefficients(), u0 + dt * v0)
    assert np.array_equal(g.velocity(), v0 + dt * ipdg)
    del pen
    ode.close()
    op.close()
    g.close()
