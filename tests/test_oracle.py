"""The CPU oracle against the reference library's own outputs (golden
fixtures from oracle/ref_harness, see tests/golden/make_golden.py) and the
reference's known-answer unit tests for the path's ingredients."""
import math

import numpy as np
import pytest

import amdg_oracle as O
from helpers import align, golden, ic_terms, manifest, rel_err

LINEAR = [n for n, m in manifest().items() if m["kind"] == "linear"]
OPER = [n for n, m in manifest().items() if m["kind"] == "oper1d"]


@pytest.mark.parametrize("name", OPER)
def test_oper1d_matches_reference(name):
    m = manifest()[name]
    z = golden(name)
    mats = O.oper1d(m["N"], m["k"])
    for key in ("u_v", "u_vx", "ulft_vjp", "urgt_vjp"):
        scale = max(1.0, np.abs(z[key]).max())
        assert np.abs(mats[key] - z[key]).max() <= 1e-13 * scale * 10, key


@pytest.mark.parametrize("name", LINEAR)
def test_linear_matches_reference(name):
    m = manifest()[name]
    z = golden(name)
    dim, N, k = m["dim"], m["N"], m["k"]
    lv, sp = O.grid(dim, N)
    assert lv.shape[0] == m["elements"] == z["level"].shape[0]
    perm = align(z["level"], z["suppt"], lv, sp)
    coef = O.project_separable(N, k, dim, ic_terms(m["ic"], dim))
    u0 = O.init_separable(dim, N, k, lv, sp, coef)
    assert rel_err(u0, z["u0"][perm]) < 1e-13
    rhs = O.linear_rhs(dim, N, k, lv, sp, m["c"], z["u0"][perm])
    assert rel_err(rhs, z["rhs0"][perm]) < 1e-12
    uT = O.linear_rk3(dim, N, k, lv, sp, m["c"], z["u0"][perm], m["dt"], m["steps"])
    assert rel_err(uT, z["uT"][perm]) < 1e-12


@pytest.mark.parametrize("name", [n for n, m in manifest().items() if m["kind"] == "linear_long"])
def test_linear_long_fixture_matches_oracle(name):
    """The full-length linear fixture (T = 1): the oracle's projection gives its initial
    coefficients, and the oracle's quadrature of its final coefficients against the exact translated
    solution sin(2 pi (sum x - sum c T)) gives the reference's L1/L2/Linf errors (1 and 2 Gauss
    points).  The run itself is compared with the GPU path (the oracle's SSP-RK3 would take over
    a minute for 2561 steps)."""
    m = manifest()[name]
    z = golden(name)
    dim, N, k = m["dim"], m["N"], m["k"]
    lv, sp = O.grid(dim, N)
    perm = align(z["level"], z["suppt"], lv, sp)
    coef = O.project_separable(N, k, dim, ic_terms(m["ic"], dim))
    u0 = O.init_separable(dim, N, k, lv, sp, coef)
    assert rel_err(u0, z["u0"][perm]) < 1e-13
    T = m["steps"] * m["dt"]
    for gp in (1, 2):
        err = O.error_burgers(dim, N, k, z["level"], z["suppt"], z["uT"], gp, a=0.0, b=1.0, c=-sum(m["c"]) * T)
        ref = z[f"normerr_g{gp}"]
        assert np.all(np.abs(err - ref) <= 1e-10 * ref), (gp, err, ref)


def test_l2_error_matches_reference():
    name = "lin3d_n4_sinprod"
    m = manifest()[name]
    z = golden(name)
    dim, N, k = m["dim"], m["N"], m["k"]
    T = m["steps"] * m["dt"]
    lv, sp = z["level"], z["suppt"]
    exact = O.project_separable(N, k, dim, [lambda x, d: math.sin(2 * math.pi * (x - m["c"][d] * T))])[0]
    err = O.l2_error_split(dim, N, k, lv, sp, z["uT"], exact, 0.5 ** (0.5 * dim))
    assert abs(err - float(z["l2err"])) <= 1e-10 * max(err, 1e-30) + 1e-15


def test_alpert_orthonormal():
    # test/test_AlptBasis.cpp:8-36: Alpert basis orthonormal on [0,1] (PMAX=2, tol 1e-14)
    mats = O.oper1d(4, 2)
    assert np.abs(mats["u_v"] - np.eye(mats["u_v"].shape[0])).max() < 1e-13


@pytest.mark.parametrize("n", [1, 2, 3, 5, 10])
def test_gauss_legendre_exactness(n):
    # test/test_Quad.cpp:13-38: n-point rule integrates x^m exactly for m <= 2n-1
    x, w = O.gauss_legendre(n)
    for m in range(2 * n):
        exact = (1 - (-1) ** (m + 1)) / (m + 1)
        assert abs(np.dot(w, x ** m) - exact) < 5e-15 * 10


@pytest.mark.parametrize("dim,N,E", [(2, 7, 576), (3, 8, 4096), (4, 8, 10496), (6, 8, 47264), (2, 3, 20)])
def test_sparse_grid_counts(dim, N, E):
    assert O.lib().amdg_oracle_grid_count(dim, N, 1) == E


def test_full_grid_count():
    assert O.lib().amdg_oracle_grid_count(2, 3, 0) == 64


def test_linear_operator_is_linear():
    dim, N, k = 3, 3, 2
    lv, sp = O.grid(dim, N)
    rng = np.random.default_rng(0)
    a = rng.standard_normal((lv.shape[0], 27))
    b = rng.standard_normal((lv.shape[0], 27))
    c = [1.0, -0.5, 0.25]
    la = O.linear_rhs(dim, N, k, lv, sp, c, a)
    lb = O.linear_rhs(dim, N, k, lv, sp, c, b)
    lab = O.linear_rhs(dim, N, k, lv, sp, c, 2.0 * a - 3.0 * b)
    assert np.abs(lab - (2.0 * la - 3.0 * lb)).max() < 1e-10 * np.abs(lab).max()


def test_constant_mode_is_conserved():
    # the level-0 constant mode carries the mean, which the periodic advection operator conserves
    dim, N, k = 2, 4, 2
    lv, sp = O.grid(dim, N)
    rng = np.random.default_rng(1)
    u = rng.standard_normal((lv.shape[0], 9))
    rhs = O.linear_rhs(dim, N, k, lv, sp, [1.0, 1.0], u)
    root = np.where((lv == 0).all(axis=1))[0][0]
    assert abs(rhs[root, 0]) < 1e-10


BURGERS = [n for n, m in manifest().items() if m["kind"] == "burgers"]


@pytest.mark.parametrize("name", BURGERS)
def test_burgers_lagrange_path_matches_reference(name):
    """Point values, flux interpolation coefficients, RHS and RK3 steps of the
    Lagrange-interpolated Burgers operator against the reference's fast LU path."""
    m = manifest()[name]
    z = golden(name)
    dim, N, k = m["dim"], m["N"], m["k"]
    lv, sp = O.grid(dim, N)
    perm = align(z["level"], z["suppt"], lv, sp)
    coef = O.project_separable(N, k, dim, O.burgers_ic_terms(dim))
    u0 = O.init_separable(dim, N, k, lv, sp, coef)
    assert rel_err(u0, z["u0"][perm]) < 1e-13
    u0 = np.ascontiguousarray(z["u0"][perm])
    rhs, up, fu = O.burgers_rhs(dim, N, k, lv, sp, u0, m["alpha"])
    assert rel_err(up, z["up0"][perm]) < 1e-13
    for d in range(dim):
        assert rel_err(fu, z[f"fu0_{d}"][perm]) < 1e-12
    assert rel_err(rhs, z["rhs0"][perm]) < 5e-12
    uT = O.burgers_rk3(dim, N, k, lv, sp, u0, m["alpha"], m["dt"], m["steps"])
    assert rel_err(uT, z["uT"][perm]) < 1e-12


@pytest.mark.parametrize("degree", [3, 4])
def test_lagrange_basis_interpolates_its_nodes(degree):
    # hierarchical Lagrange basis: 1 at its own node, 0 at the other nodes of its element
    # (degree 4 points sit 1e-13 off the nodes, relative to the element size)
    O.lagr_degree(degree)
    for n, j in [(0, 1), (1, 1), (2, 1), (2, 3), (3, 5)]:
        for p in range(degree + 1):
            for q in range(degree + 1):
                x = O.lib().amdg_oracle_lagr_point(n, j, q)
                v = O.lib().amdg_oracle_lagr_val(n, j, p, x, 0)
                assert abs(v - (1.0 if p == q else 0.0)) < 1e-11
    O.lagr_degree(O.BURGERS_LAGR_DEGREE)


ADAPT = [n for n, m in manifest().items() if m["kind"] == "burgers_adapt"]


@pytest.mark.parametrize("name", ADAPT)
def test_adaptive_burgers_matches_reference(name):
    """Element sets bit-exact and coefficients to 1e-12 after adaptive init and
    every predictor/refine/RK3/coarsen step of the reference time loop."""
    m = manifest()[name]
    z = golden(name)
    dim = m["dim"]
    hist = O.burgers_adaptive_run(dim, m["n_init"], m["nmax"], m["eps"], m["eta"], m["alpha"], m["cfl"], m["umax"],
                                  m["steps"])
    for i, (keys, u, _dt) in enumerate(hist):
        ref_keys = O.arrays_to_keys(z[f"level_{i}"], z[f"suppt_{i}"])
        assert set(ref_keys) == set(keys), f"element set differs after step {i}"
        pos = {k: j for j, k in enumerate(ref_keys)}
        perm = np.array([pos[k] for k in keys])
        assert rel_err(u, z[f"u_{i}"][perm]) < 1e-12


LONG = [n for n, m in manifest().items() if m["kind"] == "burgers_adapt_long"]


@pytest.mark.parametrize("name", LONG)
def test_adaptive_burgers_long_fixture_first_steps(name):
    """The oracle against the first two steps of the full-length 3D adaptive Burgers fixture
    (the whole run is checked on the GPU)."""
    from golden.make_golden import checksums
    m = manifest()[name]
    z = golden(name)
    dim = m["dim"]
    hist = O.burgers_adaptive_run(dim, m["n_init"], m["nmax"], m["eps"], m["eta"], m["alpha"], m["cfl"], m["umax"], 2)
    for i, (keys, u, dt) in enumerate(hist):
        ref_keys = O.arrays_to_keys(z[f"level_{i}"], z[f"suppt_{i}"])
        assert set(keys) == set(ref_keys)
        if dt is not None:
            assert dt == z["dt"][i - 1]
        lv, sp = O.keys_to_arrays(keys, dim)
        cs, ref_cs = checksums(lv, sp, u), z["checksums"][i]
        assert abs(cs[0] - ref_cs[0]) <= 1e-12 * ref_cs[0]
        assert abs(cs[2] - ref_cs[2]) <= 1e-12 * ref_cs[3]
        pos = {k: j for j, k in enumerate(ref_keys)}
        perm = np.array([pos[k] for k in keys])
        assert rel_err(u, z[f"u_{i}"][perm]) < 1e-12


def test_fast_transforms_equal_direct_sums_on_sparse_grids():
    """On a sparse grid the reference's L/U partial sums equal the direct sums
    over element pairs (an independent check of both formulations)."""
    dim, N, k = 3, 4, 2
    lv, sp = O.grid(dim, N)
    u = O.init_separable(dim, N, k, lv, sp, O.project_separable(N, k, dim, O.burgers_ic_terms(dim)))
    a = O.burgers_rhs(dim, N, k, lv, sp, u, 0.8)[0]
    b = O.burgers_rhs(dim, N, k, lv, sp, u, 0.8, direct=True)[0]
    assert rel_err(a, b) < 1e-12


def test_mlp_oracle_gradient_matches_finite_differences():
    """The CPU classifier reference: analytic backward pass against central
    finite differences in float64 (the device gradients are checked against it)."""
    rng = np.random.default_rng(0)
    dims = [12, 8, 8, 8, 3]
    n_par = sum(dims[i] * dims[i + 1] + dims[i + 1] for i in range(len(dims) - 1))
    params = rng.standard_normal(n_par) * 0.4
    x = rng.standard_normal((16, dims[0]))
    labels = rng.integers(0, 3, 16)
    _, g = O.mlp_loss_grad(params, dims, x, labels)
    h = 1e-6
    for i in rng.choice(n_par, 40, replace=False):
        p1, p2 = params.copy(), params.copy()
        p1[i] += h
        p2[i] -= h
        fd = (O.mlp_loss(p1, dims, x, labels) - O.mlp_loss(p2, dims, x, labels)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-7 + 1e-5 * abs(fd)


BURGERS = [n for n, m in manifest().items() if m["kind"] == "burgers"]


@pytest.mark.parametrize("name", BURGERS)
def test_point_values_and_exact_solution_match_reference(name):
    """DGSolution::val and BurgersExact at the reference's 48 fixed points."""
    m = manifest()[name]
    z = golden(name)
    dim = m["dim"]
    vals = z["vals"]
    x = vals[:, :dim]
    v = O.eval_points(dim, m["N"], 2, z["level"], z["suppt"], z["uT"], x)
    assert np.abs(v - vals[:, dim]).max() <= 1e-14 * max(1.0, np.abs(vals[:, dim]).max())
    ex = O.burgers_exact(dim, x, t=m["steps"] * m["dt"])
    assert np.abs(ex - vals[:, dim + 1]).max() <= 1e-15


@pytest.mark.parametrize("name", [n for n in BURGERS if manifest()[n]["N"] <= 4])
@pytest.mark.parametrize("gauss", [1, 2])
def test_quadrature_error_matches_reference(name, gauss):
    """get_error_no_separable_scalar (L1, L2, Linf) against the exact Burgers solution."""
    m = manifest()[name]
    z = golden(name)
    err = O.error_burgers(m["dim"], m["N"], 2, z["level"], z["suppt"], z["uT"], gauss, t=m["steps"] * m["dt"])
    ref = z[f"normerr_g{gauss}"]
    assert np.all(np.abs(err - ref) <= 1e-12 * ref)


def test_burgers_wave_solves_its_characteristic_equation():
    """v = sin(2 pi (x - v t)) and the odd symmetry v(x) = -v(1 - x) before the shock time."""
    rng = np.random.default_rng(3)
    for x, t in zip(rng.uniform(-2, 3, 64), rng.uniform(0.0, 0.15, 64)):
        v = O.lib().amdg_oracle_burgers_wave(x, t)
        assert abs(v - math.sin(2 * math.pi * (x - v * t))) <= 1e-12
        assert abs(v + O.lib().amdg_oracle_burgers_wave(1 - x, t)) <= 1e-12


WAVE = [n for n, m in manifest().items() if m["kind"] == "wave"]
WAVE_ADAPT = [n for n, m in manifest().items() if m["kind"] == "wave_adapt"]


@pytest.mark.parametrize("name", WAVE_ADAPT)
def test_adaptive_wave_matches_reference(name):
    """The adaptive wave loop (EulerODE2nd predictor with the IPDG-only right-hand side, refine
    on ||u|| + ||u_t||, RK4ODE2nd, coarsen): element sets bit-exact and u, u_t to 1e-12 of
    their largest entry after the adaptive initialisation and every step."""
    m = manifest()[name]
    z = golden(name)
    dim = m["dim"]
    hist = O.wave_adaptive_run(dim, m["n_init"], m["nmax"], m["eps"], m["eta"], m["sigma"], m["cfl"], 1.0, m["steps"])
    assert len(hist) == m["steps"] + 1
    for i, (keys, u, v, _dt) in enumerate(hist):
        ref_keys = O.arrays_to_keys(z[f"level_{i}"], z[f"suppt_{i}"])
        assert sorted(ref_keys) == sorted(keys), f"element set differs after step {i}"
        pos = {kk: j for j, kk in enumerate(ref_keys)}
        perm = [pos[kk] for kk in keys]
        assert np.abs(u - z[f"u_{i}"][perm]).max() <= 1e-12 * np.abs(z[f"u_{i}"]).max()
        assert np.abs(v - z[f"ut_{i}"][perm]).max() <= 1e-12 * max(np.abs(z[f"ut_{i}"]).max(), 1e-30)


@pytest.mark.parametrize("name", WAVE)
def test_wave_operator_matches_reference(name):
    """u_tt = div(K grad u): Lagrange-interpolated K grad u and K u, DiffusionRHS terms, IPDG
    penalty, RK4ODE2nd (03_wave_06_var_coeff_adapt.cpp) against the reference run."""
    m = manifest()[name]
    z = golden(name)
    dim, N = m["dim"], m["N"]
    rhs = O.wave_rhs(dim, N, 2, z["level"], z["suppt"], z["u0"], m["sigma"])
    assert rel_err(rhs, z["rhs0"]) < 1e-12
    u, v = O.wave_rk4(dim, N, 2, z["level"], z["suppt"], z["u0"], np.zeros_like(z["u0"]), m["sigma"], m["dt"],
                      m["steps"])
    assert rel_err(u, z["uT"]) < 1e-13
    assert rel_err(v, z["vT"]) < 1e-12


INTP = [n for n, m in sorted(manifest().items()) if m["kind"] == "intp_init"]


def gaussian_bump(m):
    """exp(-width |x - centre|^2) on an (n, dim) array of points, as the reference run evaluates it."""
    c, w = np.asarray(m["centre"]), m["width"]
    return lambda x: np.exp(-w * np.sum((x - c) ** 2, axis=1))


@pytest.mark.parametrize("name", INTP)
def test_adaptive_interpolation_init_matches_reference(name):
    """DGAdaptIntp::init_adaptive_intp: the adaptive Lagrange interpolation (surplus indicator
    with the Lagrange mass diagonal, refine and fill holes until nothing changes) gives the
    reference's element set bit-exact, and the fast Lagrange-to-Alpert transform its
    coefficients to 1e-12 of their largest entry."""
    m = manifest()[name]
    z = golden(name)
    keys, u, rounds = O.init_adaptive_intp(m["dim"], m["n_init"], m["nmax"], m["k"], gaussian_bump(m), m["eps"],
                                           m["lagr_degree"])
    assert rounds > 0
    ref_keys = O.arrays_to_keys(z["level"], z["suppt"])
    assert sorted(ref_keys) == sorted(keys)
    pos = {kk: j for j, kk in enumerate(ref_keys)}
    perm = [pos[kk] for kk in keys]
    assert rel_err(u, z["u"][perm]) < 1e-12


INTP_ERR = [n for n, m in sorted(manifest().items()) if m["kind"] == "intp_error"]


@pytest.mark.parametrize("name", INTP_ERR)
def test_interpolated_split_error_matches_reference(name):
    """DGAdaptIntp::get_L2_error_split_adaptive_intp_scalar of a coarse adaptive interpolation
    against a finer one: both element sets bit-exact, the error to 1e-9 relative (err^2 is a
    difference of sums of squares, so the error's own accuracy is that of the cancellation)."""
    m = manifest()[name]
    z = golden(name)
    f = gaussian_bump(m)
    ka, ua, _ = O.init_adaptive_intp(m["dim"], m["n_init"], m["nmax"], m["k"], f, m["eps_a"], m["lagr_degree"])
    kb, ub, _ = O.init_adaptive_intp(m["dim"], m["n_init"], m["nmax"], m["k"], f, m["eps_b"], m["lagr_degree"])
    assert sorted(ka) == sorted(O.arrays_to_keys(z["level_a"], z["suppt_a"]))
    assert sorted(kb) == sorted(O.arrays_to_keys(z["level_b"], z["suppt_b"]))
    err = O.l2_error_split_grids(ka, ua, kb, ub)
    assert abs(err - m["err"]) <= 1e-9 * m["err"]


HERM = [n for n, m in manifest().items() if m["kind"] == "burgers_herm"]


@pytest.mark.parametrize("name", HERM)
def test_burgers_hermite_path_matches_reference(name):
    """Cubic Hermite interpolation of the 2D Burgers flux (HermInterpolation::nonlinear_Herm_2D_fast,
    HyperbolicSameFluxHermRHS): u_h and its slopes at the Hermite points (direct sums and fast
    transforms), the flux's Hermite coefficients, the right-hand side and SSP-RK3 steps against the
    reference."""
    m = manifest()[name]
    z = golden(name)
    N, k = m["N"], m["k"]
    lv, sp = O.grid(2, N)
    perm = align(z["level"], z["suppt"], lv, sp)
    coef = O.project_separable(N, k, 2, O.burgers_ic_terms(2))
    u0 = O.init_separable(2, N, k, lv, sp, coef)
    assert rel_err(u0, z["u0"][perm]) < 1e-13
    u0 = np.ascontiguousarray(z["u0"][perm])
    assert rel_err(O.herm_point_values(2, N, k, lv, sp, u0, direct=True), z["up0"][perm]) < 1e-13
    rhs, up, fu = O.burgers_herm_rhs(N, k, lv, sp, u0, m["alpha"])
    assert rel_err(up, z["up0"][perm]) < 1e-13
    assert rel_err(fu, z["fu0"][perm]) < 1e-12
    assert rel_err(rhs, z["rhs0"][perm]) < 5e-12
    uT = O.burgers_herm_rk3(N, k, lv, sp, u0, m["alpha"], m["dt"], m["steps"])
    assert rel_err(uT, z["uT"][perm]) < 1e-12


def test_hermite_basis_interpolates_its_dofs():
    """Each Hermite function has value (or slope) 1 at its own dof and 0 at the element's other
    dofs; the points sit 1e-13 off the nodes (relative to the element size)."""
    for n, j in [(0, 1), (1, 1), (2, 1), (2, 3), (3, 5)]:
        h = 1.0 if n <= 1 else 2.0 ** (1 - n)
        for p in range(4):
            for q in range(4):
                x = O.lib().amdg_oracle_herm_point(n, j, q)
                v = O.lib().amdg_oracle_herm_val(n, j, p, q // 2, x, 0)
                assert abs(v - (1.0 if p == q else 0.0)) < 1e-11 / h, (n, j, p, q)


HERM_ADAPT = [n for n, m in manifest().items() if m["kind"] == "burgers_herm_adapt"]


@pytest.mark.parametrize("name", HERM_ADAPT)
def test_adaptive_burgers_hermite_matches_reference(name):
    """The adaptive loop of 02_hyperbolic_05_burgers_adapt.cpp (Hermite flux): element sets
    bit-exact and coefficients to 1e-12 after the adaptive init and every step; the long
    fixture's first two steps only (the whole run is checked on the GPU)."""
    from golden.make_golden import checksums
    m = manifest()[name]
    z = golden(name)
    steps = m["steps"] if m["snapshots"] is None else 2
    hist = O.burgers_herm_adaptive_run(m["n_init"], m["nmax"], m["eps"], m["eta"], m["alpha"], m["cfl"], steps)
    for i, (keys, u, dt) in enumerate(hist):
        ref_keys = O.arrays_to_keys(z[f"level_{i}"], z[f"suppt_{i}"])
        assert set(ref_keys) == set(keys), f"element set differs after step {i}"
        if dt is not None:
            assert dt == z["dt"][i - 1]
        lv, sp = O.keys_to_arrays(keys, 2)
        cs, ref_cs = checksums(lv, sp, u), z["checksums"][i]
        assert abs(cs[2] - ref_cs[2]) <= 1e-12 * ref_cs[3]
        pos = {kk: jj for jj, kk in enumerate(ref_keys)}
        perm = np.array([pos[kk] for kk in keys])
        assert rel_err(u, z[f"u_{i}"][perm]) < 1e-12
