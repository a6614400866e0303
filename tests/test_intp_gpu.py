"""Adaptive-interpolation initialisation (DGAdaptIntp::init_adaptive_intp) on the GPU: element
sets bit-exact and Alpert coefficients to 1e-12 against the reference runs (2D and 3D, Lagrange
degree 3 and 4), and against the oracle on larger grids (3D to level 8, 4D)."""
import numpy as np
import pytest

import amdg
import amdg_oracle as O
from helpers import align, golden, manifest, rel_err

pytestmark = pytest.mark.gpu

INTP = [n for n, m in sorted(manifest().items()) if m["kind"] == "intp_init"]


def bump(centre, width):
    c = np.asarray(centre)
    return lambda x: np.exp(-width * np.sum((x - c) ** 2, axis=1))


@pytest.mark.parametrize("name", INTP)
def test_init_adaptive_intp_matches_reference(ctx, name):
    m = manifest()[name]
    z = golden(name)
    g = amdg.Grid(ctx, m["dim"], m["nmax"], m["k"], level_init=m["n_init"])
    rounds = g.init_adaptive_intp(bump(m["centre"], m["width"]), m["eps"], m["lagr_degree"])
    assert rounds > 0
    lv, sp = g.elements()
    perm = align(z["level"], z["suppt"], lv, sp)
    assert rel_err(g.coefficients(), z["u"][perm]) < 1e-12
    g.close()


@pytest.mark.parametrize("dim,n_init,nmax,eps,degree,centre,width", [
    (3, 3, 8, 1e-5, 3, (0.3, 0.4, 0.5), 50.0),
    (4, 2, 6, 1e-4, 4, (0.45,) * 4, 20.0),
])
def test_init_adaptive_intp_matches_oracle(ctx, dim, n_init, nmax, eps, degree, centre, width):
    f = bump(centre, width)
    keys, u, rounds = O.init_adaptive_intp(dim, n_init, nmax, 2, f, eps, degree)
    g = amdg.Grid(ctx, dim, nmax, 2, level_init=n_init)
    assert g.init_adaptive_intp(f, eps, degree) == rounds
    lv, sp = O.keys_to_arrays(keys, dim)
    glv, gsp = g.elements()
    perm = align(lv, sp, glv, gsp)
    assert rel_err(g.coefficients(), u[perm]) < 1e-12
    g.close()


def test_init_adaptive_intp_rejects_bad_input(ctx):
    g = amdg.Grid(ctx, 2, 5, 2, level_init=2)
    with pytest.raises(RuntimeError):
        g.init_adaptive_intp(bump((0.5, 0.5), 10.0), 1e-4, degree=6)
    with pytest.raises(RuntimeError):
        g.init_adaptive_intp(lambda x: np.full(len(x), np.nan), 1e-4)
    g.close()


INTP_ERR = [n for n, m in sorted(manifest().items()) if m["kind"] == "intp_error"]


@pytest.mark.parametrize("name", INTP_ERR)
def test_interpolated_split_error_matches_reference(ctx, name):
    """DGAdaptIntp::get_L2_error_split_adaptive_intp_scalar of a coarse adaptive interpolation
    against a finer one: to 1e-9 of the reference's value (err^2 is a difference of sums of
    squares); the distance of a solution to itself is at roundoff level."""
    m = manifest()[name]
    f = bump(m["centre"], m["width"])
    grids = []
    for eps in (m["eps_a"], m["eps_b"]):
        g = amdg.Grid(ctx, m["dim"], m["nmax"], m["k"], level_init=m["n_init"])
        g.init_adaptive_intp(f, eps, m["lagr_degree"])
        grids.append(g)
    a, b = grids
    err = a.l2_error_split_grid(b)
    assert abs(err - m["err"]) <= 1e-9 * m["err"]
    assert abs(a.l2_error_split_grid(a)) < 1e-6
    other = amdg.Grid(ctx, m["dim"], m["nmax"] - 1, m["k"])
    with pytest.raises(RuntimeError):
        a.l2_error_split_grid(other)
    for g in (a, b, other):
        g.close()
