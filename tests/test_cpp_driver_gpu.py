"""The C++ mirror of the reference driver API (host/amdg_dg.hpp): the
example driver built like example/02_hyperbolic_01_scalar_const_coefficient.cpp
runs on the GPU and reproduces the oracle's L2 error."""
import math
import os
import subprocess

import numpy as np
import pytest

import amdg
import amdg_oracle as O

pytestmark = pytest.mark.gpu

EXE = os.path.join(os.path.dirname(amdg.LIB_PATH), "hyperbolic_const_coefficient")


def test_cpp_driver_matches_oracle():
    assert os.path.exists(EXE), "example driver not built"
    N, T = 5, 0.05
    out = subprocess.run([EXE, str(N), str(T)], capture_output=True, text=True, timeout=300, check=True).stdout
    fields = dict(line.split(":", 1) for line in out.splitlines() if ":" in line)
    err = float(fields["L2 error at final time"])
    head = out.splitlines()[0].split()
    steps, dt = int(head[5]), float(head[7])
    dim, k = 2, 2
    lv, sp = O.grid(dim, N)
    u0 = O.init_separable(dim, N, k, lv, sp, O.project_separable(N, k, dim, O.sin_sum_terms(dim)))
    uT = O.linear_rk3(dim, N, k, lv, sp, [1.0, 1.0], u0, dt, steps)
    exact = O.project_separable(N, k, dim, O.sin_sum_terms(dim, shift=2 * T))
    # |u - u_h|^2 = 1/2 + |u_h|^2 - 2 sum_terms <u_h, term>
    n2 = float(np.sum(uT * uT))
    cross = sum(0.5 * (1.0 + n2 - O.l2_error_split(dim, N, k, lv, sp, uT, exact[t], 1.0) ** 2) for t in range(2))
    ref = math.sqrt(max(0.0, 0.5 + n2 - 2.0 * cross))
    assert abs(err - ref) <= 1e-6 * ref
    assert ref < 1e-3


def test_cpp_wave_driver_matches_oracle():
    """The adaptive wave driver written against the C++ mirror statement by statement like
    example/03_wave_06_var_coeff_adapt.cpp (LagrInterpolation, DiffusionRHS, DiffusionAlpt,
    EulerODE2nd, RK4ODE2nd) ends on the oracle's element set and coefficients."""
    exe = os.path.join(os.path.dirname(amdg.LIB_PATH), "wave_var_coeff_adapt")
    assert os.path.exists(exe), "example driver not built"
    n_init, nmax, steps, eps, eta = 3, 5, 4, 1e-5, 1e-6
    out = subprocess.run([exe, str(n_init), str(nmax), str(steps), repr(eps), repr(eta)], capture_output=True,
                         text=True, timeout=300, check=True).stdout
    fields = dict(line.split(":", 1) for line in out.splitlines() if ":" in line)
    head = out.splitlines()[0].split()
    elements, t = int(head[5]), float(head[3])
    hist = O.wave_adaptive_run(2, n_init, nmax, eps, eta, 10.0, 0.1, 1.0, steps)
    keys, u, v, _dt = hist[-1]
    assert elements == len(keys)
    assert abs(t - sum(h[3] for h in hist[1:])) <= 1e-15
    su, sut = float(np.sum(u * u)), float(np.sum(v * v))
    assert abs(float(fields["sum of squares u"]) - su) <= 1e-12 * su
    assert abs(float(fields["sum of squares u_t"]) - sut) <= 1e-11 * sut


def test_cpp_wave_driver_matches_reference_long_run():
    """The same driver (term by term: EulerODE2nd predictor, refine, RK4ODE2nd stages of
    LagrInterpolation::var_coeff_* + DiffusionRHS + the IPDG matrix term, coarsen) over the
    reference's 24-step max-level-7 run: the final element count and the sums of squares of u and
    u_t equal the reference run's to 1e-12 / 1e-11 relative."""
    from helpers import golden, manifest
    exe = os.path.join(os.path.dirname(amdg.LIB_PATH), "wave_var_coeff_adapt")
    m = manifest()["wave_adapt2d_n7_long"]
    z = golden("wave_adapt2d_n7_long")
    out = subprocess.run([exe, str(m["n_init"]), str(m["nmax"]), str(m["steps"]), repr(m["eps"]), repr(m["eta"])],
                         capture_output=True, text=True, timeout=600, check=True).stdout
    fields = dict(line.split(":", 1) for line in out.splitlines() if ":" in line)
    head = out.splitlines()[0].split()
    assert int(head[5]) == m["elements"][-1]
    cs = z["checksums"][-1]
    assert abs(float(fields["sum of squares u"]) - cs[0]) <= 1e-12 * cs[0]
    assert abs(float(fields["sum of squares u_t"]) - cs[4]) <= 1e-11 * cs[4]


def test_cpp_intp_driver_matches_oracle():
    """The linear driver with the reference's own initialisation (adaptive Lagrange interpolation
    of degree 5, msh_case 1, of cos(2 pi (x + y))) and error (split L2 distance to the exact
    solution interpolated with refine 1e-6): the oracle's element counts and error."""
    exe = os.path.join(os.path.dirname(amdg.LIB_PATH), "hyperbolic_const_coefficient_intp")
    assert os.path.exists(exe), "example driver not built"
    N, T, dim = 5, 0.05, 2
    out = subprocess.run([exe, str(N), str(T)], capture_output=True, text=True, timeout=300, check=True).stdout
    fields = dict(line.split(":", 1) for line in out.splitlines() if ":" in line)
    err = float(fields["L2 error at final time"])
    head = out.splitlines()[0].split()
    elements, steps, dt, elements_ext = int(head[1]), int(head[5]), float(head[7]), int(head[9])

    def f(shift):
        return lambda x: np.cos(2 * np.pi * (np.sum(x, axis=1) - shift))

    keys, u0, _ = O.init_adaptive_intp(dim, N, N, 2, f(0.0), 1e10, 5)
    lv, sp = O.keys_to_arrays(keys, dim)
    uT = O.linear_rk3(dim, N, 2, lv, sp, [1.0, 1.0], u0, dt, steps)
    keys_ext, u_ext, _ = O.init_adaptive_intp(dim, N, N, 2, f(dim * T), 1e-6, 5)
    ref = O.l2_error_split_grids(keys_ext, u_ext, keys, uT)
    assert (elements, elements_ext) == (len(keys), len(keys_ext))
    assert abs(err - ref) <= 1e-7 * ref
    assert 0 < ref < 1e-2


def _read_elements(path, dim):
    rows = np.loadtxt(path, ndmin=2)
    return rows[:, :dim].astype(int), rows[:, dim:2 * dim].astype(int), rows[:, 2 * dim:]


@pytest.mark.parametrize("name", ["burgers_adapt3d", "burgers_adapt3d_config3"])
def test_cpp_burgers_driver_matches_reference(tmp_path, name):
    """The adaptive Burgers driver written call for call like the reference's loop (LagrInterpolation,
    HyperbolicLagrRHS, HyperbolicAlptRHS, ForwardEuler predictor, refine, RK3SSP stages, coarsen)
    ends on the reference's element set, coefficients to 1e-12 of their largest entry."""
    from helpers import golden, manifest, rel_err
    exe = os.path.join(os.path.dirname(amdg.LIB_PATH), "burgers_adapt")
    assert os.path.exists(exe), "example driver not built"
    m = manifest()[name]
    z = golden(name)
    out_file = str(tmp_path / "u.txt")
    args = [m["dim"], m["n_init"], m["nmax"], m["steps"], repr(m["eps"]), repr(m["eta"]), repr(m["alpha"]), out_file]
    subprocess.run([exe] + [str(a) for a in args], capture_output=True, text=True, timeout=600, check=True)
    lv, sp, u = _read_elements(out_file, m["dim"])
    s = m["steps"]
    keys = O.arrays_to_keys(lv, sp)
    ref_keys = O.arrays_to_keys(z[f"level_{s}"], z[f"suppt_{s}"])
    assert set(keys) == set(ref_keys)
    pos = {k: j for j, k in enumerate(ref_keys)}
    assert rel_err(u, z[f"u_{s}"][[pos[k] for k in keys]]) < 1e-12


@pytest.mark.parametrize("name", ["burgers_herm_adapt2d", "burgers_herm_adapt2d_n8_T003"])
def test_cpp_hermite_burgers_driver_matches_reference(tmp_path, name):
    """example/02_hyperbolic_05_burgers_adapt.cpp rewritten against amdg_dg.hpp statement by
    statement (HermInterpolation, FastHermIntp, HyperbolicSameFluxHermRHS, the Lax-Friedrichs
    matrix assembled by HyperbolicAlpt::assemble_matrix_flx_scalar and added by add_rhs_matrix,
    ForwardEuler predictor, refine, RK3SSP stages, coarsen) ends on the reference's element set,
    coefficients to 1e-12 of their largest entry."""
    from helpers import golden, manifest, rel_err
    exe = os.path.join(os.path.dirname(amdg.LIB_PATH), "burgers_herm_adapt")
    assert os.path.exists(exe), "example driver not built"
    m = manifest()[name]
    z = golden(name)
    s = m["steps"]
    out_file = str(tmp_path / "u.txt")
    args = [m["n_init"], m["nmax"], 1.0, repr(m["eps"]), repr(m["eta"]), s, out_file]
    res = subprocess.run([exe] + [str(a) for a in args], capture_output=True, text=True, timeout=600, check=True)
    assert res.stdout.startswith(f"steps {s} ")
    lv, sp, u = _read_elements(out_file, 2)
    keys = O.arrays_to_keys(lv, sp)
    ref_keys = O.arrays_to_keys(z[f"level_{s}"], z[f"suppt_{s}"])
    assert set(keys) == set(ref_keys)
    pos = {k: j for j, k in enumerate(ref_keys)}
    assert rel_err(u, z[f"u_{s}"][[pos[k] for k in keys]]) < 1e-12
