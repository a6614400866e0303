"""Checkpoint / restart of a grid (keys, coefficients, u_t, time) and the element-level dump of
IO::output_element_level_support (IO.cpp:502-517)."""
import os

import numpy as np
import pytest

import amdg
import amdg_oracle as O

pytestmark = pytest.mark.gpu


def _adaptive_wave(ctx):
    g = amdg.Grid(ctx, 2, 6, 2, level_init=3)
    g.init_separable_adaptive(O.wave_ic_terms(2), 1e-4)
    op = amdg.WaveOperator(g, 10.0)
    for _ in range(3):
        op.adaptive_step(0.1, 1.0, 1e-4, 1e-5)
    return g, op


def test_restart_reproduces_the_run(ctx, tmp_path):
    """Save after three adaptive wave steps, load, and step both copies: bitwise the same."""
    g, op = _adaptive_wave(ctx)
    path = str(tmp_path / "wave.ckpt")
    g.save(path, time=0.125)
    h, t = amdg.Grid.load(ctx, path)
    assert t == 0.125
    assert (h.dim, h.nmax, h.k, h.num_elements, h.dof) == (g.dim, g.nmax, g.k, g.num_elements, g.dof)
    for a, b in zip(g.elements(), h.elements()):
        assert np.array_equal(a, b)
    assert np.array_equal(g.coefficients(), h.coefficients())
    assert np.array_equal(g.velocity(), h.velocity())
    op2 = amdg.WaveOperator(h, 10.0)
    for _ in range(2):
        assert op.adaptive_step(0.1, 1.0, 1e-4, 1e-5) == op2.adaptive_step(0.1, 1.0, 1e-4, 1e-5)
    for a, b in zip(g.elements(), h.elements()):
        assert np.array_equal(a, b)
    assert np.array_equal(g.coefficients(), h.coefficients())
    assert np.array_equal(g.velocity(), h.velocity())
    for x in (op, op2, g, h):
        x.close()


def test_grid_without_velocity_round_trips(ctx, tmp_path):
    g = amdg.Grid(ctx, 3, 4, 2)
    rng = np.random.default_rng(0)
    g.set_coefficients(rng.standard_normal((g.num_elements, g.block)))
    path = str(tmp_path / "lin.ckpt")
    g.save(path)
    h, t = amdg.Grid.load(ctx, path)
    assert t == 0.0
    assert np.array_equal(g.coefficients(), h.coefficients())
    with pytest.raises(RuntimeError):
        h.velocity()  # no u_t stored, none created
    g.close()
    h.close()


def test_damaged_checkpoints_are_refused(ctx, tmp_path):
    g, op = _adaptive_wave(ctx)
    path = str(tmp_path / "good.ckpt")
    g.save(path)
    raw = open(path, "rb").read()
    cases = {
        "flipped": raw[:100] + bytes([raw[100] ^ 1]) + raw[101:],
        "truncated": raw[:-9],
        "magic": b"X" + raw[1:],
        "extended": raw + b"\0" * 8,
    }
    for name, data in cases.items():
        bad = str(tmp_path / f"{name}.ckpt")
        with open(bad, "wb") as f:
            f.write(data)
        with pytest.raises(RuntimeError):
            amdg.Grid.load(ctx, bad)
    with pytest.raises(RuntimeError):
        amdg.Grid.load(ctx, str(tmp_path / "missing.ckpt"))
    assert not os.path.exists(path + ".tmp")
    op.close()
    g.close()


def test_level_support_dump(ctx, tmp_path):
    g, op = _adaptive_wave(ctx)
    path = str(tmp_path / "level_support.txt")
    g.write_level_support(path)
    lines = open(path).read().splitlines()
    lv, sp = g.elements()
    assert len(lines) == g.num_elements
    for line, l_e, s_e in zip(lines, lv, sp):
        want = ""
        for n, j in zip(l_e, s_e):
            xl, xr = (0.0, 1.0) if n <= 1 else (2.0 ** (1 - n) * (j - 1) / 2, 2.0 ** (1 - n) * (j + 1) / 2)
            want += "%d %g %g " % (n, xl, xr)
        assert line == want
    op.close()
    g.close()
