"""C-ABI library: loads, exports every declared symbol, and its host-side
set-up (1D operator matrices, element enumeration) matches the reference
fixtures and the oracle.  No compute calls needing a GPU."""
import ctypes as C

import numpy as np
import pytest

import amdg
import amdg_oracle as O
from helpers import golden, manifest


def test_library_exports_every_declared_symbol():
    lib = amdg.load()
    names = amdg.declared_functions()
    assert len(names) >= 25
    for n in names:
        assert hasattr(lib, n), n


def test_abi_version():
    assert amdg.load().amdg_abi_version() == 6


@pytest.mark.parametrize("name", [n for n, m in manifest().items() if m["kind"] == "oper1d"])
def test_oper1d_matches_reference(name):
    m = manifest()[name]
    z = golden(name)
    mats = amdg.oper1d(m["N"], m["k"])
    for key in ("u_v", "u_vx", "ulft_vjp", "urgt_vjp"):
        scale = max(1.0, np.abs(z[key]).max())
        assert np.abs(mats[key] - z[key]).max() <= 1e-12 * scale, key


@pytest.mark.parametrize("dim,N,sparse", [(1, 5, 1), (2, 7, 1), (3, 4, 1), (4, 3, 1), (2, 3, 0), (6, 8, 1)])
def test_grid_enumeration_matches_oracle(dim, N, sparse):
    lv, sp = amdg.enumerate_grid(dim, N, bool(sparse))
    lv2, sp2 = O.grid(dim, N, bool(sparse))
    assert lv.shape == lv2.shape
    assert (lv == lv2).all() and (sp == sp2).all()


def test_bad_arguments_are_rejected():
    lib = amdg.load()
    n = C.c_int64()
    assert lib.amdg_grid_enumerate(0, 3, 1, C.byref(n), None, None) == 1
    assert lib.amdg_grid_enumerate(7, 3, 1, C.byref(n), None, None) == 1
    assert lib.amdg_oper1d_build(3, 5, None, None, None, None) == 1
    assert b"degree" in lib.amdg_last_error()
    assert lib.amdg_grid_destroy(None) == 0
    assert lib.amdg_linear_apply(None, None, None, 0) == 1
