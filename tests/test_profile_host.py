"""The host phase profile API: symbols, argument checks and bookkeeping that
need no device (a context is a GPU object, so only the null-argument paths
run here)."""
import ctypes as C

import numpy as np

import amdg


def test_profile_rejects_null_context():
    lib = amdg.load()
    err_arg = 1  # AMDG_ERR_ARG
    assert lib.amdg_context_profile(None, 1) == err_arg
    sec = np.zeros(8)
    assert lib.amdg_context_profile_read(None, sec.ctypes.data_as(C.c_void_p), None) == err_arg


def test_phase_names_match_header():
    import re
    hdr = open(amdg.HEADER).read()
    names = re.findall(r"AMDG_PHASE_([A-Z0-9_]+) = (\d+)", hdr)
    phases = [n.lower() for n, i in sorted(names, key=lambda t: int(t[1])) if n != "COUNT"]
    assert tuple(phases) == amdg.Context.PHASES
