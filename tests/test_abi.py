"""The C ABI library loads and exports every function include/mfree_gb300.h declares;
host-only entry points behave like the reference's set-up code.  No GPU needed."""
import ctypes
import os
import re

import numpy as np

from conftest import ROOT, gpu_available
from mfree_iwf_gb300 import scenarios as S


def declared_functions():
    names = []
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            src = open(os.path.join(ROOT, "include", f)).read()
            names += re.findall(r"MF_API\s+[\w\s\*]+?\b(mf_\w+)\s*\(", src)
    return sorted(set(names))


def test_library_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n


def test_create_without_device_reports_no_device(lib):
    import mfree_iwf_gb300 as M
    if gpu_available():
        return
    cfg = M.MfConfig(1, 0, 0, 200, 1e-6, 0.0, 0, 0)
    h = ctypes.c_void_p()
    assert lib.mf_create(ctypes.byref(cfg), ctypes.byref(h)) == -9  # MF_ERR_NO_DEVICE


def test_convex_hull_matches_reference_setup(lib):
    import mfree_iwf_gb300 as M
    from conftest import GOLDEN
    ref = S.read_case(os.path.join(GOLDEN, "rings_monaghan_contact.case"))
    for b in ref.bodies:
        h = M.convex_hull(b.arrays["x"], b.arrays["y"])
        assert np.array_equal(h, b.hull)
        assert np.array_equal(S.convex_hull(b.arrays["x"], b.arrays["y"]), b.hull)


def test_status_strings(lib):
    lib.mf_status_string.restype = ctypes.c_char_p
    assert lib.mf_status_string(0) == b"ok"
    assert b"neighbour" in lib.mf_status_string(-3)
