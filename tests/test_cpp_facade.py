"""The header-only C++ facade (include/mfree_gb300.hpp): a program written the way
the reference's scenario code is (body, add_action, set_boundary, step) compiles
against the headers, links the library, and on the GPU reproduces the reference's
golden results through the facade exactly as through the C ABI."""
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, gpu_available
from mfree_iwf_gb300 import scenarios as S

BUILD = os.path.join(ROOT, "mfree_iwf_gb300", "_build")
SRC = os.path.join(ROOT, "tests", "cpp", "facade_run.cpp")
FIELDS = ("x", "y", "vx", "vy", "rho", "Sxx", "Sxy", "Syy")


@pytest.fixture(scope="module")
def facade_bin(lib):
    os.makedirs(BUILD, exist_ok=True)
    out = os.path.join(BUILD, "facade_run")
    libdir = os.path.join(ROOT, "mfree_iwf_gb300")
    cmd = ["g++", "-std=c++14", "-O2", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"), SRC,
           "-o", out, "-L", libdir, "-lmfree_gb300", f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def test_facade_compiles_and_reports_errors(facade_bin, tmp_path):
    if gpu_available():
        pytest.skip("the no-device error path is for hosts without a GPU")
    case = os.path.join(GOLDEN, "rings_monaghan.case")
    r = subprocess.run([facade_bin, case, str(tmp_path / "o.out")], capture_output=True, text=True)
    assert r.returncode == 3, (r.returncode, r.stderr)  # mf::error carrying MF_ERR_NO_DEVICE
    assert "mf_create" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["rings_monaghan", "rings_monaghan_contact", "rings_tl_contact", "tensile_tl",
                                  "tensile_tl_weak", "rings_tl_fem_contact", "rotation_tl_weak", "rings_ul_weak_contact",
                                  "tensile_ul_fem"])
def test_facade_reproduces_the_reference(facade_bin, tmp_path, name):
    case = os.path.join(GOLDEN, f"{name}.case")
    out = str(tmp_path / "o.out")
    r = subprocess.run([facade_bin, case, out], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    got = S.read_result(out).dumps[-1]["bodies"]
    ref = S.read_result(os.path.join(GOLDEN, f"{name}.ref.out")).dumps[-1]["bodies"]
    tl = "tl" in name
    for g, w in zip(got, ref):
        for f in FIELDS:
            if tl:  # the TL path is bit-identical to the reference
                np.testing.assert_array_equal(g[f], w[f], err_msg=f)
            else:
                assert np.linalg.norm(g[f] - w[f]) <= 1e-9 * max(np.linalg.norm(w[f]), 1e-300), f
