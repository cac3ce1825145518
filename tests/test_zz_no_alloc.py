"""The allocation-free UL step (mf_ul_step_noalloc), called through the C ABI.

It serves callers that cannot allocate device memory once they are running (memory
reserved up front in their own pools, or no implicit synchronisation from cudaMalloc
allowed): they hand in device arrays and the
library works in a fixed scratch array of its own.  Checked against the regular
context-based step (mf_step) on the same body, over two calls in a row, with the
tolerance of the other FP64-strict parity tests (relative L2 < 1e-9).  The device
arrays below are created by the test, not by the entry point.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ("x", "y", "vx", "vy", "rho", "Sxx", "Sxy", "Syy")
_DP = ctypes.POINTER(ctypes.c_double)


class MfDeviceBody(ctypes.Structure):
    _fields_ = [("n", ctypes.c_uint32), ("reserved", ctypes.c_uint32)] + \
               [(f, ctypes.c_void_p) for f in FIELDS] + [(f, ctypes.c_void_p) for f in ("m", "h", "quad_weight")]


def rel_l2(a, b):
    n = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (n if n > 0 else 1.0)


def test_noalloc_step_matches_context_step(lib):
    import torch
    import mfree_iwf_gb300 as M
    from mfree_iwf_gb300 import scenarios as S

    fn = lib.mf_ul_step_noalloc
    fn.restype = ctypes.c_int32
    fn.argtypes = [ctypes.POINTER(MfDeviceBody), ctypes.POINTER(M.MfSimData), ctypes.c_double,
                   ctypes.POINTER(ctypes.c_int32), ctypes.c_uint32, ctypes.c_int32, ctypes.c_void_p]

    sc = S.c1_rings(dx=2e-3, nbh_eps=1e-6)  # ~1.1k particles, the workload's constants
    a = sc.bodies[0].arrays
    n = sc.bodies[0].n
    sim = M.from_scenario(sc, precision="fp64_strict")
    dev = {k: torch.tensor(a[k], dtype=torch.float64, device="cuda") for k in FIELDS + ("m", "h", "quad_weight")}
    body = MfDeviceBody(n, 0, *[dev[f].data_ptr() for f in FIELDS], *[dev[f].data_ptr() for f in ("m", "h", "quad_weight")])
    sd = M.SimData(sc.nu, sc.E, sc.rho0, sc.wdeltap, sc.corr_exp, sc.mghn_eps, sc.alpha, sc.beta, sc.eta,
                   sc.xsph_eps, 0)._c()
    acts = (ctypes.c_int32 * len(sc.actions))(*sc.actions)
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        st = fn(ctypes.byref(body), ctypes.byref(sd), sc.dt, acts, len(sc.actions), 5, ctypes.c_void_p(stream))
        assert st == 0, M.STATUS.get(st, st)
        torch.cuda.synchronize()
        if call > 0:  # the first call loads the kernels; later calls leave free memory as it was
            assert torch.cuda.mem_get_info()[0] == free0, "the allocation-free step changed free device memory"
        sim.step(5)
        want = sim.get_state(0, FIELDS)
        for f in FIELDS:
            got = dev[f].cpu().numpy()
            assert rel_l2(got, want[f]) < 1e-9, (call, f)
    sim.close()


def test_noalloc_rejects_too_many_particles(lib):
    import mfree_iwf_gb300 as M
    fn = lib.mf_ul_step_noalloc
    fn.restype = ctypes.c_int32
    body = MfDeviceBody(16385, 0, *([1] * 11))  # never dereferenced: the size check comes first
    sd = M.SimData(0.4, 1e7, 1200.0)._c()
    assert fn(ctypes.byref(body), ctypes.byref(sd), ctypes.c_double(1e-6), None, 0, 1, None) == -12  # MF_ERR_CAPACITY
