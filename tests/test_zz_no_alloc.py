"""The no-allocation entry point (imop_isp_run_device_noalloc) against the context entry point.

It serves callers that cannot let the library call cudaMalloc: every table and scratch buffer it
needs lives in one device array inside the library.  Two calls in a row on different frames and
parameters check that the shared array is reset between calls; outputs must equal the regular
context path bit for bit (the tolerance of every parity test here).  This file is collected last
so that a failure here leaves the rest of the suite already run.
"""
import ctypes as C

import numpy as np
import pytest

import imop_gb300 as I
from imop_gb300 import abi, workloads

pytestmark = pytest.mark.gpu


def _noalloc(pl, d_in, d_out):
    L = I.lib()
    f = L.imop_isp_run_device_noalloc
    f.restype = C.c_int
    f.argtypes = [C.POINTER(abi.IspParams), C.c_void_p, C.c_void_p, C.c_void_p]
    cp = pl.to_c()
    rc = f(C.byref(cp), d_in, d_out, None)
    assert rc == 0, L.imop_last_error_string().decode()


def test_noalloc_matches_context_path_twice():
    torch = pytest.importorskip("torch")
    cases = []
    pl1 = workloads.c2_pipeline(640, 480)                       # RAW12P, defects + chains, AMAZE, LUT
    cases.append((pl1, workloads.c2_frame(pl1, 3)))
    pl2 = workloads.c1_pipeline(642, 418, bit_depth=10)          # u16, HQLI, RGB-order WB, linear tone
    pl2.stages |= abi.STAGE_DEFECT | abi.STAGE_CCM
    pl2.ccm = workloads.random_ccm(5)
    cases.append((pl2, workloads.c1_frame(pl2, 4)))
    ctx = I.Isp()
    for pl, raw in cases:
        d_in = torch.from_numpy(raw).cuda()
        ref = torch.empty(pl.output_bytes(), dtype=torch.uint8, device="cuda")
        got = torch.full_like(ref, 0x5A)
        ctx.set_params(pl)
        ctx.run_device(d_in.data_ptr(), ref.data_ptr())
        torch.cuda.synchronize()
        _noalloc(pl, d_in.data_ptr(), got.data_ptr())
        assert torch.equal(got, ref)
    ctx.close()


def test_noalloc_rejects_beyond_limits():
    pytest.importorskip("torch")
    pl = workloads.c1_pipeline(64, 48, bit_depth=16)
    L = I.lib()
    f = L.imop_isp_run_device_noalloc
    f.restype = C.c_int
    f.argtypes = [C.POINTER(abi.IspParams), C.c_void_p, C.c_void_p, C.c_void_p]
    cp = pl.to_c()
    assert f(C.byref(cp), 1, 1, None) == abi.ERR_UNSUPPORTED
    assert b"bit depth" in L.imop_last_error_string()
