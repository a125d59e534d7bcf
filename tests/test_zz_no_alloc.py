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


def _call(pl, d_in, d_out):
    L = I.lib()
    f = L.imop_isp_run_device_noalloc
    f.restype = C.c_int
    f.argtypes = [C.POINTER(abi.IspParams), C.c_void_p, C.c_void_p, C.c_void_p]
    cp = pl.to_c()
    return f(C.byref(cp), d_in, d_out, None)


def test_noalloc_capacity_overflow_then_normal_call():
    """A frame whose defect chains need more than the array's 16384 seeds reports
    IMOP_ERR_CAPACITY; the next call, on a normal frame, starts from cleared counters and status
    and equals the context path."""
    torch = pytest.importorskip("torch")
    pl = workloads.c2_pipeline(640, 480)
    pl.dpc_threshold = 0.05
    noise = np.random.default_rng(9).integers(0, 4096, (480, 640)).astype(np.uint16)
    d_noise = torch.from_numpy(I.pack_mipi(noise, 12)).cuda()
    out = torch.zeros(pl.output_bytes(), dtype=torch.uint8, device="cuda")
    assert _call(pl, d_noise.data_ptr(), out.data_ptr()) == abi.ERR_CAPACITY
    pl2 = workloads.c2_pipeline(640, 480)
    d_in = torch.from_numpy(workloads.c2_frame(pl2, 6)).cuda()
    got = torch.zeros_like(out)
    assert _call(pl2, d_in.data_ptr(), got.data_ptr()) == 0, I.lib().imop_last_error_string().decode()
    ctx = I.Isp()
    ctx.set_params(pl2)
    ref = torch.zeros_like(out)
    ctx.run_device(d_in.data_ptr(), ref.data_ptr())
    torch.cuda.synchronize()
    ctx.close()
    assert torch.equal(got, ref)


def test_noalloc_knot_tone_and_polynomial_shading():
    torch = pytest.importorskip("torch")
    pl = workloads.c2_pipeline(322, 242)
    pl.lsc_mode = abi.LSC_POLYNOMIAL
    pl.lsc_poly = ((0.3, 0.05, 0.0), (0.25, 0.04, 0.01), (0.26, 0.03, 0.0), (0.35, -0.05, 0.1))
    pl.lsc_center = (0.47, 0.52)
    pl.tone_mode = abi.TONE_KNOTS
    pl.tone_knots = tuple(float(v) for v in (np.arange(33) / 32.0) ** 0.45)
    d_in = torch.from_numpy(workloads.c2_frame(pl, 8)).cuda()
    got = torch.zeros(pl.output_bytes(), dtype=torch.uint8, device="cuda")
    assert _call(pl, d_in.data_ptr(), got.data_ptr()) == 0, I.lib().imop_last_error_string().decode()
    ctx = I.Isp()
    ctx.set_params(pl)
    ref = torch.zeros_like(got)
    ctx.run_device(d_in.data_ptr(), ref.data_ptr())
    torch.cuda.synchronize()
    ctx.close()
    assert torch.equal(got, ref)
