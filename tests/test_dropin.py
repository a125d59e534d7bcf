"""The reference's own module dispatchers over this library: the reference's CPU sources, compiled
without its GPU glue (src/gpu_dispatch.cpp, src/algorithms/cuda_dispatch.cpp,
src/jpeg_codec/cuda_dispatch.cpp) and linked against libimop_isp.so (oracle/Makefile, target
dropin), called through black_level::process_black_level, defect_correct::process_defect_correct,
imop::demosaic, white_balance::process_white_balance, ccm::process_ccm and tone::process_tone.

Without a GPU every dispatcher must fall back to its CPU code and still equal the oracle; on a GB300
the same calls must be served by this library (imop_shim_calls_served counts them) and return the
same bytes.  The build needs the reference's sources: the reference tree named by
IMOP_REFERENCE_ROOT, or the copy `make -C oracle stage` leaves in oracle/_ref/src."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

import imop_gb300 as I
import oracle_py as O
from imop_gb300 import abi

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE = os.path.join(REPO, "oracle")
DROPIN = os.path.join(ORACLE, "_ref", "libimop_ref_dropin.so")


def _ref_root():
    for cand in (os.environ.get("IMOP_REFERENCE_ROOT"), os.path.join(ORACLE, "_ref", "src")):
        if cand and os.path.isdir(os.path.join(cand, "src", "algorithms")):
            return cand
    return None


@pytest.fixture(scope="module")
def dropin():
    root = _ref_root()
    if root is None and not os.path.exists(DROPIN):
        pytest.skip("no reference sources on this host")
    if root is not None:
        r = subprocess.run(["make", "-C", ORACLE, "dropin", "-j8", f"REF_ROOT={root}"], capture_output=True, text=True)
        assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    I.lib()  # the library the drop-in build links, loaded first
    L = C.CDLL(DROPIN)
    i, vp, fp = C.c_int, C.c_void_p, C.POINTER(C.c_float)
    L.dropin_served.restype = C.c_longlong
    L.dropin_black_level.argtypes = [vp, i, i, i, i, i, fp]
    L.dropin_defect_adaptive.argtypes = [vp, i, i, i, i, C.c_float]
    L.dropin_demosaic.argtypes = [vp, vp, i, i, i, i, i, i]
    L.dropin_white_balance.argtypes = [vp, vp, i, i, i, fp]
    L.dropin_ccm.argtypes = [vp, vp, i, i, i, fp]
    L.dropin_tone.argtypes = [vp, vp, i, i, i, i, fp]
    return L


def _f32(v):
    a = np.asarray(v, np.float32)
    return a, a.ctypes.data_as(C.POINTER(C.c_float))


def _store(a16, bd):
    """the reference's storage of u16 samples: u8 for bit depth <= 8, u16 otherwise"""
    return np.ascontiguousarray(a16.astype(np.uint8) if bd <= 8 else a16.astype(np.uint16))


def _scene(rng, w, h, bd, channels=1):
    mv = (1 << bd) - 1
    yy, xx = np.mgrid[0:h, 0:w]
    base = 0.45 + 0.3 * np.sin(0.07 * xx + rng.uniform(0, 6)) * np.cos(0.05 * yy)
    if channels > 1:
        base = np.stack([base * (0.8 + 0.2 * c) for c in range(channels)], -1)
    f = np.clip(base + rng.normal(0, 0.02, base.shape), 0, 1) * mv
    f = f.astype(np.uint16)
    k = rng.integers(0, f.size, max(1, f.size // 900))
    f.reshape(-1)[k] = rng.choice([0, mv], k.size)
    return f


def _check_all(L, expect_gpu):
    S = O.stages()
    U16P = O.U16P
    rng = np.random.default_rng(7100)
    served0 = L.dropin_served()
    calls = 0
    for (w, h, bd, pat) in ((64, 48, 8, abi.RGGB), (131, 70, 10, abi.GRBG), (1006, 758, 12, abi.BGGR)):
        mv = (1 << bd) - 1
        # black level (per channel and global), in place
        for mode in (abi.BL_PER_CHANNEL, abi.BL_GLOBAL):
            bay = _scene(rng, w, h, bd)
            off, offp = _f32([0.03 * mv, 0.05 * mv, 0.04 * mv, 17.5])
            got = _store(bay, bd)
            assert L.dropin_black_level(got.ctypes.data, w, h, pat, bd, mode, offp) == 0
            want = bay.copy()
            S.or_black_level(want.ctypes.data_as(U16P), w, h, pat, bd, mode, offp)
            assert np.array_equal(got.astype(np.uint16), want), ("black level", w, h, bd, mode)
            calls += 1
        # adaptive defect correction, in place
        bay = _scene(rng, w, h, bd)
        got = _store(bay, bd)
        assert L.dropin_defect_adaptive(got.ctypes.data, w, h, pat, bd, 0.2) == 0
        want = bay.copy()
        S.or_dpc_adaptive(want.ctypes.data_as(U16P), w, h, pat, bd, 0.2)
        assert np.array_equal(got.astype(np.uint16), want), ("defect correction", w, h, bd)
        calls += 1
        # demosaic: HQLI, MG, AMAZE on unpacked input; AMAZE on MIPI-packed input at 10 / 12 bits
        bay = _scene(rng, w, h, bd)
        for algo in (abi.HQLI, abi.MG, abi.AMAZE):
            rgb = np.zeros((h, w, 3), np.uint8 if bd <= 8 else np.uint16)
            raw = _store(bay, bd)
            assert L.dropin_demosaic(raw.ctypes.data, rgb.ctypes.data, w, h, pat, algo, bd, 0) == 0
            assert np.array_equal(rgb.astype(np.uint16), O.demosaic(bay, pat, algo, bd)), ("demosaic", algo, w, h, bd)
            calls += 1
        if bd in (10, 12):
            packed = I.pack_mipi(bay, bd)
            rgb = np.zeros((h, w, 3), np.uint16)
            assert L.dropin_demosaic(packed.ctypes.data, rgb.ctypes.data, w, h, pat, abi.AMAZE, bd, 1) == 0
            assert np.array_equal(rgb, O.demosaic(bay, pat, abi.AMAZE, bd)), ("packed demosaic", w, h, bd)
            calls += 1
        # RGB white balance and CCM
        rgb16 = _scene(rng, w, h, bd, 3)
        g, gp = _f32([1.9, 1.0, 1.6])
        inp, out = _store(rgb16, bd), np.zeros_like(_store(rgb16, bd))
        assert L.dropin_white_balance(inp.ctypes.data, out.ctypes.data, w, h, bd, gp) == 0
        want = rgb16.copy()
        S.or_wb_rgb(want.ctypes.data_as(U16P), w, h, bd, gp)
        assert np.array_equal(out.astype(np.uint16), want), ("white balance", w, h, bd)
        m, mp = _f32([1.6, -0.4, -0.2, -0.25, 1.5, -0.25, -0.1, -0.5, 1.6])
        assert L.dropin_ccm(inp.ctypes.data, out.ctypes.data, w, h, bd, mp) == 0
        want = rgb16.copy()
        S.or_ccm(want.ctypes.data_as(U16P), w, h, bd, mp)
        assert np.array_equal(out.astype(np.uint16), want), ("ccm", w, h, bd)
        calls += 2
        # tone curves: every sample through the reference's per-sample function (pinned separately
        # against the reference in test_tone_cpu.py)
        for algo in (abi.TONE_CURVE_GAMMA, abi.TONE_CURVE_S_CURVE, abi.TONE_CURVE_LEVELS, abi.TONE_CURVE_3POINT):
            p = [2.2, 0.3, 0.2, -0.1, 0.05, 0.95, 0.45]
            _, pp = _f32(p)
            assert L.dropin_tone(inp.ctypes.data, out.ctypes.data, w, h, bd, algo, pp) == 0
            table = I.tone_table(algo, bd, I.tone_params(*p))
            assert np.array_equal(out.astype(np.uint16), table[inp.astype(np.int64)]), ("tone", algo, w, h, bd)
            calls += 1
    served = L.dropin_served() - served0
    if expect_gpu:
        assert served == calls, (served, calls)
    else:
        assert served == 0


def test_reference_dispatchers_fall_back_without_gpu(dropin):
    if I.lib().imop_has_cuda() == 1:
        pytest.skip("a GPU is visible; the device path is checked by the gpu test")
    _check_all(dropin, expect_gpu=False)


@pytest.mark.gpu
def test_reference_dispatchers_served_on_gpu(dropin):
    assert I.lib().imop_has_cuda() == 1
    _check_all(dropin, expect_gpu=True)
