"""The oracle against the reference's own CPU functions, live (where oracle/_ref was built from
the reference's sources): random frames, all patterns, bit depths 8/10/12/16, every stage."""
import ctypes as C

import numpy as np
import pytest

import oracle_py as O
from imop_gb300 import abi

pytestmark = pytest.mark.skipif(not O.ref_available(), reason="reference library not built here")
U16P, U8P, F32P = O.U16P, O.U8P, O.F32P


def P(a, t=None):
    return a.ctypes.data_as(t or U16P)


def _frame(rng, w, h, bd):
    mv = (1 << bd) - 1
    f = np.clip(rng.normal(mv * 0.4, mv * 0.06, (h, w)), 0, mv).astype(np.uint16)
    k = rng.integers(0, w * h, max(1, w * h // 25))
    f.reshape(-1)[k] = rng.choice([0, mv], k.size)
    return f


@pytest.mark.parametrize("trial", range(24))
def test_stages_match_reference(trial):
    L, R = O.stages(), O.ref()
    rng = np.random.default_rng(1000 + trial)
    w, h = int(rng.integers(6, 70)), int(rng.integers(6, 60))
    bd = int(rng.choice([8, 10, 12, 16]))
    pat = int(rng.integers(0, 4))
    mv = (1 << bd) - 1
    base = _frame(rng, w, h, bd)
    off = rng.uniform(-3, mv * 0.1, 4).astype(np.float32)
    mode = int(rng.integers(0, 2))
    a, b = base.copy(), base.copy()
    L.or_black_level(P(a), w, h, pat, bd, mode, P(off, F32P))
    R.ref_black_level(P(b), w, h, pat, bd, mode, P(off, F32P))
    assert np.array_equal(a, b)
    thr = float(rng.uniform(0.0, 0.6))
    a2, b2 = a.copy(), a.copy()
    L.or_dpc_adaptive(P(a2), w, h, pat, bd, thr)
    R.ref_dpc(P(b2), w, h, pat, bd, abi.DPC_ADAPTIVE, thr, None, 0)
    assert np.array_equal(a2, b2)
    m = np.stack([rng.integers(0, w, 16), rng.integers(0, h, 16)], 1).astype(np.int32)
    m[5] = m[3]
    m[6] = m[3] + [2, 0]
    a3, b3 = a.copy(), a.copy()
    L.or_dpc_map(P(a3), w, h, pat, bd, m.ctypes.data, len(m))
    R.ref_dpc(P(b3), w, h, pat, bd, abi.DPC_MAP_BASED, 0.3, m.ctypes.data_as(C.POINTER(C.c_int)), len(m))
    assert np.array_equal(a3, b3)
    coef = rng.uniform(-0.2, 0.9, 12).astype(np.float32)
    cx, cy = float(rng.uniform(0.3, 0.7)), float(rng.uniform(0.3, 0.7))
    a4, b4 = a.copy(), a.copy()
    L.or_lsc_poly(P(a4), w, h, pat, bd, P(coef, F32P), cx, cy)
    R.ref_lsc_poly(P(b4), w, h, pat, bd, P(coef, F32P), cx, cy)
    assert np.array_equal(a4, b4)
    ff = np.clip(rng.normal(mv * 0.5, mv * 0.1, (h, w)), 1, mv).astype(np.uint16 if bd > 8 else np.uint8)
    g = O.flat_field_grid(ff, pat, bd)
    a5, b5 = a.copy(), a.copy()
    L.or_lsc_grid(P(a5), w, h, pat, bd, P(g, F32P), 32, 24)
    R.ref_lsc_flat_field(P(b5), w, h, pat, bd, P(np.ascontiguousarray(ff).view(np.uint8), U8P), w, h)
    assert np.array_equal(a5, b5)
    for algo in (abi.HQLI, abi.AMAZE, abi.MG):
        ra = O.demosaic(a, pat, algo, bd)
        rb = np.zeros((h, w, 3), np.uint16)
        R.ref_demosaic(P(a), P(rb), w, h, pat, algo, bd)
        assert np.array_equal(ra, rb), algo
    gains = rng.uniform(0.5, 2.5, 3).astype(np.float32)
    rgb = O.demosaic(a, pat, abi.AMAZE, bd)
    x, y = rgb.copy(), rgb.copy()
    L.or_wb_rgb(P(x), w, h, bd, P(gains, F32P))
    R.ref_wb_rgb(P(y), w, h, bd, P(gains, F32P))
    assert np.array_equal(x, y)
    M = rng.uniform(-0.6, 1.8, 9).astype(np.float32)
    x, y = rgb.copy(), rgb.copy()
    L.or_ccm(P(x), w, h, bd, P(M, F32P))
    R.ref_ccm(P(y), w, h, bd, P(M, F32P))
    assert np.array_equal(x, y)


@pytest.mark.parametrize("bd", [8, 9, 10, 11, 12, 14, 16])
def test_packed_unpack_matches_reference(bd):
    R = O.ref()
    rng = np.random.default_rng(bd)
    for _ in range(20):
        w, h = int(rng.integers(1, 40)), int(rng.integers(1, 9))
        size = (w * h * bd + 7) // 8
        buf = rng.integers(0, 256, size + 8, dtype=np.uint8)
        for y in range(h):
            for x in range(w):
                assert O.get_packed_raw(buf, x, y, w, h, bd) == R.ref_get_packed_raw(buf.ctypes.data_as(U8P), x, y, w, h, bd)


@pytest.mark.parametrize("bd", [8, 10, 12, 16])
@pytest.mark.parametrize("size", [2, 5, 17, 33])
def test_lut3d_matches_reference(bd, size):
    """a11: the oracle's 3D LUT stage against lut::apply_lut (trilinear), random cubes."""
    R = O.ref()
    L = O.stages()
    rng = np.random.default_rng(31 * size + bd)
    w, h = 37, 11
    mv = (1 << bd) - 1
    rgb = rng.integers(0, mv + 1, (h, w, 3)).astype(np.uint16)
    rgb[0, 0] = (0, 0, 0)
    rgb[0, 1] = (mv, mv, mv)
    lut = rng.uniform(-0.1, 1.1, (size, size, size, 3)).astype(np.float32)
    a, b = rgb.copy(), rgb.copy()
    L.or_lut3d(P(a), w, h, bd, P(lut, F32P), size)
    assert R.ref_apply_lut(P(b), w, h, bd, P(lut, F32P), size) == 0
    assert np.array_equal(a, b)
