"""Format sniffing of raw blobs (host code of the library) against the reference's analyzer
(src/analyzer.cpp), live where oracle/_ref was built: detected bit depth, packing, value range,
candidate dimensions and Bayer phase on seeded scenes in every storage format, and on blobs of
unknown sizes."""
import ctypes as C

import numpy as np
import pytest

import imop_gb300 as I
from imop_gb300 import abi
import oracle_py as O

U8P = O.U8P
IP = C.POINTER(C.c_int)


def _scene(w, h, bd, pattern, seed, lo_frac=0.05, hi_frac=0.95):
    mv = (1 << bd) - 1
    return I.scene(w, h, bd, pattern, seed, lo=mv * lo_frac, hi=mv * hi_frac)


def _blobs():
    """(name, bytes) of seeded blobs: every storage of known and unknown sizes"""
    rng = np.random.default_rng(11)
    out = []
    for (w, h) in ((1006, 758), (640, 480)):
        out.append((f"u8_{w}", _scene(w, h, 8, abi.RGGB, 1).reshape(-1)))
        for bd in (10, 12, 14, 16):
            f = _scene(w, h, bd, abi.GRBG, bd)
            out.append((f"u16_{bd}_{w}", f.view(np.uint8).reshape(-1)))
            out.append((f"packed_{bd}_{w}", I.pack_mipi(f, bd)))
    for n in (0, 3, 7, 8, 12345, 40000):
        out.append((f"random_{n}", rng.integers(0, 256, n, dtype=np.uint8)))
    out.append(("u16_unknown", rng.integers(0, 4096, 30001, dtype=np.uint16).view(np.uint8)))
    out.append(("u16_small_values", rng.integers(0, 200, 30000, dtype=np.uint16).view(np.uint8)))
    out.append(("zeros_known", np.zeros(2 * 1006 * 758, np.uint8)))
    return out


BLOBS = _blobs()


def test_known_answers():
    """Cases that follow from the rules alone (no reference needed)."""
    f = _scene(1006, 758, 12, abi.RGGB, 5)
    a = I.analyze_data(f)
    assert a["detected_bit_depth"] == 12 and not a["is_packed"] and a["pixel_count"] == 1006 * 758
    assert a["min_value"] == int(f.min()) and a["max_value"] == int(f.max())
    p = I.analyze_data(I.pack_mipi(f, 12))
    assert p["detected_bit_depth"] == 12 and p["is_packed"] and p["pixel_count"] == 1006 * 758
    assert I.analyze_data(np.zeros(640 * 480, np.uint8))["detected_bit_depth"] == 8
    assert (1920, 1080) in I.suggest_dimensions(1920 * 1080)
    assert I.suggest_dimensions(0) == []
    assert I.detect_bit_depth(np.zeros(0, np.uint8)) == 0


ref = pytest.mark.skipif(not O.ref_available(), reason="reference library not built here")


@ref
@pytest.mark.parametrize("name,blob", BLOBS, ids=[b[0] for b in BLOBS])
def test_analyze_matches_reference(name, blob):
    R = O.ref()
    b = np.ascontiguousarray(blob, np.uint8)
    ptr = b.ctypes.data_as(U8P) if b.size else None
    assert I.detect_bit_depth(b) == R.ref_detect_bit_depth(ptr, b.size)
    info = (C.c_int * 9)()
    dims = (C.c_int * 32)()
    R.ref_analyze_data(ptr, b.size, info, dims, 16)
    got = I.analyze_data(b)
    want = {"detected_bit_depth": info[0], "suggested_width": info[1], "suggested_height": info[2],
            "pixel_count": info[3], "max_value": info[4], "min_value": info[5],
            "is_likely_16bit": bool(info[6]), "is_packed": bool(info[7])}
    for k, v in want.items():
        assert got[k] == v, (k, got[k], v)
    assert got["possible_dimensions"] == [(dims[2 * k], dims[2 * k + 1]) for k in range(min(info[8], 16))]


@ref
@pytest.mark.parametrize("n", [640 * 480, 1920 * 1080, 4096 * 2160, 1006 * 758, 4024 * 3032, 5320 * 4600,
                               65536, 1000003, 123 * 456, 64 * 64, 12345 * 7, 7680 * 4320])
def test_suggest_dimensions_matches_reference(n):
    R = O.ref()
    out = (C.c_int * 64)()
    k = R.ref_suggest_dimensions(n, out, 32)
    assert I.suggest_dimensions(n) == [(out[2 * j], out[2 * j + 1]) for j in range(min(k, 16))]


@ref
@pytest.mark.parametrize("pattern", [abi.RGGB, abi.BGGR, abi.GRBG, abi.GBRG])
@pytest.mark.parametrize("fmt", ["u8", "u16_12", "u16_msb", "packed_12", "packed_10", "packed_14"])
def test_guess_pattern_matches_reference(pattern, fmt):
    R = O.ref()
    w, h = 257, 131
    if fmt == "u8":
        bd, packed = 8, False
        f = _scene(w, h, 8, pattern, 3 + pattern)
        b = f.reshape(-1)
    else:
        bd = int(fmt.split("_")[1]) if fmt != "u16_msb" else 12
        packed = fmt.startswith("packed")
        f = _scene(w, h, bd, pattern, 7 + pattern)
        if fmt == "u16_msb":
            f = (f << 4).astype(np.uint16)  # MSB-aligned 12-bit samples (align_raw_value shifts them)
        b = I.pack_mipi(f, bd) if packed else f.view(np.uint8).reshape(-1)
    b = np.ascontiguousarray(b, np.uint8)
    assert I.guess_pattern(b, w, h, bd, packed) == R.ref_guess_pattern(b.ctypes.data_as(U8P), w, h, bd, int(packed))
