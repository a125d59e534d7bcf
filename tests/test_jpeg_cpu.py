"""Baseline JPEG encode, CPU side: the oracle against the golden bytes of the reference's encoder
(tests/golden/jpeg.npz, made by tests/golden/make_golden.py from jpeg_codec::process_encode_baseline),
against the live reference where oracle/_ref was built, and the library's host-only pieces (the
header writer, the default capacity, the context without a device)."""
import ctypes as C
import json
import os

import numpy as np
import pytest

import oracle_py as O
from imop_gb300 import jpeg as J

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "jpeg.npz")


def golden():
    z = np.load(GOLD)
    meta = json.loads(bytes(z["meta"]))
    cases = []
    for i, c in enumerate(meta["cases"]):
        cases.append((c, z[f"img{c['image']}"], z[f"jpg{i}"]))
    return cases, meta["errors"]


CASES, ERRORS = golden()
IDS = [c[0]["name"] for c in CASES]


@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_oracle_matches_golden(case):
    c, img, want = case
    st, got = O.jpeg_encode(img, c["quality"], c["subsample"], c["cap"])
    assert st == 0
    assert got.size == want.size and np.array_equal(got, want)


def test_golden_properties():
    """The reference test's own expectations (tests/unit/test_jpeg_codec.cpp:164-281): SOI / EOI
    framing, flat frames smaller than raw, size non-decreasing with quality."""
    by = {c["name"]: (c, img, jpg) for c, img, jpg in CASES}
    for name, (c, img, jpg) in by.items():
        if c["cap"] == 0:
            assert jpg[0] == 0xFF and jpg[1] == 0xD8 and jpg[-2] == 0xFF and jpg[-1] == 0xD9, name
            assert jpg.size < O.jpeg_max_bytes(img.shape[1], img.shape[0])
    assert by["flat_compresses"][2].size < 64 * 64 * 3
    assert by["quality_q10"][2].size <= by["quality_q50"][2].size <= by["quality_q95"][2].size
    assert by["truncated_cap1"][2].size == 1 and by["truncated_cap700"][2].size == 700


def _oracle_status(e):
    z = np.zeros((8, 8, 3), np.uint8)
    L = O.lib()
    L.or_jpeg_encode.argtypes = [O.U8P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, O.U8P, C.POINTER(C.c_size_t)]
    buf = np.zeros(1 << 16, np.uint8)
    n = C.c_size_t(0)
    return L.or_jpeg_encode(None if e["null_in"] else z.ctypes.data_as(O.U8P), e["w"], e["h"], e["bd"], e["quality"], 1,
                            None if e["null_out"] else buf.ctypes.data_as(O.U8P), C.byref(n))


@pytest.mark.parametrize("e", ERRORS, ids=[f"{e['w']}x{e['h']}_bd{e['bd']}_q{e['quality']}_{e['null_in']}{e['null_out']}"
                                           for e in ERRORS])
def test_oracle_error_order_matches_golden(e):
    assert _oracle_status(e) == e["status"]


@pytest.mark.parametrize("case", [c for c in CASES if c[0]["cap"] == 0], ids=[c[0]["name"] for c in CASES if c[0]["cap"] == 0])
def test_header_matches_golden_prefix(case):
    c, img, want = case
    h, w = img.shape[:2]
    hdr = J.header(w, h, c["quality"], c["subsample"])
    assert hdr.size == 623 and np.array_equal(want[: hdr.size], hdr)


def test_max_bytes():
    assert J.max_bytes(640, 480) == 640 * 480 * 9 + 65536
    assert J.max_bytes(4024, 3032) == O.jpeg_max_bytes(4024, 3032)


def test_context_without_device_reports_cuda_not_available():
    import imop_gb300 as I
    if I.lib().imop_has_cuda() == 1:
        pytest.skip("a CUDA device is visible")
    with pytest.raises(J.JpegError) as ei:
        J.JpegEncoder()
    assert ei.value.code == J.CUDA_NOT_AVAILABLE


ref = pytest.mark.skipif(not O.ref_available(), reason="reference library not built here")


def _seeded(n, seed):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        w, h = int(rng.integers(8, 140)), int(rng.integers(8, 90))
        kind = k % 3
        if kind == 0:
            img = rng.integers(0, 256, (h, w, 3), dtype=np.uint8)
        elif kind == 1:
            y, x = np.mgrid[0:h, 0:w]
            img = np.stack([(x * 255) // max(w - 1, 1), (y * 255) // max(h - 1, 1), (x * y) % 256], -1).astype(np.uint8)
        else:
            img = np.clip(rng.normal(128, 60, (h, w, 3)).cumsum(1) / np.arange(1, w + 1)[None, :, None], 0, 255
                          ).astype(np.uint8)
        out.append((img, int(rng.integers(1, 101)), int(rng.integers(-1, 4))))
    return out


@ref
@pytest.mark.parametrize("k", range(60))
def test_oracle_matches_live_reference(k):
    img, q, ss = _seeded(60, 5)[k]
    a = O.ref_jpeg_encode(img, q, ss)
    b = O.jpeg_encode(img, q, ss)
    assert a[0] == b[0] == 0
    assert np.array_equal(a[1], b[1])
