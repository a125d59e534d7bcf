"""The CPU oracle against golden vectors produced by the reference's own CPU functions
(tests/golden/make_golden.py): known answers from the reference's unit tests, seeded frames
through the reference's per-module call chain, and strips of the reference's real captures."""
import ctypes as C
import hashlib
import json
import os

import numpy as np
import pytest

import oracle_py as O
from imop_gb300 import abi
from imop_gb300.params import Pipeline

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
U16P, U8P, F32P = O.U16P, O.U8P, O.F32P


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def kats():
    with open(os.path.join(GOLD, "kat.json")) as f:
        return {c["name"]: c for c in json.load(f)}


def P(a, t=None):
    return a.ctypes.data_as(t or U16P)


def test_packed_decode_known_answers():
    k = kats()
    for name in ("raw10_packed_decode", "raw12_packed_decode"):
        c = k[name]
        buf = np.array(c["bytes"], np.uint8)
        got = [O.get_packed_raw(buf, x, 0, c["w"], c["h"], c["bd"]) for x in range(4)]
        assert got == c["expect"], name
    # the reference test's own literal expectation (tests/unit/test_pixel_utils.cpp:131-134)
    assert k["raw10_packed_decode"]["expect"] == [0x2FF, 0x100, 0x001, 0x3FF]


def test_black_level_known_answers():
    L = O.stages()
    k = kats()
    for name in ("black_level_per_channel", "black_level_global_clamp"):
        c = k[name]
        d = np.full((c["h"], c["w"]), c["fill"], np.uint16)
        off = np.array(c["offsets"], np.float32)
        L.or_black_level(P(d), c["w"], c["h"], abi.RGGB, c["bd"], c["mode"], P(off, F32P))
        assert d.tolist() == c["expect"], name
    assert k["black_level_per_channel"]["expect"][0][:2] == [90, 80]   # test_black_level.cpp:57-58


def test_defect_known_answers():
    L = O.stages()
    k = kats()
    c = k["defect_adaptive_hot"]
    d = np.array(c["input"], np.uint16)
    L.or_dpc_adaptive(P(d), c["w"], c["h"], abi.RGGB, c["bd"], c["threshold"])
    assert d.tolist() == c["expect"]
    assert d[4, 4] < 200
    c = k["defect_map"]
    d = np.array(c["input"], np.uint16)
    m = np.array(c["map"], np.int32)
    L.or_dpc_map(P(d), c["w"], c["h"], abi.RGGB, c["bd"], m.ctypes.data, len(m))
    assert d.tolist() == c["expect"]


def test_lens_shading_known_answers():
    L = O.stages()
    k = kats()
    c = k["lens_shading_poly_corners"]
    d = np.full((c["h"], c["w"]), c["fill"], np.uint16)
    coef = np.array(c["coef"], np.float32)
    L.or_lsc_poly(P(d), c["w"], c["h"], abi.RGGB, c["bd"], P(coef, F32P), *c["center"])
    assert sha(d) == c["expect_sha"] and d[0, 0] > 120
    c = k["lens_shading_flat_field_identity"]
    ff = np.full((c["h"], c["w"]), c["flat"], np.uint8)
    g = O.flat_field_grid(ff, abi.RGGB, c["bd"])
    d = np.full((c["h"], c["w"]), c["fill"], np.uint16)
    L.or_lsc_grid(P(d), c["w"], c["h"], abi.RGGB, c["bd"], P(g, F32P), 32, 24)
    assert d.tolist() == c["expect"]


def test_rgb_known_answers():
    L = O.stages()
    k = kats()
    c = k["ccm_swap"]
    rgb = np.array(c["input"], np.uint16)
    m = np.array(c["m"], np.float32)
    L.or_ccm(P(rgb), c["w"], c["h"], c["bd"], P(m, F32P))
    assert rgb.tolist() == c["expect"]
    c = k["wb_manual_clamp"]
    rgb = np.array(c["input"], np.uint16)
    g = np.array(c["gains"], np.float32)
    L.or_wb_rgb(P(rgb), c["w"], c["h"], c["bd"], P(g, F32P))
    assert rgb.tolist() == c["expect"]
    c = k["hqli_12bit"]
    out = O.demosaic(np.array(c["input"], np.uint16), abi.RGGB, abi.HQLI, 12)
    assert out.tolist() == c["expect"] and out.max() <= 4095


def test_reference_call_chains():
    """Seeded frames through the reference's per-module chain: every stage hash matches."""
    z = np.load(os.path.join(GOLD, "chains.npz"))
    n = len([k for k in z.files if k.endswith("_meta")])
    assert n >= 6
    for k in range(n):
        meta = json.loads(bytes(z[f"case{k}_meta"]).decode())
        f = z[f"case{k}_input"]
        w, h, bd = meta["w"], meta["h"], meta["bd"]
        pl = Pipeline(width=w, height=h, bit_depth=bd, pattern=meta["pattern"], demosaic=meta["demosaic"],
                      stages=abi.STAGE_ALL, stage_order=abi.ORDER_RGB_WB, bl_mode=abi.BL_PER_CHANNEL,
                      bl_offset=tuple(meta["offsets"]), dpc_mode=abi.DPC_ADAPTIVE, dpc_threshold=meta["threshold"],
                      wb_gain=tuple(meta["gains"]), ccm=tuple(meta["ccm"]), out_format=abi.OUT_NATIVE)
        if meta["lsc"] == "poly":
            c = meta["coef"]
            pl.lsc_mode = abi.LSC_POLYNOMIAL
            pl.lsc_poly = tuple(tuple(c[3 * i:3 * i + 3]) for i in range(4))
            pl.lsc_center = tuple(meta["center"])
        else:
            pl.lsc_mode = abi.LSC_FLAT_FIELD
            pl.lsc_flat_field = z[f"case{k}_flat"]
        raw = f.astype(np.uint8) if bd <= 8 else f.view(np.uint8)
        _, d = O.pipeline(pl, raw.reshape(-1), dumps=True)
        for stage, digest in meta["stages"].items():
            assert sha(d[stage]) == digest, f"case {k} stage {stage}"


def test_real_capture_strips():
    """The reference's real 1006x758 captures (first 24 rows), every format, three demosaics."""
    z = np.load(os.path.join(GOLD, "real_strips.npz"))
    meta = json.loads(bytes(z["meta"]).decode())
    for tag, m in meta.items():
        for name, algo in (("HQLI", abi.HQLI), ("MG", abi.MG), ("AMAZE", abi.AMAZE)):
            pl = Pipeline(width=m["w"], height=m["h"], bit_depth=m["bd"], packed=bool(m["packed"]),
                          pattern=abi.RGGB, demosaic=algo, stages=0, out_format=abi.OUT_NATIVE)
            out, _ = O.pipeline(pl, z[tag])
            assert sha(out.astype(np.uint16)) == m["demosaic_sha"][name], f"{tag} {name}"
