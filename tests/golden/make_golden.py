"""Regenerate the golden fixtures of the oracle pin (run where the reference tree exists).

    make -C oracle ref && python tests/golden/make_golden.py [kat chains real_strips jpeg tone]

Every expected value here is produced by the reference's own CPU functions, compiled from its
sources by oracle/Makefile into oracle/_ref/libimop_ref.so (called through oracle/ref_glue.cpp):

  kat.json         known-answer cases taken from the reference's unit tests (file:line cited per
                   case), with the reference's exact outputs;
  chains.npz       small seeded frames through the reference's per-module calls in the order they
                   compose (unpack, black level, defect correction, lens shading, demosaic, RGB
                   white balance, CCM), SHA-256 of every stage output;
  real_strips.npz  the first 24 rows of each 1006x758 capture in the reference's test_data
                   (RG8, RG10, RG12, RG10 packed, RG12 packed) and the SHA-256 of
                   imop::demosaic_cpu's output on each (HQLI, MG, AMAZE), unpack included;
  tone.npz         tone::process_tone's output (GAMMA, S_CURVE, LEVELS, CURVES_3POINT) for every
                   storable sample value at several bit depths and parameter sets;
  jpeg.npz         RGB8 frames and the exact bytes of jpeg_codec::process_encode_baseline on them:
                   the images of the reference's tests/unit/test_jpeg_codec.cpp (file:line per
                   case), seeded frames over every subsampling and a range of qualities and sizes,
                   capacity truncation, and the status of each invalid argument.

The inputs are stored in the fixtures, so the tests need neither the reference tree nor the
product library to check the oracle.
"""
import ctypes as C
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, os.path.join(REPO, "im-operator_gb300"))

import oracle_py as O  # noqa: E402
from imop_gb300 import abi  # noqa: E402

REF_ROOT = os.environ.get("IMOP_REFERENCE_ROOT", "/root/reference")
U16P, U8P, F32P = O.U16P, O.U8P, O.F32P


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def P(a, t=None):
    return a.ctypes.data_as(t or U16P)


def kat_cases(R):
    cases = []
    # RAW10 packed decode, tests/unit/test_pixel_utils.cpp:111-135
    buf = np.array([0xBF, 0x40, 0x00, 0xFF, 0xD3], np.uint8)
    vals = [R.ref_get_packed_raw(P(buf, U8P), x, 0, 4, 1, 10) for x in range(4)]
    cases.append({"name": "raw10_packed_decode", "cite": "tests/unit/test_pixel_utils.cpp:111-135",
                  "w": 4, "h": 1, "bd": 10, "bytes": buf.tolist(), "expect": vals})
    # RAW12 packed decode: bytes of the reference's 12-bit packer (tools/synthetic_test.cpp:416-427)
    # for the pixel pair (0xABC, 0x123): b0 = 0xAB, b1 = 0x3C, b2 = 0x12
    buf12 = np.array([0xAB, 0x3C, 0x12, 0x00, 0xFF, 0x0F], np.uint8)
    vals12 = [R.ref_get_packed_raw(P(buf12, U8P), x, 0, 4, 1, 12) for x in range(4)]
    cases.append({"name": "raw12_packed_decode", "cite": "include/imop/pixel_utils.hpp:69-80",
                  "w": 4, "h": 1, "bd": 12, "bytes": buf12.tolist(), "expect": vals12})
    # black level per channel, tests/unit/test_black_level.cpp:46-61
    d = np.full((8, 8), 100, np.uint16)
    off = np.array([10, 20, 30, 40], np.float32)
    R.ref_black_level(P(d), 8, 8, abi.RGGB, 8, abi.BL_PER_CHANNEL, P(off, F32P))
    cases.append({"name": "black_level_per_channel", "cite": "tests/unit/test_black_level.cpp:46-61",
                  "w": 8, "h": 8, "bd": 8, "fill": 100, "offsets": off.tolist(), "mode": abi.BL_PER_CHANNEL,
                  "expect": d.tolist()})
    # black level global clamp, tests/unit/test_black_level.cpp:36-44
    d = np.full((8, 8), 40, np.uint16)
    off = np.array([100, 0, 0, 0], np.float32)
    R.ref_black_level(P(d), 8, 8, abi.RGGB, 8, abi.BL_GLOBAL, P(off, F32P))
    cases.append({"name": "black_level_global_clamp", "cite": "tests/unit/test_black_level.cpp:36-44",
                  "w": 8, "h": 8, "bd": 8, "fill": 40, "offsets": off.tolist(), "mode": abi.BL_GLOBAL,
                  "expect": d.tolist()})
    # adaptive defect correction of a hot pixel, tests/unit/test_defect_correct.cpp:23-36
    d = np.full((8, 8), 50, np.uint16)
    d[4, 4] = 255
    inp = d.copy()
    R.ref_dpc(P(d), 8, 8, abi.RGGB, 8, abi.DPC_ADAPTIVE, 0.3, None, 0)
    cases.append({"name": "defect_adaptive_hot", "cite": "tests/unit/test_defect_correct.cpp:23-36",
                  "w": 8, "h": 8, "bd": 8, "input": inp.tolist(), "threshold": 0.3, "expect": d.tolist()})
    # map-based defect correction, tests/unit/test_defect_correct.cpp:49-62
    d = np.full((8, 8), 100, np.uint16)
    d[3, 3] = 255
    inp = d.copy()
    m = np.array([[3, 3]], np.int32)
    R.ref_dpc(P(d), 8, 8, abi.RGGB, 8, abi.DPC_MAP_BASED, 0.3, m.ctypes.data_as(C.POINTER(C.c_int)), 1)
    cases.append({"name": "defect_map", "cite": "tests/unit/test_defect_correct.cpp:49-62",
                  "w": 8, "h": 8, "bd": 8, "input": inp.tolist(), "map": m.tolist(), "expect": d.tolist()})
    # polynomial lens shading brightens corners, tests/unit/test_lens_shading.cpp:33-50
    d = np.full((100, 100), 120, np.uint16)
    coef = np.array([0.8, 0, 0] * 4, np.float32)
    R.ref_lsc_poly(P(d), 100, 100, abi.RGGB, 8, P(coef, F32P), 0.5, 0.5)
    cases.append({"name": "lens_shading_poly_corners", "cite": "tests/unit/test_lens_shading.cpp:33-50",
                  "w": 100, "h": 100, "bd": 8, "fill": 120, "coef": coef.tolist(), "center": [0.5, 0.5],
                  "expect_sha": sha(d), "expect_corner": int(d[0, 0]), "expect_center": int(d[50, 50])})
    # flat-field identity, tests/unit/test_lens_shading.cpp:92-106
    ff = np.full((32, 32), 200, np.uint8)
    d = np.full((32, 32), 150, np.uint16)
    R.ref_lsc_flat_field(P(d), 32, 32, abi.RGGB, 8, P(ff, U8P), 32, 32)
    cases.append({"name": "lens_shading_flat_field_identity", "cite": "tests/unit/test_lens_shading.cpp:92-106",
                  "w": 32, "h": 32, "bd": 8, "fill": 150, "flat": 200, "expect": d.tolist()})
    # CCM channel swap, tests/unit/test_ccm.cpp:108-126 (R<->B)
    rgb = np.arange(4 * 4 * 3, dtype=np.uint16).reshape(4, 4, 3) * 5
    inp = rgb.copy()
    m = np.array([0, 0, 1, 0, 1, 0, 1, 0, 0], np.float32)
    R.ref_ccm(P(rgb), 4, 4, 8, P(m, F32P))
    cases.append({"name": "ccm_swap", "cite": "tests/unit/test_ccm.cpp:108-126", "w": 4, "h": 4, "bd": 8,
                  "input": inp.tolist(), "m": m.tolist(), "expect": rgb.tolist()})
    # manual WB clamps out of range, tests/unit/test_white_balance.cpp:372-393
    rgb = np.full((4, 4, 3), 200, np.uint16)
    inp = rgb.copy()
    g = np.array([2.0, 1.0, 3.0], np.float32)
    R.ref_wb_rgb(P(rgb), 4, 4, 8, P(g, F32P))
    cases.append({"name": "wb_manual_clamp", "cite": "tests/unit/test_white_balance.cpp:372-393", "w": 4, "h": 4,
                  "bd": 8, "input": inp.tolist(), "gains": g.tolist(), "expect": rgb.tolist()})
    # 12-bit HQLI stays in range, tests/unit/test_correctness.cpp:210-240
    rng = np.random.default_rng(1)
    bay = rng.integers(0, 4096, (16, 16)).astype(np.uint16)
    out = np.zeros((16, 16, 3), np.uint16)
    R.ref_demosaic(P(bay), P(out), 16, 16, abi.RGGB, abi.HQLI, 12)
    cases.append({"name": "hqli_12bit", "cite": "tests/unit/test_correctness.cpp:210-240", "w": 16, "h": 16,
                  "bd": 12, "input": bay.tolist(), "expect": out.tolist()})
    return cases


def chain_cases(R):
    """Seeded frames through the reference's per-module calls in call order."""
    rng = np.random.default_rng(20261203)
    out = {}
    specs = [(40, 30, 10, abi.RGGB, abi.HQLI), (41, 33, 12, abi.BGGR, abi.AMAZE), (38, 29, 8, abi.GRBG, abi.MG),
             (44, 26, 12, abi.GBRG, abi.MG), (36, 36, 8, abi.RGGB, abi.AMAZE), (50, 31, 10, abi.GRBG, abi.AMAZE)]
    for k, (w, h, bd, pat, dm) in enumerate(specs):
        mv = (1 << bd) - 1
        f = np.clip(rng.normal(mv * 0.45, mv * 0.12, (h, w)), 0, mv).astype(np.uint16)
        idx = rng.integers(0, w * h, 8)
        f.reshape(-1)[idx] = rng.choice([0, mv], 8)
        off = rng.uniform(0, mv * 0.06, 4).astype(np.float32)
        thr = float(rng.uniform(0.1, 0.4))
        coef = rng.uniform(-0.1, 0.7, 12).astype(np.float32)
        cx, cy = float(rng.uniform(0.4, 0.6)), float(rng.uniform(0.4, 0.6))
        gains = rng.uniform(0.7, 2.2, 3).astype(np.float32)
        m = rng.uniform(-0.4, 1.5, 9).astype(np.float32)
        use_poly = k % 2 == 0
        ff = np.clip(rng.normal(mv * 0.6, mv * 0.05, (h, w)), 1, mv).astype(np.uint16 if bd > 8 else np.uint8)
        stages = {}
        d = f.copy()
        stages["unpacked"] = sha(d)
        R.ref_black_level(P(d), w, h, pat, bd, abi.BL_PER_CHANNEL, P(off, F32P))
        stages["black_level"] = sha(d)
        R.ref_dpc(P(d), w, h, pat, bd, abi.DPC_ADAPTIVE, thr, None, 0)
        stages["defect"] = sha(d)
        if use_poly:
            R.ref_lsc_poly(P(d), w, h, pat, bd, P(coef, F32P), cx, cy)
        else:
            ffb = np.ascontiguousarray(ff).view(np.uint8)
            R.ref_lsc_flat_field(P(d), w, h, pat, bd, P(ffb, U8P), w, h)
        stages["lens_shading"] = sha(d)
        rgb = np.zeros((h, w, 3), np.uint16)
        R.ref_demosaic(P(d), P(rgb), w, h, pat, dm, bd)
        stages["demosaic"] = sha(rgb)
        R.ref_wb_rgb(P(rgb), w, h, bd, P(gains, F32P))
        stages["white_balance"] = sha(rgb)
        R.ref_ccm(P(rgb), w, h, bd, P(m, F32P))
        stages["ccm"] = sha(rgb)
        meta = dict(w=w, h=h, bd=bd, pattern=pat, demosaic=dm, offsets=off.tolist(), threshold=thr,
                    lsc="poly" if use_poly else "flat_field", coef=coef.tolist(), center=[cx, cy],
                    gains=gains.tolist(), ccm=m.tolist(), stages=stages)
        out[f"case{k}_input"] = f
        out[f"case{k}_flat"] = ff
        out[f"case{k}_meta"] = np.frombuffer(json.dumps(meta).encode(), np.uint8)
    return out


def real_strips(R):
    td = os.path.join(REF_ROOT, "test_data")
    files = {
        "RG8": ("Image_20260510144302933_w1006_h758_pBayerRG8.raw", 8, 0),
        "RG10": ("Image_20260510144219156_w1006_h758_pBayerRG10.raw", 10, 0),
        "RG12": ("Image_20260510144315897_w1006_h758_pBayerRG12.raw", 12, 0),
        "RG10P": ("Image_20260510144329680_w1006_h758_pBayerRG10_Packed.raw", 10, 1),
        "RG12P": ("Image_20260510144339211_w1006_h758_pBayerRG12_Packed.raw", 12, 1),
    }
    w, rows = 1006, 24
    out = {}
    meta = {}
    for tag, (fn, bd, packed) in files.items():
        raw = np.fromfile(os.path.join(td, fn), np.uint8)
        n = w * rows
        nbytes = (n * bd + 7) // 8 if packed else n * (1 if bd <= 8 else 2)
        strip = raw[:nbytes].copy()
        out[tag] = strip
        hashes = {}
        for name, algo in (("HQLI", abi.HQLI), ("MG", abi.MG), ("AMAZE", abi.AMAZE)):
            rgb = np.zeros((rows, w, 3), np.uint16)
            st = R.ref_demosaic_raw(P(strip, U8P), P(rgb), w, rows, abi.RGGB, algo, bd, packed)
            assert st == 0
            hashes[name] = sha(rgb)
        meta[tag] = {"file": fn, "bd": bd, "packed": packed, "w": w, "h": rows, "demosaic_sha": hashes}
    out["meta"] = np.frombuffer(json.dumps(meta).encode(), np.uint8)
    return out


def jpeg_image(kind, w, h, seed=0, colour=(0, 0, 0)):
    """the reference test's image makers (tests/unit/test_jpeg_codec.cpp:11-38) and seeded ones"""
    if kind == "flat":
        return np.broadcast_to(np.array(colour, np.uint8), (h, w, 3)).copy()
    if kind == "gradient":
        y, x = np.mgrid[0:h, 0:w]
        return np.stack([(x * 255) // (w - 1), (y * 255) // (h - 1), np.full_like(x, 128)], -1).astype(np.uint8)
    if kind == "pattern":
        return ((np.arange(w * h * 3, dtype=np.int64) * 37 + 127) % 256).astype(np.uint8).reshape(h, w, 3)
    rng = np.random.default_rng(seed)
    if kind == "noise":
        return rng.integers(0, 256, (h, w, 3), dtype=np.uint8)
    # smooth scene: sinusoids, edges and mild noise
    y, x = np.mgrid[0:h, 0:w].astype(np.float64)
    f = rng.uniform(0.02, 0.2, 3)
    base = np.stack([128 + 100 * np.sin(f[c] * x + (c + 1) * 0.7 * np.cos(f[2 - c] * y)) for c in range(3)], -1)
    base += np.where((x // 13 + y // 11) % 2 == 0, 30.0, -30.0)[..., None]
    base += rng.normal(0, 4, base.shape)
    return np.clip(base, 0, 255).astype(np.uint8)


def jpeg_cases(R):
    """(name, image, quality, subsample, cap, cite) per case"""
    T = "tests/unit/test_jpeg_codec.cpp"
    pat32 = jpeg_image("pattern", 32, 32)
    cases = [
        ("flat_roundtrip", jpeg_image("flat", 32, 32, colour=(80, 120, 200)), 90, 1, 0, f"{T}:283-316"),
        ("flat_compresses", jpeg_image("flat", 64, 64, colour=(128, 128, 128)), 90, 1, 0, f"{T}:191-209"),
        ("quality_q10", pat32, 10, 1, 0, f"{T}:211-260"),
        ("quality_q50", pat32, 50, 1, 0, f"{T}:211-260"),
        ("quality_q95", pat32, 95, 1, 0, f"{T}:211-260"),
        ("non_multiple_37x29", jpeg_image("pattern", 37, 29), 90, 1, 0, f"{T}:262-281"),
        ("gradient_48", jpeg_image("gradient", 48, 48), 95, 1, 0, f"{T}:318-350"),
        ("small_16", jpeg_image("pattern", 16, 16), 90, 1, 0, f"{T}:352-376"),
        ("odd_33x27", jpeg_image("pattern", 33, 27), 90, 1, 0, f"{T}:378-405"),
    ]
    k = 0
    for (w, h) in ((8, 8), (9, 8), (8, 15), (61, 47), (96, 64), (120, 40)):
        for ss in (0, 1, 2):
            for kind in (("scene", "noise") if w * h <= 61 * 47 else ("scene", "pattern")):
                q = (1, 25, 50, 75, 90, 100)[k % 6]
                cases.append((f"seed{k}_{kind}_{w}x{h}_q{q}_ss{ss}", jpeg_image(kind, w, h, seed=k), q, ss, 0, "seeded"))
                k += 1
    sc = jpeg_image("scene", 64, 48, seed=99)
    for cap in (1, 300, 700, 2000):
        cases.append((f"truncated_cap{cap}", sc, 80, 1, cap, "capacity"))
    cases.append(("subsample_clamp_hi", sc, 80, 7, 0, "clamped to 2"))
    cases.append(("subsample_clamp_lo", sc, 80, -4, 0, "clamped to 0"))
    out, meta, stored = {}, [], {}
    for i, (name, img, q, ss, cap, cite) in enumerate(cases):
        st, data = O.ref_jpeg_encode(img, q, ss, cap)
        assert st == 0, (name, st)
        key = id(img)
        if key not in stored:  # frames shared by several cases are stored once
            stored[key] = len(stored)
            out[f"img{stored[key]}"] = img
        out[f"jpg{i}"] = data
        meta.append({"name": name, "image": stored[key], "quality": q, "subsample": ss, "cap": cap, "cite": cite})
    # invalid arguments: (w, h, bit depth, quality, null input, null output) -> status
    errs = []
    z = np.zeros((8, 8, 3), np.uint8)
    for (w, h, bd, q, nin, nout) in ((8, 8, 8, 90, 1, 0), (8, 8, 8, 90, 0, 1), (0, 8, 8, 90, 0, 0), (8, -1, 8, 90, 0, 0),
                                     (8, 8, 16, 90, 0, 0), (8, 8, 7, 90, 0, 0), (4, 4, 8, 90, 0, 0), (7, 8, 8, 90, 0, 0),
                                     (8, 8, 8, 0, 0, 0), (8, 8, 8, 101, 0, 0), (4, 4, 16, 0, 1, 1), (8, 8, 8, 0, 0, 1)):
        buf = np.zeros(1 << 16, np.uint8)
        n = C.c_size_t(0)
        st = R.ref_jpeg_encode(None if nin else P(z, U8P), w, h, bd, q, 1, None if nout else P(buf, U8P), C.byref(n))
        errs.append({"w": w, "h": h, "bd": bd, "quality": q, "null_in": nin, "null_out": nout, "status": int(st)})
    out["meta"] = np.frombuffer(json.dumps({"cases": meta, "errors": errs}).encode(), np.uint8)
    return out


def tone_cases(R):
    """tone::process_tone on a ramp of every storable sample value (a n x 1 RGB frame with R = G = B)"""
    sets = [(2.2, 0.0, 0.0, 0.0, 0.0, 1.0, 0.5), (0.45, 0.8, -0.4, 0.6, 0.1, 0.9, 0.3),
            (10.5, -1.3, 1.1, -1.1, 0.5, 0.4, 0.95), (1.0, 2.4, 0.2, 0.2, -0.05, 1.05, 0.02)]
    out, bds, algos, params = {}, [], [], []
    k = 0
    for bd in (1, 8, 12, 16):
        for algo in range(4):
            for p in (sets[(bd + algo) % 4],):
                n = 256 if bd <= 8 else 65536
                ramp = np.repeat(np.arange(n, dtype=np.uint16), 3)
                res = np.zeros_like(ramp)
                pa = np.asarray(p, np.float32)
                st = R.ref_tone(P(ramp), P(res), n, 1, bd, algo, P(pa, F32P))
                assert st == 0
                out[f"table{k}"] = res.reshape(n, 3)[:, 0].copy()
                bds.append(bd)
                algos.append(algo)
                params.append(p)
                k += 1
    out.update(n=np.int32(k), bd=np.array(bds, np.int32), algo=np.array(algos, np.int32),
               params=np.array(params, np.float32))
    return out


def main():
    R = O.ref()
    only = set(sys.argv[1:])
    if not only or "kat" in only:
        with open(os.path.join(HERE, "kat.json"), "w") as f:
            json.dump(kat_cases(R), f)
    for name, fn in (("chains", chain_cases), ("real_strips", real_strips), ("jpeg", jpeg_cases), ("tone", tone_cases)):
        if not only or name in only:
            np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **fn(R))
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
