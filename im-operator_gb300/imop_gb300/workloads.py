"""Seeded synthetic workloads of the RAW->RGB path.

C1  1006x758 RGGB, 10-bit in u16; BL 64; WB (1.9, 1.0, 1.6) on RGB after demosaic (the order the
    reference's per-module calls compose); HQLI; linear tone -> RGB8.
C2  4024x3032 RGGB MIPI RAW12; BL 256; 0.01 % hot/dead pixels, adaptive defect correction t=0.3;
    17x13x4 radial lens-shading grid (1.0 centre -> 2.0 corners); Bayer WB (2.1, 1.0, 1.5);
    AMAZE; CCM with rows summing to 1 (diagonal U(1.4, 1.8)); 4096-entry gamma-2.2 LUT -> RGB8.
C3  5320x4600, one 8-bit and one 12-bit u16 frame, the C1 pipeline.
Scenes come from imop_scene_render (seed = 20261203 + frame index).
"""
import numpy as np

from . import abi
from .params import Pipeline

BASE_SEED = 20261203


def radial_grid(width, height, gw=17, gh=13, corner_gain=2.0):
    """gw x gh x 4 gain grid: 1 + (corner_gain-1) * (r / r_corner)^2 at each node."""
    gx = np.arange(gw) * (width - 1) / (gw - 1)
    gy = np.arange(gh) * (height - 1) / (gh - 1)
    cx, cy = (width - 1) / 2.0, (height - 1) / 2.0
    rc = np.hypot(cx, cy)
    r = np.hypot(gx[None, :] - cx, gy[:, None] - cy)
    g = 1.0 + (corner_gain - 1.0) * (r / rc) ** 2
    return np.repeat(g[:, :, None], 4, axis=2).astype(np.float32)


def gamma_lut(bit_depth, gamma=2.2):
    mv = (1 << bit_depth) - 1
    return (np.arange(mv + 1, dtype=np.float64) / mv) ** (1.0 / gamma)


def random_ccm(seed, lo=1.4, hi=1.8):
    rng = np.random.default_rng(seed)
    m = np.zeros((3, 3))
    for i in range(3):
        d = rng.uniform(lo, hi)
        a = rng.uniform(0.0, 1.0)
        others = [j for j in range(3) if j != i]
        m[i, i] = d
        m[i, others[0]] = (1.0 - d) * a
        m[i, others[1]] = (1.0 - d) * (1.0 - a)
    return tuple(float(v) for v in m.astype(np.float32).reshape(-1))


def c1_pipeline(width=1006, height=758, bit_depth=10, demosaic=abi.HQLI):
    lo = (1 << bit_depth) // 16
    return Pipeline(width=width, height=height, bit_depth=bit_depth, packed=False, pattern=abi.RGGB,
                    demosaic=demosaic, stages=abi.STAGE_BLACK_LEVEL | abi.STAGE_WHITE_BALANCE,
                    stage_order=abi.ORDER_RGB_WB, bl_offset=(lo,) * 4, wb_gain=(1.9, 1.0, 1.6),
                    tone_mode=abi.TONE_LINEAR)


def c1_frame(pl, index=0):
    from . import scene
    mv = (1 << pl.bit_depth) - 1
    f = scene(pl.width, pl.height, pl.bit_depth, pl.pattern, BASE_SEED + index, lo=(mv + 1) // 16, hi=mv)
    return f.view(np.uint8).reshape(-1)


def c2_pipeline(width=4024, height=3032, seed=BASE_SEED, defect_frac=1e-4, defects=None):
    """defects: the defect-position generator (default the library's imop_scene_defects)"""
    if defects is None:
        from . import defects
    n_def = int(round(defect_frac * width * height))
    return Pipeline(width=width, height=height, bit_depth=12, packed=True, pattern=abi.RGGB,
                    demosaic=abi.AMAZE, stages=abi.STAGE_ALL, stage_order=abi.ORDER_BAYER_WB,
                    bl_offset=(256.0,) * 4, dpc_mode=abi.DPC_ADAPTIVE, dpc_threshold=0.3,
                    dpc_map=defects(width, height, n_def, seed) if n_def else None,
                    lsc_mode=abi.LSC_GRID, lsc_grid=radial_grid(width, height),
                    wb_gain=(2.1, 1.0, 1.5), ccm=random_ccm(seed), tone_mode=abi.TONE_LUT,
                    tone_lut=gamma_lut(12).astype(np.float32))


def c2_frame(pl, index=0, gen=None):
    """RAW12P bytes of one C2 frame: scene in [256, 4095], defects burnt in, MIPI packed.  gen: a
    module with scene / apply_defects / pack_mipi (default this package's, i.e. the library's)."""
    if gen is None:
        from . import scene, apply_defects, pack_mipi
    else:
        scene, apply_defects, pack_mipi = gen.scene, gen.apply_defects, gen.pack_mipi
    f = scene(pl.width, pl.height, 12, pl.pattern, BASE_SEED + index, lo=256, hi=4095)
    if pl.dpc_map is not None:
        apply_defects(f, pl.dpc_map, 12)
    return pack_mipi(f, 12) if pl.packed else f.view(np.uint8).reshape(-1)


def c3_pipelines():
    return [c1_pipeline(5320, 4600, 8), c1_pipeline(5320, 4600, 12)]


def c3_frame(pl, index=0):
    """A C3 frame (8-bit or 12-bit u16, seeded scene) for one of c3_pipelines()."""
    return c1_frame(pl, index)


# ---- C5: calibration of the differentiable chain ------------------------------------------------
# 16 x 1006x758 RGGB 12-bit frames (u16 unpacked), 933 parameters (BL 4, WB 3, CCM 9, 17x13x4
# lens-shading grid, 33 tone knots); the target is the FP64 forward at the true parameters, the
# start point the true parameters scaled by 1 + U(-0.2, 0.2).
C5_SCENE = (256, 1400)  # scene range: the true gains keep nearly every sample below 2^12 - 1


def c5_desc(n_frames=16, width=1006, height=758, demosaic=abi.AMAZE, grid=(17, 13)):
    return abi.AdjointDesc(width, height, 12, 0, abi.RGGB, demosaic, grid[0], grid[1], n_frames)


def c5_theta_true(desc):
    gw, gh = desc.grid_w, desc.grid_h
    knots = (np.arange(33) / 32.0) ** (1.0 / 2.2)
    th = np.concatenate([
        np.array([240.0, 256.0, 256.0, 272.0]),
        np.array([1.9, 1.0, 1.6]),
        np.array(random_ccm(BASE_SEED + 5)),
        radial_grid(desc.width, desc.height, gw, gh, 1.8).reshape(-1).astype(np.float64),
        knots,
    ])
    return th.astype(np.float32)


def c5_theta_init(theta_true, seed=BASE_SEED + 7, spread=0.2):
    rng = np.random.default_rng(seed)
    return (theta_true * (1.0 + rng.uniform(-spread, spread, theta_true.shape))).astype(np.float32)


def c5_frames(desc, first=0):
    """Raw bytes of desc.n_frames frames back to back (u16 LSB-aligned)."""
    from . import scene
    out = [scene(desc.width, desc.height, 12, desc.pattern, BASE_SEED + 500 + first + k, lo=C5_SCENE[0],
                 hi=C5_SCENE[1]).view(np.uint8).reshape(-1) for k in range(desc.n_frames)]
    return np.concatenate(out)


# ---- C4: uneven batch ------------------------------------------------------------------------------
C4_SIZES = [(1006, 758), (4024, 3032), (5320, 4600)]
C4_FORMATS = [(8, False), (10, True), (10, False), (12, True), (12, False)]


def c4_batch(n_frames=96, seed=BASE_SEED + 4):
    """(Pipeline, raw bytes) per frame: sizes and formats cycle through C4_SIZES x C4_FORMATS;
    black level 64 or 256, WB R ~ U(1.5, 2.4), B ~ U(1.2, 2.0), own CCM; BL, Bayer WB, AMAZE,
    CCM, linear tone -> RGB8.  Scenes are rendered once per (size, bit depth) and shared."""
    from . import scene, pack_mipi
    rng = np.random.default_rng(seed)
    cache = {}
    out = []
    for k in range(n_frames):
        w, h = C4_SIZES[k % len(C4_SIZES)]
        bd, packed = C4_FORMATS[(k // len(C4_SIZES)) % len(C4_FORMATS)]
        bl = float(rng.choice([64.0, 256.0])) * ((1 << bd) / 4096.0 if bd < 12 else 1.0)
        pl = Pipeline(width=w, height=h, bit_depth=bd, packed=packed, pattern=abi.RGGB, demosaic=abi.AMAZE,
                      stages=abi.STAGE_BLACK_LEVEL | abi.STAGE_WHITE_BALANCE | abi.STAGE_CCM,
                      stage_order=abi.ORDER_BAYER_WB, bl_offset=(round(bl),) * 4,
                      wb_gain=(float(rng.uniform(1.5, 2.4)), 1.0, float(rng.uniform(1.2, 2.0))),
                      ccm=random_ccm(int(rng.integers(0, 2**31))), tone_mode=abi.TONE_LINEAR)
        key = (w, h, bd, packed)
        if key not in cache:
            mv = (1 << bd) - 1
            f = scene(w, h, bd, abi.RGGB, BASE_SEED + 400 + k, lo=mv // 16, hi=mv)
            cache[key] = pack_mipi(f, bd) if packed else f.view(np.uint8).reshape(-1)
        out.append((pl, cache[key]))
    return out
