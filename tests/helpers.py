"""Shared helpers of the parity tests: random pipelines and frames, comparisons."""
import numpy as np

import imop_gb300 as I
from imop_gb300 import abi


def max_abs(a, b):
    return int(np.max(np.abs(a.astype(np.int64) - b.astype(np.int64)))) if a.size else 0


def psnr(a, b, peak=255.0):
    d = a.astype(np.float64) - b.astype(np.float64)
    mse = float(np.mean(d * d))
    return float("inf") if mse == 0 else 10.0 * np.log10(peak * peak / mse)


def random_pipeline(rng, w, h, bd, packed, demosaic, pattern, stages=abi.STAGE_ALL, order=None,
                    dpc_mode=abi.DPC_ADAPTIVE, lsc_mode=abi.LSC_GRID, tone=None, out=abi.OUT_RGB8):
    mv = (1 << bd) - 1
    gw, gh = int(rng.integers(2, 9)), int(rng.integers(2, 7))
    pl = I.Pipeline(width=w, height=h, bit_depth=bd, packed=packed, pattern=pattern, demosaic=demosaic,
                    stages=stages,
                    stage_order=int(rng.integers(0, 2)) if order is None else order,
                    bl_mode=int(rng.integers(0, 2)),
                    bl_offset=tuple(float(v) for v in rng.uniform(0, mv * 0.08, 4)),
                    dpc_mode=dpc_mode, dpc_threshold=float(rng.uniform(0.05, 0.5)),
                    lsc_mode=lsc_mode,
                    lsc_grid=rng.uniform(0.8, 2.2, (gh, gw, 4)).astype(np.float32),
                    lsc_poly=tuple(tuple(float(v) for v in rng.uniform(-0.2, 0.9, 3)) for _ in range(4)),
                    lsc_center=(float(rng.uniform(0.3, 0.7)), float(rng.uniform(0.3, 0.7))),
                    wb_gain=tuple(float(v) for v in rng.uniform(0.6, 2.4, 3)),
                    ccm=tuple(float(v) for v in rng.uniform(-0.5, 1.6, 9)),
                    out_format=out)
    t = int(rng.integers(0, 3)) if tone is None else tone
    pl.tone_mode = t
    if t == abi.TONE_LUT:
        pl.tone_lut = np.sort(rng.uniform(-0.05, 1.05, mv + 1)).astype(np.float32)
    elif t == abi.TONE_KNOTS:
        pl.tone_knots = tuple(float(v) for v in np.sort(rng.uniform(0, 1, 33)))
    if dpc_mode == abi.DPC_MAP_BASED:
        n = int(rng.integers(1, 12))
        m = np.stack([rng.integers(0, w, n), rng.integers(0, h, n)], 1).astype(np.int32)
        if n > 3:
            m[1] = m[0]                       # repeated entry
            m[2] = m[0] + np.array([2, 0])    # same-colour neighbour
        pl.dpc_map = m
    return pl


def random_frame(rng, pl, defect_frac=0.01):
    """Unpacked scene with planted hot/dead pixels, in the pipeline's input format (bytes)."""
    bd = pl.bit_depth
    mv = (1 << bd) - 1
    f = I.scene(pl.width, pl.height, bd, pl.pattern, int(rng.integers(0, 2**62)), lo=mv * 0.05, hi=mv * 0.95)
    n = max(1, int(defect_frac * f.size))
    idx = rng.integers(0, f.size, n)
    f.reshape(-1)[idx] = rng.choice([0, mv], n)
    if rng.random() < 0.5 and pl.width > 8 and pl.height > 8:
        # a same-colour cluster: defects two pixels apart (sequential defect semantics)
        x, y = int(rng.integers(2, pl.width - 6)), int(rng.integers(2, pl.height - 6))
        f[y, x] = mv
        f[y, x + 2] = mv
        f[y + 2, x] = mv
        f[y + 2, x + 2] = 0
    if pl.packed:
        return I.pack_mipi(f, bd)
    return f.view(np.uint8).reshape(-1).copy()
