"""The light-chain kernel (HQLI without defect correction, lens shading or CCM; isp_lite.cuh)
against the CPU oracle, bit for bit: every input format it takes, bit depths 1-12, both
white-balance orders, integral and fractional black levels (the latter through the general
kernel), every tone mode, all Bayer patterns, frames from 6x6 up to the 5320x4600 frames of the
large-frame workload, widths that are not
multiples of the tile, unaligned input and output pointers, samples above the bit depth's maximum
(the reference's MSB-aligned read), and batches that mix it with the general kernel.  The
direct-read variant (aligned frames whose rows start on a word) separately: its launches
counted, widths that are not multiples of 8 with every output phase, segments continued and bands
taken from the back under extreme tuning entries, and batches of frames of several widths in one
launch."""
import dataclasses

import numpy as np
import pytest

import imop_gb300 as I
from imop_gb300 import abi, workloads
import oracle_py as O

from helpers import max_abs

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

SIZES = [(6, 6), (7, 6), (6, 9), (9, 7), (8, 9), (33, 17), (131, 70), (255, 129), (256, 16), (257, 20), (259, 19),
         (260, 23), (520, 300), (771, 37), (1006, 758)]


def _pipeline(rng, w, h, allow_frac=True):
    fmt = int(rng.integers(0, 4))
    if fmt == 0:
        bd, packed = int(rng.integers(1, 9)), False
    elif fmt == 1:
        bd, packed = int(rng.integers(9, 13)), False
    elif fmt == 2:
        bd, packed = 10, True
    else:
        bd, packed = 12, True
    mv = (1 << bd) - 1
    stages = 0
    if rng.random() < 0.8:
        stages |= abi.STAGE_BLACK_LEVEL
    if rng.random() < 0.8:
        stages |= abi.STAGE_WHITE_BALANCE
    frac = allow_frac and rng.random() < 0.3
    off = [float(v) if frac else float(round(v)) for v in rng.uniform(0, mv * 0.08, 4)]
    pl = I.Pipeline(width=w, height=h, bit_depth=bd, packed=packed, pattern=int(rng.integers(0, 4)),
                    demosaic=abi.HQLI, stages=stages, stage_order=int(rng.integers(0, 2)),
                    bl_mode=int(rng.integers(0, 2)), bl_offset=tuple(off),
                    wb_gain=tuple(float(v) for v in rng.uniform(0.6, 2.4, 3)))
    t = int(rng.integers(0, 3))
    pl.tone_mode = t
    if t == abi.TONE_LUT:
        pl.tone_lut = np.sort(rng.uniform(-0.05, 1.05, mv + 1)).astype(np.float32)
    elif t == abi.TONE_KNOTS:
        pl.tone_knots = tuple(float(v) for v in np.sort(rng.uniform(0, 1, 33)))
    return pl


def _frame(rng, pl, over=False):
    bd = pl.bit_depth
    mv = (1 << bd) - 1
    f = I.scene(pl.width, pl.height, bd, pl.pattern, int(rng.integers(0, 2**62)), lo=mv * 0.05, hi=mv * 0.95)
    if over and not pl.packed:
        # samples above the bit depth's maximum: u8 frames of depth < 8 carry larger bytes, u16
        # frames MSB-aligned samples (the reference's get_raw shifts them when nothing clamped)
        k = rng.integers(0, f.size, max(1, f.size // 7))
        if bd <= 8:
            f.reshape(-1)[k] = rng.integers(mv, 256, k.size)
        else:
            f.reshape(-1)[k] = (f.reshape(-1)[k].astype(np.uint32) << (16 - bd)).astype(np.uint16)
    if pl.packed:
        return I.pack_mipi(f, bd)
    return f.view(np.uint8).reshape(-1).copy()


def _run(isp, pl, raw, in_off=0, out_off=0):
    buf = torch.zeros(raw.size + 16, dtype=torch.uint8, device="cuda")
    buf[in_off:in_off + raw.size].copy_(torch.from_numpy(raw))
    out = torch.full((pl.output_bytes() + 16,), 0x5A, dtype=torch.uint8, device="cuda")
    isp.set_params(pl)
    isp.run_device(buf.data_ptr() + in_off, out.data_ptr() + out_off)
    isp.sync_status()
    o = out.cpu().numpy()
    # bytes outside the frame untouched
    assert (o[:out_off] == 0x5A).all() and (o[out_off + pl.output_bytes():] == 0x5A).all()
    return o[out_off:out_off + pl.output_bytes()].reshape(pl.output_shape())


@pytest.fixture(scope="module")
def isp():
    """a context, with the built-in launch parameters while the module runs (the measured table
    may send a class to the tile kernel; the tests that change the table restore these)"""
    from imop_gb300 import tuning
    ctx = I.Isp()
    saved = tuning.get_table()
    tuning.set_table([])
    yield ctx
    tuning.set_table(saved)
    ctx.close()


@pytest.mark.parametrize("trial", range(30))
def test_lite_matches_oracle(isp, trial):
    rng = np.random.default_rng(9100 + trial)
    w, h = SIZES[trial % len(SIZES)]
    pl = _pipeline(rng, w, h)
    raw = _frame(rng, pl, over=(trial % 3 == 2 and pl.stages == 0))
    ref, _ = O.pipeline(pl, raw)
    in_off = int(rng.integers(0, 16)) if trial % 4 == 1 else 0
    out_off = int(rng.integers(0, 16)) if trial % 2 == 1 else 0
    got = _run(isp, pl, raw, in_off, out_off)
    assert max_abs(got, ref) == 0, (w, h, pl.bit_depth, pl.packed, pl.stages, pl.stage_order, in_off, out_off)


def test_lite_values_above_max_without_clamping_stages(isp):
    rng = np.random.default_rng(9200)
    for bd, packed in ((6, False), (8, False), (10, False), (12, False)):
        pl = I.Pipeline(width=131, height=70, bit_depth=bd, packed=packed, pattern=abi.GBRG, demosaic=abi.HQLI,
                        stages=0)
        raw = _frame(rng, pl, over=True)
        ref, _ = O.pipeline(pl, raw)
        assert max_abs(_run(isp, pl, raw), ref) == 0, bd
    # u16 samples above 32767 with black level on (the per-sample path of the lanes holding them)
    for bd in (10, 12):
        pl = I.Pipeline(width=300, height=41, bit_depth=bd, packed=False, pattern=abi.RGGB, demosaic=abi.HQLI,
                        stages=abi.STAGE_BLACK_LEVEL | abi.STAGE_WHITE_BALANCE, stage_order=abi.ORDER_RGB_WB,
                        bl_offset=(20.0, 21.0, 22.0, 23.0), wb_gain=(1.7, 1.0, 1.4))
        raw = _frame(rng, pl, over=True)
        ref, _ = O.pipeline(pl, raw)
        assert max_abs(_run(isp, pl, raw), ref) == 0, bd


@pytest.mark.parametrize("which", ["c1", "c3_8", "c3_12"])
def test_lite_full_frames(isp, which):
    if which == "c1":
        pl = workloads.c1_pipeline()
        raw = workloads.c1_frame(pl, 2)
    else:
        pl = workloads.c3_pipelines()[0 if which == "c3_8" else 1]
        raw = workloads.c3_frame(pl, 1)
    ref, _ = O.pipeline(pl, raw)
    assert max_abs(_run(isp, pl, raw), ref) == 0


def test_lite_in_mixed_batch(isp):
    """HQLI light-chain frames and general-kernel frames in one batch: both kernels, every frame
    against the oracle, recorded and replayed."""
    rng = np.random.default_rng(9300)
    frames = []
    for k in range(12):
        w, h = SIZES[(3 * k + 5) % len(SIZES)]
        pl = _pipeline(rng, w, h)
        if k % 3 == 2:
            pl.demosaic = abi.AMAZE  # general kernel
        if k % 4 == 3:
            pl.stages |= abi.STAGE_CCM
            pl.ccm = workloads.random_ccm(k)
        raw = _frame(rng, pl)
        ref, _ = O.pipeline(pl, raw)
        frames.append((pl, raw, ref))
    dev = [(pl, torch.from_numpy(raw).cuda(), torch.zeros(pl.output_bytes(), dtype=torch.uint8, device="cuda"))
           for pl, raw, _ in frames]
    for flags in (0, abi.BATCH_GRAPH, abi.BATCH_GRAPH):
        for _, _, d_out in dev:
            d_out.zero_()
        isp.batch_submit(dev, flags=flags)
        isp.sync_status()
        for k, ((pl, _, ref), (_, _, d_out)) in enumerate(zip(frames, dev)):
            got = d_out.cpu().numpy().reshape(ref.shape)
            assert max_abs(got, ref) == 0, (k, pl.width, pl.height, pl.demosaic, flags)


def test_lite_host_batch(isp):
    rng = np.random.default_rng(9400)
    frames = []
    for k in range(6):
        pl = workloads.c1_pipeline(1006 - 2 * k, 758 - k, bit_depth=10)
        raw = _frame(rng, pl)
        ref, _ = O.pipeline(pl, raw)
        frames.append((pl, raw, ref))
    outs = [np.zeros(ref.shape, ref.dtype) for _, _, ref in frames]
    isp.run_host_batch([(pl, raw, o) for (pl, raw, _), o in zip(frames, outs)])
    for (_, _, ref), o in zip(frames, outs):
        assert max_abs(o, ref) == 0


# widths that are multiples of 8: one strip and several, a last strip narrower than 256, up to the
# large-frame width
DIRECT_SIZES = [(8, 6), (16, 9), (64, 33), (248, 40), (256, 17), (264, 31), (512, 64), (520, 300), (1000, 77),
                (2048, 129), (5320, 57), (776, 6)]


def _direct_launches():
    return I.lib().imop_kernel_launches(abi.KERNEL_LITE_DIRECT)


def _word_rows(pl):
    """rows that start on a word: the direct-read variant's condition on the width"""
    return pl.width % 8 == 0 or (not pl.packed and pl.bit_depth > 8 and pl.width % 2 == 0) or \
        (not pl.packed and pl.bit_depth <= 8 and pl.width % 4 == 0)


def _bounded(pl):
    """the light-chain kernel's condition on the samples reaching HQLI: a clamping stage (black
    level, Bayer-order white balance), a format without spare bits, or full 8-bit bytes"""
    return bool(pl.stages & abi.STAGE_BLACK_LEVEL or (pl.stages & abi.STAGE_WHITE_BALANCE and pl.stage_order == 0)
                or pl.packed or pl.bit_depth >= 8)


@pytest.mark.parametrize("trial", range(24))
def test_direct_matches_oracle(isp, trial):
    rng = np.random.default_rng(9500 + trial)
    w, h = DIRECT_SIZES[trial % len(DIRECT_SIZES)]
    pl = _pipeline(rng, w, h, allow_frac=False)
    raw = _frame(rng, pl, over=(trial % 3 == 2 and pl.stages == 0))
    ref, _ = O.pipeline(pl, raw)
    out_off = int(rng.integers(0, 16)) if trial % 2 == 1 else 0
    n0 = _direct_launches()
    got = _run(isp, pl, raw, 0, out_off)
    assert (_direct_launches() > n0) == (_bounded(pl) and _word_rows(pl)), (w, h)
    assert max_abs(got, ref) == 0, (w, h, pl.bit_depth, pl.packed, pl.stages, pl.stage_order, out_off)


# widths that are not multiples of 8: rows that start on a word (u8: multiples of 4, u16: even)
WORD_SIZES = [(12, 7), (20, 9), (268, 31), (1004, 40), (6, 6), (10, 11), (262, 33), (1006, 758), (2054, 19)]


@pytest.mark.parametrize("trial", range(18))
def test_direct_word_rows_matches_oracle(isp, trial):
    """the direct-read variant on rows that start on a word: word copies of each lane's samples
    limited to the row, output rows stored by their 8-byte phase (odd phases, from odd output
    offsets, through the staging row)"""
    rng = np.random.default_rng(9900 + trial)
    w, h = WORD_SIZES[trial % len(WORD_SIZES)]
    u8 = w % 4 == 0 and trial % 2 == 0
    bd = int(rng.integers(1, 9)) if u8 else int(rng.integers(9, 13))
    pl = I.Pipeline(width=w, height=h, bit_depth=bd, packed=False, pattern=int(rng.integers(0, 4)), demosaic=abi.HQLI,
                    stages=abi.STAGE_BLACK_LEVEL | (abi.STAGE_WHITE_BALANCE if rng.random() < 0.8 else 0),
                    stage_order=int(rng.integers(0, 2)),
                    bl_offset=tuple(float(round(v)) for v in rng.uniform(0, ((1 << bd) - 1) * 0.08, 4)),
                    wb_gain=tuple(float(v) for v in rng.uniform(0.6, 2.4, 3)))
    raw = _frame(rng, pl)
    ref, _ = O.pipeline(pl, raw)
    out_off = int(rng.integers(0, 16))
    n0 = _direct_launches()
    got = _run(isp, pl, raw, 0, out_off)
    assert _direct_launches() > n0, (w, h, bd)
    assert max_abs(got, ref) == 0, (w, h, bd, pl.stages, pl.stage_order, out_off)


def test_direct_unaligned_input_takes_staged_kernel(isp):
    rng = np.random.default_rng(9600)
    pl = _pipeline(rng, 520, 40, allow_frac=False)
    raw = _frame(rng, pl)
    ref, _ = O.pipeline(pl, raw)
    n0 = _direct_launches()
    got = _run(isp, pl, raw, 3, 0)
    assert _direct_launches() == n0
    assert max_abs(got, ref) == 0


@pytest.mark.parametrize("band,seg", [(4, 10), (4, 1000), (1024, 100), (8, 50)])
def test_direct_segments_and_stolen_bands(isp, band, seg):
    """segments much shorter than a warp's share (most bands taken from the back by warps that
    own none), much longer (warps without a segment steal), one band per segment, and the default
    spread: every frame against the oracle"""
    from imop_gb300 import tuning
    old = tuning.get_table()
    try:
        tuning.set_table([{"kernel": abi.KERNEL_LITE, "fmt": -1, "max_width": 1 << 30, "enabled": 1,
                           "band_rows": band, "seg_percent": seg}])
        rng = np.random.default_rng(9700 + band + seg)
        for w, h in ((2048, 300), (264, 1001), (5320, 97)):
            pl = _pipeline(rng, w, h, allow_frac=False)
            pl.stages |= abi.STAGE_BLACK_LEVEL
            raw = _frame(rng, pl)
            ref, _ = O.pipeline(pl, raw)
            n0 = _direct_launches()
            got = _run(isp, pl, raw)
            assert _direct_launches() > n0
            assert max_abs(got, ref) == 0, (w, h, band, seg)
    finally:
        tuning.set_table(old)


def test_direct_batch_of_widths(isp):
    """frames of six widths in one recorded direct-read launch (one rectangle each), replayed"""
    rng = np.random.default_rng(9800)
    base = _pipeline(rng, 64, 64, allow_frac=False)
    base.stages |= abi.STAGE_BLACK_LEVEL
    frames = []
    for k, (w, h) in enumerate(((64, 40), (256, 77), (520, 33), (1000, 64), (2048, 19), (264, 150))):
        pl = dataclasses.replace(base, width=w, height=h)
        raw = _frame(rng, pl)
        ref, _ = O.pipeline(pl, raw)
        frames.append((pl, raw, ref))
    dev = [(pl, torch.from_numpy(raw).cuda(), torch.zeros(pl.output_bytes(), dtype=torch.uint8, device="cuda"))
           for pl, raw, _ in frames]
    n0 = _direct_launches()
    for flags in (0, abi.BATCH_GRAPH, abi.BATCH_GRAPH):
        for _, _, d_out in dev:
            d_out.zero_()
        isp.batch_submit(dev, flags=flags)
        isp.sync_status()
        for k, ((pl, _, ref), (_, _, d_out)) in enumerate(zip(frames, dev)):
            assert max_abs(d_out.cpu().numpy().reshape(ref.shape), ref) == 0, (k, pl.width, pl.height, flags)
    assert _direct_launches() > n0
