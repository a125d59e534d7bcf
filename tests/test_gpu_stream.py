"""The warp-streamed kernel (the interior of AMAZE frames, isp_stream.cu) with the tile kernel on
the border rows and columns, against the CPU oracle, bit for bit: every input format it takes, bit
depths 5-12, every stage on and off (integral black level, adaptive defect correction with planted
defects and same-colour clusters that need the raster-order fix-up, grid lens shading, Bayer-order
white balance, CCM), every tone mode, all Bayer patterns, widths from one strip to many, bands of
one to several, unaligned output pointers, u16 samples above 32767, batches of several streamed
frames mixed with other kernels (recorded and replayed), and a full 4024x3032 RAW12 frame of the
headline workload.  Each case also checks that the streaming kernel was launched."""
import numpy as np
import pytest

import imop_gb300 as I
from imop_gb300 import abi, workloads
import oracle_py as O

from helpers import max_abs

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

SIZES = [(64, 32), (72, 40), (256, 64), (264, 45), (496, 130), (504, 97), (520, 300), (1000, 133), (1288, 260),
         (2048, 96), (248, 250), (752, 41)]
STREAM = 2  # IMOP_KERNEL_STREAM


def _launches():
    return I.lib().imop_kernel_launches(STREAM)


def _pipeline(rng, w, h, fmt=None, stages=None):
    fmt = int(rng.integers(0, 4)) if fmt is None else fmt
    if fmt == 0:
        bd, packed = int(rng.integers(5, 9)), False
    elif fmt == 1:
        bd, packed = int(rng.integers(9, 13)), False
    elif fmt == 2:
        bd, packed = 10, True
    else:
        bd, packed = 12, True
    mv = (1 << bd) - 1
    if stages is None:
        stages = abi.STAGE_BLACK_LEVEL
        for s in (abi.STAGE_DEFECT, abi.STAGE_LENS_SHADING, abi.STAGE_WHITE_BALANCE, abi.STAGE_CCM):
            if rng.random() < 0.7:
                stages |= s
        if bd == 8 and rng.random() < 0.3:
            stages &= ~abi.STAGE_BLACK_LEVEL
    gw, gh = int(rng.integers(2, 18)), int(rng.integers(2, 14))
    pl = I.Pipeline(width=w, height=h, bit_depth=bd, packed=packed, pattern=int(rng.integers(0, 4)),
                    demosaic=abi.AMAZE, stages=stages, stage_order=abi.ORDER_BAYER_WB,
                    bl_mode=int(rng.integers(0, 2)),
                    bl_offset=tuple(float(round(v)) for v in rng.uniform(0, mv * 0.08, 4)),
                    dpc_mode=abi.DPC_ADAPTIVE, dpc_threshold=float(rng.uniform(0.05, 0.5)),
                    lsc_mode=abi.LSC_GRID, lsc_grid=rng.uniform(0.6, 2.4, (gh, gw, 4)).astype(np.float32),
                    wb_gain=tuple(float(v) for v in rng.uniform(0.6, 2.4, 3)),
                    ccm=tuple(float(v) for v in rng.uniform(-0.5, 1.6, 9)))
    t = int(rng.integers(0, 3))
    pl.tone_mode = t
    if t == abi.TONE_LUT:
        pl.tone_lut = np.sort(rng.uniform(-0.05, 1.05, mv + 1)).astype(np.float32)
    elif t == abi.TONE_KNOTS:
        pl.tone_knots = tuple(float(v) for v in np.sort(rng.uniform(0, 1, 33)))
    return pl


def _frame(rng, pl, defect_frac=0.004, clusters=3, over=False):
    bd = pl.bit_depth
    mv = (1 << bd) - 1
    f = I.scene(pl.width, pl.height, bd, pl.pattern, int(rng.integers(0, 2**62)), lo=mv * 0.05, hi=mv * 0.95)
    n = max(1, int(defect_frac * f.size))
    idx = rng.integers(0, f.size, n)
    f.reshape(-1)[idx] = rng.choice([0, mv], n)
    for _ in range(clusters):
        # defects two pixels apart: the raster-order (sequential) semantics differ from Jacobi
        x, y = int(rng.integers(8, pl.width - 12)), int(rng.integers(7, pl.height - 10))
        f[y, x] = mv
        f[y, x + 2] = mv
        f[y + 2, x] = mv
        f[y + 2, x + 2] = 0
    if over and not pl.packed and bd > 8:
        # MSB-aligned u16 samples above 32767 (the per-sample black-level path)
        k = rng.integers(0, f.size, max(1, f.size // 50))
        f.reshape(-1)[k] = 0x8000 | (f.reshape(-1)[k].astype(np.uint32) << (16 - bd)).astype(np.uint16)
    if pl.packed:
        return I.pack_mipi(f, bd)
    return f.view(np.uint8).reshape(-1).copy()


def _run(isp, pl, raw, out_off=0):
    d_in = torch.from_numpy(raw).cuda()
    out = torch.full((pl.output_bytes() + 16,), 0x5A, dtype=torch.uint8, device="cuda")
    isp.set_params(pl)
    isp.run_device(d_in.data_ptr(), out.data_ptr() + out_off)
    isp.sync_status()
    o = out.cpu().numpy()
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


@pytest.mark.parametrize("trial", range(36))
def test_stream_matches_oracle(isp, trial):
    rng = np.random.default_rng(12100 + trial)
    w, h = SIZES[trial % len(SIZES)]
    pl = _pipeline(rng, w, h, fmt=trial % 4)
    raw = _frame(rng, pl, over=(trial % 4 == 1 and trial % 3 == 0))
    ref, _ = O.pipeline(pl, raw)
    out_off = [0, 4, 3, 8][trial % 4]
    n0 = _launches()
    got = _run(isp, pl, raw, out_off)
    assert _launches() > n0, "the streaming kernel did not run"
    assert max_abs(got, ref) == 0, (w, h, pl.bit_depth, pl.packed, pl.stages, pl.pattern, out_off)


@pytest.mark.parametrize("stages", [0, abi.STAGE_BLACK_LEVEL, abi.STAGE_DEFECT | abi.STAGE_BLACK_LEVEL,
                                    abi.STAGE_LENS_SHADING | abi.STAGE_WHITE_BALANCE,
                                    abi.STAGE_ALL & ~abi.STAGE_LUT3D])
def test_stream_stage_sets(isp, stages):
    rng = np.random.default_rng(12300 + stages)
    pl = _pipeline(rng, 520, 300, fmt=3, stages=stages)
    raw = _frame(rng, pl)
    ref, _ = O.pipeline(pl, raw)
    n0 = _launches()
    got = _run(isp, pl, raw)
    assert _launches() > n0
    assert max_abs(got, ref) == 0, stages


def test_stream_dense_defects(isp):
    """1 % defects and many same-colour clusters: the median path on many lanes at once and
    defect-chain seeds in most bands."""
    rng = np.random.default_rng(12400)
    for fmt in (1, 3):
        pl = _pipeline(rng, 1000, 133, fmt=fmt, stages=abi.STAGE_ALL & ~abi.STAGE_LUT3D)
        raw = _frame(rng, pl, defect_frac=0.01, clusters=40)
        ref, _ = O.pipeline(pl, raw)
        assert max_abs(_run(isp, pl, raw), ref) == 0, fmt


def test_stream_ineligible_frames_take_the_tile_kernel(isp):
    """A width not a multiple of 8, a fractional black level, RGB-order white balance: the tile kernel
    alone, same bytes as the oracle."""
    rng = np.random.default_rng(12500)
    cases = []
    pl = _pipeline(rng, 522, 96, fmt=3)
    cases.append(pl)
    pl = _pipeline(rng, 520, 96, fmt=1, stages=abi.STAGE_ALL & ~abi.STAGE_LUT3D)
    pl.bl_offset = (20.5, 21.0, 22.0, 23.0)
    cases.append(pl)
    pl = _pipeline(rng, 520, 96, fmt=3, stages=abi.STAGE_ALL & ~abi.STAGE_LUT3D)
    pl.stage_order = abi.ORDER_RGB_WB
    cases.append(pl)
    for pl in cases:
        raw = _frame(rng, pl)
        ref, _ = O.pipeline(pl, raw)
        n0 = _launches()
        got = _run(isp, pl, raw)
        assert _launches() == n0
        assert max_abs(got, ref) == 0


def test_stream_batch_mixed(isp):
    """Streamed frames of two formats among HQLI and MG frames in one batch submission, recorded
    into a graph and replayed."""
    rng = np.random.default_rng(12600)
    frames = []
    for k in range(10):
        w, h = SIZES[(5 * k + 3) % len(SIZES)]
        pl = _pipeline(rng, w, h, fmt=3 if k % 2 else 1)
        if k % 5 == 4:
            pl.demosaic = abi.MG
        if k % 5 == 2:
            pl.demosaic = abi.HQLI
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


def test_stream_full_c2_frame(isp):
    pl = workloads.c2_pipeline()
    raw = workloads.c2_frame(pl, 3)
    ref, _ = O.pipeline(pl, raw)
    n0 = _launches()
    got = _run(isp, pl, raw)
    assert _launches() > n0
    assert max_abs(got, ref) == 0


def test_defect_chains_beyond_shared_memory(isp):
    """Thousands of same-colour defect clusters in one frame: more chain overrides than the
    resolution keeps in shared memory, so it falls back to its global-memory lists; the bytes must
    still equal the oracle's raster-order result."""
    rng = np.random.default_rng(12700)
    pl = _pipeline(rng, 1008, 760, fmt=3, stages=abi.STAGE_ALL & ~abi.STAGE_LUT3D)
    pl.dpc_threshold = 0.1
    raw = _frame(rng, pl, defect_frac=0.02, clusters=5000)
    ref, _ = O.pipeline(pl, raw)
    assert max_abs(_run(isp, pl, raw), ref) == 0


@pytest.mark.parametrize("entry", [
    {"kernel": abi.KERNEL_STREAM, "enabled": 1, "band_rows": 16, "seg_percent": 50},
    {"kernel": abi.KERNEL_STREAM, "enabled": 1, "band_rows": 4, "seg_percent": 10},
    {"kernel": abi.KERNEL_STREAM, "enabled": 1, "band_rows": 64, "seg_percent": 200},
    {"kernel": abi.KERNEL_STREAM, "enabled": 0, "band_rows": 32, "seg_percent": 100},
    {"kernel": abi.KERNEL_LITE, "enabled": 1, "band_rows": 8, "seg_percent": 100},
    {"kernel": abi.KERNEL_LITE, "enabled": 1, "band_rows": 48, "seg_percent": 100},
    {"kernel": abi.KERNEL_LITE, "enabled": 0, "band_rows": 16, "seg_percent": 100}])
def test_tuned_launches_same_bytes(isp, entry):
    """Every tuning choice (band rows, segment size, the tile kernel instead) leaves the output
    equal to the oracle's; a disabled class takes the tile kernel.  At 10 % segments outnumber
    the launch's warps, so most are adopted by warps done with their own."""
    from imop_gb300 import tuning
    rng = np.random.default_rng(12800 + entry["band_rows"] + entry["seg_percent"] + 7 * entry["enabled"])
    saved = tuning.get_table()
    try:
        tuning.set_table([dict(entry, fmt=-1, max_width=1 << 30)])
        if entry["kernel"] == abi.KERNEL_STREAM:
            w, h = (2048, 1200) if entry["seg_percent"] < 50 else (1288, 260)
            pl = _pipeline(rng, w, h, fmt=3, stages=abi.STAGE_ALL & ~abi.STAGE_LUT3D)
        else:
            pl = workloads.c1_pipeline(1006, 303)
        raw = _frame(rng, pl) if entry["kernel"] == abi.KERNEL_STREAM else workloads.c1_frame(pl, 5)
        ref, _ = O.pipeline(pl, raw)
        n0 = I.lib().imop_kernel_launches(entry["kernel"])
        got = _run(isp, pl, raw)
        ran = I.lib().imop_kernel_launches(entry["kernel"]) > n0
        assert ran == bool(entry["enabled"])
        assert max_abs(got, ref) == 0
    finally:
        tuning.set_table(saved)
