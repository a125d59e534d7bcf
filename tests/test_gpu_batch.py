"""GPU parity of the batch entry points: mixed sizes, formats and parameter sets in one persistent
launch (more than one launch group, both output widths), the recorded-graph replay, the plain
per-frame comparator, and the pipelined host batch - every frame against the CPU oracle."""
import numpy as np
import pytest

import imop_gb300 as I
from imop_gb300 import abi, workloads
import oracle_py as O

from helpers import max_abs, random_frame, random_pipeline

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

MIX = [(6, 6, 8, False), (7, 9, 12, True), (33, 17, 10, True), (131, 70, 12, False), (200, 97, 10, False),
       (67, 35, 16, False), (250, 130, 12, True), (64, 32, 9, False), (1006, 758, 10, False),
       (121, 25, 12, True), (120, 24, 8, False), (241, 49, 12, True)]
DEMOSAICS = [abi.HQLI, abi.AMAZE, abi.MG]


def _mixed(seed, n):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        w, h, bd, packed = MIX[k % len(MIX)]
        dm = DEMOSAICS[k % 3]
        dpc = abi.DPC_MAP_BASED if k % 5 == 3 else abi.DPC_ADAPTIVE
        lsc = [abi.LSC_GRID, abi.LSC_POLYNOMIAL, abi.LSC_GRID][k % 3]
        out_fmt = abi.OUT_NATIVE if k % 7 == 6 else abi.OUT_RGB8
        pl = random_pipeline(rng, w, h, bd, packed, dm, int(rng.integers(0, 4)), dpc_mode=dpc, lsc_mode=lsc,
                             out=out_fmt)
        raw = random_frame(rng, pl)
        ref, _ = O.pipeline(pl, raw)
        out.append((pl, raw, ref))
    return out


def _device(frames):
    d = []
    for pl, raw, _ in frames:
        d_in = torch.from_numpy(raw).cuda()
        d_out = torch.zeros(pl.output_bytes(), dtype=torch.uint8, device="cuda")
        d.append((pl, d_in, d_out))
    return d


def _check(frames, dev):
    for k, ((pl, _, ref), (_, _, d_out)) in enumerate(zip(frames, dev)):
        got = d_out.cpu().numpy().view(ref.dtype).reshape(ref.shape)
        assert max_abs(got, ref) == 0, f"frame {k}: {pl.width}x{pl.height} bd {pl.bit_depth} demosaic {pl.demosaic}"


@pytest.fixture(scope="module")
def isp():
    ctx = I.Isp()
    yield ctx
    ctx.close()


@pytest.mark.parametrize("flags", [0, abi.BATCH_PLAIN])
def test_mixed_batch(isp, flags):
    frames = _mixed(3 + flags, 22)  # 22 frames: two launch groups, two output widths
    dev = _device(frames)
    isp.batch_submit(dev, flags=flags)
    isp.sync_status()
    _check(frames, dev)


def test_graph_replay(isp):
    """The first call records, later calls with the same descriptors replay: new input contents
    in the same buffers must give the new outputs."""
    frames = _mixed(11, 9)
    dev = _device(frames)
    isp.batch_submit(dev, flags=abi.BATCH_GRAPH)
    isp.sync_status()
    _check(frames, dev)
    rng = np.random.default_rng(12)
    frames2 = []
    for (pl, _, _), (_, d_in, d_out) in zip(frames, dev):
        raw = random_frame(rng, pl)
        d_in.copy_(torch.from_numpy(raw))
        d_out.zero_()
        ref, _ = O.pipeline(pl, raw)
        frames2.append((pl, raw, ref))
    for _ in range(2):
        isp.batch_submit(dev, flags=abi.BATCH_GRAPH)
    isp.sync_status()
    _check(frames2, dev)


def test_batch_defect_chains_per_frame(isp):
    """Frames with defect chains in one launch each keep their own seed list and fix-up."""
    rng = np.random.default_rng(5)
    frames = []
    for k in range(4):
        w, h, bd = 150 + 2 * k, 90, 12
        pl = random_pipeline(rng, w, h, bd, True, abi.AMAZE, abi.RGGB, order=abi.ORDER_BAYER_WB)
        pl.dpc_threshold = 0.1
        f = I.scene(w, h, bd, abi.RGGB, 40 + k, lo=800, hi=2000)
        f[10:80:2, 40 + 2 * k] = 4095
        f[30 + k, 20:140:2] = 0
        raw = I.pack_mipi(f, bd)
        ref, _ = O.pipeline(pl, raw)
        frames.append((pl, raw, ref))
    dev = _device(frames)
    isp.batch_submit(dev)
    isp.sync_status()
    _check(frames, dev)


def test_run_host_batch(isp):
    frames = _mixed(21, 10)
    outs = [np.zeros(ref.shape, ref.dtype) for _, _, ref in frames]
    isp.run_host_batch([(pl, raw, o) for (pl, raw, _), o in zip(frames, outs)])
    for (pl, _, ref), o in zip(frames, outs):
        assert max_abs(o, ref) == 0


def test_run_host_batch_mixed_memory(isp):
    """Page-locked and pageable host frames in one call, more frames than device slots."""
    frames = _mixed(33, 8)
    descs, outs = [], []
    for k, (pl, raw, ref) in enumerate(frames):
        inp = torch.from_numpy(raw.reshape(-1).view(np.uint8)).pin_memory() if k % 3 == 1 else raw
        if k % 2 == 0:
            out = torch.zeros(ref.nbytes, dtype=torch.uint8).pin_memory()
        else:
            out = np.zeros(ref.shape, ref.dtype)
        descs.append((pl, inp, out))
        outs.append(out)
    isp.run_host_batch(descs)
    for (pl, _, ref), o in zip(frames, outs):
        got = o.numpy().view(ref.dtype).reshape(ref.shape) if isinstance(o, torch.Tensor) else o
        assert max_abs(got, ref) == 0


def test_run_host_pinned_output(isp):
    """Single-frame host call filling a page-locked output frame in place."""
    pl, raw, ref = _mixed(34, 1)[0]
    isp.set_params(pl)
    out = torch.zeros(ref.nbytes, dtype=torch.uint8).pin_memory()
    isp.run_host(raw, out)
    assert max_abs(out.numpy().view(ref.dtype).reshape(ref.shape), ref) == 0


def test_run_host_batch_pinned_c2(isp):
    """Page-locked host frames of the 4024x3032 RAW12P workload through the pipelined host batch."""
    pl = workloads.c2_pipeline()
    raws = [workloads.c2_frame(pl, k) for k in range(3)]
    ins = [torch.from_numpy(r).pin_memory() for r in raws]
    outs = [torch.empty(pl.output_bytes(), dtype=torch.uint8).pin_memory() for _ in raws]
    isp.run_host_batch([(pl, i.data_ptr(), o.data_ptr()) for i, o in zip(ins, outs)])
    ref, _ = O.pipeline(pl, raws[2])
    assert np.array_equal(outs[2].numpy().reshape(ref.shape), ref)
    d_in = torch.from_numpy(raws[0]).cuda()
    d_out = torch.empty(pl.output_bytes(), dtype=torch.uint8, device="cuda")
    isp.set_params(pl)
    isp.run_device(d_in, d_out)
    torch.cuda.synchronize()
    assert torch.equal(d_out.cpu(), outs[0])


def test_c4_batch_at_its_own_configuration(isp):
    """The 96-frame uneven batch the bench times (1006x758 / 4024x3032 / 5320x4600, RAW8 and
    RAW10 / RAW12 packed and unpacked, each frame its own BL / WB / CCM), as one recorded batch:
    every frame equals the plain per-operator path, and one frame of each (size, format) pair
    equals the CPU oracle."""
    frames = workloads.c4_batch()
    assert len(frames) == 96
    dev = []
    for pl, raw in frames:
        d_in = torch.from_numpy(raw).cuda()
        dev.append((pl, d_in, torch.zeros(pl.output_bytes(), dtype=torch.uint8, device="cuda")))
    isp.batch_submit(dev, flags=abi.BATCH_GRAPH)
    isp.batch_submit(dev, flags=abi.BATCH_GRAPH)  # recorded on the first call, replayed here
    isp.sync_status()
    fused = [d_out.clone() for _, _, d_out in dev]
    for _, _, d_out in dev:
        d_out.zero_()
    isp.batch_submit(dev, flags=abi.BATCH_PLAIN)
    isp.sync_status()
    for k, (f, (pl, _, d_out)) in enumerate(zip(fused, dev)):
        assert torch.equal(f, d_out), f"frame {k}: {pl.width}x{pl.height} bd {pl.bit_depth} packed {pl.packed}"
    seen = set()
    for k, (pl, raw) in enumerate(frames):
        key = (pl.width, pl.height, pl.bit_depth, pl.packed)
        if key in seen:
            continue
        seen.add(key)
        ref, _ = O.pipeline(pl, raw)
        got = fused[k].cpu().numpy().reshape(ref.shape)
        assert np.array_equal(got, ref), f"frame {k} vs oracle: {key}"
    assert len(seen) == 15
