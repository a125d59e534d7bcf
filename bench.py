#!/usr/bin/env python3
"""Throughput of the fused RAW->RGB pipeline on one GB300 (or N independent replicas).

Workload (one step): a batch of FRAMES distinct 4024x3032 RGGB RAW12-packed frames through the full
pipeline (BL 256, 0.01 % defects + adaptive correction, 17x13 lens-shading grid, Bayer WB, AMAZE,
CCM, 4096-entry gamma LUT -> RGB8).  The batch is larger than L2 (FRAMES x 55 MB), so no L2 flush
is needed between steps.

  value       Mpix/s of the fused path with inputs resident in HBM (whole job, all ranks): one
              recorded batch per step (the streaming kernel over all frames' interiors, the
              border tile launches, the defect-chain fix-up)
  e2e         the same through the host-buffer batch API: pinned frames, copies in / kernels /
              copies out pipelined over four device slots
  roofline    dominant kernel: algorithmic bytes per launch / CUDA-event launch time vs the
              measured HBM copy bandwidth
  plain       the same batch through the plain per-operator kernels (one kernel per stage)
  cpu_baseline  the reference's own CPU per-module calls (oracle/_ref, compiled from its sources
              staged beside the oracle) on a bounded sample of the same frames on this host's cores,
              or the plain-C restatement where those sources were not staged
  c3          one 5320x4600 frame per step (8-bit and 12-bit), per-frame time and HBM GB/s
  jpeg        the step's RGB8 frames encoded to baseline JPEG (quality 90, 4:2:0, the reference's
              JpegParams defaults), byte-identical to the reference's encoder: device-resident
              frames, the host entry point with pinned buffers (e2e), RAW -> JPEG on the device
              (ISP step + encodes), and the CPU restatement of the reference's encoder

`--impl reference` times the reference's CPU algorithm for this path (its own per-module calls
compiled from the staged sources, else the oracle port) with all host threads, same metric / config.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "im-operator_gb300"))

METRIC = "ISP Mpix/s & % HBM peak, fused-batched vs plain (1 GB300, <=1 LSB); adjoint Mpix/s"
W_C2, H_C2 = 4024, 3032
# ncu smsp__inst_executed.sum of one recorded C2 step over 8 frames: the claim-word init kernel
# (0.01e6), the streaming kernel (363.24e6), the border-column (16.66e6) and border-row (10.51e6)
# tile launches, the defect-chain resolution (0.01e6) and window re-rendering (0.04e6)
WARP_INST_PER_STEP_8 = 3.905e8
# ncu dram__bytes_read.sum + dram__bytes_write.sum of the streaming kernel's launch over 8 frames
STREAM_DRAM_BYTES_8 = 391222528
# HBM bytes per C2 pixel of the plain per-operator chain (planes between its kernels)
PLAIN_BYTES_PER_PX = 62.5


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--frames", type=int, default=8, help="frames per step (batch)")
    ap.add_argument("--cpu-sample-frames", type=int, default=8)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer leg")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain per-operator leg")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint leg")
    ap.add_argument("--no-c4", action="store_true", help="skip the uneven 96-frame batch leg")
    ap.add_argument("--no-jpeg", action="store_true", help="skip the JPEG encode leg")
    ap.add_argument("--no-c3", action="store_true", help="skip the per-frame 5320x4600 leg")
    return ap.parse_args()


def peaks():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def warm_up(step, warmup, torch, seconds=0.3):
    """at least max(3, warmup) steps and `seconds` of them, for the short legs: the host-side set-up
    before a leg leaves the GPU idle long enough for its clocks to drop, and a timed region of a
    few milliseconds would otherwise begin before they are back"""
    n, t0 = 0, time.perf_counter()
    while n < max(3, warmup) or time.perf_counter() - t0 < seconds:
        step()
        n += 1
        if n % 8 == 0:
            torch.cuda.synchronize()
    torch.cuda.synchronize()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = str(gpu_index)
        self.rows = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        try:
            p = subprocess.Popen(["nvidia-smi", "-i", self.gpu, f"--query-gpu={self.FIELDS}",
                                  "--format=csv,noheader,nounits", "-lms", "200"],
                                 stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            return
        while not self._stop.is_set():
            line = p.stdout.readline()
            if not line:
                break
            self.rows.append([c.strip() for c in line.split(",")])
        p.terminate()
        try:
            p.wait(timeout=2)
        except subprocess.TimeoutExpired:
            p.kill()

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=5)

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
                for k, n in enumerate(names):
                    if r[5 + k].lower() == "active":
                        reasons.add(n)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


class CpuChain:
    """The CPU implementation of the C2 path, timed as the reference arm and as the GPU arm's
    cpu_baseline: the reference's own per-module calls (oracle/_ref, compiled from the reference's
    sources; kind "reference") where that library exists, else the oracle's C restatement (kind
    "port").  A batch of frames runs on all host cores: frames concurrently in threads (the
    reference's defect correction is sequential within a frame), each with an equal share of the
    OpenMP threads its demosaic and per-row stages use."""

    def __init__(self, pl):
        sys.path.insert(0, os.path.join(REPO, "oracle"))
        import ctypes
        import oracle_py as O
        self.O, self.pl = O, pl
        self.kind = "reference" if O.ref_available() else "port"
        self.cores = os.cpu_count() or 1
        try:
            self._omp = ctypes.CDLL("libgomp.so.1").omp_set_num_threads
        except OSError:
            self._omp = None

    def frame(self, raw):
        if self.kind == "reference":
            return self.O.ref_chain(self.pl, raw)
        return self.O.pipeline(self.pl, raw)[0]

    def batch(self, frames):
        """all frames of one step; returns the outputs"""
        n = len(frames)
        conc = max(1, min(n, self.cores))
        inner = max(1, self.cores // conc)
        out = [None] * n

        def worker(j):
            if self._omp is not None:
                self._omp(inner)
            for k in range(j, n, conc):
                out[k] = self.frame(frames[k])

        ts = [threading.Thread(target=worker, args=(j,)) for j in range(conc)]
        for t in ts:
            t.start()
        for t in ts:
            t.join()
        return out

    def describe(self):
        what = ("the reference's own per-module calls (unpack, black level, adaptive defect correction, AMAZE, "
                "CCM; compiled from its sources) with the oracle's restated grid shading, Bayer WB and LUT"
                if self.kind == "reference" else "the oracle's C restatement of the reference's chain")
        return what


def cpu_chain_rate(pl, frames, min_seconds=10.0):
    """Mpix/s of the CPU chain on batches of `frames` (all host cores), repeated until at least
    `min_seconds` of work are timed; returns (rate, frames done, seconds, CpuChain)."""
    ch = CpuChain(pl)
    ch.batch(frames[:1])  # warm-up (page-in, OpenMP pool)
    t0 = time.perf_counter()
    done = 0
    while done == 0 or time.perf_counter() - t0 < min_seconds:
        ch.batch(frames)
        done += len(frames)
    dt = time.perf_counter() - t0
    return done * pl.pixels / dt / 1e6, done, dt, ch


def cpu_jpeg_rate(rgb, quality, subsample, min_seconds=10.0):
    """Mpix/s of the CPU restatement of the reference's baseline JPEG encoder (one thread, as the
    reference's encoder) on whole frames, repeated until at least `min_seconds` are timed."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle_py as O
    h, w = rgb.shape[:2]
    t0 = time.perf_counter()
    done = 0
    while done == 0 or time.perf_counter() - t0 < min_seconds:
        O.jpeg_encode(rgb, quality, subsample)
        done += 1
    dt = time.perf_counter() - t0
    return done * w * h / dt / 1e6, done, dt


def jpeg_leg(args, torch, stream, barrier, max_over_ranks, world, rank, step_device, d_rgb, h_rgb, isp, h_raw, peak,
             peak_kind):
    """Baseline JPEG encode of the step's B RGB8 frames (4024x3032, quality 90, 4:2:0)."""
    from imop_gb300 import jpeg as J
    B = d_rgb.shape[0]
    w, h, q, ss = W_C2, H_C2, 90, 1
    enc = J.JpegEncoder()
    cap = J.max_bytes(w, h)
    d_jpg = torch.empty((B, cap), dtype=torch.uint8, device="cuda")
    sh = stream.cuda_stream
    sizes = []

    batch = [(d_rgb[i], w, h, d_jpg[i], cap, q, ss, None) for i in range(B)]

    def encode_all():  # one batch call: the frames alternate over the encoder's two streams
        enc.encode_device_batch(batch, stream=sh)

    for i in range(B):  # sizes of this step's frames, and the host entry point agrees byte for byte
        enc.encode_device(d_rgb[i], w, h, d_jpg[i], cap, q, ss, stream=sh)
        sizes.append(enc.last_size()[1])
    host0 = enc.encode(h_rgb[0].numpy().reshape(h, w, 3), q, ss)
    same = bool(host0.size == sizes[0] and (d_jpg[0, :sizes[0]].cpu().numpy() == host0).all())
    for _ in range(max(3, args.warmup)):
        encode_all()
    torch.cuda.synchronize()
    steps = args.steps
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(steps):
        encode_all()
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = max_over_ranks(ev0.elapsed_time(ev1)) / steps
    # RAW -> JPEG on the device: the ISP step, then the encodes of its frames
    barrier()
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(steps):
        step_device()
        encode_all()
    ev1.record(stream)
    torch.cuda.synchronize()
    ms_chain = max_over_ranks(ev0.elapsed_time(ev1)) / steps
    # e2e: the host batch entry point from pinned RGB8 frames into pinned JPEG buffers (frame k's
    # input copy and kernels overlap frame k-1's output copy)
    h_jpg = torch.empty((B, cap), dtype=torch.uint8).pin_memory()
    host_frames = [(h_rgb[i].view(h, w, 3), q, ss, h_jpg[i]) for i in range(B)]

    def host_all():
        res = enc.encode_host_batch(host_frames)
        if any(st for st, _ in res):
            raise RuntimeError(f"jpeg encode status {res}")

    host_all()
    barrier()
    t0 = time.perf_counter()
    for _ in range(steps):
        host_all()
    ms_e2e = max_over_ranks((time.perf_counter() - t0) * 1e3) / steps
    barrier()
    # RAW -> JPEG end to end: pinned RAW12P frames in, pinned JPEG bytes out, the RGB8 frames
    # staying in HBM (chunks of two frames: raw copies, fused batch, encoder batch, JPEG copies)
    raw_frames = [(None, h_raw[i], q, ss, h_jpg[i]) for i in range(B)]
    rj_sizes = J.raw_to_jpeg_host_batch(isp, enc, raw_frames)
    rj_same = bool(rj_sizes == sizes and (h_jpg[0, :sizes[0]].numpy() == d_jpg[0, :sizes[0]].cpu().numpy()).all())
    barrier()
    t0 = time.perf_counter()
    for _ in range(steps):
        J.raw_to_jpeg_host_batch(isp, enc, raw_frames)
    ms_rj = max_over_ranks((time.perf_counter() - t0) * 1e3) / steps
    barrier()
    px = B * w * h
    jpeg_bytes = sum(sizes)
    alg = B * w * h * 3 + jpeg_bytes  # RGB8 in, JPEG out
    out = {"value": round(world * px / (ms / 1e3) / 1e6, 2), "unit": "Mpix/s", "ms_per_step": round(ms, 4),
           "frames_per_step": B, "jpeg_bytes_per_step": jpeg_bytes, "device_equals_host_entry": same,
           "gpu_launches_per_step": 5 * B, "api": "imop_jpeg_encode_device_batch",
           "roofline": {"bound": "hbm", "achieved": round(alg / (ms / 1e3) / 1e9, 1), "peak": peak, "unit": "GB/s",
                        "frac": round(alg / (ms / 1e3) / 1e9 / peak, 4), "peak_kind": peak_kind,
                        "note": "algorithmic bytes = RGB8 in + JPEG out; the transform kernel is bound by "
                                "instruction issue (exact float DCT order), not by HBM"},
           "e2e": {"value": round(world * px / (ms_e2e / 1e3) / 1e6, 2), "unit": "Mpix/s",
                   "h2d_bytes_per_step": B * w * h * 3, "d2h_bytes_per_step": jpeg_bytes,
                   "api": "imop_jpeg_encode_host_batch (pinned RGB8 in, pinned JPEG out)"},
           "raw_to_jpeg": {"value": round(world * px / (ms_chain / 1e3) / 1e6, 2), "unit": "Mpix/s",
                           "ms_per_step": round(ms_chain, 4)},
           "raw_to_jpeg_e2e": {"value": round(world * px / (ms_rj / 1e3) / 1e6, 2), "unit": "Mpix/s",
                               "ms_per_step": round(ms_rj, 4), "h2d_bytes_per_step": int(h_raw.numel()),
                               "d2h_bytes_per_step": jpeg_bytes, "bytes_equal_device_chain": rj_same,
                               "api": "imop_isp_run_host_jpeg_batch (pinned RAW12P in, pinned JPEG out)"},
           "config": "4024x3032 RGB8 from the fused ISP step, quality 90, 4:2:0, bytes equal to "
                     "jpeg_codec::process_encode_baseline"}
    if rank == 0 and not args.no_cpu:
        rate, done, dt = cpu_jpeg_rate(h_rgb[0].numpy().reshape(h, w, 3), q, ss)
        out["cpu_baseline"] = {"value": round(rate, 3), "unit": "Mpix/s", "cores": 1, "kind": "port",
                               "sample": f"{done} frames in {dt:.1f} s (plain-C restatement of the reference's "
                                         f"single-threaded baseline encoder)"}
    enc.close()
    return out


def c3_leg(args, torch, stream, barrier, max_over_ranks, world, peak, peak_kind):
    """C3: one 5320x4600 frame per step, 8-bit and 12-bit u16 (BL, RGB WB, HQLI, linear tone ->
    RGB8), device-resident, one recorded single-frame batch per step; per-frame time and HBM
    GB/s against the measured peak.  Inputs and outputs of one frame (98 / 122 MB) are larger than
    half the L2; a 256 MB buffer is rewritten between steps so each step starts cold."""
    import imop_gb300 as I
    from imop_gb300 import abi, workloads
    out = {}
    # the earlier legs' cached blocks go back to the device first, so this leg's frames are
    # fresh allocations rather than pieces of blocks split by other legs
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    sh = stream.cuda_stream
    for pl in workloads.c3_pipelines():
        isp = I.Isp(pl)
        d_in = torch.from_numpy(workloads.c3_frame(pl, 0)).cuda()
        d_out = torch.empty(pl.output_bytes(), dtype=torch.uint8, device="cuda")
        desc = [(None, d_in.data_ptr(), d_out.data_ptr())]
        isp.batch_submit(desc, flags=abi.BATCH_GRAPH, stream=sh)
        fused = d_out.clone()
        isp.batch_submit(desc, flags=abi.BATCH_PLAIN, stream=sh)
        isp.sync_status(sh)
        same = bool(torch.equal(fused, d_out))
        del fused
        warm_up(lambda: isp.batch_submit(desc, flags=abi.BATCH_GRAPH, stream=sh), args.warmup, torch)
        steps = max(1, min(2 * args.steps, 20))  # short steps: more of them for a steadier mean
        # per step, in one stream: the L2 flush, then the frame's graph between two events; the
        # steps are queued without host waits, so the events bracket the frame's device work alone
        # (the host-side submission overlaps the flush before it)
        evs = []
        barrier()
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            for _ in range(steps):
                flush.fill_(1)
                ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                ev0.record(stream)
                isp.batch_submit(desc, flags=abi.BATCH_GRAPH, stream=sh)
                ev1.record(stream)
                evs.append((ev0, ev1))
        torch.cuda.synchronize()
        total = sum(max_over_ranks(a.elapsed_time(b)) for a, b in evs)
        isp.sync_status(sh)
        isp.close()
        ms = total / steps
        alg = pl.input_bytes() + pl.output_bytes()
        gbs = alg / (ms / 1e3) / 1e9
        if not same:
            out[f"{pl.bit_depth}bit"] = {"value": None, "error": "fused frame differs from the plain path"}
            continue
        out[f"{pl.bit_depth}bit"] = {"ms_per_frame": round(ms, 4), "Mpix/s": round(world * pl.pixels / (ms / 1e3) / 1e6, 1),
                                     "gbs_algorithmic": round(gbs, 1), "hbm_frac": round(gbs / peak, 4),
                                     "bytes_per_frame": alg, "fused_equals_plain": same}
    out["config"] = ("C3: 5320x4600 RGGB, an 8-bit frame and a 12-bit u16 frame, BL, RGB-order WB, HQLI, "
                     "linear tone -> RGB8; L2 flushed between steps; peak " + peak_kind)
    return out


def c1_leg(args, torch, stream, barrier, max_over_ranks, world, peak, peak_kind, n_frames=64):
    """C1: 1006x758 RGGB 10-bit u16 frames (BL 64, RGB-order WB, HQLI, linear tone -> RGB8), a
    batch of n_frames distinct frames per step (244 MB in and out, larger than L2), device-resident,
    one recorded batch per step; Mpix/s and HBM GB/s against the measured peak.  Every frame is
    checked against the plain per-operator path before timing."""
    import imop_gb300 as I
    from imop_gb300 import abi, workloads
    pl = workloads.c1_pipeline()
    isp = I.Isp(pl)
    d_in = torch.stack([torch.from_numpy(workloads.c1_frame(pl, k)) for k in range(n_frames)]).cuda()
    d_out = torch.empty((n_frames, pl.output_bytes()), dtype=torch.uint8, device="cuda")
    sh = stream.cuda_stream
    desc = [(None, d_in[k].data_ptr(), d_out[k].data_ptr()) for k in range(n_frames)]
    isp.batch_submit(desc, flags=abi.BATCH_GRAPH, stream=sh)
    fused = d_out.clone()
    isp.batch_submit(desc, flags=abi.BATCH_PLAIN, stream=sh)
    isp.sync_status(sh)
    same = bool(torch.equal(fused, d_out))
    del fused
    warm_up(lambda: isp.batch_submit(desc, flags=abi.BATCH_GRAPH, stream=sh), args.warmup, torch)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(args.steps):
        isp.batch_submit(desc, flags=abi.BATCH_GRAPH, stream=sh)
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = max_over_ranks(ev0.elapsed_time(ev1)) / args.steps
    isp.sync_status(sh)
    isp.close()
    if not same:
        return {"value": None, "error": "fused batch differs from the plain path"}
    px = n_frames * pl.pixels
    alg = n_frames * (pl.input_bytes() + pl.output_bytes())
    gbs = alg / (ms / 1e3) / 1e9
    return {"value": round(world * px / (ms / 1e3) / 1e6, 1), "unit": "Mpix/s", "ms_per_step": round(ms, 4),
            "frames_per_step": n_frames, "gbs_algorithmic": round(world * gbs, 1), "hbm_frac": round(gbs / peak, 4),
            "bytes_per_step": alg, "fused_equals_plain": same,
            "config": f"C1: {n_frames} x 1006x758 RGGB 10-bit u16, BL 64, RGB-order WB, HQLI, linear tone -> RGB8; "
                      f"peak {peak_kind}"}


def adjoint_leg(isp, args, torch, stream, barrier, max_over_ranks, world):
    """Adjoint of the calibration chain on C5: 16 x 1006x758 RGGB 12-bit frames, AMAZE, 933
    parameters; one step = forward recompute + back-propagation + parameter reduction against an
    FP32 target (the loss and dL/dtheta), CUDA events on the launching stream."""
    from imop_gb300 import abi, workloads
    from imop_gb300 import adjoint as A
    d = workloads.c5_desc()
    th_true = workloads.c5_theta_true(d)
    raw = torch.from_numpy(workloads.c5_frames(d)).cuda()
    theta_true = torch.from_numpy(th_true).cuda()
    target = A.render_forward(isp, d, theta_true, raw)
    theta = torch.from_numpy(workloads.c5_theta_init(th_true)).cuda()
    for _ in range(args.warmup):
        A.backward(isp, d, theta, raw, target, abi.ADJ_TARGET)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(args.steps):
        A.backward(isp, d, theta, raw, target, abi.ADJ_TARGET)
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier()
    ms = max_over_ranks(ev0.elapsed_time(ev1))
    px = d.n_frames * d.width * d.height
    alg = px * (2 + 12) + 2 * 933 * 4  # raw u16 + FP32 RGB target per pixel, parameters in and out
    return {"value": round(world * args.steps * px / (ms / 1e3) / 1e6, 2), "unit": "Mpix/s",
            "ms_per_step": round(ms / args.steps, 4), "bytes_per_step": alg,
            "gbs_algorithmic": round(world * args.steps * alg / (ms / 1e3) / 1e9, 1),
            "config": "C5: 16 x 1006x758 RGGB 12-bit u16, AMAZE, 17x13 grid, 933 parameters, L2 to an FP32 target",
            "gpu_launches_per_step": 2}


def c4_leg(isp, args, torch, stream, barrier, max_over_ranks, world):
    """C4: 96 frames of three sizes (1006x758, 4024x3032, 5320x4600) and five formats (RAW8,
    RAW10/RAW12 packed and unpacked), each with its own BL / WB / CCM, as one recorded batch
    (one persistent launch per 16 frames) against 96 plain per-operator pipelines."""
    from imop_gb300 import abi, workloads
    frames = workloads.c4_batch()
    dev = []
    for pl, raw in frames:
        d_in = torch.from_numpy(raw).cuda()
        d_out = torch.empty(pl.output_bytes(), dtype=torch.uint8, device="cuda")
        dev.append((pl, d_in, d_out))
    descs = [(pl, d_in.data_ptr(), d_out.data_ptr()) for pl, d_in, d_out in dev]
    px = sum(pl.pixels for pl, _ in frames)
    alg = sum(pl.input_bytes() + pl.output_bytes() for pl, _ in frames)
    sh = stream.cuda_stream
    steps = max(1, min(args.steps, 3))

    def run(flags):
        for _ in range(2):
            isp.batch_submit(descs, flags=flags, stream=sh)
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        barrier()
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(steps):
            isp.batch_submit(descs, flags=flags, stream=sh)
        ev1.record(stream)
        torch.cuda.synchronize()
        barrier()
        return max_over_ranks(ev0.elapsed_time(ev1)) / steps

    ms = run(abi.BATCH_GRAPH)
    isp.sync_status(sh)
    fused = [d_out.clone() for _, _, d_out in dev]
    ms_plain = run(abi.BATCH_PLAIN)
    isp.sync_status(sh)
    # correctness gate: every frame of the recorded batch equals the plain per-operator path
    bad = [k for k, (f, (_, _, d_out)) in enumerate(zip(fused, dev)) if not torch.equal(f, d_out)]
    del fused
    if bad:
        return {"value": None, "error": f"recorded batch differs from the plain path on frames {bad[:8]}",
                "frames": len(frames)}
    # the same batch with the built-in launch parameters, and with the tile kernel alone (both
    # streamed kernels disabled), against the measured table loaded at start-up
    from imop_gb300 import tuning
    table = tuning.get_table()
    try:
        tuning.set_table([])
        ms_fixed = run(abi.BATCH_GRAPH)
        off = {"fmt": -1, "max_width": 1 << 30, "enabled": 0, "band_rows": 16, "seg_percent": 100}
        tuning.set_table([dict(off, kernel=abi.KERNEL_LITE), dict(off, kernel=abi.KERNEL_STREAM)])
        ms_tile = run(abi.BATCH_GRAPH)
    finally:
        tuning.set_table(table)
    isp.sync_status(sh)
    tuned = {"table_entries": len(table), "ms_per_step": round(ms, 3), "fixed_ms_per_step": round(ms_fixed, 3),
             "tile_kernel_only_ms_per_step": round(ms_tile, 3),
             "note": "fixed: the built-in launch parameters; tile kernel only: every frame in the general "
                     "tiled kernel, one launch per instantiation group of up to 32 frames"}
    return {"value": round(world * px / (ms / 1e3) / 1e6, 2), "unit": "Mpix/s", "ms_per_step": round(ms, 3),
            "fused_equals_plain": True, "tuning": tuned,
            "plain": {"value": round(world * px / (ms_plain / 1e3) / 1e6, 2), "ms_per_step": round(ms_plain, 3)},
            "gbs_algorithmic": round(world * alg / (ms / 1e3) / 1e9, 1), "frames": len(frames),
            "megapixels_per_step": round(px / 1e6, 1), "steps": steps,
            "config": "C4: 96 frames, sizes 1006x758 / 4024x3032 / 5320x4600, RAW8 and RAW10/RAW12 packed and "
                      "unpacked, own BL (64 or 256) / WB / CCM each, AMAZE, recorded graph vs 96 plain pipelines"}


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def frame_indices(rank, frames_per_rank):
    """scene indices of a replica's frames: every rank renders frames of its own"""
    return [rank * frames_per_rank + i for i in range(frames_per_rank)]


def rank_sync(world, device):
    """(barrier, max_over_ranks) of a replica run: no-ops for one rank; otherwise a process-group
    barrier and an all-reduce MAX of a time in ms (the tensor on `device`: "cuda" under NCCL,
    "cpu" under gloo)"""
    import torch

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    def max_over_ranks(ms):
        if world > 1:
            t = torch.tensor([ms], dtype=torch.float64, device=device)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            ms = float(t.item())
        return ms

    return barrier, max_over_ranks


def c2_config(B, world, in_b, out_b):
    """the `config` of both arms: the C2 workload with B frames per step"""
    return {"workload": "C2 4024x3032 RGGB RAW12P full pipeline (BL, adaptive DPC, 17x13 LSC grid, "
                        "Bayer WB, AMAZE, CCM, gamma LUT -> RGB8)",
            "frames_per_step": B, "pixels_per_frame": W_C2 * H_C2,
            "l2": f"inputs larger than L2: {B} distinct frames, {B * (in_b + out_b) / 1e6:.0f} MB per step",
            "parallelism": f"replicas x{world}"}


def run_reference(args):
    """The reference arm: the CPU chain (CpuChain) on the same B frames per step as the GPU arm
    (the frames of rank 0), rendered by the oracle's copy of the workloads' generator, so no part
    of the product library is loaded.  Rank 0 alone runs; the other ranks exit without work."""
    world, rank, _ = dist_init()
    if rank != 0:
        return
    from imop_gb300 import workloads
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle_py as O
    B = args.frames
    pl = workloads.c2_pipeline(defects=O.defects)
    frames = [workloads.c2_frame(pl, k, gen=O) for k in frame_indices(0, B)]
    ch = CpuChain(pl)
    for _ in range(max(0, args.warmup)):
        ch.batch(frames)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ch.batch(frames)
    dt = time.perf_counter() - t0
    rate = args.steps * B * pl.pixels / dt / 1e6
    sample = (f"{args.steps} steps of the step's {B} C2 frames: {ch.describe()}; frames concurrently in "
              f"{min(B, ch.cores)} threads sharing {ch.cores} host cores")
    ref_cuda = reference_cuda_leg(args, pl, frames, O)
    line = {
        "impl": "reference", "metric": METRIC, "value": round(rate, 3), "unit": "Mpix/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1000 * dt / args.steps, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u16/f32", "data": "synthetic (seeded sinusoid scene + shot/read noise + "
                                                         "0.01% hot/dead pixels)",
        "config": c2_config(B, world, pl.input_bytes(), pl.output_bytes()),
        "cpu_baseline": {"value": round(rate, 3), "unit": "Mpix/s", "cores": ch.cores, "kind": ch.kind,
                         "sample": sample},
        "e2e": {"value": round(rate, 3), "unit": "Mpix/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "reference_cuda": ref_cuda,
    }
    print(json.dumps(line), flush=True)


def reference_cuda_leg(args, pl, frames, O):
    """The reference's own GPU path on this GB300, timed beside its CPU path: each frame through
    the calls its dispatchers make on a CUDA host (oracle_py.ref_chain_cuda: its GPU black level,
    adaptive defect correction and AMAZE, each with its own host copies; its CPU unpack and CCM; the
    restated grid shading, Bayer WB and LUT), one frame after the other as its synchronous calls
    run.  Timing only."""
    if not (O.ref_available() and O.refcuda_available()):
        return {"value": None, "unavailable": "the reference's sources were not staged on this host"}
    if O.refcuda().refcuda_has_cuda() != 1:
        return {"value": None, "unavailable": "no CUDA device"}
    O.ref_chain_cuda(pl, frames[0])  # context, workspaces
    n = max(1, min(len(frames), 8))
    t0 = time.perf_counter()
    for _ in range(max(1, min(args.steps, 3))):
        for f in frames[:n]:
            O.ref_chain_cuda(pl, f)
    dt = time.perf_counter() - t0
    done = max(1, min(args.steps, 3)) * n
    return {"value": round(done * pl.pixels / dt / 1e6, 3), "unit": "Mpix/s", "frames": done,
            "seconds": round(dt, 3),
            "on_gpu": "black_level::process_black_level_cuda, defect_correct::process_defect_correct_cuda "
                      "(adaptive), imop::demosaic_cuda (AMAZE; the reference's GPU demosaic takes no packed input)",
            "not_run": "ccm::process_ccm_cuda and the reference's other kern_gpu_pipeline stages: their parameter "
                       "buffer is never allocated on that path (GpuWorkspace::ensure(w, h, bd, 0)), so the kernel "
                       "would read through a null pointer; the CCM runs on the reference's CPU code",
            "note": "timing only: the reference's GPU kernels do not reproduce its CPU results"}


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    world, rank, local = dist_init()
    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    import imop_gb300 as I
    from imop_gb300 import abi, workloads

    pl = workloads.c2_pipeline()
    B = args.frames
    in_b, out_b = pl.input_bytes(), pl.output_bytes()
    host_frames = [workloads.c2_frame(pl, k) for k in frame_indices(rank, B)]
    h_in = torch.empty((B, in_b), dtype=torch.uint8).pin_memory()
    for i, f in enumerate(host_frames):
        h_in[i].copy_(torch.from_numpy(f))
    h_out = torch.empty((B, out_b), dtype=torch.uint8).pin_memory()
    d_in = h_in.cuda()
    d_out = torch.empty((B, out_b), dtype=torch.uint8, device="cuda")
    isp = I.Isp(pl)
    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream
    dev_frames = [(None, d_in[i].data_ptr(), d_out[i].data_ptr()) for i in range(B)]
    host_batch = [(None, h_in[i].data_ptr(), h_out[i].data_ptr()) for i in range(B)]

    def step_device():
        # one recorded graph per step: seed-counter reset, the claim-word init, the streaming
        # launch over all B frames' interiors with the two border tile launches beside it, the
        # defect-chain resolution and window re-rendering launches
        isp.batch_submit(dev_frames, flags=abi.BATCH_GRAPH, stream=sh)

    def step_plain():
        isp.batch_submit(dev_frames, flags=abi.BATCH_PLAIN, stream=sh)

    barrier, max_over_ranks = rank_sync(world, "cuda")

    def timed(fn, steps):
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        barrier()
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(steps):
            fn()
        ev1.record(stream)
        torch.cuda.synchronize()
        barrier()
        return max_over_ranks(ev0.elapsed_time(ev1))

    # correctness gate before timing: the fused batch equals the plain per-operator batch
    step_device()
    fused = d_out.clone()
    step_plain()
    torch.cuda.synchronize()
    parity_ok = bool(torch.equal(fused, d_out))
    isp.sync_status(sh)

    for _ in range(args.warmup):
        step_device()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        ms = timed(step_device, args.steps)
    isp.sync_status(sh)
    ms_e2e = None
    if not args.no_e2e:
        # end to end through the host-buffer batch call: pinned frames, copies in, kernels and
        # copies out pipelined over four device slots; synchronous, so wall-clock timed
        for _ in range(max(1, args.warmup // 2)):
            isp.run_host_batch(host_batch)
        barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            isp.run_host_batch(host_batch)
        torch.cuda.synchronize()
        ms_e2e = max_over_ranks((time.perf_counter() - t0) * 1e3)
        barrier()
    ms_plain = None
    if not args.no_plain:
        for _ in range(max(1, args.warmup // 2)):
            step_plain()
        ms_plain = timed(step_plain, args.steps)

    jpeg = None
    if not args.no_jpeg:
        pk, pk_kind = peaks()
        if args.no_e2e:  # the host frames of the JPEG e2e leg are the ISP's outputs
            isp.run_host_batch(host_batch)
        jpeg = jpeg_leg(args, torch, stream, barrier, max_over_ranks, world, rank, step_device,
                        d_out.view(B, H_C2, W_C2, 3), h_out, isp, h_in, pk, pk_kind)

    c3 = None
    if not args.no_c3:
        pk, pk_kind = peaks()
        with ClockSampler(local) as clk3:
            c3 = c3_leg(args, torch, stream, barrier, max_over_ranks, world, pk, pk_kind)
            c3["c1"] = c1_leg(args, torch, stream, barrier, max_over_ranks, world, pk, pk_kind)
        c3["clocks"] = clk3.summary()

    adjoint = None
    if not args.no_adjoint:
        adjoint = adjoint_leg(isp, args, torch, stream, barrier, max_over_ranks, world)
    c4 = None
    if not args.no_c4:
        c4 = c4_leg(isp, args, torch, stream, barrier, max_over_ranks, world)

    px_step = B * pl.pixels
    mpix = world * args.steps * px_step / (ms / 1e3) / 1e6
    alg_bytes = in_b + out_b + 4096 * 4 + 17 * 13 * 4 * 4  # per frame: RAW12P in, RGB8 out, LUT, grid
    # the launch time of the roofline is the recorded step of the timed region (CUDA events on the
    # launching stream): the streaming kernel over the frames' interiors (85 % of the step in the
    # ncu launch list), the border-column and border-row tile launches and the two fix-up launches
    per_launch_ms = ms / args.steps
    achieved = B * alg_bytes / (per_launch_ms / 1e3) / 1e9
    peak, peak_kind = peaks()

    line = {
        "metric": METRIC, "value": round(mpix, 2), "unit": "Mpix/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u16/f32",
        "data": "synthetic (seeded sinusoid scene + shot/read noise + 0.01% hot/dead pixels)",
        "config": c2_config(B, world, in_b, out_b),
        "gbs_algorithmic": round(world * args.steps * B * alg_bytes / (ms / 1e3) / 1e9, 1),
        "hbm_frac": round(world * args.steps * B * alg_bytes / (ms / 1e3) / 1e9 / peak, 4),
        "fused_equals_plain": parity_ok,
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": int(STREAM_DRAM_BYTES_8 * B / 8),
                     "peak_kind": peak_kind,
                     "kernel": "stream_kernel (warp-streamed strips of the frames' interiors, one launch "
                               "over the step's frames), timed as the recorded step with its claim-word "
                               "init, the border tile launches beside it and the two defect fix-up launches",
                     "bytes_per_launch": B * alg_bytes, "launch_ms": round(per_launch_ms, 4),
                     "traffic_note": "ncu: 391.2 MB DRAM read+write of the streaming kernel's launch over "
                                     "8 frames (the last writes still in L2 when it ends; profiles/)"},
        "gpu_launches": 6 * args.steps,
        "clocks": clk.summary(),
    }
    # the ceiling that binds this kernel: warp-instruction issue (4 per SM per clock)
    sm_mhz = line["clocks"]["sm_mhz"] or line["clocks"]["sm_max_mhz"] or 2070.0
    n_sm = torch.cuda.get_device_properties(0).multi_processor_count
    issue_peak = n_sm * 4 * sm_mhz * 1e6
    issue_achieved = WARP_INST_PER_STEP_8 * B / 8 / (per_launch_ms / 1e3)
    line["roofline"]["issue"] = {
        "achieved": round(issue_achieved / 1e12, 4), "peak": round(issue_peak / 1e12, 4),
        "unit": "T warp instructions/s", "frac": round(issue_achieved / issue_peak, 4),
        "warp_instructions_per_launch": int(WARP_INST_PER_STEP_8 * B / 8),
        "note": f"ncu smsp__inst_executed.sum of the step's six kernels over 8 frames (profiles/); peak = {n_sm} SMs x 4 "
                f"schedulers x the median SM clock sampled in the timed region"}
    if ms_e2e is not None:
        line["e2e"] = {"value": round(world * args.steps * px_step / (ms_e2e / 1e3) / 1e6, 2), "unit": "Mpix/s",
                       "h2d_bytes_per_step": B * in_b, "d2h_bytes_per_step": B * out_b,
                       "api": "imop_isp_run_host_batch (pinned host frames)"}
    if ms_plain is not None:
        # the plain path's own HBM traffic: u16 planes between its kernels (bytes per C2 pixel:
        # unpack 1.5 + 2, black level 2 + 2, Jacobi 2 + 2, seeds 2 + 2, lens shading 2 + 2, white
        # balance 2 + 2, green 2 + 4, demosaic 2 + 4 + 6, CCM 6 + 6, output 6 + 3)
        plain_gbs = world * args.steps * px_step * PLAIN_BYTES_PER_PX / (ms_plain / 1e3) / 1e9
        line["plain"] = {"value": round(world * args.steps * px_step / (ms_plain / 1e3) / 1e6, 2), "unit": "Mpix/s",
                         "ms_per_step": round(ms_plain / args.steps, 4), "bytes_per_pixel": PLAIN_BYTES_PER_PX,
                         "gbs_traffic": round(plain_gbs, 1), "hbm_frac": round(plain_gbs / peak, 4)}
    if adjoint is not None:
        line["adjoint"] = adjoint
    if c4 is not None:
        line["c4"] = c4
    if jpeg is not None:
        line["jpeg"] = jpeg
    if c3 is not None:
        line["c3"] = c3
    if rank == 0 and not args.no_cpu:
        rate, done, dt, ch = cpu_chain_rate(pl, host_frames[: max(1, args.cpu_sample_frames)])
        line["cpu_baseline"] = {"value": round(rate, 3), "unit": "Mpix/s", "cores": ch.cores, "kind": ch.kind,
                                "sample": f"{done} C2 frames in {dt:.1f} s ({ch.describe()}; frames "
                                          f"concurrently on all host cores)"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    isp.close()
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
