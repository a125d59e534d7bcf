"""Launch tuning of the two streamed kernels (ImopTuneEntry, imop_tuning_set).

Per (kernel, input format, width class) the table says whether frames of that class take the
kernel at all (otherwise the general tile kernel), the rows of a band (the light-chain kernel's
unit of work, the streaming kernel's claim granule) and the streaming kernel's segment size.

    python -m imop_gb300.tuning --out tuning_gb300.json    # measure on this GPU, write the table
    python -m imop_gb300.tuning --kernels lite             # re-measure one kernel's classes

measures every candidate of every class on the device (CUDA events over replayed batch graphs)
and writes the best entry per class together with every timing, the built-in default's among
them, so the table states what tuning won against the fixed parameters.  `load()` applies a
table; importing the package loads `tuning_gb300.json` beside this file when the device's name
matches the one the table was measured on.
"""
import argparse
import ctypes as C
import json
import os

from . import abi

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_TABLE = os.path.join(HERE, "tuning_gb300.json")
FMT_NAMES = {0: "u8", 1: "u16", 2: "raw10p", 3: "raw12p"}
# width classes: the widths of the workloads (1006, 4024, 5320) each in its own class
WIDTH_CLASSES = [1024, 4096, 1 << 30]
DEFAULTS = {abi.KERNEL_LITE: (1, 16, 100), abi.KERNEL_STREAM: (1, 32, 100)}


def _lib():
    from . import lib
    return lib()


def set_table(entries):
    """entries: dicts with kernel, fmt, max_width, enabled, band_rows, seg_percent"""
    from . import check
    arr = (abi.TuneEntry * max(1, len(entries)))()
    for k, e in enumerate(entries):
        arr[k] = abi.TuneEntry(int(e["kernel"]), int(e["fmt"]), int(e["max_width"]), int(e["enabled"]),
                               int(e["band_rows"]), int(e["seg_percent"]))
    check(_lib().imop_tuning_set(arr, len(entries)))


def get_table():
    n = _lib().imop_tuning_get(None, 0)
    arr = (abi.TuneEntry * max(1, n))()
    _lib().imop_tuning_get(arr, n)
    return [{f: getattr(arr[k], f) for f, _ in abi.TuneEntry._fields_} for k in range(n)]


def load(path=DEFAULT_TABLE, device_name=None):
    """Apply the table in `path` (when its device matches `device_name`, if given); returns the
    number of entries applied (0: no table or another device)."""
    if not os.path.exists(path):
        return 0
    with open(path) as f:
        t = json.load(f)
    if device_name is not None and t.get("device") != device_name:
        return 0
    set_table(t["entries"])
    return len(t["entries"])


def _classes():
    """(kernel, fmt, width class, [(pipeline, raw bytes)], frames per step): the workloads' frames
    grouped the way a launch groups them"""
    from . import workloads
    out = []
    c1 = workloads.c1_pipeline()
    out.append((abi.KERNEL_LITE, 1, 1024, [(c1, workloads.c1_frame(c1, k)) for k in range(16)]))
    for pl in workloads.c3_pipelines():
        out.append((abi.KERNEL_LITE, 0 if pl.bit_depth <= 8 else 1, 1 << 30, [(pl, workloads.c3_frame(pl, 0))]))
    c2 = workloads.c2_pipeline()
    out.append((abi.KERNEL_STREAM, 3, 4096, [(c2, workloads.c2_frame(c2, k)) for k in range(8)]))
    # the C4 frames by (format, width class): each class as the batch its launch would be
    groups = {}
    for pl, raw in workloads.c4_batch():
        fmt = 2 if (pl.packed and pl.bit_depth == 10) else 3 if pl.packed else (0 if pl.bit_depth <= 8 else 1)
        wc = next(c for c in WIDTH_CLASSES if pl.width <= c)
        if (fmt, wc) == (3, 4096):
            continue  # the C2 class above
        groups.setdefault((fmt, wc), []).append((pl, raw))
    for (fmt, wc), frames in sorted(groups.items()):
        out.append((abi.KERNEL_STREAM, fmt, wc, frames[:8]))
    return out


def _candidates(kernel):
    if kernel == abi.KERNEL_LITE:
        # the staged variant takes only the band; the direct-read one also the segment spread
        return [(1, b, s) for b in (4, 8, 16, 32) for s in (50, 100, 200)] + [(0, 16, 100)]
    return [(1, b, s) for b in (16, 32, 64) for s in (50, 100, 200)] + [(0, 32, 100)]


def tune(out_path, steps=5, warmup=2, verbose=True, kernels=None):
    """Measure every candidate of every class on the current device; write and apply the table.
    kernels: the kernels whose classes are measured (default both); the entries and measurements
    of the others are kept from the table at out_path."""
    import torch
    from . import Isp
    dev = torch.cuda.get_device_name(0)
    isp = Isp()
    rows, entries = [], []
    if kernels is not None and os.path.exists(out_path):
        with open(out_path) as f:
            old = json.load(f)
        if old.get("device") == dev:
            entries = [e for e in old["entries"] if e["kernel"] not in kernels]
            names = {abi.KERNEL_LITE: "lite", abi.KERNEL_STREAM: "stream"}
            rows = [r for r in old.get("measurements", []) if r["kernel"] not in {names[k] for k in kernels}]
    for kernel, fmt, wc, frames in _classes():
        if kernels is not None and kernel not in kernels:
            continue
        d = [(pl, torch.from_numpy(raw).cuda(), torch.empty(pl.output_bytes(), dtype=torch.uint8, device="cuda"))
             for pl, raw in frames]
        px = sum(pl.width * pl.height for pl, _ in frames)
        timings = []
        for cand in _candidates(kernel):
            en, band, seg = cand
            set_table([{"kernel": kernel, "fmt": fmt, "max_width": wc, "enabled": en, "band_rows": band,
                        "seg_percent": seg}])
            for _ in range(warmup):
                isp.batch_submit(d, flags=abi.BATCH_GRAPH)
            isp.sync_status()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record()
            for _ in range(steps):
                isp.batch_submit(d, flags=abi.BATCH_GRAPH)
            e1.record()
            torch.cuda.synchronize()
            isp.sync_status()
            ms = e0.elapsed_time(e1) / steps
            timings.append({"enabled": en, "band_rows": band, "seg_percent": seg, "ms": round(ms, 4),
                            "gpix_s": round(px / (ms / 1e3) / 1e9, 2)})
        best = min(timings, key=lambda t: t["ms"])
        dflt = DEFAULTS[kernel]
        fixed = next(t for t in timings if (t["enabled"], t["band_rows"], t["seg_percent"]) == dflt)
        entries.append({"kernel": kernel, "fmt": fmt, "max_width": wc, "enabled": best["enabled"],
                        "band_rows": best["band_rows"], "seg_percent": best["seg_percent"]})
        rows.append({"kernel": "lite" if kernel == abi.KERNEL_LITE else "stream", "fmt": FMT_NAMES[fmt],
                     "max_width": wc, "frames": len(frames), "megapixels": round(px / 1e6, 2),
                     "best": best, "fixed": fixed, "speedup_vs_fixed": round(fixed["ms"] / best["ms"], 4),
                     "timings": timings})
        if verbose:
            print(f"{rows[-1]['kernel']:6s} {FMT_NAMES[fmt]:6s} w<={wc:<10d} fixed {fixed['ms']:.4f} ms  "
                  f"best {best['ms']:.4f} ms {best}", flush=True)
    isp.close()
    entries.sort(key=lambda e: (e["kernel"], e["fmt"], e["max_width"]))
    table = {"device": dev, "entries": entries, "measurements": rows,
             "method": f"CUDA events over {steps} replayed batch graphs after {warmup} warm-up, per candidate"}
    with open(out_path, "w") as f:
        json.dump(table, f, indent=1)
    set_table(entries)
    return table


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--out", default=DEFAULT_TABLE)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--kernels", choices=["lite", "stream"], nargs="*",
                    help="measure these kernels' classes only (the others' entries are kept)")
    args = ap.parse_args()
    ks = None if not args.kernels else [abi.KERNEL_LITE if k == "lite" else abi.KERNEL_STREAM for k in args.kernels]
    tune(args.out, steps=args.steps, kernels=ks)


if __name__ == "__main__":
    main()
