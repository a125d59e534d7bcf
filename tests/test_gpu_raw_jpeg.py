"""RAW host frames to JPEG host bytes (imop_isp_run_host_jpeg_batch): every frame's bytes equal the
oracle's encoder run on the oracle's pipeline output, across chunks (more than four frames, two
full-size 4024x3032 frames that fill a chunk alone), mixed formats and parameters (defect maps,
polynomial lens shading, both white-balance orders), the context's
parameters, pinned and pageable buffers, a truncating capacity; and the argument checks."""
import numpy as np
import pytest

import imop_gb300 as I
from imop_gb300 import abi
from imop_gb300 import jpeg as J
from imop_gb300 import workloads
import oracle_py as O

from helpers import random_frame, random_pipeline

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctxs():
    isp, enc = I.Isp(), J.JpegEncoder()
    yield isp, enc
    enc.close()
    isp.close()


def _want(pl, raw, q, ss, cap=0):
    rgb, _ = O.pipeline(pl, raw)
    st, want = O.jpeg_encode(rgb.reshape(pl.height, pl.width, 3), q, ss, cap)
    assert st == 0
    return want


def test_mixed_frames_across_chunks(ctxs):
    import torch
    isp, enc = ctxs
    rng = np.random.default_rng(77)
    frames, wants = [], []
    specs = [(640, 480, 12, True, abi.AMAZE), (333, 217, 10, False, abi.HQLI), (1006, 758, 8, False, abi.MG),
             (96, 64, 10, True, abi.AMAZE), (517, 389, 12, False, abi.HQLI), (128, 8, 14, True, abi.MG),
             (800, 600, 12, True, abi.AMAZE)]
    specs += [(720, 404, 12, False, abi.AMAZE), (301, 255, 10, True, abi.MG)]
    for k, (w, h, bd, packed, dm) in enumerate(specs):
        extra = {}
        if k == 7:  # a defect list (map-based correction)
            extra = dict(dpc_mode=abi.DPC_MAP_BASED, lsc_mode=abi.LSC_POLYNOMIAL)
        elif k == 8:
            extra = dict(lsc_mode=abi.LSC_POLYNOMIAL, order=abi.ORDER_RGB_WB)
        pl = random_pipeline(rng, w, h, bd, packed, dm, k % 4, **extra)
        raw = random_frame(rng, pl)
        q, ss = (90, 75, 50, 100, 20, 95, 85, 70, 99)[k], k % 3
        cap = J.max_bytes(w, h) if k != 4 else 900  # frame 4 truncated
        raw_h = torch.from_numpy(np.ascontiguousarray(raw)).pin_memory() if k % 2 else raw
        out = torch.zeros(cap, dtype=torch.uint8).pin_memory() if k % 3 == 0 else np.zeros(cap, np.uint8)
        frames.append((pl, raw_h, q, ss, out))
        wants.append(_want(pl, raw, q, ss, cap))
    sizes = J.raw_to_jpeg_host_batch(isp, enc, frames)
    for k, want in enumerate(wants):
        out = frames[k][4]
        got = (out.numpy() if hasattr(out, "numpy") else out)[: sizes[k]]
        assert sizes[k] == want.size and np.array_equal(got, want), k
    # the same call again: slots and lanes reused
    sizes2 = J.raw_to_jpeg_host_batch(isp, enc, frames)
    assert sizes2 == sizes


def test_full_size_frames_with_context_params(ctxs):
    """two 4024x3032 RAW12-packed frames (one per chunk) on the parameters set on the context"""
    isp, enc = ctxs
    pl = workloads.c2_pipeline(4024, 3032)
    raws = [workloads.c2_frame(pl, k) for k in range(2)]
    isp.set_params(pl)
    outs = [np.zeros(J.max_bytes(4024, 3032), np.uint8) for _ in raws]
    sizes = J.raw_to_jpeg_host_batch(isp, enc, [(None, raw, 90, 1, out) for raw, out in zip(raws, outs)])
    for raw, out, n in zip(raws, outs, sizes):
        want = _want(pl, raw, 90, 1)
        assert n == want.size and np.array_equal(out[:n], want)


def test_argument_checks(ctxs):
    isp, enc = ctxs
    rng = np.random.default_rng(5)
    pl = random_pipeline(rng, 64, 48, 10, False, abi.HQLI, 0)
    raw = random_frame(rng, pl)
    out = np.zeros(J.max_bytes(64, 48), np.uint8)
    native = random_pipeline(rng, 64, 48, 10, False, abi.HQLI, 0, out=abi.OUT_NATIVE)
    for frames, code in (([(native, raw, 90, 1, out)], abi.ERR_UNSUPPORTED),
                         ([(pl, raw, 0, 1, out)], abi.ERR_INVALID_ARGUMENT),
                         ([(pl, raw, 101, 1, out)], abi.ERR_INVALID_ARGUMENT)):
        with pytest.raises(I.IspError) as ei:
            J.raw_to_jpeg_host_batch(isp, enc, frames)
        assert ei.value.code == code
    assert J.raw_to_jpeg_host_batch(isp, enc, []) == []
