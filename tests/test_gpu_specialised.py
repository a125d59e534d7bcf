"""The fused kernel's instantiations per launch configuration against the oracle: every input
format the per-format kernels serve (u8, u16, RAW10 and RAW12 packed) x every demosaic algorithm x
{all stages, black level + white balance + CCM only (the copies without defect correction and
lens shading)} x both white-balance orders, on frames with full and border tiles; and one batch
mixing all of them, which the host groups by instantiation."""
import numpy as np
import pytest

import imop_gb300 as I
from imop_gb300 import abi
import oracle_py as O

from helpers import max_abs, random_frame, random_pipeline

pytestmark = pytest.mark.gpu

FORMATS = [(8, False), (12, False), (10, True), (12, True)]
DEMOSAICS = [abi.HQLI, abi.MG, abi.AMAZE]
LITE = abi.STAGE_BLACK_LEVEL | abi.STAGE_WHITE_BALANCE | abi.STAGE_CCM


def _case(k, bd, packed, dm, lite, order, w=300, h=130):
    rng = np.random.default_rng(900 + k)
    pl = random_pipeline(rng, w, h, bd, packed, dm, int(rng.integers(0, 4)), stages=LITE if lite else abi.STAGE_ALL,
                         order=order)
    return pl, random_frame(rng, pl)


CASES = [(bd, packed, dm, lite, order) for (bd, packed) in FORMATS for dm in DEMOSAICS for lite in (False, True)
         for order in (abi.ORDER_BAYER_WB, abi.ORDER_RGB_WB)]


@pytest.fixture(scope="module")
def isp():
    ctx = I.Isp()
    yield ctx
    ctx.close()


@pytest.mark.parametrize("k,case", list(enumerate(CASES)),
                         ids=[f"bd{c[0]}{'p' if c[1] else 'u'}_dm{c[2]}_{'lite' if c[3] else 'all'}_wb{c[4]}" for c in CASES])
def test_per_configuration_kernel_matches_oracle(isp, k, case):
    pl, raw = _case(k, *case)
    ref, _ = O.pipeline(pl, raw)
    isp.set_params(pl)
    assert max_abs(isp.run_host(raw), ref) == 0


def test_mixed_batch_grouped_by_instantiation(isp):
    import torch
    frames = []
    for k, case in enumerate(CASES[::3]):
        pl, raw = _case(100 + k, *case, w=260 + 8 * k, h=100 + 2 * k)
        frames.append((pl, raw))
    d_in = [torch.from_numpy(np.ascontiguousarray(raw)).cuda() for _, raw in frames]
    d_out = [torch.zeros(pl.output_bytes(), dtype=torch.uint8, device="cuda") for pl, _ in frames]
    isp.batch_submit([(pl, d_in[k].data_ptr(), d_out[k].data_ptr()) for k, (pl, _) in enumerate(frames)],
                     flags=abi.BATCH_GRAPH, stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    isp.sync_status(torch.cuda.current_stream().cuda_stream)
    for k, (pl, raw) in enumerate(frames):
        ref, _ = O.pipeline(pl, raw)
        got = d_out[k].cpu().numpy().reshape(ref.shape)
        assert max_abs(got, ref) == 0, k
