"""GPU parity: the fused kernel and the plain per-operator kernels against the CPU oracle.

Integer and floating-point stages alike are compared bit-exactly (max-abs 0): every FP stage of
the CUDA path evaluates the reference's expressions in the same order with round-to-nearest
intrinsics, so the gate of the task (<= 1 LSB max-abs for FP stages) is met with margin.
"""
import numpy as np
import pytest

import imop_gb300 as I
from imop_gb300 import abi, workloads
import oracle_py as O

from helpers import max_abs, psnr, random_frame, random_pipeline

pytestmark = pytest.mark.gpu

SIZES = [(6, 6), (7, 9), (9, 7), (33, 17), (64, 32), (67, 35), (68, 36), (131, 70), (200, 97)]
FORMATS = [(8, False), (10, False), (12, False), (10, True), (12, True), (16, False), (9, False)]
DEMOSAICS = [abi.HQLI, abi.AMAZE, abi.MG]


def _cases(n, seed):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        w, h = SIZES[i % len(SIZES)]
        bd, packed = FORMATS[(i // 2) % len(FORMATS)]
        dm = DEMOSAICS[i % 3]
        pat = int(rng.integers(0, 4))
        out.append((w, h, bd, packed, dm, pat, int(rng.integers(0, 2**31))))
    return out


@pytest.fixture(scope="module")
def isp():
    ctx = I.Isp()
    yield ctx
    ctx.close()


@pytest.mark.parametrize("w,h,bd,packed,dm,pat,seed", _cases(63, 1))
def test_fused_matches_oracle(isp, w, h, bd, packed, dm, pat, seed):
    rng = np.random.default_rng(seed)
    pl = random_pipeline(rng, w, h, bd, packed, dm, pat)
    raw = random_frame(rng, pl)
    ref, _ = O.pipeline(pl, raw)
    isp.set_params(pl)
    got = isp.run_host(raw)
    assert max_abs(got, ref) == 0, f"psnr {psnr(got, ref):.2f}"


@pytest.mark.parametrize("w,h", [(7, 9), (67, 35), (268, 80), (301, 77)])
@pytest.mark.parametrize("bd", [8, 9, 11, 13, 14, 16])
def test_bitstream_packed_matches_oracle(isp, w, h, bd):
    """Packed depths other than MIPI RAW10 / RAW12: one LSB-first bit stream per frame
    (pixel::get_packed_raw's generic case), odd widths included, full and border tiles."""
    rng = np.random.default_rng(1000 * bd + w)
    dm = DEMOSAICS[(w + bd) % 3]
    pl = random_pipeline(rng, w, h, bd, True, dm, int(rng.integers(0, 4)))
    raw = random_frame(rng, pl)
    assert raw.size == pl.input_bytes()
    ref, _ = O.pipeline(pl, raw)
    isp.set_params(pl)
    got = isp.run_host(raw)
    assert max_abs(got, ref) == 0, f"psnr {psnr(got, ref):.2f}"
    torch = pytest.importorskip("torch")
    d_out = torch.zeros(pl.output_bytes(), dtype=torch.uint8, device="cuda")
    isp.run_device_plain(torch.from_numpy(raw).cuda(), d_out)
    torch.cuda.synchronize()
    assert np.array_equal(d_out.cpu().numpy(), got.view(np.uint8).reshape(-1))


@pytest.mark.parametrize("w,h,bd,dm,size", [(67, 35, 10, abi.HQLI, 17), (268, 80, 12, abi.AMAZE, 33),
                                              (131, 70, 8, abi.MG, 5), (301, 77, 16, abi.AMAZE, 2)])
def test_lut3d_stage_matches_oracle(isp, w, h, bd, dm, size):
    """The optional 3D LUT after the CCM (lut::apply_lut): fused, plain and batched paths."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(7 * size + bd)
    pl = random_pipeline(rng, w, h, bd, False, dm, int(rng.integers(0, 4)))
    pl.stages |= abi.STAGE_LUT3D
    pl.lut3d = rng.uniform(-0.1, 1.1, (size, size, size, 3)).astype(np.float32)
    raw = random_frame(rng, pl)
    ref, _ = O.pipeline(pl, raw)
    isp.set_params(pl)
    got = isp.run_host(raw)
    assert max_abs(got, ref) == 0, f"psnr {psnr(got, ref):.2f}"
    d_in = torch.from_numpy(raw).cuda()
    d_out = torch.zeros(pl.output_bytes(), dtype=torch.uint8, device="cuda")
    isp.run_device_plain(d_in, d_out)
    torch.cuda.synchronize()
    assert np.array_equal(d_out.cpu().numpy(), got.view(np.uint8).reshape(-1))
    d_out.zero_()
    isp.batch_submit([(pl, d_in, d_out)])
    isp.sync_status()
    assert np.array_equal(d_out.cpu().numpy(), got.view(np.uint8).reshape(-1))


@pytest.mark.parametrize("w,h,bd,packed,dm,pat,seed", _cases(21, 2))
def test_stage_dumps_match_oracle(isp, w, h, bd, packed, dm, pat, seed):
    rng = np.random.default_rng(seed)
    pl = random_pipeline(rng, w, h, bd, packed, dm, pat)
    raw = random_frame(rng, pl)
    ref_out, ref = O.pipeline(pl, raw, dumps=True)
    isp.set_params(pl)
    got = isp.dump_stages(raw)
    for k in O.STAGES:
        if k == "white_balance" and not (pl.stages & abi.STAGE_WHITE_BALANCE):
            continue
        assert np.array_equal(got[k], ref[k]), f"stage {k}: max-abs {max_abs(got[k], ref[k])}"
    assert np.array_equal(got["output"], ref_out)


@pytest.mark.parametrize("mode", [abi.OUT_NATIVE, abi.OUT_RGB8])
@pytest.mark.parametrize("lsc", [abi.LSC_POLYNOMIAL, abi.LSC_GRID])
@pytest.mark.parametrize("dpc", [abi.DPC_ADAPTIVE, abi.DPC_MAP_BASED])
def test_modes(isp, mode, lsc, dpc):
    rng = np.random.default_rng(7 + mode + 3 * lsc + 11 * dpc)
    for bd, packed, dm in [(12, True, abi.AMAZE), (8, False, abi.AMAZE), (10, False, abi.MG), (8, False, abi.HQLI)]:
        pl = random_pipeline(rng, 77, 53, bd, packed, dm, int(rng.integers(0, 4)), dpc_mode=dpc, lsc_mode=lsc,
                             out=mode)
        raw = random_frame(rng, pl)
        ref, _ = O.pipeline(pl, raw)
        isp.set_params(pl)
        got = isp.run_host(raw)
        assert max_abs(got, ref) == 0


def test_flat_field_mode(isp):
    rng = np.random.default_rng(3)
    pl = random_pipeline(rng, 96, 64, 12, False, abi.AMAZE, abi.RGGB, lsc_mode=abi.LSC_FLAT_FIELD)
    pl.lsc_flat_field = I.scene(96, 64, 12, abi.RGGB, 99, lo=1500, hi=3800)
    raw = random_frame(rng, pl)
    ref, _ = O.pipeline(pl, raw)
    isp.set_params(pl)
    assert max_abs(isp.run_host(raw), ref) == 0


def test_defect_chains(isp):
    """Defect clusters and lines: pixels whose raster-earlier same-colour neighbours were
    corrected must see the corrected values (sequential semantics of the reference)."""
    rng = np.random.default_rng(11)
    w, h, bd = 150, 90, 12
    mv = 4095
    pl = random_pipeline(rng, w, h, bd, True, abi.AMAZE, abi.RGGB, order=abi.ORDER_BAYER_WB)
    pl.dpc_threshold = 0.1
    f = I.scene(w, h, bd, abi.RGGB, 5, lo=800, hi=2000)
    f[10:80:2, 40] = mv          # same-colour column line
    f[30, 20:140:2] = 0          # same-colour row line
    f[50:60:2, 100:110:2] = mv   # 5x5 block of hot same-colour pixels
    f[5, 5] = mv; f[7, 7] = mv; f[5, 7] = 0
    raw = I.pack_mipi(f, bd)
    ref, d = O.pipeline(pl, raw, dumps=True)
    isp.set_params(pl)
    got = isp.run_host(raw)
    seeds, overrides = isp.last_stats()
    assert seeds > 0 and overrides > 0
    assert max_abs(got, ref) == 0
    dumps = isp.dump_stages(raw)
    assert np.array_equal(dumps["defect"], d["defect"])


def test_c1_full_frame(isp):
    pl = workloads.c1_pipeline()
    raw = workloads.c1_frame(pl, 0)
    ref, _ = O.pipeline(pl, raw)
    isp.set_params(pl)
    assert max_abs(isp.run_host(raw), ref) == 0


def test_c2_full_frame(isp):
    pl = workloads.c2_pipeline()
    raw = workloads.c2_frame(pl, 0)
    ref, _ = O.pipeline(pl, raw)
    isp.set_params(pl)
    got = isp.run_host(raw)
    assert max_abs(got, ref) == 0


@pytest.mark.parametrize("k", [0, 1], ids=["c3_8bit", "c3_12bit_u16"])
def test_c3_full_frame(isp, k):
    """5320x4600 frames (8-bit and 12-bit unpacked) through the C1 pipeline."""
    pl = workloads.c3_pipelines()[k]
    raw = workloads.c3_frame(pl, k)
    ref, _ = O.pipeline(pl, raw)
    isp.set_params(pl)
    assert max_abs(isp.run_host(raw), ref) == 0


def test_plain_equals_fused_device(isp):
    torch = pytest.importorskip("torch")
    pl = workloads.c2_pipeline(1200, 900)
    raw = workloads.c2_frame(pl, 1)
    isp.set_params(pl)
    d_in = torch.from_numpy(raw).cuda()
    a = torch.empty(pl.output_bytes(), dtype=torch.uint8, device="cuda")
    b = torch.empty_like(a)
    isp.run_device(d_in, a)
    isp.run_device_plain(d_in, b)
    torch.cuda.synchronize()
    assert torch.equal(a, b)
    ref, _ = O.pipeline(pl, raw)
    assert np.array_equal(a.cpu().numpy().reshape(ref.shape), ref)


def test_real_capture_strips(isp):
    """Strips of the reference's real 1006x758 captures (RG8/10/12, RG10/12 packed) through the
    full fused pipeline, each demosaic, against the oracle."""
    import json
    import os
    z = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "real_strips.npz"))
    meta = json.loads(bytes(z["meta"]).decode())
    rng = np.random.default_rng(17)
    for tag, m in meta.items():
        for dm in DEMOSAICS:
            pl = random_pipeline(rng, m["w"], m["h"], m["bd"], bool(m["packed"]), dm, abi.RGGB)
            raw = z[tag]
            ref, _ = O.pipeline(pl, raw)
            isp.set_params(pl)
            assert max_abs(isp.run_host(raw), ref) == 0, f"{tag} demosaic {dm}"
