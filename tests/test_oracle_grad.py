"""The FP64 differentiable chain of the oracle: its analytic gradient against central finite
differences (h = 1e-6) for every parameter, HQLI and AMAZE, target and upstream-gradient modes.
CPU only; the adjoint kernel is checked against this gradient in the GPU tests."""
import numpy as np
import pytest

import imop_gb300 as I
from imop_gb300 import abi, workloads
import oracle_py as O

H = 1e-6
TOL = 1e-4


def _case(demosaic, seed, w=44, h=34, grid=(5, 4), frames=2):
    d = workloads.c5_desc(frames, w, h, demosaic, grid)
    th_true = workloads.c5_theta_true(d).astype(np.float64)
    th = workloads.c5_theta_init(th_true.astype(np.float32), seed).astype(np.float64)
    raw = workloads.c5_frames(d, seed)
    return d, th_true, th, raw


def _fd_check(d, th, raw, ref, mode):
    loss, g = O.adj_loss_grad(d, th, raw, ref, mode)
    fd = np.zeros_like(g)
    for k in range(th.size):
        tp, tm = th.copy(), th.copy()
        tp[k] += H
        tm[k] -= H
        fd[k] = (O.adj_loss(d, tp, raw, ref, mode) - O.adj_loss(d, tm, raw, ref, mode)) / (2 * H)
    scale = max(1e-2 * np.max(np.abs(fd)), 1e-12)
    rel = np.abs(g - fd) / np.maximum(np.abs(fd), scale)
    return loss, g, fd, rel


@pytest.mark.parametrize("demosaic", [abi.HQLI, abi.AMAZE])
def test_oracle_gradient_matches_finite_differences(demosaic):
    d, th_true, th, raw = _case(demosaic, 3)
    target = O.adj_forward(d, th_true, raw).astype(np.float32)
    loss, g, fd, rel = _fd_check(d, th, raw, target, abi.ADJ_TARGET)
    assert loss > 0
    assert np.max(rel) <= TOL, f"worst parameter {int(np.argmax(rel))}: {g[np.argmax(rel)]} vs {fd[np.argmax(rel)]}"
    assert np.count_nonzero(g) > 0.9 * g.size


def test_oracle_gradient_upstream_mode():
    d, th_true, th, raw = _case(abi.AMAZE, 5, w=38, h=30, grid=(3, 3))
    rng = np.random.default_rng(1)
    up = rng.normal(size=(d.n_frames, d.height, d.width, 3)).astype(np.float32)
    loss, g, fd, rel = _fd_check(d, th, raw, up, abi.ADJ_UPSTREAM)
    t = O.adj_forward(d, th, raw)
    assert abs(loss - float(np.sum(t * up))) <= 1e-9 * max(1.0, abs(loss))
    assert np.max(rel) <= TOL


def test_forward_matches_rgb8_path_before_rounding():
    """At parameters the product path can express (integral BL, tone knots), the differentiable
    forward stays within the rounding the product path adds between stages."""
    d, th_true, _, raw = _case(abi.AMAZE, 9, w=64, h=48, grid=(5, 4), frames=1)
    t = O.adj_forward(d, th_true, raw)[0]
    pl = I.Pipeline(width=d.width, height=d.height, bit_depth=12, packed=False, pattern=d.pattern,
                    demosaic=d.demosaic, stages=abi.STAGE_BLACK_LEVEL | abi.STAGE_LENS_SHADING |
                    abi.STAGE_WHITE_BALANCE | abi.STAGE_CCM, stage_order=abi.ORDER_BAYER_WB,
                    bl_offset=tuple(float(v) for v in th_true[0:4]), lsc_mode=abi.LSC_GRID,
                    lsc_grid=th_true[16:16 + 80].reshape(4, 5, 4).astype(np.float32),
                    wb_gain=tuple(float(v) for v in th_true[4:7]), ccm=tuple(float(v) for v in th_true[7:16]),
                    tone_mode=abi.TONE_KNOTS, tone_knots=tuple(float(v) for v in th_true[96:129]))
    out, _ = O.pipeline(pl, raw)
    q = np.clip(np.floor(t * 255 + 0.5), 0, 255)
    # stage-wise rounding moves a value by a few DN at 12 bit; through the gamma curve and the
    # 8-bit quantiser that is at most a few codes
    assert np.mean(np.abs(q - out)) < 0.6
    assert np.max(np.abs(q - out)) <= 6
