"""GPU adjoint of the differentiable calibration chain against the FP64 oracle: forward values,
the analytic gradient (all parameters), central finite differences at the 16-frame 1006x758
calibration size, the torch.autograd wrappers, and a 200-step Adam calibration."""
import numpy as np
import pytest

import imop_gb300 as I
from imop_gb300 import abi, workloads
import oracle_py as O

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
from imop_gb300 import adjoint as A  # noqa: E402

TOL = 1e-4


def _rel(g, ref):
    scale = max(1e-2 * float(np.max(np.abs(ref))), 1e-12)
    return np.abs(g - ref) / np.maximum(np.abs(ref), scale)


@pytest.fixture(scope="module")
def isp():
    ctx = I.Isp()
    yield ctx
    ctx.close()


CASES = [  # w, h, frames, demosaic, pattern, grid, packed, bd
    (44, 34, 2, abi.AMAZE, abi.RGGB, (5, 4), 0, 12),
    (67, 39, 1, abi.HQLI, abi.BGGR, (3, 3), 0, 12),
    (131, 70, 2, abi.AMAZE, abi.GRBG, (17, 13), 1, 12),
    (70, 19, 1, abi.AMAZE, abi.GBRG, (4, 2), 1, 10),
    (66, 68, 1, abi.HQLI, abi.RGGB, (6, 5), 0, 10),
]


def _setup(case, seed):
    w, h, n, dm, pat, grid, packed, bd = case
    d = abi.AdjointDesc(w, h, bd, packed, pat, dm, grid[0], grid[1], n)
    rng = np.random.default_rng(seed)
    mv = (1 << bd) - 1
    frames = []
    for k in range(n):
        f = I.scene(w, h, bd, pat, 1000 + seed + k, lo=mv * 0.06, hi=mv * 0.34)
        frames.append(I.pack_mipi(f, bd) if packed else f.view(np.uint8).reshape(-1))
    raw = np.concatenate(frames)
    d12 = workloads.c5_desc(1, w, h, dm, grid)
    th_true = workloads.c5_theta_true(d12).astype(np.float64)
    th_true[0:4] *= mv / 4095.0
    th = workloads.c5_theta_init(th_true.astype(np.float32), seed + 1).astype(np.float64)
    target = O.adj_forward(d, th_true, raw).astype(np.float32)
    return d, raw, th, target, rng


@pytest.mark.parametrize("case", CASES)
def test_render_matches_fp64(isp, case):
    d, raw, th, _, _ = _setup(case, 1)
    ref = O.adj_forward(d, th, raw)
    t = A.render_forward(isp, d, torch.tensor(th, dtype=torch.float32, device="cuda"),
                         torch.from_numpy(raw).cuda())
    torch.cuda.synchronize()
    assert np.max(np.abs(t.cpu().numpy() - ref)) < 2e-4


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("mode", [abi.ADJ_TARGET, abi.ADJ_UPSTREAM])
def test_gradient_matches_fp64(isp, case, mode):
    d, raw, th, target, rng = _setup(case, 2)
    # an upstream gradient of one sign keeps the FP32 sums well conditioned
    ref = target if mode == abi.ADJ_TARGET else rng.uniform(0.2, 1.0, size=target.shape).astype(np.float32)
    loss64, g64 = O.adj_loss_grad(d, th, raw, ref, mode)
    loss, g = A.backward(isp, d, torch.tensor(th, dtype=torch.float32, device="cuda"),
                         torch.from_numpy(raw).cuda(), torch.from_numpy(ref).cuda(), mode)
    torch.cuda.synchronize()
    g = g.cpu().numpy().astype(np.float64)
    assert abs(float(loss) - loss64) <= 1e-4 * max(abs(loss64), 1e-3)
    rel = _rel(g, g64)
    assert np.max(rel) <= TOL, f"parameter {int(np.argmax(rel))}: {g[np.argmax(rel)]} vs {g64[np.argmax(rel)]}"


@pytest.fixture(scope="module")
def c5():
    d = workloads.c5_desc()
    th_true = workloads.c5_theta_true(d)
    th0 = workloads.c5_theta_init(th_true)
    raw = workloads.c5_frames(d)
    target = O.adj_forward(d, th_true.astype(np.float64), raw).astype(np.float32)
    return d, th_true, th0, raw, target


def test_c5_gradient_all_parameters_vs_fp64(isp, c5):
    d, _, th0, raw, target = c5
    loss64, g64 = O.adj_loss_grad(d, th0.astype(np.float64), raw, target, abi.ADJ_TARGET)
    loss, g = A.backward(isp, d, torch.from_numpy(th0).cuda(), torch.from_numpy(raw).cuda(),
                         torch.from_numpy(target).cuda(), abi.ADJ_TARGET)
    g = g.cpu().numpy().astype(np.float64)
    assert g.size == 933
    assert abs(float(loss) - loss64) <= 1e-4 * loss64
    assert np.max(_rel(g, g64)) <= TOL


def test_c5_gradient_vs_finite_differences(isp, c5):
    """Central differences (h = 1e-6) of the FP64 loss for BL, WB, CCM and a spread of grid
    nodes and knots, against the FP32 adjoint."""
    d, _, th0, raw, target = c5
    _, g = A.backward(isp, d, torch.from_numpy(th0).cuda(), torch.from_numpy(raw).cuda(),
                      torch.from_numpy(target).cuda(), abi.ADJ_TARGET)
    g = g.cpu().numpy().astype(np.float64)
    th = th0.astype(np.float64)
    idx = list(range(16)) + [16 + k for k in (0, 37, 250, 441, 700, 883)] + [900 + k for k in (0, 5, 11, 20, 27, 32)]
    h = 1e-6
    fd = []
    for k in idx:
        tp, tm = th.copy(), th.copy()
        tp[k] += h
        tm[k] -= h
        fd.append((O.adj_loss(d, tp, raw, target) - O.adj_loss(d, tm, raw, target)) / (2 * h))
    fd = np.array(fd)
    scale = max(1e-2 * float(np.max(np.abs(fd))), 1e-12)
    rel = np.abs(g[idx] - fd) / np.maximum(np.abs(fd), scale)
    assert np.max(rel) <= TOL, f"parameter {idx[int(np.argmax(rel))]}: {g[idx][np.argmax(rel)]} vs {fd[np.argmax(rel)]}"


def test_repeated_launches_of_different_sizes(isp, c5):
    """Tiles past the first wave of a launch are claimed from a counter that the launch's last CTA
    clears: C5 launches (more tiles than CTAs) alternating with a 16-tile launch give the
    gradients of their first runs every time (to the rounding of the shared-memory sums)."""
    d, _, th0, raw, target = c5
    ds, raws, ths, tgts, _ = _setup(CASES[2], 5)
    big = (d, torch.from_numpy(th0).cuda(), torch.from_numpy(raw).cuda(), torch.from_numpy(target).cuda())
    small = (ds, torch.tensor(ths, dtype=torch.float32, device="cuda"), torch.from_numpy(raws).cuda(),
             torch.from_numpy(tgts).cuda())

    def grads():
        return [A.backward(isp, *a, abi.ADJ_TARGET)[1].cpu().numpy() for a in (big, small)]

    first = grads()
    for _ in range(3):
        for g, f in zip(grads(), first):
            assert np.allclose(g, f, rtol=1e-5, atol=1e-6 * float(np.abs(f).max()))


def test_autograd_wrappers(isp):
    d, raw, th, target, rng = _setup(CASES[2], 4)
    theta = torch.tensor(th, dtype=torch.float32, device="cuda", requires_grad=True)
    raw_t = torch.from_numpy(raw).cuda()
    tgt = torch.from_numpy(target).cuda()
    t = A.render(isp, d, theta, raw_t)
    ((t - tgt) ** 2).sum().backward()
    g_render = theta.grad.clone()
    theta.grad = None
    A.l2_loss(isp, d, theta, raw_t, tgt).backward()
    g_l2 = theta.grad.clone()
    _, g64 = O.adj_loss_grad(d, th, raw, target, abi.ADJ_TARGET)
    assert np.max(_rel(g_render.cpu().numpy().astype(np.float64), g64)) <= TOL
    assert np.max(_rel(g_l2.cpu().numpy().astype(np.float64), g64)) <= TOL


def test_adam_calibration_c5(isp, c5):
    """200 Adam steps from the perturbed start: the loss falls by orders of magnitude."""
    d, th_true, th0, raw, target = c5
    theta = torch.from_numpy(th0.copy()).cuda().requires_grad_(True)
    raw_t = torch.from_numpy(raw).cuda()
    tgt = torch.from_numpy(target).cuda()
    scale = torch.from_numpy(np.abs(th_true) + 1e-3).cuda()
    phi = (theta.detach() / scale).clone().requires_grad_(True)
    opt = torch.optim.Adam([phi], lr=3e-3)
    losses = []
    for _ in range(200):
        opt.zero_grad()
        loss = A.l2_loss(isp, d, (phi * scale).contiguous(), raw_t, tgt)
        loss.backward()
        opt.step()
        losses.append(float(loss.detach()))
    assert losses[-1] < 1e-2 * losses[0], f"loss {losses[0]:.4g} -> {losses[-1]:.4g}"
    # parameter recovery, on the quantities the chain identifies: the black levels, the effective
    # lens gain per node and CFA colour (grid gain x white-balance gain: the chain multiplies them,
    # so only the product is determined), the CCM and the tone knots.  Start: BL 19 %, effective
    # gain 17 % RMS, CCM 0.29, knots 0.091 RMS.
    th = (phi * scale).detach().cpu().numpy().astype(np.float64)
    tt = th_true.astype(np.float64)
    ng = d.grid_w * d.grid_h * 4
    bl_err = np.max(np.abs(th[0:4] - tt[0:4]) / tt[0:4])
    wb4 = lambda w: np.array([w[0], w[1], w[1], w[2]])
    eff = th[16:16 + ng].reshape(-1, 4) * wb4(th[4:7])
    eff_true = tt[16:16 + ng].reshape(-1, 4) * wb4(tt[4:7])
    eff_rms = float(np.sqrt(np.mean(((eff - eff_true) / eff_true) ** 2)))
    ccm_err = float(np.max(np.abs(th[7:16] - tt[7:16])))
    knot_rms = float(np.sqrt(np.mean((th[16 + ng:] - tt[16 + ng:]) ** 2)))
    assert bl_err <= 0.10, bl_err
    assert eff_rms <= 0.07, eff_rms
    assert ccm_err <= 0.15, ccm_err
    assert knot_rms <= 0.01, knot_rms
