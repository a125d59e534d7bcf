"""CCM from patch measurements (host, against the reference's process_solve_ccm where oracle/_ref
was built) and its refinement on raw frames through the adjoint (GPU)."""
import ctypes as C

import numpy as np
import pytest

import imop_gb300 as I
from imop_gb300 import abi, calibration as K, workloads
import oracle_py as O

ref = pytest.mark.skipif(not O.ref_available(), reason="reference library not built here")


def _patches(rng, n, noise=0.01):
    meas = rng.uniform(0.02, 0.95, (n, 3)).astype(np.float32)
    M = np.array([[1.6, -0.4, -0.2], [-0.3, 1.5, -0.2], [-0.1, -0.5, 1.6]], np.float32)
    refc = (meas @ M.T + rng.normal(0, noise, (n, 3))).astype(np.float32)
    return meas, refc, M


def test_exact_patches_give_the_matrix():
    rng = np.random.default_rng(1)
    meas, refc, M = _patches(rng, 24, noise=0.0)
    out = K.solve_ccm(meas, refc, K.LINEAR_3X3)
    assert out["rows"] == 3 and out["cols"] == 3
    assert np.allclose(out["m"], M, atol=1e-4)
    with pytest.raises(I.IspError) as e:
        K.solve_ccm(meas[:2], refc[:2])
    assert e.value.code == 106
    # all-zero measurements: the 1e-9 ridge keeps the system solvable (all-zero colour terms)
    z = K.solve_ccm(np.zeros((5, 3)), refc[:5], K.LINEAR_4X3)
    assert np.all(z["m"][:, :3] == 0)


@ref
@pytest.mark.parametrize("mtype", [K.LINEAR_3X3, K.LINEAR_4X3, K.POLY_3X9])
@pytest.mark.parametrize("n", [3, 10, 24, 60])
def test_solve_matches_reference(mtype, n):
    R = O.ref()
    rng = np.random.default_rng(100 * n + mtype)
    meas, refc, _ = _patches(rng, n)
    m = (C.c_float * 27)()
    rows, cols = C.c_int(), C.c_int()
    e = R.ref_solve_ccm(meas.ctypes.data_as(O.F32P), refc.ctypes.data_as(O.F32P), n, mtype, m,
                        C.byref(rows), C.byref(cols))
    if e != 0:
        with pytest.raises(I.IspError):
            K.solve_ccm(meas, refc, mtype)
        return
    out = K.solve_ccm(meas, refc, mtype)
    assert (out["rows"], out["cols"]) == (rows.value, cols.value)
    want = np.array(m[: rows.value * cols.value], np.float32).reshape(rows.value, cols.value)
    assert np.array_equal(out["m"], want)


@pytest.mark.gpu
def test_fit_ccm_on_raw_frames():
    """The CCM refit through the adjoint: from a 20 % perturbed matrix, and from a patch seed."""
    torch = pytest.importorskip("torch")
    from imop_gb300 import adjoint as A
    isp = I.Isp()
    d = workloads.c5_desc(2, 256, 192)
    th_true = workloads.c5_theta_true(d)
    raw = torch.from_numpy(workloads.c5_frames(d)).cuda()
    target = A.render_forward(isp, d, torch.from_numpy(th_true).cuda(), raw)
    th0 = th_true.copy()
    rng = np.random.default_rng(5)
    th0[K.CCM_SLICE] *= (1 + rng.uniform(-0.2, 0.2, 9)).astype(np.float32)
    th, ccm, losses = K.fit_ccm(isp, d, raw, target, torch.from_numpy(th0).cuda(), steps=200, lr=0.02)
    assert losses[-1] < 1e-3 * losses[0], f"loss {losses[0]:.4g} -> {losses[-1]:.4g}"
    true = th_true[K.CCM_SLICE].reshape(3, 3)
    assert np.max(np.abs(ccm - true)) < 2e-2 * np.max(np.abs(true))
    # other parameters untouched when only the CCM is free
    assert torch.equal(th[:7].cpu(), torch.from_numpy(th0[:7]))
    # a 3x3 patch solve of linear patches made with the true matrix seeds it at once
    meas = rng.uniform(0.05, 0.9, (24, 3)).astype(np.float32)
    patches = (meas, (meas @ true.T).astype(np.float32))
    assert np.max(np.abs(K.solve_ccm(*patches)["m"] - true)) < 1e-4
    _, _, losses2 = K.fit_ccm(isp, d, raw, target, torch.from_numpy(th0).cuda(), steps=1, patches=patches)
    assert losses2[0] < 1e-3 * losses[0]
    isp.close()
