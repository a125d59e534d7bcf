"""Colour-correction matrix: the reference's patch least-squares solve, and its refinement on raw
frames through the adjoint of the differentiable chain.

    solve_ccm(measured, reference, matrix_type)   -> {"type", "m", "rows", "cols"}  (host, FP64)
    fit_ccm(isp, desc, raw, target, theta, ...)   -> (theta, ccm 3x3, losses)        (GPU adjoint)

solve_ccm gives what color_calibration::process_solve_ccm gives for the same patches (a 3x3, 3x4
with bias, or 3x9 polynomial matrix).  fit_ccm starts from theta (optionally with its CCM seeded
by a 3x3 patch solve) and minimises sum((render(theta) - target)^2) over the raw frames with Adam,
moving only the CCM entries of theta or every parameter; the 3x3 it returns is in the layout of
SolvedMatrix (type LINEAR_3X3, row-major).
"""
import ctypes as C

import numpy as np

from . import abi, check, lib

LINEAR_3X3, LINEAR_4X3, POLY_3X9 = 0, 1, 2
CCM_SLICE = slice(7, 16)  # theta layout: bl[4], wb[3], ccm[9], grid, knots


class PatchColor(C.Structure):
    _fields_ = [("r", C.c_float), ("g", C.c_float), ("b", C.c_float)]


class SolvedMatrix(C.Structure):
    _fields_ = [("type", C.c_int), ("m", C.c_float * 27), ("rows", C.c_int), ("cols", C.c_int)]


def _patches(a):
    a = np.ascontiguousarray(a, np.float32).reshape(-1, 3)
    arr = (PatchColor * len(a))()
    C.memmove(arr, a.ctypes.data, a.nbytes)
    return arr, len(a)


def solve_ccm(measured, reference, matrix_type=LINEAR_3X3):
    """Least-squares CCM of N >= 3 patch pairs ((N, 3) arrays of linear RGB)."""
    L = lib()
    L.imop_solve_ccm.argtypes = [C.POINTER(PatchColor), C.POINTER(PatchColor), C.c_int, C.c_int,
                                 C.POINTER(SolvedMatrix)]
    L.imop_solve_ccm.restype = C.c_int
    m_arr, n = _patches(measured)
    r_arr, n2 = _patches(reference)
    if n != n2:
        raise ValueError("measured and reference hold different patch counts")
    out = SolvedMatrix()
    check(L.imop_solve_ccm(m_arr, r_arr, n, matrix_type, C.byref(out)))
    m = np.array(out.m[: out.rows * out.cols], np.float32).reshape(out.rows, out.cols)
    return {"type": out.type, "m": m, "rows": out.rows, "cols": out.cols}


def fit_ccm(isp, desc, raw, target, theta, steps=150, lr=0.01, free="ccm", patches=None):
    """Adam on sum((render(theta) - target)^2) through the fused adjoint.

    free: "ccm" moves only the 9 CCM entries, "all" every parameter.  patches: optional
    (measured, reference) linear-RGB patch pairs whose 3x3 solve seeds the CCM first.  Returns the
    final theta, its CCM as a 3x3 array and the loss of every step."""
    import torch

    from . import adjoint as A

    th = theta.detach().clone().contiguous()
    if patches is not None:
        seed = solve_ccm(patches[0], patches[1], LINEAR_3X3)["m"]
        th[CCM_SLICE] = torch.from_numpy(seed.reshape(-1)).to(th.device)
    mask = torch.zeros_like(th)
    if free == "ccm":
        mask[CCM_SLICE] = 1.0
    elif free == "all":
        mask[:] = 1.0
    else:
        raise ValueError("free must be 'ccm' or 'all'")
    # per-parameter step scale: relative to the magnitude of each parameter
    scale = th.abs() + 1e-3
    m1 = torch.zeros_like(th)
    m2 = torch.zeros_like(th)
    b1, b2, eps = 0.9, 0.999, 1e-12
    losses = []
    for k in range(1, steps + 1):
        loss, g = A.backward(isp, desc, th, raw, target, abi.ADJ_TARGET)
        losses.append(float(loss))
        g = g * mask * scale
        m1.mul_(b1).add_(g, alpha=1 - b1)
        m2.mul_(b2).addcmul_(g, g, value=1 - b2)
        step = (m1 / (1 - b1 ** k)) / ((m2 / (1 - b2 ** k)).sqrt() + eps)
        th.sub_(lr * scale * step)
    return th, th[CCM_SLICE].reshape(3, 3).cpu().numpy(), losses
