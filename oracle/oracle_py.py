"""ctypes binding of the CPU oracle.  TEST INFRASTRUCTURE ONLY.

Imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg, as the checker
and the timed CPU baseline; never by the product package.

  liboracle_isp.so        the C restatement (oracle/isp_oracle.c), built by `make -C oracle`
  _ref/libimop_ref.so     the reference's own CPU functions compiled from its sources
                          (`make -C oracle ref`); present only where the reference tree is
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(REPO, "im-operator_gb300"))

from imop_gb300 import abi  # noqa: E402  (struct layouts only)

_lib = None
_ref = None

U16P = C.POINTER(C.c_uint16)
U8P = C.POINTER(C.c_uint8)
F32P = C.POINTER(C.c_float)


def _p(a, t=C.c_void_p):
    return a.ctypes.data_as(t) if a is not None else None


class OracleDumps(C.Structure):
    _fields_ = [(n, U16P) for n in ("unpacked", "black_level", "defect", "lens_shading",
                                    "white_balance", "demosaic", "ccm")]


def lib():
    global _lib
    if _lib is None:
        path = os.path.join(HERE, "liboracle_isp.so")
        if not os.path.exists(path):
            raise RuntimeError("oracle not built: run `make -C oracle`")
        _lib = C.CDLL(path)
        _lib.or_pipeline.argtypes = [C.POINTER(abi.IspParams), C.c_void_p, C.c_void_p, C.POINTER(OracleDumps)]
        _lib.or_pipeline.restype = C.c_int
        _lib.or_get_packed_raw.argtypes = [U8P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
        _lib.or_get_packed_raw.restype = C.c_int
        _lib.or_tone_value.argtypes = [C.c_int, F32P, F32P, C.c_int, C.c_int]
        _lib.or_tone_value.restype = C.c_float
        _lib.or_tone_to_u8.argtypes = [C.c_float]
        _lib.or_tone_to_u8.restype = C.c_uint8
        _lib.or_lsc_flat_field_grid.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, F32P]
        _lib.or_lsc_flat_field_grid.restype = C.c_int
    return _lib


def ref_available():
    return os.path.exists(os.path.join(HERE, "_ref", "libimop_ref.so"))


def ref():
    global _ref
    if _ref is None:
        path = os.path.join(HERE, "_ref", "libimop_ref.so")
        if not os.path.exists(path):
            raise RuntimeError("reference library not built: run `make -C oracle ref`")
        _ref = C.CDLL(path)
        i = C.c_int
        _ref.ref_get_packed_raw.argtypes = [U8P, i, i, i, i, i]
        _ref.ref_get_raw.argtypes = [U8P, i, i, i, i, i, i]
        _ref.ref_black_level.argtypes = [U16P, i, i, i, i, i, F32P]
        _ref.ref_dpc.argtypes = [U16P, i, i, i, i, i, C.c_float, C.POINTER(C.c_int), i]
        _ref.ref_lsc_poly.argtypes = [U16P, i, i, i, i, F32P, C.c_float, C.c_float]
        _ref.ref_lsc_flat_field.argtypes = [U16P, i, i, i, i, U8P, i, i]
        _ref.ref_demosaic.argtypes = [U16P, U16P, i, i, i, i, i]
        _ref.ref_demosaic_raw.argtypes = [U8P, U16P, i, i, i, i, i, i]
        _ref.ref_wb_rgb.argtypes = [U16P, i, i, i, F32P]
        _ref.ref_ccm.argtypes = [U16P, i, i, i, F32P]
        _ref.ref_tone.argtypes = [U16P, U16P, i, i, i, i, F32P]
        IP = C.POINTER(C.c_int)
        _ref.ref_detect_bit_depth.argtypes = [U8P, C.c_size_t]
        _ref.ref_suggest_dimensions.argtypes = [C.c_size_t, IP, i]
        _ref.ref_analyze_data.argtypes = [U8P, C.c_size_t, IP, IP, i]
        _ref.ref_guess_pattern.argtypes = [U8P, i, i, i, i]
        _ref.ref_solve_ccm.argtypes = [F32P, F32P, i, i, F32P, IP, IP]
        _ref.ref_apply_lut.argtypes = [U16P, i, i, i, F32P, i]
        SP = C.POINTER(C.c_size_t)
        _ref.ref_jpeg_encode.argtypes = [U8P, i, i, i, i, i, U8P, SP]
        _ref.ref_jpeg_decode.argtypes = [U8P, C.c_size_t, U8P, IP, IP, IP]
    return _ref


def jpeg_max_bytes(w, h):
    """The reference's default output capacity (get_max_jpeg_size)."""
    return w * h * 9 + 65536


def _jpeg_call(fn, rgb, quality, subsample, cap, bd):
    rgb = np.ascontiguousarray(rgb, np.uint8)
    h, w = rgb.shape[:2]
    out = np.zeros(max(cap or jpeg_max_bytes(w, h), 1), np.uint8)
    n = C.c_size_t(cap)
    st = fn(rgb.ctypes.data_as(U8P), w, h, bd, quality, subsample, out.ctypes.data_as(U8P), C.byref(n))
    return st, out[: n.value].copy() if st == 0 else None


def ref_jpeg_encode(rgb, quality=90, subsample=1, cap=0, bd=8):
    """(status, bytes) of the reference's process_encode_baseline on an (h, w, 3) u8 frame."""
    return _jpeg_call(ref().ref_jpeg_encode, rgb, quality, subsample, cap, bd)


def ref_jpeg_decode(data):
    """(status, (h, w, 3) u8) of the reference's process_decode_baseline."""
    data = np.ascontiguousarray(data, np.uint8)
    w, h, c = C.c_int(0), C.c_int(0), C.c_int(0)
    # the decoder needs the frame size up front: read it from SOF0 (FF C0, len, prec, h, w)
    k = bytes(data).find(b"\xff\xc0")
    hh, ww = (int(data[k + 5]) << 8 | int(data[k + 6]), int(data[k + 7]) << 8 | int(data[k + 8])) if k >= 0 else (1, 1)
    out = np.zeros((hh, ww, 3), np.uint8)
    st = ref().ref_jpeg_decode(data.ctypes.data_as(U8P), data.size, out.ctypes.data_as(U8P), C.byref(w), C.byref(h),
                               C.byref(c))
    return st, out


def jpeg_encode(rgb, quality=90, subsample=1, cap=0, bd=8):
    """(status, bytes) of the oracle's restatement of process_encode_baseline."""
    L = lib()
    L.or_jpeg_encode.argtypes = [U8P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, U8P, C.POINTER(C.c_size_t)]
    return _jpeg_call(L.or_jpeg_encode, rgb, quality, subsample, cap, bd)


# ---- oracle ---------------------------------------------------------------------------------
STAGES = ("unpacked", "black_level", "defect", "lens_shading", "white_balance", "demosaic", "ccm")


def pipeline(pl, raw, dumps=False):
    """Run the oracle chain for a `Pipeline` on one input frame (bytes as np.uint8).
    Returns (output ndarray, dict of stage dumps or None)."""
    p = pl.to_c()
    raw = np.ascontiguousarray(raw, dtype=np.uint8)
    if raw.size < pl.input_bytes():
        raise ValueError("input smaller than one frame")
    out = np.zeros(pl.output_shape(), dtype=pl.output_dtype())
    d = None
    dd = None
    if dumps:
        n = pl.pixels
        wb_rgb = pl.stage_order == abi.ORDER_RGB_WB
        d = {
            "unpacked": np.zeros((pl.height, pl.width), np.uint16),
            "black_level": np.zeros((pl.height, pl.width), np.uint16),
            "defect": np.zeros((pl.height, pl.width), np.uint16),
            "lens_shading": np.zeros((pl.height, pl.width), np.uint16),
            "white_balance": np.zeros((pl.height, pl.width, 3) if wb_rgb else (pl.height, pl.width), np.uint16),
            "demosaic": np.zeros((pl.height, pl.width, 3), np.uint16),
            "ccm": np.zeros((pl.height, pl.width, 3), np.uint16),
        }
        del n
        dd = OracleDumps(*[d[k].ctypes.data_as(U16P) for k in STAGES])
    st = lib().or_pipeline(C.byref(p), raw.ctypes.data, out.ctypes.data, C.byref(dd) if dd else None)
    if st != 0:
        raise RuntimeError(f"oracle pipeline failed with status {st}")
    return out, d


def get_packed_raw(buf, x, y, w, h, bd):
    buf = np.ascontiguousarray(buf, dtype=np.uint8)
    return lib().or_get_packed_raw(_p(buf, U8P), x, y, w, h, bd)


def flat_field_grid(ff, pattern, bd):
    ff = np.ascontiguousarray(ff)
    g = np.zeros((24, 32, 4), np.float32)
    st = lib().or_lsc_flat_field_grid(ff.ctypes.data, ff.shape[1], ff.shape[0], pattern, bd, _p(g, F32P))
    if st:
        raise RuntimeError(f"flat field grid failed: {st}")
    return g


# ---- per-stage bindings (the tests pin each restated stage) ------------------------------------
def stages():
    """ctypes handles of the oracle's per-stage functions."""
    L = lib()
    i = C.c_int
    L.or_black_level.argtypes = [U16P, i, i, i, i, i, F32P]
    L.or_dpc_adaptive.argtypes = [U16P, i, i, i, i, C.c_float]
    L.or_dpc_map.argtypes = [U16P, i, i, i, i, C.c_void_p, i]
    L.or_lsc_poly.argtypes = [U16P, i, i, i, i, F32P, C.c_float, C.c_float]
    L.or_lsc_grid.argtypes = [U16P, i, i, i, i, F32P, i, i]
    L.or_wb_bayer.argtypes = [U16P, i, i, i, i, F32P]
    for f in (L.or_demosaic_hqli, L.or_demosaic_amaze, L.or_demosaic_mg):
        f.argtypes = [U16P, U16P, i, i, i, i]
    L.or_wb_rgb.argtypes = [U16P, i, i, i, F32P]
    L.or_ccm.argtypes = [U16P, i, i, i, F32P]
    L.or_lut3d.argtypes = [U16P, i, i, i, F32P, i]
    L.or_unpack.argtypes = [U8P, i, i, i, i, U16P]
    return L


def demosaic(bay, pattern, algo, bd):
    L = stages()
    h, w = bay.shape
    bay = np.ascontiguousarray(bay, np.uint16)
    out = np.zeros((h, w, 3), np.uint16)
    fn = {1: L.or_demosaic_hqli, 6: L.or_demosaic_amaze, 2: L.or_demosaic_mg}[algo]
    fn(bay.ctypes.data_as(U16P), out.ctypes.data_as(U16P), w, h, pattern, bd)
    return out


# ---- FP64 differentiable calibration chain ------------------------------------------------------
def _adj_lib():
    L = lib()
    D = C.POINTER(abi.AdjointDesc)
    DP = C.POINTER(C.c_double)
    L.or_adj_param_count.argtypes = [D]
    L.or_adj_param_count.restype = C.c_int
    L.or_adj_forward.argtypes = [D, DP, U8P, DP]
    L.or_adj_loss_grad.argtypes = [D, DP, U8P, F32P, C.c_int, DP, DP]
    L.or_adj_loss.argtypes = [D, DP, U8P, F32P, C.c_int, DP]
    return L


def adj_forward(desc, theta, raw):
    """t of every pixel (n_frames, h, w, 3) in FP64."""
    L = _adj_lib()
    th = np.ascontiguousarray(theta, np.float64)
    raw = np.ascontiguousarray(raw, np.uint8)
    out = np.zeros((desc.n_frames, desc.height, desc.width, 3), np.float64)
    st = L.or_adj_forward(C.byref(desc), th.ctypes.data_as(C.POINTER(C.c_double)), _p(raw, U8P),
                          out.ctypes.data_as(C.POINTER(C.c_double)))
    if st:
        raise RuntimeError(f"or_adj_forward: {st}")
    return out


def adj_loss_grad(desc, theta, raw, ref, mode=0):
    """(loss, dL/dtheta) in FP64 against a target (mode 0) or an upstream gradient (mode 1)."""
    L = _adj_lib()
    th = np.ascontiguousarray(theta, np.float64)
    raw = np.ascontiguousarray(raw, np.uint8)
    ref = np.ascontiguousarray(ref, np.float32)
    g = np.zeros(L.or_adj_param_count(C.byref(desc)), np.float64)
    loss = C.c_double()
    st = L.or_adj_loss_grad(C.byref(desc), th.ctypes.data_as(C.POINTER(C.c_double)), _p(raw, U8P), _p(ref, F32P),
                            mode, C.byref(loss), g.ctypes.data_as(C.POINTER(C.c_double)))
    if st:
        raise RuntimeError(f"or_adj_loss_grad: {st}")
    return loss.value, g


def adj_loss(desc, theta, raw, ref, mode=0):
    L = _adj_lib()
    th = np.ascontiguousarray(theta, np.float64)
    raw = np.ascontiguousarray(raw, np.uint8)
    ref = np.ascontiguousarray(ref, np.float32)
    loss = C.c_double()
    st = L.or_adj_loss(C.byref(desc), th.ctypes.data_as(C.POINTER(C.c_double)), _p(raw, U8P), _p(ref, F32P), mode,
                       C.byref(loss))
    if st:
        raise RuntimeError(f"or_adj_loss: {st}")
    return loss.value
