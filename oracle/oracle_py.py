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


# ---- seeded synthetic frames, without the product library (timed CPU baseline) ------------------
def _scene_lib():
    L = lib()
    L.or_scene_render.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_uint64, C.c_float, C.c_float, C.c_float,
                                  C.c_float, C.c_void_p]
    L.or_scene_defects.argtypes = [C.c_int, C.c_int, C.c_uint64, C.c_int, C.c_void_p]
    L.or_scene_apply_defects.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int]
    L.or_pack_mipi.argtypes = [C.c_void_p, C.c_size_t, C.c_int, C.c_void_p]
    return L


def scene(width, height, bit_depth, pattern=0, seed=20261203, lo=None, hi=None, gain=0.5, read_sigma=2.0):
    """The workloads' seeded Bayer frame (uint8 for bd <= 8, uint16 otherwise), equal to the
    product's imop_scene_render byte for byte."""
    mv = (1 << bit_depth) - 1
    lo = float(lo if lo is not None else 0.0625 * (mv + 1))
    hi = float(hi if hi is not None else mv)
    out = np.empty((height, width), np.uint8 if bit_depth <= 8 else np.uint16)
    if _scene_lib().or_scene_render(width, height, bit_depth, pattern, seed, lo, hi, gain, read_sigma,
                                    out.ctypes.data) != 0:
        raise ValueError("bad scene arguments")
    return out


def defects(width, height, count, seed=20261203):
    xy = np.zeros((max(1, count), 2), np.int32)
    if _scene_lib().or_scene_defects(width, height, seed, count, xy.ctypes.data) != 0:
        raise ValueError("bad defect arguments")
    return xy[:count]


def apply_defects(frame, pts, bit_depth):
    pts = np.ascontiguousarray(pts, np.int32).reshape(-1, 2)
    assert frame.dtype == np.uint16 and frame.flags.c_contiguous
    _scene_lib().or_scene_apply_defects(frame.ctypes.data, frame.shape[1], bit_depth, pts.ctypes.data, pts.shape[0])
    return frame


def pack_mipi(frame, bit_depth):
    """MIPI RAW10 / RAW12 bytes of an unpacked frame"""
    assert bit_depth in (10, 12)
    f = np.ascontiguousarray(frame, np.uint16)
    out = np.empty((f.size * bit_depth + 7) // 8, np.uint8)
    _scene_lib().or_pack_mipi(f.ctypes.data, f.size, bit_depth, out.ctypes.data)
    return out


# ---- the reference's own CPU chain for the C2 configuration (timed reference arm) ---------------
def _ref_chain_lib():
    R = ref()
    i, vp = C.c_int, C.c_void_p
    R.ref_unpack_packed.argtypes = [vp, C.c_size_t, vp, i, i, i]
    R.ref_black_level_store.argtypes = [vp, i, i, i, i, F32P]
    R.ref_dpc_adaptive_store.argtypes = [vp, i, i, i, i, C.c_float]
    R.ref_demosaic_store.argtypes = [vp, vp, i, i, i, i, i]
    R.ref_ccm_store.argtypes = [vp, vp, i, i, i, F32P]
    return R


def ref_chain(pl, raw):
    """RGB8 of one frame through the reference's per-module calls in the order they compose
    (packed unpack by pixel::get_packed_raw, black_level::process_black_level, the adaptive
    defect_correct::process_defect_correct, imop::demosaic_cpu, ccm::process_ccm), with the
    oracle's restatements for the three stages the reference has no function for (explicit-grid
    lens shading, Bayer-domain white balance, the 1-D LUT to RGB8).  Serves the C2 configuration:
    a packed 12-bit (or 10-bit) frame, per-channel black level, adaptive defect correction, grid
    lens shading, Bayer WB, any of the three demosaics, CCM, LUT tone."""
    assert pl.packed and pl.bit_depth in (10, 12) and pl.stage_order == abi.ORDER_BAYER_WB
    assert pl.bl_mode == abi.BL_PER_CHANNEL and pl.dpc_mode == abi.DPC_ADAPTIVE and pl.lsc_mode == abi.LSC_GRID
    assert pl.stages == abi.STAGE_ALL and pl.tone_mode == abi.TONE_LUT and pl.out_format == abi.OUT_RGB8
    R, L = _ref_chain_lib(), stages()
    L.or_tone_rgb8.argtypes = [U16P, U8P, C.c_int, C.c_int, C.c_int, C.c_int, F32P, F32P]
    w, h, bd, pat = pl.width, pl.height, pl.bit_depth, pl.pattern
    raw = np.ascontiguousarray(raw, np.uint8)
    bay = np.empty((h, w), np.uint16)
    R.ref_unpack_packed(raw.ctypes.data, raw.size, bay.ctypes.data, w, h, bd)
    off = np.asarray(pl.bl_offset, np.float32)
    R.ref_black_level_store(bay.ctypes.data, w, h, pat, bd, off.ctypes.data_as(F32P))
    R.ref_dpc_adaptive_store(bay.ctypes.data, w, h, pat, bd, float(pl.dpc_threshold))
    grid = np.ascontiguousarray(pl.lsc_grid, np.float32)
    L.or_lsc_grid(bay.ctypes.data_as(U16P), w, h, pat, bd, grid.ctypes.data_as(F32P), grid.shape[1], grid.shape[0])
    wb = np.asarray(pl.wb_gain, np.float32)
    L.or_wb_bayer(bay.ctypes.data_as(U16P), w, h, pat, bd, wb.ctypes.data_as(F32P))
    rgb = np.empty((h, w, 3), np.uint16)
    R.ref_demosaic_store(bay.ctypes.data, rgb.ctypes.data, w, h, pat, pl.demosaic, bd)
    m = np.asarray(pl.ccm, np.float32)
    rgb2 = np.empty_like(rgb)
    R.ref_ccm_store(rgb.ctypes.data, rgb2.ctypes.data, w, h, bd, m.ctypes.data_as(F32P))
    out = np.empty((h, w, 3), np.uint8)
    lut = np.ascontiguousarray(pl.tone_lut, np.float32)
    L.or_tone_rgb8(rgb2.ctypes.data_as(U16P), out.ctypes.data_as(U8P), w, h, bd, pl.tone_mode,
                   lut.ctypes.data_as(F32P), None)
    return out


_refcuda = None


def refcuda_available():
    return os.path.exists(os.path.join(HERE, "_ref", "libimop_refcuda.so"))


def refcuda():
    """the reference's own GPU path (`make -C oracle refcuda`; timing only)"""
    global _refcuda
    if _refcuda is None:
        path = os.path.join(HERE, "_ref", "libimop_refcuda.so")
        if not os.path.exists(path):
            raise RuntimeError("reference GPU library not built: run `make -C oracle refcuda`")
        _refcuda = C.CDLL(path)
        i, vp = C.c_int, C.c_void_p
        _refcuda.refcuda_has_cuda.argtypes = []
        _refcuda.refcuda_black_level.argtypes = [vp, i, i, i, i, F32P]
        _refcuda.refcuda_defect_adaptive.argtypes = [vp, i, i, i, i, C.c_float]
        _refcuda.refcuda_demosaic.argtypes = [vp, vp, i, i, i, i, i]
    return _refcuda


def ref_chain_cuda(pl, raw):
    """RGB8 of one frame through the calls the reference's dispatchers make on a CUDA host: its GPU
    black level, adaptive defect correction and demosaic (each copying the frame in and out, as the
    reference's glue does), its CPU unpack and CCM, and the oracle's restatements of the stages the
    reference has no function for (as ref_chain).  Timing only: the reference's GPU kernels do not
    reproduce its CPU results.  Raises when a GPU call reports an error."""
    assert pl.packed and pl.bit_depth in (10, 12) and pl.stage_order == abi.ORDER_BAYER_WB
    assert pl.bl_mode == abi.BL_PER_CHANNEL and pl.dpc_mode == abi.DPC_ADAPTIVE and pl.lsc_mode == abi.LSC_GRID
    assert pl.stages == abi.STAGE_ALL and pl.tone_mode == abi.TONE_LUT and pl.out_format == abi.OUT_RGB8
    R, G, L = _ref_chain_lib(), refcuda(), stages()
    L.or_tone_rgb8.argtypes = [U16P, U8P, C.c_int, C.c_int, C.c_int, C.c_int, F32P, F32P]
    w, h, bd, pat = pl.width, pl.height, pl.bit_depth, pl.pattern
    raw = np.ascontiguousarray(raw, np.uint8)
    bay = np.empty((h, w), np.uint16)
    R.ref_unpack_packed(raw.ctypes.data, raw.size, bay.ctypes.data, w, h, bd)
    off = np.asarray(pl.bl_offset, np.float32)
    for rc, what in ((G.refcuda_black_level(bay.ctypes.data, w, h, pat, bd, off.ctypes.data_as(F32P)), "black level"),
                     (G.refcuda_defect_adaptive(bay.ctypes.data, w, h, pat, bd, float(pl.dpc_threshold)), "defects")):
        if rc != 0:
            raise RuntimeError(f"reference GPU {what}: status {rc}")
    grid = np.ascontiguousarray(pl.lsc_grid, np.float32)
    L.or_lsc_grid(bay.ctypes.data_as(U16P), w, h, pat, bd, grid.ctypes.data_as(F32P), grid.shape[1], grid.shape[0])
    wb = np.asarray(pl.wb_gain, np.float32)
    L.or_wb_bayer(bay.ctypes.data_as(U16P), w, h, pat, bd, wb.ctypes.data_as(F32P))
    rgb = np.empty((h, w, 3), np.uint16)
    rc = G.refcuda_demosaic(bay.ctypes.data, rgb.ctypes.data, w, h, pat, pl.demosaic, bd)
    if rc != 0:
        raise RuntimeError(f"reference GPU demosaic: status {rc}")
    m = np.asarray(pl.ccm, np.float32)
    rgb2 = np.empty_like(rgb)
    R.ref_ccm_store(rgb.ctypes.data, rgb2.ctypes.data, w, h, bd, m.ctypes.data_as(F32P))
    out = np.empty((h, w, 3), np.uint8)
    lut = np.ascontiguousarray(pl.tone_lut, np.float32)
    L.or_tone_rgb8(rgb2.ctypes.data_as(U16P), out.ctypes.data_as(U8P), w, h, bd, pl.tone_mode,
                   lut.ctypes.data_as(F32P), None)
    return out
