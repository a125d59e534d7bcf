"""imop_gb300 - Python host mirror of the GB300 RAW->RGB ISP library (libimop_isp.so).

Thin ctypes layer over the C ABI declared in include/imop_isp.h.  Device buffers are passed as
raw addresses (for example torch.Tensor.data_ptr()), streams as raw cudaStream_t handles.  The
library is required: importing `lib()` raises when libimop_isp.so has not been built, so no
caller can silently fall back to a CPU path.
"""
import ctypes as C
import os

import numpy as np

from . import abi
from .abi import *  # noqa: F401,F403
from .params import Pipeline  # noqa: F401

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libimop_isp.so")
_lib = None


class IspError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"imop status {code}: {msg}")
        self.code = code


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with __graft_entry__.build()")
        L = C.CDLL(LIB_PATH)
        i, vp, sz = C.c_int, C.c_void_p, C.c_size_t
        PP = C.POINTER(abi.IspParams)
        sig = {
            "imop_isp_params_default": (None, [PP, i, i, i, i]),
            "imop_isp_input_bytes": (sz, [PP]),
            "imop_isp_output_bytes": (sz, [PP]),
            "imop_isp_create": (i, [C.POINTER(vp)]),
            "imop_isp_destroy": (i, [vp]),
            "imop_isp_set_params": (i, [vp, PP]),
            "imop_isp_run_host": (i, [vp, vp, sz, vp, sz]),
            "imop_isp_run_device": (i, [vp, vp, vp, vp]),
            "imop_isp_run_device_plain": (i, [vp, vp, vp, vp]),
            "imop_isp_dump_stages": (i, [vp, vp, sz, C.POINTER(abi.StageDumps)]),
            "imop_isp_set_tile": (i, [vp, i, i]),
            "imop_isp_last_stats": (i, [vp, C.POINTER(i), C.POINTER(i)]),
            "imop_isp_sync_status": (i, [vp, vp]),
            "imop_isp_batch_submit": (i, [vp, C.POINTER(abi.FrameDesc), i, C.c_uint, vp]),
            "imop_isp_run_host_batch": (i, [vp, C.POINTER(abi.FrameDesc), i]),
            "imop_adjoint_param_count": (i, [C.POINTER(abi.AdjointDesc)]),
            "imop_isp_render_device": (i, [vp, C.POINTER(abi.AdjointDesc), vp, vp, vp, vp]),
            "imop_isp_backward_device": (i, [vp, C.POINTER(abi.AdjointDesc), vp, vp, vp, i, vp, vp, vp]),
            "imop_scene_render": (i, [i, i, i, i, C.c_uint64, C.c_float, C.c_float, C.c_float, C.c_float, vp]),
            "imop_scene_defects": (i, [i, i, C.c_uint64, i, C.POINTER(abi.DefectPoint)]),
            "imop_scene_apply_defects": (i, [vp, i, i, i, C.POINTER(abi.DefectPoint), i]),
            "imop_packed_bytes": (sz, [i, i, i]),
            "imop_pack_mipi": (i, [vp, i, i, i, vp]),
            "imop_analyze_data": (i, [vp, sz, C.POINTER(abi.DataInfo)]),
            "imop_detect_bit_depth": (i, [vp, sz]),
            "imop_suggest_dimensions": (i, [sz, C.POINTER(C.c_int * 2), i]),
            "imop_guess_pattern": (i, [vp, i, i, i, i]),
            "imop_last_error_string": (C.c_char_p, []),
            "imop_abi_version": (i, []),
            "imop_has_cuda": (i, []),
            "imop_device_name": (C.c_char_p, []),
            "imop_shim_calls_served": (C.c_longlong, []),
            "imop_kernel_launches": (C.c_longlong, [i]),
            "imop_tuning_set": (i, [C.POINTER(abi.TuneEntry), i]),
            "imop_tuning_get": (i, [C.POINTER(abi.TuneEntry), i]),
            "imop_tone_table_entries": (sz, [i]),
            "imop_tone_table": (i, [i, i, C.POINTER(abi.ToneParams), vp, sz]),
            "imop_op_rgb_table": (i, [vp, i, i, i, vp, vp, vp]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(code):
    if code != 0:
        raise IspError(code, lib().imop_last_error_string().decode(errors="replace"))
    return code


def _addr(x):
    """device / host address of a tensor, ndarray or integer"""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    if isinstance(x, np.ndarray):
        return x.ctypes.data
    raise TypeError(type(x))


_tuning_loaded = False


def _load_tuning():
    """Once per process: the measured launch-tuning table beside the package (tuning.py), when it
    was measured on this device; IMOP_TUNING_FILE names another table, IMOP_TUNING_FILE="" none."""
    global _tuning_loaded
    if _tuning_loaded:
        return
    _tuning_loaded = True
    from . import tuning
    path = os.environ.get("IMOP_TUNING_FILE", tuning.DEFAULT_TABLE)
    if path:
        tuning.load(path, device_name=lib().imop_device_name().decode())


class Isp:
    """One pipeline context (imop_isp_t)."""

    def __init__(self, pipeline=None):
        h = C.c_void_p()
        check(lib().imop_isp_create(C.byref(h)))
        _load_tuning()
        self.h = h
        self.pipeline = None
        self._cparams = None
        if pipeline is not None:
            self.set_params(pipeline)

    def close(self):
        if self.h:
            lib().imop_isp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, pl):
        cp = pl.to_c()
        check(lib().imop_isp_set_params(self.h, C.byref(cp)))
        self.pipeline = pl
        self._cparams = cp

    def run_host(self, raw, out=None):
        """One host frame, synchronous; `out` (ndarray or host tensor, e.g. page-locked) is filled
        in place when given, else a new array is returned."""
        pl = self.pipeline
        raw = np.ascontiguousarray(raw).view(np.uint8).reshape(-1)
        if out is None:
            out = np.empty(pl.output_shape(), dtype=pl.output_dtype())
        nbytes = out.nbytes if isinstance(out, np.ndarray) else out.numel() * out.element_size()
        check(lib().imop_isp_run_host(self.h, raw.ctypes.data, raw.nbytes, _addr(out), nbytes))
        return out

    def run_device(self, d_in, d_out, stream=0):
        check(lib().imop_isp_run_device(self.h, _addr(d_in), _addr(d_out), stream))

    def run_device_plain(self, d_in, d_out, stream=0):
        check(lib().imop_isp_run_device_plain(self.h, _addr(d_in), _addr(d_out), stream))

    def dump_stages(self, raw):
        pl = self.pipeline
        raw = np.ascontiguousarray(raw).view(np.uint8).reshape(-1)
        h, w = pl.height, pl.width
        rgb_wb = pl.stage_order == abi.ORDER_RGB_WB
        d = {
            "unpacked": np.zeros((h, w), np.uint16),
            "black_level": np.zeros((h, w), np.uint16),
            "defect": np.zeros((h, w), np.uint16),
            "lens_shading": np.zeros((h, w), np.uint16),
            "white_balance": np.zeros((h, w, 3) if rgb_wb else (h, w), np.uint16),
            "demosaic": np.zeros((h, w, 3), np.uint16),
            "ccm": np.zeros((h, w, 3), np.uint16),
            "output": np.zeros(pl.output_shape(), pl.output_dtype()),
        }
        sd = abi.StageDumps(*[d[k].ctypes.data for k in ("unpacked", "black_level", "defect", "lens_shading",
                                                         "white_balance", "demosaic", "ccm", "output")])
        check(lib().imop_isp_dump_stages(self.h, raw.ctypes.data, raw.nbytes, C.byref(sd)))
        return d

    def last_stats(self):
        s, o = C.c_int(), C.c_int()
        check(lib().imop_isp_last_stats(self.h, C.byref(s), C.byref(o)))
        return s.value, o.value

    def sync_status(self, stream=0):
        check(lib().imop_isp_sync_status(self.h, stream))

    @staticmethod
    def _descs(frames):
        """frames: list of (Pipeline or None, input, output); returns the C array and its keep-alive"""
        keep = []
        arr = (abi.FrameDesc * max(1, len(frames)))()
        for k, (pl, inp, out) in enumerate(frames):
            cp = None
            if pl is not None:
                cp = pl.to_c()
                keep.append(cp)
            arr[k].params = C.pointer(cp) if cp is not None else None
            arr[k].inp = _addr(inp)
            arr[k].out = _addr(out)
        return arr, keep

    def batch_submit(self, frames, flags=0, stream=0):
        """Device frames: list of (Pipeline or None, d_in, d_out); asynchronous on `stream`."""
        arr, keep = self._descs(frames)
        check(lib().imop_isp_batch_submit(self.h, arr, len(frames), flags, stream))
        del keep

    def run_host_batch(self, frames):
        """Host frames: list of (Pipeline or None, input ndarray, output ndarray); synchronous."""
        arr, keep = self._descs(frames)
        check(lib().imop_isp_run_host_batch(self.h, arr, len(frames)))
        del keep


# ---- synthetic scenes ---------------------------------------------------------------------------
def scene(width, height, bit_depth, pattern=abi.RGGB, seed=20261203, lo=None, hi=None, gain=0.5,
          read_sigma=2.0):
    """Seeded Bayer frame (uint8 for bd <= 8, uint16 otherwise) as an (h, w) array."""
    mv = (1 << bit_depth) - 1
    lo = float(lo if lo is not None else 0.0625 * (mv + 1))
    hi = float(hi if hi is not None else mv)
    out = np.empty((height, width), np.uint8 if bit_depth <= 8 else np.uint16)
    check(lib().imop_scene_render(width, height, bit_depth, pattern, seed, lo, hi, gain, read_sigma,
                                  out.ctypes.data))
    return out


def defects(width, height, count, seed=20261203):
    pts = (abi.DefectPoint * max(1, count))()
    check(lib().imop_scene_defects(width, height, seed, count, pts))
    return np.array([(pts[i].x, pts[i].y) for i in range(count)], np.int32).reshape(-1, 2)


def apply_defects(frame, pts, bit_depth):
    pts = np.ascontiguousarray(pts, np.int32).reshape(-1, 2)
    h, w = frame.shape
    check(lib().imop_scene_apply_defects(frame.ctypes.data, w, h, bit_depth,
                                         pts.ctypes.data_as(C.POINTER(abi.DefectPoint)), pts.shape[0]))
    return frame


def pack_mipi(frame, bit_depth):
    h, w = frame.shape
    f = np.ascontiguousarray(frame, np.uint16)
    out = np.empty(lib().imop_packed_bytes(w, h, bit_depth), np.uint8)
    check(lib().imop_pack_mipi(f.ctypes.data, w, h, bit_depth, out.ctypes.data))
    return out


# ---- format sniffing (the reference's analyzer heuristics) ----------------------------------------
def _bytes(buf):
    a = np.ascontiguousarray(buf).view(np.uint8).reshape(-1)
    return a, a.nbytes


def analyze_data(buf):
    """dict of the detected bit depth, packing, pixel count, value range and candidate sizes"""
    a, n = _bytes(buf)
    info = abi.DataInfo()
    check(lib().imop_analyze_data(a.ctypes.data if n else None, n, C.byref(info)))
    dims = [(info.dims[k][0], info.dims[k][1]) for k in range(info.n_dims)]
    return {"detected_bit_depth": info.detected_bit_depth, "suggested_width": info.suggested_width,
            "suggested_height": info.suggested_height, "pixel_count": info.pixel_count,
            "max_value": info.max_value, "min_value": info.min_value,
            "is_likely_16bit": bool(info.is_likely_16bit), "is_packed": bool(info.is_packed),
            "possible_dimensions": dims}


def detect_bit_depth(buf):
    a, n = _bytes(buf)
    return lib().imop_detect_bit_depth(a.ctypes.data if n else None, n)


def suggest_dimensions(pixel_count):
    out = ((C.c_int * 2) * abi.ANALYZE_MAX_DIMS)()
    k = lib().imop_suggest_dimensions(pixel_count, out, abi.ANALYZE_MAX_DIMS)
    return [(out[j][0], out[j][1]) for j in range(min(k, abi.ANALYZE_MAX_DIMS))]


def guess_pattern(buf, width, height, bit_depth=8, packed=False):
    a, _ = _bytes(buf)
    return lib().imop_guess_pattern(a.ctypes.data, width, height, bit_depth, int(bool(packed)))


def tone_params(gamma=1.0, contrast=0.0, shadows=0.0, highlights=0.0, black_point=0.0, white_point=1.0,
                mid_point=0.5):
    """tone::ToneParams with the reference's defaults (include/tone/types.hpp:50-58)."""
    return abi.ToneParams(gamma, contrast, shadows, highlights, black_point, white_point, mid_point)


def tone_table(algorithm, bit_depth, params):
    """Output sample of one of the reference's tone curves for every storable input sample value
    (uint16, 256 entries for bit depth <= 8, 65536 otherwise)."""
    n = lib().imop_tone_table_entries(bit_depth)
    t = np.zeros(n, np.uint16)
    check(lib().imop_tone_table(algorithm, bit_depth, C.byref(params), t.ctypes.data, n))
    return t
