"""Baseline JPEG encode of RGB8 frames on the device (the imop_jpeg_* C ABI).

    enc = JpegEncoder()
    data = enc.encode(rgb, quality=90, subsample=1)             # host (h, w, 3) u8 -> bytes array
    n = enc.encode_device(d_rgb, w, h, d_out, cap, stream=s)    # device in, device out, no sync
    enc.last_size()                                             # (jpeg bytes, written)
    raw_to_jpeg_host_batch(isp, enc, [(None, raw, 90, 1, out)])  # host RAW -> host JPEG via HBM

The bytes are those of jpeg_codec::process_encode_baseline for the same frame, quality and
subsampling (0 = 4:4:4, 1 = 4:2:0, 2 = 4:2:2).  Status codes are jpeg_codec::JpegError values;
a non-zero status raises JpegError (or is returned by the *_status variants).
"""
import ctypes as C

import numpy as np

from . import _addr, lib

OK, NULL_INPUT, NULL_OUTPUT, INVALID_DIMENSIONS, INVALID_BIT_DEPTH, INVALID_CHANNELS = 0, 1, 2, 3, 4, 5
INVALID_QUALITY, IMAGE_TOO_SMALL, ENCODE_FAILED, DECODE_FAILED, INVALID_DATA = 6, 7, 8, 9, 10
CUDA_NOT_AVAILABLE, INTERNAL_ERROR = 11, 12


class JpegFrame(C.Structure):
    _fields_ = [("d_rgb", C.c_void_p), ("width", C.c_int), ("height", C.c_int), ("quality", C.c_int),
                ("subsample", C.c_int), ("d_out", C.c_void_p), ("out_cap", C.c_size_t), ("d_out_size", C.c_void_p)]


class JpegHostFrame(C.Structure):
    _fields_ = [("rgb", C.c_void_p), ("width", C.c_int), ("height", C.c_int), ("quality", C.c_int),
                ("subsample", C.c_int), ("out", C.c_void_p), ("out_cap", C.c_size_t), ("out_size", C.c_size_t),
                ("status", C.c_int)]


class RawJpegFrame(C.Structure):
    _fields_ = [("params", C.c_void_p), ("raw", C.c_void_p), ("quality", C.c_int), ("subsample", C.c_int),
                ("out", C.c_void_p), ("out_cap", C.c_size_t), ("out_size", C.c_size_t)]


class JpegError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"jpeg status {code}: {msg}")
        self.code = code


_bound = False


def _L():
    global _bound
    L = lib()
    if not _bound:
        i, vp, sz = C.c_int, C.c_void_p, C.c_size_t
        SP = C.POINTER(C.c_size_t)
        for name, res, args in (
            ("imop_jpeg_create", i, [C.POINTER(vp)]),
            ("imop_jpeg_destroy", i, [vp]),
            ("imop_jpeg_max_bytes", sz, [i, i]),
            ("imop_jpeg_header", i, [i, i, i, i, vp, sz]),
            ("imop_jpeg_encode_host", i, [vp, vp, i, i, i, i, i, vp, SP]),
            ("imop_jpeg_encode_device", i, [vp, vp, i, i, i, i, i, vp, sz, vp, vp]),
            ("imop_jpeg_last_size", i, [vp, SP, SP]),
            ("imop_jpeg_encode_device_batch", i, [vp, C.POINTER(JpegFrame), i, vp]),
            ("imop_jpeg_encode_host_batch", i, [vp, C.POINTER(JpegHostFrame), i]),
            ("imop_jpeg_last_error_string", C.c_char_p, []),
            ("imop_isp_run_host_jpeg_batch", i, [vp, vp, C.POINTER(RawJpegFrame), i]),
        ):
            f = getattr(L, name)
            f.restype, f.argtypes = res, args
        _bound = True
    return L


def _check(code):
    if code != 0:
        raise JpegError(code, _L().imop_jpeg_last_error_string().decode(errors="replace"))
    return code


def max_bytes(width, height):
    """jpeg_codec::get_max_jpeg_size: the default output capacity"""
    return int(_L().imop_jpeg_max_bytes(width, height))


def header(width, height, quality=90, subsample=1):
    """the header bytes (SOI .. SOS) of an encode"""
    n = _L().imop_jpeg_header(width, height, quality, subsample, None, 0)
    out = np.zeros(n, np.uint8)
    _L().imop_jpeg_header(width, height, quality, subsample, out.ctypes.data, n)
    return out


class JpegEncoder:
    """One encoder context (imop_jpeg_t): device scratch grown on demand, reused across calls."""

    def __init__(self):
        h = C.c_void_p()
        _check(_L().imop_jpeg_create(C.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            _L().imop_jpeg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def encode_status(self, rgb, quality=90, subsample=1, cap=0, bit_depth=8, width=None, height=None):
        """(status, bytes or None) of a host frame; rgb an (h, w, 3) u8 array (or None with
        width / height given, to exercise the null-input check)"""
        if rgb is None:
            w, h, ptr = width, height, None
        else:
            rgb = np.ascontiguousarray(rgb, np.uint8)
            h, w = rgb.shape[:2]
            w, h = width if width is not None else w, height if height is not None else h
            ptr = rgb.ctypes.data
        out = np.zeros(max(cap or max_bytes(max(w, 1), max(h, 1)), 1), np.uint8)
        n = C.c_size_t(cap)
        st = _L().imop_jpeg_encode_host(self.h, ptr, w, h, bit_depth, quality, subsample, out.ctypes.data, C.byref(n))
        return st, (out[: n.value].copy() if st == 0 else None)

    def encode(self, rgb, quality=90, subsample=1, cap=0):
        st, data = self.encode_status(rgb, quality, subsample, cap)
        _check(st)
        return data

    def encode_device(self, d_rgb, width, height, d_out, out_cap, quality=90, subsample=1, d_size=None, stream=0):
        """Device RGB8 at d_rgb -> the JPEG at d_out (addresses or tensors) on `stream`; returns
        without synchronising.  d_size: optional device size_t receiving the bytes written."""
        _check(_L().imop_jpeg_encode_device(self.h, _addr(d_rgb), width, height, 8, quality, subsample,
                                            _addr(d_out), out_cap, _addr(d_size), stream or None))

    def encode_device_batch(self, frames, stream=0):
        """frames: (d_rgb, width, height, d_out, out_cap, quality, subsample, d_size or None) per
        frame (addresses or tensors); encoded on two internal streams after `stream` reaches the
        call, `stream` continues after the last; no host synchronisation."""
        arr = (JpegFrame * len(frames))()
        for k, (d_rgb, w, h, d_out, cap, q, ss, d_size) in enumerate(frames):
            arr[k] = JpegFrame(_addr(d_rgb), w, h, q, ss, _addr(d_out), cap, _addr(d_size))
        _check(_L().imop_jpeg_encode_device_batch(self.h, arr, len(frames), stream or None))

    def encode_host_batch(self, frames):
        """frames: (rgb, quality, subsample, out) per frame, rgb an (h, w, 3) u8 array or host
        tensor, out a u8 array / host tensor with room for the JPEG; returns [(status, size)]."""
        arr = (JpegHostFrame * len(frames))()
        for k, (rgb, q, ss, out) in enumerate(frames):
            h, w = rgb.shape[:2]
            cap = out.nbytes if isinstance(out, np.ndarray) else out.numel()
            arr[k] = JpegHostFrame(_addr(rgb), w, h, q, ss, _addr(out), cap, 0, 0)
        _L().imop_jpeg_encode_host_batch(self.h, arr, len(frames))
        return [(arr[k].status, arr[k].out_size) for k in range(len(frames))]

    def last_size(self):
        """(JPEG bytes, bytes written) of the last encode (synchronises a pending device call)"""
        a, b = C.c_size_t(0), C.c_size_t(0)
        _check(_L().imop_jpeg_last_size(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value


def raw_to_jpeg_host_batch(isp, enc, frames):
    """RAW host frames -> JPEG host bytes through an ISP context (imop_gb300.Isp) and an encoder
    (imop_isp_run_host_jpeg_batch); the RGB8 frames stay on the device.  frames: (Pipeline or
    None, raw, quality, subsample, out) per frame, out a u8 array or host tensor with room for
    the JPEG (its size is the capacity).  Synchronous; returns the bytes written per frame and
    raises imop_gb300.ImopError on a non-zero status."""
    from . import check
    arr = (RawJpegFrame * max(1, len(frames)))()
    keep = []
    for k, (pl, raw, q, ss, out) in enumerate(frames):
        cp = pl.to_c() if pl is not None else None
        keep.append(cp)
        cap = out.nbytes if isinstance(out, np.ndarray) else out.numel()
        arr[k] = RawJpegFrame(C.addressof(cp) if cp is not None else None, _addr(raw), q, ss, _addr(out), cap, 0)
    check(_L().imop_isp_run_host_jpeg_batch(isp.h, enc.h, arr, len(frames)))
    del keep
    return [arr[k].out_size for k in range(len(frames))]
