"""CPU-side checks of the C ABI: the library loads and exports every function that
include/imop_isp.h declares; parameter validation returns the reference's status codes; the
seeded scene is deterministic; the MIPI packers invert the reference unpackers."""
import ctypes as C
import hashlib
import os
import re
import subprocess

import numpy as np
import pytest

import imop_gb300 as I
import oracle_py as O
from imop_gb300 import abi, workloads

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    with open(os.path.join(REPO, "include", "imop_isp.h")) as f:
        src = f.read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(imop_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_function():
    L = I.lib()
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(L, n), f"{n} declared in include/imop_isp.h but not exported"
    assert L.imop_abi_version() == 4


def _validate(pl_or_none):
    f = I.lib().imop_isp_run_device_noalloc
    f.restype = C.c_int
    f.argtypes = [C.POINTER(abi.IspParams), C.c_void_p, C.c_void_p, C.c_void_p]
    if pl_or_none is None:
        return f(None, 1, 1, None)
    cp = pl_or_none.to_c() if isinstance(pl_or_none, I.Pipeline) else pl_or_none
    return f(C.byref(cp), 1, 1, None)


def test_validation_codes_follow_the_reference():
    # src/algorithms/dispatch.cpp:14-20 order: null, dimensions, bit depth, pattern, too small
    assert _validate(None) == abi.ERR_NULL_INPUT
    assert _validate(I.Pipeline(width=0, height=10)) == abi.ERR_INVALID_DIMENSIONS
    assert _validate(I.Pipeline(width=10, height=10, bit_depth=0)) == abi.ERR_INVALID_BIT_DEPTH
    assert _validate(I.Pipeline(width=10, height=10, bit_depth=17)) == abi.ERR_INVALID_BIT_DEPTH
    assert _validate(I.Pipeline(width=10, height=10, pattern=7)) == abi.ERR_INVALID_PATTERN
    assert _validate(I.Pipeline(width=5, height=10)) == abi.ERR_IMAGE_TOO_SMALL
    # a packed depth other than 10 / 12 is a bit stream: valid (this host then reports no device)
    assert _validate(I.Pipeline(width=10, height=10, bit_depth=11, packed=True)) == abi.ERR_NO_DEVICE
    assert _validate(I.Pipeline(width=10, height=10, demosaic=3)) == abi.ERR_UNSUPPORTED
    pl = I.Pipeline(width=10, height=10, bit_depth=12, out_format=abi.OUT_RGB8, tone_mode=abi.TONE_LUT)
    pl.tone_lut = np.zeros(100, np.float32)
    assert _validate(pl) == abi.ERR_INVALID_ARGUMENT


def test_raw_to_jpeg_argument_checks_without_device():
    """the host checks of imop_isp_run_host_jpeg_batch come before any device work"""
    from imop_gb300 import jpeg as J
    f = J._L().imop_isp_run_host_jpeg_batch
    assert f(None, None, None, 0) == abi.ERR_NULL_INPUT
    fake = C.c_void_p(1)  # never dereferenced: the frame checks fail first
    assert f(fake, fake, None, -1) == abi.ERR_INVALID_ARGUMENT
    assert f(fake, fake, None, 0) == abi.OK
    assert f(fake, fake, None, 2) == abi.ERR_NULL_INPUT


def test_adjoint_argument_checks_without_device():
    """The adjoint's host checks (context, descriptor, pointers, mode) come before any device
    work, with the library's status codes; the parameter vector holds 16 + 4 x grid nodes + 33."""
    L = I.lib()
    d = abi.AdjointDesc(1006, 758, 12, 0, abi.RGGB, abi.AMAZE, 17, 13, 16)
    assert L.imop_adjoint_param_count(C.byref(d)) == 933
    assert L.imop_adjoint_param_count(None) == 0
    fake = C.c_void_p(1)  # never dereferenced: the checks fail first

    def backward(desc, ctx=fake, ptr=fake, mode=abi.ADJ_TARGET):
        return L.imop_isp_backward_device(ctx, None if desc is None else C.byref(desc), ptr, ptr, ptr, mode, None,
                                          ptr, None)

    def render(desc, ctx=fake, ptr=fake):
        return L.imop_isp_render_device(ctx, None if desc is None else C.byref(desc), ptr, ptr, ptr, None)

    for call in (backward, render):
        assert call(d, ctx=None) == abi.ERR_NULL_INPUT
        assert call(None) == abi.ERR_NULL_INPUT
        assert call(d, ptr=None) == abi.ERR_NULL_INPUT
        for field, value, code in [("width", 0, abi.ERR_INVALID_DIMENSIONS),
                                   ("bit_depth", 17, abi.ERR_INVALID_BIT_DEPTH),
                                   ("pattern", 4, abi.ERR_INVALID_PATTERN),
                                   ("height", 5, abi.ERR_IMAGE_TOO_SMALL),
                                   ("demosaic", abi.MG, abi.ERR_UNSUPPORTED),
                                   ("grid_w", 1, abi.ERR_INVALID_ARGUMENT),
                                   ("grid_h", 33, abi.ERR_INVALID_ARGUMENT),
                                   ("n_frames", 0, abi.ERR_INVALID_ARGUMENT)]:
            bad = abi.AdjointDesc(*(getattr(d, n) for n, _ in abi.AdjointDesc._fields_))
            setattr(bad, field, value)
            assert call(bad) == code, (call.__name__, field)
        big = abi.AdjointDesc(*(getattr(d, n) for n, _ in abi.AdjointDesc._fields_))
        big.grid_w, big.grid_h = 17, 17  # 289 nodes: more than the 256 the kernels hold
        assert call(big) == abi.ERR_INVALID_ARGUMENT
    assert backward(d, mode=2) == abi.ERR_INVALID_ARGUMENT


def test_params_default_and_sizes():
    L = I.lib()
    p = abi.IspParams()
    L.imop_isp_params_default(C.byref(p), 4024, 3032, 12, 1)
    assert p.width == 4024 and p.demosaic == abi.HQLI and p.ccm[0] == 1.0 and p.tone_knots[32] == 1.0
    assert L.imop_isp_input_bytes(C.byref(p)) == 18301152
    assert L.imop_isp_output_bytes(C.byref(p)) == 36602304
    p.packed, p.bit_depth, p.out_format = 0, 12, abi.OUT_NATIVE
    assert L.imop_isp_input_bytes(C.byref(p)) == 2 * 4024 * 3032
    assert L.imop_isp_output_bytes(C.byref(p)) == 6 * 4024 * 3032


def test_scene_is_seeded_and_in_range():
    a = I.scene(257, 131, 12, abi.GRBG, seed=7, lo=256, hi=4095)
    b = I.scene(257, 131, 12, abi.GRBG, seed=7, lo=256, hi=4095)
    c = I.scene(257, 131, 12, abi.GRBG, seed=8, lo=256, hi=4095)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    assert a.dtype == np.uint16 and a.max() <= 4095 and a.min() >= 0
    assert abs(float(a.mean()) - (256 + 4095) / 2) < 400
    pts = I.defects(4024, 3032, 1220, seed=3)
    assert len({(x, y) for x, y in pts}) == 1220
    assert pts[:, 0].min() >= 2 and pts[:, 0].max() < 4022 and pts[:, 1].max() < 3030


def test_mipi_packers_invert_the_unpacker():
    rng = np.random.default_rng(5)
    for bd in (10, 12):
        for (w, h) in ((8, 4), (7, 5), (33, 3), (1006, 4)):
            f = rng.integers(0, 1 << bd, (h, w)).astype(np.uint16)
            buf = I.pack_mipi(f, bd)
            assert buf.size == (w * h * bd + 7) // 8
            got = np.array([[O.get_packed_raw(buf, x, y, w, h, bd) for x in range(w)] for y in range(h)])
            # pixels of an incomplete trailing group read as 0 (include/imop/pixel_utils.hpp:71,85)
            n = w * h
            full = n - (n % (4 if bd == 10 else 2))
            assert np.array_equal(got.reshape(-1)[:full], f.reshape(-1)[:full])
            assert not got.reshape(-1)[full:].any()
    # other depths: one LSB-first bit stream (the reference's generic case), every sample returns
    for bd in (8, 9, 11, 13, 14, 16):
        for (w, h) in ((8, 4), (7, 5), (33, 3)):
            f = rng.integers(0, 1 << bd, (h, w)).astype(np.uint16)
            buf = I.pack_mipi(f, bd)
            assert buf.size == (w * h * bd + 7) // 8
            got = np.array([[O.get_packed_raw(buf, x, y, w, h, bd) for x in range(w)] for y in range(h)])
            assert np.array_equal(got, f)


def test_c2_workload_shape():
    pl = workloads.c2_pipeline()
    assert pl.input_bytes() == 18301152 and pl.output_bytes() == 36602304
    assert pl.dpc_map.shape == (1220, 2)
    g = workloads.radial_grid(4024, 3032)
    assert g.shape == (13, 17, 4) and abs(g[6, 8, 0] - 1.0) < 0.01 and abs(g[0, 0, 0] - 2.0) < 1e-5
    m = np.array(pl.ccm).reshape(3, 3)
    assert np.allclose(m.sum(1), 1.0, atol=1e-6) and (np.diag(m) >= 1.4).all()


def test_reference_shim_symbols_link(tmp_path):
    """The reference-compatible C++ symbols resolve against the library (link only; no GPU)."""
    from shim_build import build_shim_check
    r = build_shim_check(str(tmp_path / "shim_check"))
    assert r.returncode == 0, r.stderr


def test_reference_headers_link_against_library():
    """The reference's own declarations of its GPU glue (every module's process_*_cuda and
    has_cuda, imop::demosaic_cuda and friends) resolve against this library: the link recipe
    oracle/Makefile `shimlink` compiles a probe with the reference's headers."""
    import oracle_py as O
    if not O.ref_available():
        pytest.skip("the reference tree is not on this host")
    r = subprocess.run(["make", "-C", os.path.join(REPO, "oracle"), "shimlink"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr


def test_c_abi_header_is_plain_c(tmp_path):
    """include/imop_isp.h compiles as strict C99 (the ABI carries no C++ types), and a C caller of
    the RAW-to-JPEG batch call links against the library."""
    src = tmp_path / "caller.c"
    src.write_text('#include "imop_isp.h"\n'
                   "int run(imop_isp_t isp, imop_jpeg_t j, const void* raw, uint8_t* out, size_t cap) {\n"
                   "    ImopRawJpegFrame f = {0};\n"
                   "    f.raw = raw; f.quality = 90; f.subsample = 1; f.out = out; f.out_cap = cap;\n"
                   "    int st = imop_isp_run_host_jpeg_batch(isp, j, &f, 1);\n"
                   "    return st ? st : (int)f.out_size;\n"
                   "}\n"
                   "int main(void) { return imop_abi_version() == IMOP_ISP_ABI_VERSION ? 0 : 1; }\n")
    lib_dir = os.path.dirname(I.lib()._name)
    exe = tmp_path / "caller"
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", os.path.join(REPO, "include"),
                        str(src), "-o", str(exe), "-L", lib_dir, "-limop_isp", f"-Wl,-rpath,{lib_dir}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert subprocess.run([str(exe)]).returncode == 0
