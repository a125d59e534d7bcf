"""ctypes mirror of include/imop_isp.h (structs and constants only; no library is loaded here)."""
import ctypes as C

OK = 0
ERR_NULL_INPUT = 1
ERR_INVALID_DIMENSIONS = 2
ERR_INVALID_BIT_DEPTH = 3
ERR_INVALID_PATTERN = 4
ERR_IMAGE_TOO_SMALL = 5
ERR_INTERNAL = 6
ERR_INVALID_ARGUMENT = 100
ERR_UNSUPPORTED = 101
ERR_CUDA = 102
ERR_TIMEOUT = 103
ERR_CAPACITY = 104
ERR_NO_DEVICE = 105

RGGB, BGGR, GRBG, GBRG = 0, 1, 2, 3
PATTERNS = {"RGGB": RGGB, "BGGR": BGGR, "GRBG": GRBG, "GBRG": GBRG}

HQLI, MG, AMAZE = 1, 2, 6

STAGE_BLACK_LEVEL = 1 << 0
STAGE_DEFECT = 1 << 1
STAGE_LENS_SHADING = 1 << 2
STAGE_WHITE_BALANCE = 1 << 3
STAGE_CCM = 1 << 4
STAGE_ALL = 0x1F
STAGE_LUT3D = 1 << 5  # optional 3D LUT after the CCM, not in STAGE_ALL

ORDER_BAYER_WB = 0
ORDER_RGB_WB = 1

BL_PER_CHANNEL, BL_GLOBAL = 0, 1
DPC_ADAPTIVE, DPC_MAP_BASED = 0, 1
LSC_GRID, LSC_POLYNOMIAL, LSC_FLAT_FIELD = 0, 1, 2
TONE_LINEAR, TONE_LUT, TONE_KNOTS = 0, 1, 2
OUT_RGB8, OUT_NATIVE = 0, 1


class DefectPoint(C.Structure):
    _fields_ = [("x", C.c_int), ("y", C.c_int)]


class IspParams(C.Structure):
    _fields_ = [
        ("width", C.c_int), ("height", C.c_int),
        ("bit_depth", C.c_int), ("packed", C.c_int),
        ("pattern", C.c_int), ("demosaic", C.c_int),
        ("stages", C.c_uint), ("stage_order", C.c_int),
        ("bl_mode", C.c_int), ("bl_offset", C.c_float * 4),
        ("dpc_mode", C.c_int), ("dpc_threshold", C.c_float),
        ("dpc_map", C.POINTER(DefectPoint)), ("dpc_map_count", C.c_int),
        ("lsc_mode", C.c_int),
        ("lsc_grid", C.POINTER(C.c_float)), ("lsc_grid_w", C.c_int), ("lsc_grid_h", C.c_int),
        ("lsc_poly", (C.c_float * 3) * 4), ("lsc_center", C.c_float * 2),
        ("lsc_flat_field", C.c_void_p), ("lsc_flat_w", C.c_int), ("lsc_flat_h", C.c_int),
        ("wb_gain", C.c_float * 3),
        ("ccm", C.c_float * 9),
        ("tone_mode", C.c_int),
        ("tone_lut", C.POINTER(C.c_float)), ("tone_lut_len", C.c_int),
        ("tone_knots", C.c_float * 33),
        ("out_format", C.c_int),
        ("lut3d", C.POINTER(C.c_float)), ("lut3d_size", C.c_int),
    ]


ANALYZE_MAX_DIMS = 16


class DataInfo(C.Structure):
    _fields_ = [("detected_bit_depth", C.c_int), ("suggested_width", C.c_int), ("suggested_height", C.c_int),
                ("pixel_count", C.c_int), ("max_value", C.c_int), ("min_value", C.c_int),
                ("is_likely_16bit", C.c_int), ("is_packed", C.c_int), ("n_dims", C.c_int),
                ("dims", (C.c_int * 2) * ANALYZE_MAX_DIMS)]


class StageDumps(C.Structure):
    _fields_ = [
        ("unpacked", C.c_void_p), ("black_level", C.c_void_p), ("defect", C.c_void_p),
        ("lens_shading", C.c_void_p), ("white_balance", C.c_void_p), ("demosaic", C.c_void_p),
        ("ccm", C.c_void_p), ("output", C.c_void_p),
    ]


class FrameDesc(C.Structure):
    _fields_ = [("params", C.POINTER(IspParams)), ("inp", C.c_void_p), ("out", C.c_void_p)]


BATCH_GRAPH = 1
BATCH_PLAIN = 2


class AdjointDesc(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("bit_depth", C.c_int), ("packed", C.c_int),
                ("pattern", C.c_int), ("demosaic", C.c_int), ("grid_w", C.c_int), ("grid_h", C.c_int),
                ("n_frames", C.c_int)]


ADJ_TARGET = 0
ADJ_UPSTREAM = 1

# the reference's tone curves (tone::ToneAlgorithm) and their parameters (tone::ToneParams)
TONE_CURVE_GAMMA, TONE_CURVE_S_CURVE, TONE_CURVE_LEVELS, TONE_CURVE_3POINT, TONE_CURVE_SHADOWS_HIGHLIGHTS = range(5)


class ToneParams(C.Structure):
    _fields_ = [("gamma", C.c_float), ("contrast", C.c_float), ("shadows", C.c_float), ("highlights", C.c_float),
                ("black_point", C.c_float), ("white_point", C.c_float), ("mid_point", C.c_float)]


KERNEL_TILE, KERNEL_LITE, KERNEL_STREAM, KERNEL_LITE_DIRECT = 0, 1, 2, 3


class TuneEntry(C.Structure):
    """ImopTuneEntry: launch parameters of a streamed kernel for one (kernel, format, width) class"""
    _fields_ = [("kernel", C.c_int), ("fmt", C.c_int), ("max_width", C.c_int), ("enabled", C.c_int),
                ("band_rows", C.c_int), ("seg_percent", C.c_int)]
