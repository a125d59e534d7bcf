"""High-level pipeline description -> the C ABI's ImopIspParams.

`Pipeline` keeps the numpy arrays that the C struct points at alive for as long as the
struct is used, so callers never hand a dangling pointer across the boundary.
"""
import ctypes as C
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from . import abi


@dataclass
class Pipeline:
    width: int
    height: int
    bit_depth: int = 12
    packed: bool = False
    pattern: int = abi.RGGB
    demosaic: int = abi.HQLI
    stages: int = 0
    stage_order: int = abi.ORDER_BAYER_WB
    bl_mode: int = abi.BL_PER_CHANNEL
    bl_offset: tuple = (0.0, 0.0, 0.0, 0.0)
    dpc_mode: int = abi.DPC_ADAPTIVE
    dpc_threshold: float = 0.3
    dpc_map: Optional[np.ndarray] = None          # (n, 2) int32 (x, y)
    lsc_mode: int = abi.LSC_GRID
    lsc_grid: Optional[np.ndarray] = None         # (gh, gw, 4) float32
    lsc_poly: tuple = ((0.0, 0.0, 0.0),) * 4
    lsc_center: tuple = (0.5, 0.5)
    lsc_flat_field: Optional[np.ndarray] = None   # (fh, fw) uint8/uint16
    wb_gain: tuple = (1.0, 1.0, 1.0)
    ccm: tuple = (1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0)
    tone_mode: int = abi.TONE_LINEAR
    tone_lut: Optional[np.ndarray] = None         # (2^bd,) float32
    tone_knots: tuple = tuple(i / 32.0 for i in range(33))
    out_format: int = abi.OUT_RGB8
    lut3d: Optional[np.ndarray] = None            # (n, n, n, 3) float32, R-major (stage STAGE_LUT3D)
    _keep: list = field(default_factory=list, repr=False)

    # ---- sizes ----------------------------------------------------------------------------
    @property
    def pixels(self) -> int:
        return self.width * self.height

    def input_bytes(self) -> int:
        n = self.pixels
        if self.packed:
            return (n * self.bit_depth + 7) // 8
        return n if self.bit_depth <= 8 else 2 * n

    def output_bytes(self) -> int:
        if self.out_format == abi.OUT_NATIVE and self.bit_depth > 8:
            return self.pixels * 6
        return self.pixels * 3

    def output_shape(self):
        return (self.height, self.width, 3)

    def output_dtype(self):
        if self.out_format == abi.OUT_NATIVE and self.bit_depth > 8:
            return np.uint16
        return np.uint8

    # ---- C struct ---------------------------------------------------------------------------
    def to_c(self) -> abi.IspParams:
        p = abi.IspParams()
        p.width, p.height = self.width, self.height
        p.bit_depth, p.packed = self.bit_depth, int(bool(self.packed))
        p.pattern, p.demosaic = self.pattern, self.demosaic
        p.stages, p.stage_order = self.stages, self.stage_order
        p.bl_mode = self.bl_mode
        for i in range(4):
            p.bl_offset[i] = float(self.bl_offset[i])
        p.dpc_mode, p.dpc_threshold = self.dpc_mode, float(self.dpc_threshold)
        if self.dpc_map is not None and len(self.dpc_map):
            m = np.ascontiguousarray(self.dpc_map, dtype=np.int32).reshape(-1, 2)
            self._keep.append(m)
            p.dpc_map = m.ctypes.data_as(C.POINTER(abi.DefectPoint))
            p.dpc_map_count = m.shape[0]
        p.lsc_mode = self.lsc_mode
        if self.lsc_grid is not None:
            g = np.ascontiguousarray(self.lsc_grid, dtype=np.float32)
            self._keep.append(g)
            p.lsc_grid = g.ctypes.data_as(C.POINTER(C.c_float))
            p.lsc_grid_h, p.lsc_grid_w = g.shape[0], g.shape[1]
        for c in range(4):
            for k in range(3):
                p.lsc_poly[c][k] = float(self.lsc_poly[c][k])
        p.lsc_center[0], p.lsc_center[1] = float(self.lsc_center[0]), float(self.lsc_center[1])
        if self.lsc_flat_field is not None:
            f = np.ascontiguousarray(self.lsc_flat_field)
            self._keep.append(f)
            p.lsc_flat_field = f.ctypes.data
            p.lsc_flat_h, p.lsc_flat_w = f.shape[0], f.shape[1]
        for i in range(3):
            p.wb_gain[i] = float(self.wb_gain[i])
        for i in range(9):
            p.ccm[i] = float(self.ccm[i])
        p.tone_mode = self.tone_mode
        if self.tone_lut is not None:
            t = np.ascontiguousarray(self.tone_lut, dtype=np.float32)
            self._keep.append(t)
            p.tone_lut = t.ctypes.data_as(C.POINTER(C.c_float))
            p.tone_lut_len = t.shape[0]
        for i in range(33):
            p.tone_knots[i] = float(self.tone_knots[i])
        p.out_format = self.out_format
        if self.lut3d is not None:
            lt = np.ascontiguousarray(self.lut3d, dtype=np.float32)
            self._keep.append(lt)
            p.lut3d = lt.ctypes.data_as(C.POINTER(C.c_float))
            p.lut3d_size = lt.shape[0]
        return p
