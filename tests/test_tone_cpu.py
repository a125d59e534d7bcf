"""The reference's RGB tone curves (tone::process_tone) as per-sample tables (imop_tone_table):
every storable sample value through the table equals the reference's own function on a ramp of
all those values (live, where oracle/_ref was built from the reference's sources) and the
reference outputs stored in tests/golden/tone.npz."""
import os

import numpy as np
import pytest

import imop_gb300 as I
import oracle_py as O
from imop_gb300 import abi

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "tone.npz")
CURVES = [abi.TONE_CURVE_GAMMA, abi.TONE_CURVE_S_CURVE, abi.TONE_CURVE_LEVELS, abi.TONE_CURVE_3POINT]


def _params(rng):
    return [float(rng.uniform(0.05, 11.0)), float(rng.uniform(-1.5, 2.5)), float(rng.uniform(-1.2, 1.2)),
            float(rng.uniform(-1.2, 1.2)), float(rng.uniform(-0.1, 1.0)), float(rng.uniform(0.0, 1.1)),
            float(rng.uniform(-0.1, 1.1))]


def _ref_ramp(bd, algo, p):
    """the reference's process_tone on a (n x 1) RGB ramp of every storable sample value"""
    n = 256 if bd <= 8 else 65536
    ramp = np.repeat(np.arange(n, dtype=np.uint16), 3)
    out = np.zeros_like(ramp)
    st = O.ref().ref_tone(ramp.ctypes.data_as(O.U16P), out.ctypes.data_as(O.U16P), n, 1, bd, algo,
                          np.asarray(p, np.float32).ctypes.data_as(O.F32P))
    assert st == 0
    rgb = out.reshape(n, 3)
    assert (rgb[:, 0] == rgb[:, 1]).all() and (rgb[:, 0] == rgb[:, 2]).all()
    return rgb[:, 0]


@pytest.mark.skipif(not O.ref_available(), reason="reference library not built here")
@pytest.mark.parametrize("trial", range(12))
def test_tables_match_reference_live(trial):
    rng = np.random.default_rng(4400 + trial)
    for bd in ([1, 4, 7, 8, 9, 10, 12, 14, 16] if trial == 0 else [int(rng.choice([8, 10, 12, 16]))]):
        for algo in CURVES:
            p = [2.2, 0.4, 0.3, -0.2, 0.05, 0.95, 0.45] if trial == 0 else _params(rng)
            got = I.tone_table(algo, bd, I.tone_params(*p))
            assert np.array_equal(got, _ref_ramp(bd, algo, p)), (bd, algo, p)


def test_tables_match_reference_golden():
    g = np.load(GOLDEN)
    for k in range(int(g["n"])):
        bd, algo = int(g["bd"][k]), int(g["algo"][k])
        got = I.tone_table(algo, bd, I.tone_params(*[float(v) for v in g["params"][k]]))
        assert np.array_equal(got, g[f"table{k}"]), (bd, algo)


def test_luminance_curve_and_bad_arguments_refused():
    p = I.tone_params()
    t = np.zeros(65536, np.uint16)
    L = I.lib()
    import ctypes as C
    assert L.imop_tone_table(abi.TONE_CURVE_SHADOWS_HIGHLIGHTS, 12, C.byref(p), t.ctypes.data, t.size) == abi.ERR_UNSUPPORTED
    assert L.imop_tone_table(abi.TONE_CURVE_GAMMA, 0, C.byref(p), t.ctypes.data, t.size) == abi.ERR_INVALID_BIT_DEPTH
    assert L.imop_tone_table(abi.TONE_CURVE_GAMMA, 12, C.byref(p), t.ctypes.data, 4096) == abi.ERR_INVALID_ARGUMENT
    assert L.imop_tone_table(abi.TONE_CURVE_GAMMA, 12, None, t.ctypes.data, t.size) == abi.ERR_NULL_INPUT
    assert L.imop_tone_table_entries(8) == 256 and L.imop_tone_table_entries(9) == 65536


def test_table_stage_reports_no_device_without_gpu():
    if I.lib().imop_has_cuda() == 1:
        pytest.skip("a GPU is visible")
    t = np.zeros(256, np.uint16)
    img = np.zeros(6 * 6 * 3, np.uint8)
    # no context can be made without a device; the call checks its arguments and the device before
    # it touches the handle, so any non-null handle reaches the device check
    handle = np.zeros(64, np.uint8)
    rc = I.lib().imop_op_rgb_table(handle.ctypes.data, 6, 6, 8, t.ctypes.data, img.ctypes.data, img.ctypes.data)
    assert rc == abi.ERR_NO_DEVICE
