"""The oracle's copy of the workloads' frame generator (oracle/isp_oracle_scene.c) against the
product's (imop_scene_render, imop_scene_defects, imop_pack_mipi): identical bytes, so the timed
CPU baseline renders the same frames without loading the product library."""
import numpy as np
import pytest

import imop_gb300 as I
import oracle_py as O
from imop_gb300 import workloads


@pytest.mark.parametrize("w,h,bd,pat", [(64, 48, 8, 0), (131, 70, 10, 1), (200, 97, 12, 2), (33, 17, 16, 3),
                                        (1006, 758, 12, 0)])
def test_scene_equals_product(w, h, bd, pat):
    a = I.scene(w, h, bd, pat, 77 + w, lo=10, hi=(1 << bd) - 100)
    b = O.scene(w, h, bd, pat, 77 + w, lo=10, hi=(1 << bd) - 100)
    assert a.dtype == b.dtype and np.array_equal(a, b)


def test_defects_and_packing_equal_product():
    assert np.array_equal(I.defects(300, 200, 60, 5), O.defects(300, 200, 60, 5))
    f = I.scene(130, 41, 12, 0, 9)
    for bd in (10, 12):
        g = (f >> (12 - bd)).astype(np.uint16)
        assert np.array_equal(I.pack_mipi(g, bd), O.pack_mipi(g, bd))
    pts = I.defects(130, 41, 20, 3)
    a, b = f.copy(), f.copy()
    assert np.array_equal(I.apply_defects(a, pts, 12), O.apply_defects(b, pts, 12))


def test_c2_frame_without_the_library():
    pl = workloads.c2_pipeline(402, 303)
    pl_o = workloads.c2_pipeline(402, 303, defects=O.defects)
    assert np.array_equal(pl.dpc_map, pl_o.dpc_map)
    assert np.array_equal(workloads.c2_frame(pl, 3), workloads.c2_frame(pl_o, 3, gen=O))


@pytest.mark.skipif(not O.ref_available(), reason="reference library not built here")
def test_reference_chain_equals_oracle_pipeline():
    """The timed reference arm's composition of the reference's own per-module calls (with the
    oracle's restated grid shading, Bayer WB and LUT) gives the oracle pipeline's bytes."""
    pl = workloads.c2_pipeline(402, 303, defects=O.defects)
    pl.dpc_threshold = 0.1
    for k in range(2):
        raw = workloads.c2_frame(pl, k, gen=O)
        want, _ = O.pipeline(pl, raw)
        assert np.array_equal(O.ref_chain(pl, raw), want)
