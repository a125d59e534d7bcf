"""The launch-tuning table (imop_tuning_set / _get) and its JSON form, without a GPU: entries round
trip, out-of-range entries are refused and leave the table unchanged, a table measured on another
device is not applied."""
import json

import pytest

import imop_gb300 as I
from imop_gb300 import abi, tuning


def _entry(**kw):
    e = {"kernel": abi.KERNEL_STREAM, "fmt": 3, "max_width": 4096, "enabled": 1, "band_rows": 32, "seg_percent": 100}
    e.update(kw)
    return e


def test_set_get_roundtrip():
    entries = [_entry(), _entry(kernel=abi.KERNEL_LITE, fmt=-1, max_width=1 << 30, band_rows=24),
               _entry(fmt=0, enabled=0)]
    tuning.set_table(entries)
    try:
        assert tuning.get_table() == entries
    finally:
        tuning.set_table([])
    assert tuning.get_table() == []


@pytest.mark.parametrize("bad", [dict(kernel=0), dict(kernel=3), dict(fmt=4), dict(fmt=-2), dict(max_width=0),
                                 dict(band_rows=3), dict(band_rows=2000), dict(seg_percent=5),
                                 dict(seg_percent=5000)])
def test_out_of_range_refused(bad):
    tuning.set_table([_entry()])
    try:
        with pytest.raises(I.IspError):
            tuning.set_table([_entry(), _entry(**bad)])
        assert tuning.get_table() == [_entry()]
    finally:
        tuning.set_table([])


def test_load_checks_device(tmp_path):
    p = tmp_path / "t.json"
    p.write_text(json.dumps({"device": "some other GPU", "entries": [_entry()]}))
    assert tuning.load(str(p), device_name="NVIDIA GB300") == 0
    assert tuning.get_table() == []
    assert tuning.load(str(p), device_name="some other GPU") == 1
    try:
        assert tuning.get_table() == [_entry()]
    finally:
        tuning.set_table([])
    assert tuning.load(str(tmp_path / "missing.json")) == 0


def test_shipped_table_is_well_formed():
    if not __import__("os").path.exists(tuning.DEFAULT_TABLE):
        pytest.skip("no measured table shipped")
    t = json.load(open(tuning.DEFAULT_TABLE))
    assert t["device"] and t["entries"]
    tuning.set_table(t["entries"])  # every entry in range
    tuning.set_table([])
    for m in t["measurements"]:
        assert m["best"]["ms"] <= m["fixed"]["ms"]
