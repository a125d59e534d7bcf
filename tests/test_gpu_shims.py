"""The C++ entry points with the reference's names and signatures (include/imop_ref_shims.hpp):
each one on seeded frames (3 sizes x bit depths 8/10/12, rotating patterns) against the CPU
oracle, byte for byte; unsupported algorithms return InternalError (the CPU fallback signal)."""
import subprocess

import pytest

from shim_build import build_shim_check

pytestmark = pytest.mark.gpu


def test_reference_shims_match_oracle(tmp_path):
    exe = str(tmp_path / "shim_check")
    r = build_shim_check(exe)
    assert r.returncode == 0, r.stderr
    run = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    print(run.stdout)
    assert run.returncode == 0, run.stdout[-3000:] + run.stderr
    assert "ALL OK" in run.stdout
