"""The reference's own MVS unit test, run on the GB300 engine.

tests/unit/test_mvs.cpp of the reference (unmodified: camera model, NCC
known answers, source-view selection, and the plane-scene PatchMatchStereo
+ RefineSubpixel + FuseDepthMaps accuracy gates of test_mvs.cpp:337-466) is
linked against the C++ binding that replaces patchmatch_stereo.cpp and run
as a program; its main (test_mvs.cpp:504-517) returns 0 only when every check
passed.  It runs once with the engine's default plane mode and once with
RECON_MVS_MODE=compat (the reference's own search)."""
import os
import subprocess

import pytest

import ref_unit

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def binary():
    out = ref_unit.build_reference_unit_test()
    if out is None:
        pytest.skip("neither the reference tree nor its staged copy is present")
    return out


@pytest.mark.parametrize("mode", ["plane", "compat"])
def test_reference_unit_test_passes(binary, mode):
    env = dict(os.environ)
    env.pop("RECON_MVS_MODE", None)
    if mode == "compat":
        env["RECON_MVS_MODE"] = "compat"
    r = subprocess.run([binary], capture_output=True, text=True, env=env, timeout=600)
    print(r.stdout[-3000:])
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-2000:]
    assert "全部通过" in r.stdout
