"""Builds the reference's own MVS unit test against the GB300 binding.

The reference's unmodified tests/unit/test_mvs.cpp is compiled together with
recon-scanner_gb300/bindings/patchmatch_stereo_gb300.cpp (which replaces
core/src/mvs/patchmatch_stereo.cpp), the reference's camera.cpp / linalg.cpp
and librecon_mvs_gb300.so.  The sources come from the reference tree or its
staged copy (oracle.reference_tree()); the binary goes to the package's
_build folder.  Test infrastructure only.
"""
from __future__ import annotations

import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHIM = os.path.join(ROOT, "recon-scanner_gb300", "bindings", "patchmatch_stereo_gb300.cpp")
OUT = os.path.join(ROOT, "recon-scanner_gb300", "_build", "test_mvs_gb300")


def build_reference_unit_test() -> str | None:
    """Path of the built binary, or None when no reference tree is present."""
    import oracle
    import recon_mvs

    ref = oracle.reference_tree()
    if ref is None:
        return None
    lib = recon_mvs.LIB_PATH
    recon_mvs.load_library()
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(ref, "core", "include"), "-I", os.path.join(ROOT, "include"),
           os.path.join(ref, "tests", "unit", "test_mvs.cpp"), SHIM, os.path.join(ref, "core", "src", "util", "camera.cpp"),
           os.path.join(ref, "core", "src", "util", "linalg.cpp"), lib, "-Wl,-rpath," + os.path.dirname(lib), "-o", OUT]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("building the reference unit test failed:\n" + r.stderr[-3000:])
    return OUT
