"""CPU: the ctypes mirror of the C ABI has the C header's struct layouts.

A small C program, compiled with the host compiler against
include/recon_mvs_gb300.h, prints sizeof of every public struct and offsetof
of every field; the ctypes classes of recon_mvs.py must agree field by field
(names, order, offsets) and in size -- a field added to one side only would
shift every later field of every call that passes the struct.
"""
import ctypes as C
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

# ctypes class name -> C struct name
PAIRS = {
    "Intrinsics": "recon_camera_intrinsics",
    "Pose": "recon_pose",
    "MvsConfig": "recon_mvs_config",
    "Options": "recon_mvs_options",
    "Views": "recon_mvs_views",
    "DepthMapC": "recon_mvs_depth_map",
    "NccResult": "recon_mvs_ncc_result",
    "PointCloudC": "recon_mvs_point_cloud",
    "DeviceCloudC": "recon_mvs_device_cloud",
    "TsdfConfig": "recon_tsdf_config",
    "Stats": "recon_mvs_stats",
    "StageParams": "recon_mvs_stage_params",
}


@pytest.fixture(scope="module")
def mirror():
    import recon_mvs

    return recon_mvs


@pytest.fixture(scope="module")
def c_layout(mirror, tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no host C compiler")
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "recon_mvs_gb300.h"', "int main(void) {"]
    for py, cname in PAIRS.items():
        cls = getattr(mirror, py)
        lines.append(f'  printf("{py} size %zu\\n", sizeof({cname}));')
        for field in cls._fields_:
            name = field[0]
            lines.append(f'  printf("{py} {name} %zu\\n", offsetof({cname}, {name}));')
    lines += ["  return 0;", "}"]
    d = tmp_path_factory.mktemp("abi")
    src, exe = d / "layout.c", d / "layout"
    src.write_text("\n".join(lines) + "\n")
    r = subprocess.run([cc, "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    table = {}
    for line in out.splitlines():
        cls, key, val = line.split()
        table[(cls, key)] = int(val)
    return table


@pytest.mark.parametrize("py", sorted(PAIRS))
def test_struct_layout_matches_header(mirror, c_layout, py):
    cls = getattr(mirror, py)
    assert C.sizeof(cls) == c_layout[(py, "size")], f"{py}: sizeof differs from {PAIRS[py]}"
    for field in cls._fields_:
        name = field[0]
        assert getattr(cls, name).offset == c_layout[(py, name)], f"{py}.{name}: offset differs"
