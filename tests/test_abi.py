"""CPU checks of the C ABI: the library builds, loads without a GPU and
exports every function include/*.h declares; the configuration and
parameter-registry entry points (host-only) behave like the reference's;
the reference-side C++ binding compiles against the reference's headers and
links the reference's unit test."""
import ctypes as C
import glob
import os
import re
import subprocess

import numpy as np
import pytest

import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def M():
    import recon_mvs

    recon_mvs.load_library()
    return recon_mvs


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        names |= set(re.findall(r"RECON_API\s+[\w\s\*]+?\b(recon_mvs_\w+)\s*\(", text))
    return names


def test_library_exports_every_declared_symbol(M):
    lib = M.load_library()
    names = declared_functions()
    assert len(names) >= 20
    for n in sorted(names):
        assert hasattr(lib, n), n
    # and the Python mirror binds each of them
    assert names <= set(M.exported_symbols())
    assert lib.recon_mvs_abi_version() == 1


def test_config_defaults_match_mvsconfig(M):
    """recon_mvs_config_default == MvsConfig{} (mvs.h:24-67), field by field."""
    c = M.MvsConfig()
    for name, value in O.CONFIG_DEFAULTS.items():
        assert getattr(c, name) == pytest.approx(value), name
    assert C.sizeof(M.MvsConfig) == C.sizeof(O.Config)


def test_param_registry_clamps_and_maps_like_stagemvs(M):
    c = M.MvsConfig()
    c.set_param("mvs_patch_size", 99)  # clamped to [3, 21] (params.cpp:397)
    assert c.patch_size == 21
    c.set_param("mvs_patch_iterations", 0)
    assert c.iterations == 1
    c.set_param("mvs_photo_threshold", 0.35)
    assert c.photo_threshold == pytest.approx(0.35)
    # StageMvs writes the integer radius key into the ratio field (orchestrator.cpp:959-960)
    c.set_param("mvs_patch_random_search_radius", 4)
    assert c.random_search_radius_ratio == 4.0
    c.set_param("mvs_max_depth_m", 9.0)
    assert c.max_depth_m == 5.0
    before = c.patch_size
    c.set_param("mvs_gpu_tile_size", 512)  # registered, not read by StageMvs
    assert c.patch_size == before
    with pytest.raises(M.MvsError) as e:
        c.set_param("not_a_key", 1)
    assert e.value.status == M.RECON_ERR_INVALID_ARGUMENT


@pytest.mark.parametrize("preset,expect", [(0, (7, 3, 5, 1.5)), (1, (7, 3, 5, 1.5)), (2, (11, 6, 8, 2.0))])
def test_presets(M, preset, expect):
    c = M.MvsConfig()
    c.apply_preset(preset)
    assert (c.patch_size, c.iterations, c.num_views, c.max_depth_m) == expect


def test_select_source_views_matches_oracle(M, orc):
    """Host-side SelectSourceViews equals the reference's on its unit-test
    poses and a ring (golden vectors)."""
    import ast

    import golden_io as G

    d = G.load("select.npz")
    cfgs = [ast.literal_eval(s) for s in d["cfgs"]]
    k = 0
    for pose_set, set_cfgs in ((d["poses"], cfgs[:3]), (d["ring"], cfgs[3:])):
        for cd in set_cfgs:
            sel = M.SelectSourceViews(pose_set[0], list(pose_set), [400.0, 400, 80, 60, 0, 0, 0, 0, 0, 160, 120],
                                      M.MvsConfig(**cd))
            assert sel == [int(i) for i in d["sel"][k] if i >= 0]
            k += 1


def test_reference_binding_links():
    """The reference-side binding replaces patchmatch_stereo.cpp: it compiles
    against the reference's own headers and the reference's unmodified unit
    test links against it and the engine library (it runs on the GPU in
    test_gpu_reference_unit.py)."""
    import ref_unit

    out = ref_unit.build_reference_unit_test()
    if out is None:
        pytest.skip("reference tree not present")
    syms = subprocess.run(["nm", "-C", out], capture_output=True, text=True).stdout
    assert "recon::PatchMatchStereo" in syms and "recon_mvs_patchmatch" in syms
