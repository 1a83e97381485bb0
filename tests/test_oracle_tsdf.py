"""CPU: the oracle's TSDF fusion (oracle/tsdf_oracle.c, a restatement of
core/src/rgbd/tsdf_fusion.cpp and tsdf_internal.h) against the reference.

  * golden vectors recorded from the reference's own code
    (tests/golden/tsdf.npz: the reference TSDF test's tilted wall, three
    frames; a 320x240 sphere capture with holes and low-confidence pixels,
    four frames): pixels fused per frame, the grid (tsdf and weight, by
    digest) and the extracted surface points, bit for bit;
  * the live reference library, where the reference sources are present, on
    a scene outside the fixture (no confidence map, other poses);
  * the extracted points lie on the scene's surfaces.
"""
import ast

import numpy as np
import pytest

import golden_io as G
import oracle as O


def fixture_scene(d, name):
    cfgd = {k: ast.literal_eval(v) for k, v in d[name + "_cfg"]}
    frames = [(d[name + "_depth"][i], d[name + "_conf"][i], d[name + "_w2c"][i], float(d[name + "_unc"][i]))
              for i in range(len(d[name + "_unc"]))]
    return O.tsdf_config(**cfgd), frames


@pytest.mark.parametrize("name", ["wall", "capture"])
def test_oracle_tsdf_matches_reference_goldens(name):
    d = G.load("tsdf.npz")
    cfg, frames = fixture_scene(d, name)
    r = O.tsdf_fuse(cfg, frames)
    assert r["integrated"] == [int(v) for v in d[name + "_integrated"]]
    assert int((r["weight"] > 0).sum()) == int(d[name + "_fused_voxels"])
    assert G.digest(r["tsdf"], r["weight"]) == str(d[name + "_grid_digest"])
    assert len(r["positions"]) == int(d[name + "_count"]) > 1000
    assert G.digest(r["positions"], r["normals"], r["confidences"]) == str(d[name + "_digest"])


def test_oracle_tsdf_matches_live_reference():
    if not O.reference_available():
        pytest.skip("reference sources not present on this host")
    import synthetic as S

    cfgd, frames = S.tsdf_capture(width=200, height=150, f=190.0, n_frames=3, seed=5, voxel=0.003)
    frames = [(dd, None, p, u) for dd, _, p, u in frames]
    cfg = O.tsdf_config(**cfgd)
    a, b = O.tsdf_fuse(cfg, frames), O.tsdf_reference(cfg, frames)
    assert a["integrated"] == b["integrated"]
    assert np.array_equal(a["tsdf"], b["tsdf"]) and np.array_equal(a["weight"], b["weight"])
    for k in ("positions", "normals", "confidences"):
        assert np.array_equal(a[k], b[k]), k


def test_tsdf_points_on_the_surfaces():
    import synthetic as S

    cfgd, frames = S.tsdf_capture(seed=2)
    r = O.tsdf_fuse(O.tsdf_config(**cfgd), frames)
    p = r["positions"]
    d_wall = np.abs(p[:, 2] - 0.45)
    d_sphere = np.abs(np.linalg.norm(p - [0.0, 0.0, 0.35], axis=1) - 0.05)
    dist = np.minimum(d_wall, d_sphere)
    print("points", len(p), "median distance to the surfaces (m)", np.median(dist))
    assert len(p) > 10_000
    # zero crossings are voxel centres: within a voxel of the surface
    assert np.median(dist) < cfgd["voxel_size_m"]
    assert np.mean(dist < 2 * cfgd["voxel_size_m"]) > 0.95
