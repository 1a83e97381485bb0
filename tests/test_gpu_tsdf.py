"""GPU: TSDF fusion on the device (recon_tsdf_*), the reference's TsdfVolume
(core/src/rgbd/tsdf_fusion.cpp) with its grid in HBM.

Bar: bit for bit -- pixels fused per frame, the whole grid (tsdf and
weight) and the extracted surface points (positions, normals, confidences,
in the reference's (iz, iy, ix) order) equal the reference's goldens and the
oracle's results, including frames without a confidence map, with holes,
low-confidence and out-of-range pixels, and an empty frame.
"""
import ast

import numpy as np
import pytest

import golden_io as G
import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mvs():
    import recon_mvs

    recon_mvs.load_library()
    return recon_mvs


def gpu_fuse(mvs, cfgd, frames):
    vol = mvs.TsdfVolume(mvs.TsdfConfig(**cfgd))
    try:
        integ = [vol.IntegrateDepthFrame(d, c, p, u) for d, c, p, u in frames]
        t, w = vol.grid()
        pc = vol.ExtractPoints()
        return dict(integrated=integ, tsdf=t, weight=w, positions=pc.positions, normals=pc.normals,
                    confidences=pc.confidences, keys=pc.keys, dims=vol.dims())
    finally:
        vol.close()


@pytest.mark.parametrize("name", ["wall", "capture"])
def test_tsdf_matches_reference_goldens(mvs, name):
    d = G.load("tsdf.npz")
    cfgd = {k: ast.literal_eval(v) for k, v in d[name + "_cfg"]}
    frames = [(d[name + "_depth"][i], d[name + "_conf"][i], d[name + "_w2c"][i], float(d[name + "_unc"][i]))
              for i in range(len(d[name + "_unc"]))]
    r = gpu_fuse(mvs, cfgd, frames)
    assert r["integrated"] == [int(v) for v in d[name + "_integrated"]]
    assert G.digest(r["tsdf"], r["weight"]) == str(d[name + "_grid_digest"])
    assert len(r["positions"]) == int(d[name + "_count"])
    assert G.digest(r["positions"], r["normals"], r["confidences"]) == str(d[name + "_digest"])


def test_tsdf_matches_oracle_at_capture_size(mvs):
    """640x480 frames into a 2 mm grid (16 M voxels), one frame without a
    confidence map, one empty, one entirely beyond max_depth."""
    import synthetic as S

    cfgd, frames = S.tsdf_capture(width=640, height=480, f=600.0, n_frames=4, seed=9, voxel=0.002,
                                  truncation=0.01)
    frames[1] = (frames[1][0], None, frames[1][2], frames[1][3])
    empty = (np.zeros_like(frames[0][0]), frames[0][1], frames[0][2], 0.003)
    far = (np.full_like(frames[0][0], 2500), frames[0][1], frames[0][2], 0.003)
    frames = frames + [empty, far]
    cfg = O.tsdf_config(**cfgd)
    want = O.tsdf_fuse(cfg, frames)
    got = gpu_fuse(mvs, cfgd, frames)
    print("dims", got["dims"], "integrated", got["integrated"], "points", len(got["positions"]))
    assert got["dims"] == O.tsdf_dims(cfg)
    assert got["integrated"] == want["integrated"] and got["integrated"][-2:] == [0, 0]
    np.testing.assert_array_equal(got["tsdf"], want["tsdf"])
    np.testing.assert_array_equal(got["weight"], want["weight"])
    for k in ("positions", "normals", "confidences"):
        np.testing.assert_array_equal(got[k], want[k], err_msg=k)
    np.testing.assert_array_equal(got["keys"], want["voxel_index"])
    assert len(got["positions"]) > 20_000


def test_tsdf_empty_volume_and_errors(mvs):
    import recon_mvs

    vol = mvs.TsdfVolume(mvs.TsdfConfig(voxel_size_m=0.01, fx=100.0, fy=100.0))
    try:
        dims = vol.dims()
        assert dims == O.tsdf_dims(O.tsdf_config(voxel_size_m=0.01, fx=100.0, fy=100.0))
        assert vol.ExtractPoints().size() == 0
        assert vol.MemoryUsageBytes() == dims[0] * dims[1] * dims[2] * 8
    finally:
        vol.close()
    with pytest.raises(recon_mvs.MvsError):
        mvs.TsdfVolume(mvs.TsdfConfig(voxel_size_m=0.0005, bbox_max_x=2.0, bbox_max_y=2.0, bbox_max_z=2.0))
