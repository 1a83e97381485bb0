"""GPU: the headline size -- 1920x1440 views, 8 sources, the tabletop
capture -- through properties that do not depend on the size:

  * plane cost vs the FP64 oracle on 20 000 seeded hypotheses spread over
    the full frame (the small-size bound: |dc| <= 1e-5 |c| + 2e-6 for
    99.9 %, never above 1e-3);
  * a batch of two maps equals one launch per map, bit for bit, in the
    chosen form (FP16 storage, texture-unit interpolation, Gauss-Newton
    refinement) on the distorted capture undistorted on the device;
  * the chosen form's map 0 after 8 iterations: median relative depth error
    vs analytic truth <= 0.1 %, Gauss-Newton no worse than golden section,
    and median and P95 no worse than the reference's own algorithm
    (PatchMatchStereo + RefineSubpixel with its parabola fit, restated on
    the device as COMPAT mode) on the same views;
  * consistency counts bit-exact vs the oracle over nine full-size maps
    with distortion, and the fused cloud of three of them point for point
    equal to the oracle's.
"""
import numpy as np
import pytest

import oracle as O
from test_gpu_parity import assert_costs_close, consistency_maps, plane_hypotheses

pytestmark = pytest.mark.gpu

W, H, F = 1920, 1440, 1450.0


@pytest.fixture(scope="module")
def mvs():
    import recon_mvs

    recon_mvs.load_library()
    return recon_mvs


@pytest.fixture(scope="module")
def pinhole():
    import synthetic as S

    return S.tabletop(width=W, height=H, f=F, num_sources=8, k1=0.0, k2=0.0, seed=12, device="cuda:0")


@pytest.fixture(scope="module")
def distorted():
    import synthetic as S

    return S.tabletop(width=W, height=H, f=F, num_sources=8, seed=2, device="cuda:0")


def cfg_of(mvs, sc, iterations=8):
    return mvs.MvsConfig(min_depth_m=sc.min_depth, max_depth_m=sc.max_depth, iterations=iterations, patch_size=11,
                         subpixel_iterations=4)


def chosen(mvs, **kw):
    d = dict(mode=mvs.MODE_PLANE, best_k=3, storage=mvs.STORAGE_FP16, interp=1, refine=2, device=0)
    d.update(kw)
    return mvs.Options(**d)


def run_maps(mvs, scenes, opts, iterations):
    eng = mvs.Engine(opts)
    try:
        jobs = [eng.stage(mvs.ViewArgs.from_cameras(sc.ref.image, [s.image for s in sc.sources], sc.ref.camera,
                                                    [s.camera for s in sc.sources]),
                          cfg_of(mvs, sc, iterations), undistort=True) for sc in scenes]
        eng.run_many(jobs)
        return [eng.download(j) for j in jobs]
    finally:
        eng.close()


def err_stats(depth, truth, margin=16):
    e = np.abs(depth.astype(np.float64) - truth)[margin:-margin, margin:-margin]
    rel = (e / truth[margin:-margin, margin:-margin])[np.isfinite(e)]
    return float(np.median(rel)), float(np.quantile(rel, 0.95))


def test_plane_cost_full_frame(mvs, orc, pinhole):
    sc = pinhole
    cams = sc.cameras
    imgs = [v.image for v in sc.views]
    px, py, inv, nrm = plane_hypotheses(sc, 20_000, 17)
    # the hypotheses the device evaluates: FP32 inverse depth and normal
    inv = inv.astype(np.float32).astype(np.float64)
    nrm = nrm.astype(np.float32).astype(np.float64)
    cfg_d = dict(min_depth_m=sc.min_depth, max_depth_m=sc.max_depth, patch_size=11)
    vs_o = O.ViewSet(imgs[0], imgs[1:], cams[0], cams[1:])
    want, _, want_view = orc.plane_costs(vs_o, O.make_config(**cfg_d), 3, px, py, inv, nrm)
    va = mvs.ViewArgs.from_cameras(imgs[0], imgs[1:], cams[0], cams[1:])
    got, _, view = mvs.Evaluate(va, mvs.MvsConfig(**cfg_d), chosen(mvs, interp=0), px, py, inv,
                                nrm.astype(np.float32), per_view=True)
    assert_costs_close(got, want, "full-frame plane cost")
    assert_costs_close(view.ravel(), want_view.ravel(), "full-frame per-view")


def test_batched_equals_per_view_full_size(mvs, distorted):
    import synthetic as S

    scenes = [S.as_reference(distorted, 0), S.as_reference(distorted, 5)]
    a = run_maps(mvs, scenes, chosen(mvs), 2)
    b = run_maps(mvs, scenes, chosen(mvs, per_view=1), 2)
    for x, y in zip(a, b):
        assert x.filled == y.filled > 0.9 * x.depth.size
        np.testing.assert_array_equal(x.depth, y.depth)
        np.testing.assert_array_equal(x.cost, y.cost)
        np.testing.assert_array_equal(x.normal, y.normal)


def test_accuracy_vs_reference_algorithm_full_size(mvs, distorted):
    import synthetic as S

    sc = S.as_reference(distorted, 0)
    truth = sc.ref.depth
    gn = run_maps(mvs, [sc], chosen(mvs), 8)[0]
    golden = run_maps(mvs, [sc], chosen(mvs, refine=1), 8)[0]
    # the reference's algorithm on the same views: undistorted on the device,
    # rounded to its 8-bit input type, pinhole cameras
    vs = sc.views
    imgs = [np.clip(np.rint(mvs.Undistort(v.image, v.camera.intrinsics_array())), 0, 255).astype(np.uint8)
            for v in vs]
    cams = [v.camera.undistorted() for v in vs]
    va = mvs.ViewArgs.from_cameras(imgs[0], imgs[1:], cams[0], cams[1:])
    copts = mvs.Options(mode=mvs.MODE_COMPAT, device=0)
    ref_map = mvs.PatchMatchStereo(va, cfg_of(mvs, sc), options=copts)
    mvs.RefineSubpixel(va, cfg_of(mvs, sc), ref_map, options=copts)
    g_med, g_p95 = err_stats(gn.depth, truth)
    s_med, s_p95 = err_stats(golden.depth, truth)
    r_med, r_p95 = err_stats(ref_map.depth, truth)
    print(f"median / p95 relative depth error: gauss-newton {g_med:.3e} / {g_p95:.3e}, golden {s_med:.3e} / "
          f"{s_p95:.3e}, reference algorithm {r_med:.3e} / {r_p95:.3e}")
    assert g_med <= 1e-3
    assert g_med <= s_med
    assert g_med <= r_med and g_p95 <= r_p95


def test_consistency_and_fusion_full_size(mvs, distorted):
    views = distorted.views
    depths = consistency_maps(views)
    poses = [v.camera.pose_array() for v in views]
    intr = [v.camera.intrinsics_array() for v in views]
    ones = [np.full(d.shape, 3, np.uint8) for d in depths]
    conf = [np.full(d.shape, 0.9, np.float32) for d in depths]
    oracle_maps = list(zip(depths, ones, conf))
    gpu_maps = [mvs.DepthMap(d, s, c) for d, s, c in zip(depths, ones, conf)]
    for r in (0, 4):
        want_c, want_k = O.geo_consistency(oracle_maps, poses, intr, r, 0.01, 1.0, 3)
        got_c, got_k = mvs.GeometricConsistency(gpu_maps, poses, intr, r, 0.01, 1.0, 3)
        assert np.array_equal(got_c, want_c) and np.array_equal(got_k, want_k)
        assert want_k.mean() > 0.3
    cfg = mvs.MvsConfig(min_depth_m=distorted.min_depth, max_depth_m=distorted.max_depth, fusion_voxel_size_m=0.002)
    ocfg = O.make_config(min_depth_m=distorted.min_depth, max_depth_m=distorted.max_depth,
                         fusion_voxel_size_m=0.002)
    # fusion of the first three maps (the oracle's output buffers grow with
    # the pixel count)
    pos, nrm, cf = O.fuse_depth_maps("oracle", oracle_maps[:3], poses[:3], intr[:3], ocfg)
    pc = mvs.FuseDepthMaps(gpu_maps[:3], poses[:3], intr[:3], cfg)
    order = np.lexsort((pc.positions[:, 2], pc.positions[:, 1], pc.positions[:, 0]))
    print("fused points", len(pos))
    assert len(pos) > 100_000
    np.testing.assert_array_equal(pc.positions[order], pos)
    np.testing.assert_array_equal(pc.normals[order], nrm)
    np.testing.assert_array_equal(pc.confidences[order], cf)
