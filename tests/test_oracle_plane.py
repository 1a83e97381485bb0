"""CPU: properties of the oracle's plane-induced homography cost (the FP64
restatement the device's plane mode is checked against).

  * a plane within ~3 degrees of grazing the pixel ray is not a hypothesis:
    every view and the aggregate are infinite, as on the device;
  * NCC ignores an affine change of a source's intensities;
  * the analytic surface scores better than random planes at the same pixels;
  * best_k = k is the mean of the k lowest view costs;
  * the engine's exact shortcuts, restated in the FP64 search, leave its maps
    bit-identical.
"""
import numpy as np
import pytest

import oracle as O

INF = 1e29


@pytest.fixture(scope="module")
def scene():
    import synthetic as S

    return S.sphere_on_backdrop(width=96, height=72, f=90.0, num_sources=4, seed=51)


def views(sc, srcs=None):
    cams = sc.cameras
    imgs = [sc.ref.image] + (srcs if srcs is not None else [s.image for s in sc.sources])
    return O.ViewSet(imgs[0], imgs[1:], cams[0], cams[1:])


def cfg(sc):
    return O.make_config(min_depth_m=sc.min_depth, max_depth_m=sc.max_depth, patch_size=11)


def interior_truth(sc, n, seed):
    rng = np.random.default_rng(seed)
    h, w = sc.ref.depth.shape
    px = rng.integers(12, w - 12, n)
    py = rng.integers(12, h - 12, n)
    d = sc.ref.depth[py, px]
    nrm = sc.ref.normal[py, px]
    ok = np.isfinite(d) & np.isfinite(nrm).all(1)
    return px[ok], py[ok], 1.0 / d[ok], nrm[ok]


def test_grazing_planes_are_not_hypotheses(orc, scene):
    sc = scene
    cam = sc.ref.camera
    px = np.array([20, 48, 70], np.int32)
    py = np.array([30, 36, 50], np.int32)
    rays = np.stack([(px + 0.5 - cam.cx) / cam.fx, (py + 0.5 - cam.cy) / cam.fy, np.ones(3)], 1)
    rn = np.linalg.norm(rays, axis=1)
    u = rays / rn[:, None]
    # a unit normal at angle a from -u (cos a = -n.u): n.ray = -cos(a) |ray|
    side = np.cross(u, [0.0, 1.0, 0.0])
    side /= np.linalg.norm(side, axis=1, keepdims=True)
    inv = np.full(3, 1.0 / 0.4)
    for cos_a, finite in ((0.049, False), (0.0, False), (0.2, True), (1.0, True)):
        sin_a = np.sqrt(1.0 - cos_a * cos_a)
        nrm = -cos_a * u + sin_a * side
        cost, _, view = orc.plane_costs(views(sc), cfg(sc), 0, px, py, inv, nrm)
        if finite:
            assert np.any(cost < INF), cos_a
        else:
            assert np.all(cost >= INF) and np.all(view >= INF), cos_a


def test_ncc_ignores_affine_intensity_change(orc, scene):
    sc = scene
    px, py, inv, nrm = interior_truth(sc, 300, 1)
    # FP32 source images both times (the oracle's float-image path)
    srcs = [s.image.astype(np.float32) for s in sc.sources]
    vs = O.ViewSet(sc.ref.image.astype(np.float32), srcs, sc.cameras[0], sc.cameras[1:])
    base, _, vb = orc.plane_costs(vs, cfg(sc), 0, px, py, inv, nrm)
    # a darker, lower-contrast first source (exact in FP32)
    srcs = list(srcs)
    srcs[0] = 0.5 * srcs[0] + 40.0
    vs = O.ViewSet(sc.ref.image.astype(np.float32), srcs, sc.cameras[0], sc.cameras[1:])
    got, _, vg = orc.plane_costs(vs, cfg(sc), 0, px, py, inv, nrm)
    ok = (vb[:, 0] < INF) & (vg[:, 0] < INF)
    assert ok.mean() > 0.5
    np.testing.assert_allclose(vg[ok, 0], vb[ok, 0], atol=1e-12)
    np.testing.assert_allclose(vg[:, 1:], vb[:, 1:], atol=0)


def test_truth_beats_random_planes(orc, scene):
    sc = scene
    px, py, inv, nrm = interior_truth(sc, 400, 2)
    truth, _, _ = orc.plane_costs(views(sc), cfg(sc), 2, px, py, inv, nrm)
    rng = np.random.default_rng(3)
    rinv = rng.uniform(1.0 / sc.max_depth, 1.0 / sc.min_depth, len(px))
    rn = rng.normal(0, 1, (len(px), 3))
    rn[:, 2] = -np.abs(rn[:, 2]) - 0.5
    rn /= np.linalg.norm(rn, axis=1, keepdims=True)
    rand, _, _ = orc.plane_costs(views(sc), cfg(sc), 2, px, py, rinv, rn)
    both = (truth < INF) & (rand < INF)
    assert both.mean() > 0.5
    assert np.median(truth[both]) < 0.5 * np.median(rand[both])
    assert np.mean(truth[both] < rand[both]) > 0.9


def test_best_k_is_the_mean_of_the_lowest_views(orc, scene):
    sc = scene
    px, py, inv, nrm = interior_truth(sc, 200, 4)
    for k in (1, 2, 3):
        cost, valid, view = orc.plane_costs(views(sc), cfg(sc), k, px, py, inv, nrm)
        for i in range(len(px)):
            v = np.sort(view[i][view[i] < INF])
            if len(v) == 0:
                assert cost[i] >= INF
                continue
            want = v[: min(k, len(v))].mean()
            assert cost[i] == pytest.approx(want, rel=1e-12, abs=1e-15)
            assert valid[i] == len(v)


@pytest.mark.parametrize("best_k", [0, 2, 3])
def test_exact_shortcuts_leave_the_fp64_search_unchanged(orc, scene, best_k):
    """The engine's shortcuts restated in the FP64 search (a candidate stops
    once its views bound its cost above the pixel's; a repeated propagation
    candidate is skipped): the maps are bit-identical to the full search."""
    sc = scene
    c = O.make_config(min_depth_m=sc.min_depth, max_depth_m=sc.max_depth, iterations=3, patch_size=11,
                      subpixel_iterations=3, num_threads=4)
    full = orc.plane_patchmatch(views(sc), c, best_k=best_k, refine=1, prune=False)
    fast = orc.plane_patchmatch(views(sc), c, best_k=best_k, refine=1, prune=True)
    assert full[0] == fast[0] > 0.5 * sc.ref.depth.size
    for a, b in zip(full[1:], fast[1:]):
        np.testing.assert_array_equal(a, b)


def test_exploration_schedule_in_the_fp64_search(orc, scene):
    """The engine's exploration schedule restated in the FP64 search: a
    cutoff at the iteration count is the full schedule bit for bit (the
    exploration candidates are drawn either way); an early cutoff keeps the
    maps' accuracy against analytic truth."""
    sc = scene
    c = O.make_config(min_depth_m=sc.min_depth, max_depth_m=sc.max_depth, iterations=4, patch_size=11,
                      subpixel_iterations=3, num_threads=4)
    full = orc.plane_patchmatch(views(sc), c, best_k=3, refine=1, prune=True)
    late = orc.plane_patchmatch(views(sc), c, best_k=3, refine=1, prune=True, explore=4)
    for a, b in zip(full, late):
        np.testing.assert_array_equal(a, b)
    early = orc.plane_patchmatch(views(sc), c, best_k=3, refine=1, prune=True, explore=2)
    assert early[0] >= 0.98 * full[0]
    truth = sc.ref.depth

    def med(d):
        ok = np.isfinite(d) & np.isfinite(truth)
        return float(np.median(np.abs(d[ok] - truth[ok]) / truth[ok]))

    assert med(early[1]) <= 1.5 * med(full[1])
