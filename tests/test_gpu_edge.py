"""GPU: edge cases of the batched plane-mode path.

Every case runs as one batch and as one launch per view and must give
bit-identical maps: images smaller than a tile or a window, a degenerate job
(zero baseline) inside a batch, a job with zero iterations, mixed window
sizes (two groups in one plan), 32 sources (the maximum; per-thread ray cache
above 48 KB of shared memory), Gauss-Newton refinement on BF16 storage.
The sweep's exact shortcuts (repeated candidates skipped, hopeless windows
pruned) are checked the same way: with and without them the maps are
bit-identical while fewer source windows are sampled.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mvs():
    import recon_mvs

    recon_mvs.load_library()
    return recon_mvs


def views_of(mvs, sc):
    cams = [sc.ref.camera] + [s.camera for s in sc.sources]
    imgs = [sc.ref.image] + [s.image for s in sc.sources]
    return mvs.ViewArgs.from_cameras(imgs[0], imgs[1:], cams[0], cams[1:])


def run(mvs, items, per_view, **opt):
    eng = mvs.Engine(mvs.Options(mode=mvs.MODE_PLANE, best_k=3, device=0, per_view=int(per_view), **opt))
    try:
        jobs = [eng.stage(v, c) for v, c in items]
        eng.run_many(jobs)
        return [eng.download(j) for j in jobs]
    finally:
        eng.close()


def same(a, b):
    for x, y in zip(a, b):
        assert x.filled == y.filled
        np.testing.assert_array_equal(x.depth, y.depth)
        np.testing.assert_array_equal(x.cost, y.cost)
        np.testing.assert_array_equal(x.normal, y.normal)


def scene(w, h, ns, seed):
    import synthetic as S

    return S.sphere_on_backdrop(width=w, height=h, f=150.0 * w / 160, num_sources=ns, seed=seed)


def cfg(mvs, sc, **kw):
    d = dict(min_depth_m=sc.min_depth, max_depth_m=sc.max_depth, iterations=3, patch_size=11)
    d.update(kw)
    return mvs.MvsConfig(**d)


def test_tiny_images_and_zero_iterations(mvs):
    tiny = scene(9, 5, 2, 31)      # smaller than a window and a tile
    small = scene(70, 9, 3, 32)    # ragged: 70 columns, 9 rows
    base = scene(96, 72, 3, 33)
    items = [(views_of(mvs, tiny), cfg(mvs, tiny)), (views_of(mvs, small), cfg(mvs, small)),
             (views_of(mvs, base), cfg(mvs, base, iterations=0))]
    a = run(mvs, items, False)
    b = run(mvs, items, True)
    same(a, b)
    assert a[2].filled > 0  # initialisation + refinement only


def test_degenerate_job_inside_a_batch(mvs):
    good = scene(96, 72, 3, 34)
    bad = scene(96, 72, 3, 35)
    bad_views = views_of(mvs, bad)
    # every source at the reference's own pose: zero baseline
    bad_views = mvs.ViewArgs(bad.ref.image, [s.image for s in bad.sources], bad.ref.camera.pose_array(),
                             [bad.ref.camera.pose_array()] * len(bad.sources), bad.ref.camera.intrinsics_array(),
                             [s.camera.intrinsics_array() for s in bad.sources], list(range(len(bad.sources))))
    items = [(views_of(mvs, good), cfg(mvs, good)), (bad_views, cfg(mvs, bad)),
             (views_of(mvs, good), cfg(mvs, good))]
    a = run(mvs, items, False)
    b = run(mvs, items, True)
    same(a, b)
    assert a[1].filled == 0 and np.all(np.isnan(a[1].depth))
    same([a[0]], [a[2]])


def test_mixed_window_sizes(mvs):
    s1, s2 = scene(96, 72, 3, 36), scene(80, 64, 4, 37)
    items = [(views_of(mvs, s1), cfg(mvs, s1, patch_size=11)), (views_of(mvs, s2), cfg(mvs, s2, patch_size=7)),
             (views_of(mvs, s2), cfg(mvs, s2, patch_size=9))]
    same(run(mvs, items, False), run(mvs, items, True))


@pytest.mark.parametrize("rows", [2, 8])
def test_thirty_two_sources(mvs, rows):
    sc = scene(128, 96, 32, 38)
    items = [(views_of(mvs, sc), cfg(mvs, sc, iterations=2))]
    a = run(mvs, items, False, tile_rows=rows)
    b = run(mvs, items, True, tile_rows=4)
    same(a, b)
    assert a[0].filled > 0.8 * a[0].depth.size


def test_gauss_newton_on_bf16(mvs):
    sc = scene(128, 96, 4, 39)
    items = [(views_of(mvs, sc), cfg(mvs, sc))]
    a = run(mvs, items, False, refine=2, storage=mvs.STORAGE_BF16)
    b = run(mvs, items, True, refine=2, storage=mvs.STORAGE_BF16)
    same(a, b)
    err = np.abs(a[0].depth - sc.ref.depth)[8:-8, 8:-8]
    assert np.nanmedian(err) < 2e-3


@pytest.mark.parametrize("best_k,refine,interp", [(3, 2, 1), (0, 1, 0), (8, 2, 0), (4, 1, 1)])
def test_pruning_is_exact(mvs, best_k, refine, interp):
    import synthetic as S

    cap = S.tabletop(width=240, height=180, f=1450.0 * 240 / 1920, num_sources=8, seed=41)
    sph = scene(128, 96, 4, 42)
    items = [(views_of(mvs, S.as_reference(cap, 0)), cfg(mvs, cap, iterations=4)),
             (views_of(mvs, sph), cfg(mvs, sph, iterations=4))]
    common = dict(mode=mvs.MODE_PLANE, best_k=best_k, device=0, refine=refine, interp=interp,
                  storage=mvs.STORAGE_FP16 if interp else mvs.STORAGE_FP32)
    out, stats = [], []
    for exhaustive in (0, 1):
        eng = mvs.Engine(mvs.Options(exhaustive=exhaustive, **common))
        try:
            jobs = [eng.stage(v, c, undistort=True) for v, c in items]
            eng.run_many(jobs)
            out.append([eng.download(j) for j in jobs])
            stats.append(eng.stats())
        finally:
            eng.close()
    same(out[0], out[1])
    pruned, full = stats[0], stats[1]
    print(f"best_k={best_k}: hypotheses {pruned.hypotheses_evaluated} / {full.hypotheses_evaluated}, windows "
          f"{pruned.windows_evaluated} / {full.windows_evaluated}")
    assert pruned.hypotheses_evaluated <= full.hypotheses_evaluated
    assert pruned.windows_evaluated < full.windows_evaluated
