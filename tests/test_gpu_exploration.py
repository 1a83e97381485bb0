"""GPU: the exploration schedule of the plane sweep (options.exploration_iterations).

The exploration candidates -- a uniformly random plane and the current depth
on a fronto-parallel plane -- are drawn in every iteration whatever the
schedule, so a cutoff at or beyond the iteration count gives the maps of the
full schedule bit for bit; an early cutoff (after the coarse level and one
full-resolution iteration) keeps the accuracy against analytic truth.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mvs():
    import recon_mvs

    recon_mvs.load_library()
    return recon_mvs


@pytest.fixture(scope="module")
def sphere():
    import synthetic as S

    return S.sphere_on_backdrop(width=640, height=480, f=600.0, num_sources=4, seed=5)


def run(mvs, sc, explore, coarse=2, iters=6):
    opts = mvs.Options(mode=mvs.MODE_PLANE, best_k=3, device=0, storage=mvs.STORAGE_FP16, interp=1, refine=2,
                       coarse_iterations=coarse, exploration_iterations=explore)
    eng = mvs.Engine(opts)
    try:
        cams = [sc.ref.camera] + [s.camera for s in sc.sources]
        imgs = [sc.ref.image] + [s.image for s in sc.sources]
        v = mvs.ViewArgs.from_cameras(imgs[0], imgs[1:], cams[0], cams[1:])
        cfg = mvs.MvsConfig(min_depth_m=sc.min_depth, max_depth_m=sc.max_depth, iterations=iters, patch_size=11)
        j = eng.stage(v, cfg)
        eng.run(j)
        return eng.download(j), eng.stats()
    finally:
        eng.close()


def rel_err(dm, truth):
    d = dm.depth.astype(np.float64)
    ok = np.isfinite(d) & np.isfinite(truth)
    return np.abs(d[ok] - truth[ok]) / truth[ok]


def test_cutoff_beyond_the_schedule_is_the_full_schedule(mvs, sphere):
    full, _ = run(mvs, sphere, 0)
    late, _ = run(mvs, sphere, 6)
    np.testing.assert_array_equal(late.depth, full.depth)
    np.testing.assert_array_equal(late.cost, full.cost)
    np.testing.assert_array_equal(late.normal, full.normal)


def test_early_cutoff_keeps_accuracy(mvs, sphere):
    full, st_full = run(mvs, sphere, 0)
    early, st_early = run(mvs, sphere, 3)
    truth = sphere.ref.depth
    e_full, e_early = rel_err(full, truth), rel_err(early, truth)
    print(f"median {np.median(e_full):.3e} -> {np.median(e_early):.3e}, p95 {np.quantile(e_full, 0.95):.3e} -> "
          f"{np.quantile(e_early, 0.95):.3e}, hypotheses {st_full.hypotheses_evaluated} -> "
          f"{st_early.hypotheses_evaluated}")
    assert st_early.hypotheses_evaluated < st_full.hypotheses_evaluated
    assert early.filled >= 0.99 * full.filled
    assert np.median(e_early) <= 1.2 * np.median(e_full)
    assert np.quantile(e_early, 0.95) <= 1.2 * np.quantile(e_full, 0.95)


def test_negative_cutoff_is_refused(mvs):
    with pytest.raises(mvs.MvsError) as e:
        mvs.Engine(mvs.Options(mode=mvs.MODE_PLANE, device=0, exploration_iterations=-1))
    assert e.value.status == mvs.RECON_ERR_INVALID_ARGUMENT
