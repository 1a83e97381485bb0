"""GPU: the staged-window schedule of the plane sweep.

With exact interpolation a warp may read the source windows its pixels share
from a box it copies into shared memory by TMA instead of from the texture
(options.window_staging).  Both read the same texels and do the same FP32
arithmetic, so the bar is bit-identity: every map of the staged schedule
equals the texture schedule's, for every tile shape, storage format and
window size, and on the full-size tabletop capture -- and the staged run did
read windows from its boxes.
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
def scenes():
    import synthetic as S

    specs = [(160, 120, 4, 21, 4), (200, 150, 3, 22, 3), (96, 80, 5, 23, 4), (130, 98, 2, 24, 2)]
    return [(S.sphere_on_backdrop(width=w, height=h, f=150.0 * w / 160, num_sources=ns, seed=seed), iters)
            for w, h, ns, seed, iters in specs]


def views_of(mvs, sc):
    cams = [sc.ref.camera] + [s.camera for s in sc.sources]
    imgs = [sc.ref.image] + [s.image for s in sc.sources]
    return mvs.ViewArgs.from_cameras(imgs[0], imgs[1:], cams[0], cams[1:])


def run_all(mvs, scenes, staging, tile_rows=0, storage=None, patch=11):
    opts = mvs.Options(mode=mvs.MODE_PLANE, best_k=3, device=0, tile_rows=tile_rows, interp=0,
                       window_staging=staging)
    if storage is not None:
        opts.storage = storage
    eng = mvs.Engine(opts)
    try:
        jobs = []
        for sc, iters in scenes:
            cfg = mvs.MvsConfig(min_depth_m=sc.min_depth, max_depth_m=sc.max_depth, iterations=iters,
                                patch_size=patch)
            jobs.append(eng.stage(views_of(mvs, sc), cfg))
        eng.run_many(jobs)
        return [eng.download(j) for j in jobs], eng.stats()
    finally:
        eng.close()


def assert_same(a, b, label):
    for k, (x, y) in enumerate(zip(a, b)):
        assert x.filled == y.filled, (label, k)
        np.testing.assert_array_equal(x.depth, y.depth, err_msg=f"{label} depth {k}")
        np.testing.assert_array_equal(x.cost, y.cost, err_msg=f"{label} cost {k}")
        np.testing.assert_array_equal(x.normal, y.normal, err_msg=f"{label} normal {k}")
        np.testing.assert_array_equal(x.support_count, y.support_count, err_msg=f"{label} support {k}")


@pytest.mark.parametrize("rows", [2, 4, 8])
def test_staged_equals_texture_reads(mvs, scenes, rows):
    tex, st_t = run_all(mvs, scenes, staging=1, tile_rows=rows)
    box, st_b = run_all(mvs, scenes, staging=2, tile_rows=rows)
    assert st_t.window_staging == 0 and st_t.windows_staged == 0
    assert st_b.window_staging == 1
    print(f"rows={rows}: windows {st_b.windows_evaluated}, staged {st_b.windows_staged} "
          f"({st_b.windows_staged / max(st_b.windows_evaluated, 1):.1%})")
    assert st_b.windows_staged > 0
    assert st_b.windows_evaluated == st_t.windows_evaluated
    assert_same(box, tex, f"staged rows={rows}")


def test_staged_fp16_and_7x7(mvs, scenes):
    for storage, patch in ((mvs.STORAGE_FP16, 11), (mvs.STORAGE_FP32, 7)):
        tex, _ = run_all(mvs, scenes, staging=1, storage=storage, patch=patch)
        box, st = run_all(mvs, scenes, staging=2, storage=storage, patch=patch)
        assert st.window_staging == 1 and st.windows_staged > 0
        assert_same(box, tex, f"storage={storage} patch={patch}")


def test_autotuned_schedule_equals_texture_reads(mvs, scenes):
    tex, _ = run_all(mvs, scenes, staging=1)
    auto, st = run_all(mvs, scenes, staging=0)
    assert st.window_staging in (0, 1)
    assert_same(auto, tex, "autotuned schedule")


def test_staged_fullsize_tabletop(mvs):
    """Two tabletop scenes at 1920x1440, 8 sources each, distorted and
    undistorted on the device, FP16 storage with Gauss-Newton refinement:
    the staged schedule's maps equal the texture schedule's bit for bit."""
    import synthetic as S

    scenes = [S.tabletop(width=1920, height=1440, f=1450.0, num_sources=8, seed=s, device="cuda:0") for s in (31, 32)]
    out = {}
    for staging in (1, 2):
        opts = mvs.Options(mode=mvs.MODE_PLANE, storage=mvs.STORAGE_FP16, best_k=4, refine=2, device=0, interp=0,
                           window_staging=staging)
        eng = mvs.Engine(opts)
        try:
            jobs = [eng.stage(views_of(mvs, sc),
                              mvs.MvsConfig(min_depth_m=sc.min_depth, max_depth_m=sc.max_depth, iterations=4,
                                            patch_size=11), undistort=True) for sc in scenes]
            eng.run_many(jobs)
            out[staging] = ([eng.download(j) for j in jobs], eng.stats())
        finally:
            eng.close()
    (tex, _), (box, st) = out[1], out[2]
    print(f"full size: windows {st.windows_evaluated}, staged {st.windows_staged} "
          f"({st.windows_staged / max(st.windows_evaluated, 1):.1%})")
    assert st.window_staging == 1 and st.windows_staged > 0
    assert_same(box, tex, "full-size staged")


def test_staging_option_checks(mvs):
    bad = (dict(window_staging=3), dict(window_staging=-1), dict(window_staging=2, interp=1),
           dict(window_staging=2, storage=mvs.STORAGE_BF16), dict(window_staging=2, storage=mvs.STORAGE_U8))
    for kw in bad:
        with pytest.raises(mvs.MvsError) as e:
            mvs.Engine(mvs.Options(mode=mvs.MODE_PLANE, device=0, **kw))
        assert e.value.status == mvs.RECON_ERR_INVALID_ARGUMENT, kw
