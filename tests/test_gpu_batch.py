"""GPU: the batched plane-mode form.

Many reference views of uneven size, source count and iteration count run
as one batch -- one launch per stage over all of them, the half-sweeps a
persistent kernel, the run captured as a CUDA graph.  Red-black sweeps make
every pixel's result independent of scheduling, so the bar is bit-identity:
every batched map equals the same view run alone, one launch per view,
whatever the autotuner's tile shape.
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

    # uneven sizes (one not a multiple of any tile), source counts and seeds
    specs = [(160, 120, 4, 11, 4), (200, 150, 3, 12, 3), (96, 80, 5, 13, 4), (130, 98, 2, 14, 2)]
    out = []
    for w, h, ns, seed, iters in specs:
        sc = S.sphere_on_backdrop(width=w, height=h, f=150.0 * w / 160, num_sources=ns, seed=seed)
        out.append((sc, iters))
    return out


def views_of(mvs, sc):
    cams = [sc.ref.camera] + [s.camera for s in sc.sources]
    imgs = [sc.ref.image] + [s.image for s in sc.sources]
    return mvs.ViewArgs.from_cameras(imgs[0], imgs[1:], cams[0], cams[1:])


def run_all(mvs, scenes, batched, tile_rows=0, storage=None, interp=0, repeat=1):
    opts = mvs.Options(mode=mvs.MODE_PLANE, best_k=3, device=0, per_view=0 if batched else 1, tile_rows=tile_rows,
                       interp=interp)
    if storage is not None:
        opts.storage = storage
    eng = mvs.Engine(opts)
    try:
        jobs = []
        for sc, iters in scenes:
            cfg = mvs.MvsConfig(min_depth_m=sc.min_depth, max_depth_m=sc.max_depth, iterations=iters, patch_size=11)
            jobs.append(eng.stage(views_of(mvs, sc), cfg))
        for _ in range(repeat):
            eng.run_many(jobs)
        maps = [eng.download(j) for j in jobs]
        return maps, eng.stats()
    finally:
        eng.close()


def assert_same(a, b, label):
    for k, (x, y) in enumerate(zip(a, b)):
        assert x.filled == y.filled, (label, k)
        np.testing.assert_array_equal(x.depth, y.depth, err_msg=f"{label} depth {k}")
        np.testing.assert_array_equal(x.cost, y.cost, err_msg=f"{label} cost {k}")
        np.testing.assert_array_equal(x.normal, y.normal, err_msg=f"{label} normal {k}")
        np.testing.assert_array_equal(x.support_count, y.support_count, err_msg=f"{label} support {k}")


def test_batched_equals_per_view(mvs, scenes):
    single, st1 = run_all(mvs, scenes, batched=False, tile_rows=4)
    batch, st2 = run_all(mvs, scenes, batched=True)
    assert st1.last_run_ms > 0 and st2.last_run_ms > 0 and st2.last_sweep_ms > 0
    print("per-view", st1.last_sweep_launches, "batched", st2.last_sweep_launches, "rows", st2.tile_rows,
          "ctas/SM", st2.ctas_per_sm)
    assert st2.last_sweep_launches == 2 * max(it for _, it in scenes)
    assert st1.last_sweep_launches == 2 * sum(it for _, it in scenes)
    assert st2.graph_launches == 1 and st1.graph_launches == 0
    assert_same(batch, single, "batched vs per-view")
    for m, (sc, _) in zip(batch, scenes):
        assert m.filled > 0.7 * m.depth.size


@pytest.mark.parametrize("rows", [2, 8])
def test_tile_shape_does_not_change_results(mvs, scenes, rows):
    base, _ = run_all(mvs, scenes, batched=True, tile_rows=4)
    other, st = run_all(mvs, scenes, batched=True, tile_rows=rows)
    assert st.tile_rows == rows
    assert_same(other, base, f"rows={rows}")


def test_graph_replay_is_deterministic(mvs, scenes):
    once, _ = run_all(mvs, scenes, batched=True)
    thrice, st = run_all(mvs, scenes, batched=True, repeat=3)
    assert st.graph_launches == 3
    assert_same(thrice, once, "graph replay")


def test_batched_fp16_texture_interp_matches_per_view(mvs, scenes):
    single, _ = run_all(mvs, scenes, batched=False, storage=mvs.STORAGE_FP16, interp=1, tile_rows=4)
    batch, _ = run_all(mvs, scenes, batched=True, storage=mvs.STORAGE_FP16, interp=1)
    assert_same(batch, single, "fp16+interp batched vs per-view")


def test_batch_larger_than_one_table(mvs):
    """More jobs than one launch's job table (64): the batch splits into
    groups, still bit-identical to the per-view runs."""
    import synthetic as S

    sc = S.sphere_on_backdrop(width=64, height=48, f=60.0, num_sources=2, seed=21)
    many = [(sc, 1)] * 70
    single, _ = run_all(mvs, many[:1], batched=False, tile_rows=2)
    batch, st = run_all(mvs, many, batched=True, tile_rows=2)
    assert st.last_sweep_launches == 4  # two groups x one iteration x two colours
    for m in batch:
        np.testing.assert_array_equal(m.depth, single[0].depth)


def test_shared_image_staging_matches_per_job_staging(mvs):
    """A capture staged once (each view the reference of one job and a source
    of the others) gives the same maps as staging every job's images."""
    import synthetic as S

    cap = S.tabletop(width=200, height=150, f=1450.0 * 200 / 1920, num_sources=3, seed=6)
    scenes = [S.as_reference(cap, k) for k in range(len(cap.views))]
    opts = mvs.Options(mode=mvs.MODE_PLANE, best_k=3, device=0)

    def cfg(sc):
        return mvs.MvsConfig(min_depth_m=sc.min_depth, max_depth_m=sc.max_depth, iterations=3, patch_size=11)

    eng = mvs.Engine(opts)
    own = [eng.stage(views_of(mvs, sc), cfg(sc), undistort=True) for sc in scenes]
    eng.run_many(own)
    a = [eng.download(j) for j in own]
    eng.close()
    eng = mvs.Engine(opts)
    ids = [eng.stage_image(v.image, v.camera.intrinsics_array(), undistort=True) for v in cap.views]
    jobs = []
    for k, sc in enumerate(scenes):
        others = [i for i in range(len(cap.views)) if i != k]
        jobs.append(eng.stage_images(ids[k], [ids[i] for i in others], cap.views[k].camera.pose_array(),
                                     [cap.views[i].camera.pose_array() for i in others], cfg(sc)))
    for i in ids:
        eng.release_image(i)  # the jobs keep their images
    eng.run_many(jobs)
    b = [eng.download(j) for j in jobs]
    eng.close()
    assert_same(b, a, "shared staging")


def test_contexts_on_concurrent_host_threads(mvs, scenes):
    """One context per host thread (the boundary's rule): two threads run the
    same batch at the same time on their own contexts and streams; each gets
    the maps of the batch run alone."""
    import threading

    base, _ = run_all(mvs, scenes, batched=True)
    results, errors = [None, None], []

    def worker(i):
        try:
            results[i] = run_all(mvs, scenes, batched=True, repeat=2)[0]
        except Exception as e:  # surfaced on the main thread
            errors.append(e)

    threads = [threading.Thread(target=worker, args=(i,)) for i in range(2)]
    for t in threads:
        t.start()
    for t in threads:
        t.join(300)
    assert not errors, errors
    for r in results:
        assert r is not None
        assert_same(r, base, "concurrent context")
