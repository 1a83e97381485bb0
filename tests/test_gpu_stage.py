"""GPU: the MVS stage over a capture (recon_mvs_stage_run), the batched
restatement of Orchestrator::StageMvs (orchestrator.cpp:942-1071).

Bar: the fused cloud is bit-identical to the same pipeline assembled from
the per-job entry points (SelectSourceViews without the keyframe itself, at
most num_views sources, one PatchMatch job per keyframe, FuseDepthMaps);
cancel and progress callbacks behave as StageMvs's (cancel checked before
each batch -> RECON_ERR_CANCELLED; progress after each batch); fewer than two
keyframes -> RECON_ERR_MVS_NO_DEPTH.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RECON_ERR_CANCELLED = 5
RECON_ERR_MVS_NO_DEPTH = 500


@pytest.fixture(scope="module")
def mvs():
    import recon_mvs

    recon_mvs.load_library()
    return recon_mvs


@pytest.fixture(scope="module")
def capture():
    import synthetic as S

    cap = S.tabletop(width=200, height=150, f=1450.0 * 200 / 1920, num_sources=4, k1=0.0, k2=0.0, seed=8)
    return cap


def cfg_of(mvs, cap):
    return mvs.MvsConfig(min_depth_m=cap.min_depth, max_depth_m=cap.max_depth, iterations=3, patch_size=11,
                         num_views=3, fusion_voxel_size_m=0.002)


def test_stage_run_matches_assembled_pipeline(mvs, capture):
    cams = [v.camera for v in capture.views]
    imgs = [v.image for v in capture.views]
    poses = [c.pose_array() for c in cams]
    intr = [c.intrinsics_array() for c in cams]
    cfg = cfg_of(mvs, capture)
    opts = mvs.Options(mode=mvs.MODE_PLANE, best_k=3, device=0)

    eng = mvs.Engine(opts)
    fractions = []
    cloud, nmaps = eng.stage_run(imgs, poses, intr, cfg, batch_size=2, progress=fractions.append)
    eng.close()

    eng = mvs.Engine(opts)
    maps, mposes, mintr = [], [], []
    for r in range(len(cams)):
        sel = [i for i in mvs.SelectSourceViews(poses[r], poses, intr[r], cfg) if i != r][: cfg.num_views]
        if not sel:
            continue
        views = mvs.ViewArgs.from_cameras(imgs[r], [imgs[i] for i in sel], cams[r], [cams[i] for i in sel])
        j = eng.stage(views, cfg)
        eng.run(j)
        dm = eng.download(j)
        eng.release(j)
        if dm.filled > 0:
            maps.append(dm)
            mposes.append(poses[r])
            mintr.append(intr[r])
    eng.close()
    want = mvs.FuseDepthMaps(maps, mposes, mintr, cfg)
    print("maps", nmaps, "points", cloud.size(), "progress", fractions)
    assert nmaps == len(maps)
    assert cloud.size() == want.size() > 1000
    np.testing.assert_array_equal(cloud.keys, want.keys)
    np.testing.assert_array_equal(cloud.counts, want.counts)
    np.testing.assert_array_equal(cloud.positions, want.positions)
    np.testing.assert_array_equal(cloud.normals, want.normals)
    assert fractions == pytest.approx([2 / nmaps, 4 / nmaps, 1.0])


def test_stage_run_consistency_filter_drops_points(mvs, capture):
    cams = [v.camera for v in capture.views]
    args = ([v.image for v in capture.views], [c.pose_array() for c in cams], [c.intrinsics_array() for c in cams],
            cfg_of(mvs, capture))
    eng = mvs.Engine(mvs.Options(mode=mvs.MODE_PLANE, best_k=3, device=0))
    all_pts, _ = eng.stage_run(*args)
    kept, _ = eng.stage_run(*args, consistency_views=2, rel_depth=0.01, reproj_px=1.0)
    eng.close()
    print("points", all_pts.size(), "consistent", kept.size())
    assert 0 < kept.size() < all_pts.size()


def test_stage_run_cancel_and_no_depth(mvs, capture):
    cams = [v.camera for v in capture.views]
    imgs = [v.image for v in capture.views]
    poses = [c.pose_array() for c in cams]
    intr = [c.intrinsics_array() for c in cams]
    cfg = cfg_of(mvs, capture)
    eng = mvs.Engine(mvs.Options(mode=mvs.MODE_PLANE, best_k=3, device=0))
    with pytest.raises(mvs.MvsError) as e:
        eng.stage_run(imgs, poses, intr, cfg, cancel=lambda: True)
    assert e.value.status == RECON_ERR_CANCELLED
    with pytest.raises(mvs.MvsError) as e:
        eng.stage_run(imgs[:1], poses[:1], intr[:1], cfg)
    assert e.value.status == RECON_ERR_MVS_NO_DEPTH
    # the context stays usable
    cloud, n = eng.stage_run(imgs, poses, intr, cfg)
    eng.close()
    assert n > 0 and cloud.size() > 0


def test_stage_run_plane_normals(mvs, capture):
    """Fused normals from the plane hypotheses: same points, and on the
    table (world z = 0, away from the objects) they point along +z where the
    reference's -ray normals follow the viewing directions."""
    cams = [v.camera for v in capture.views]
    args = ([v.image for v in capture.views], [c.pose_array() for c in cams], [c.intrinsics_array() for c in cams],
            cfg_of(mvs, capture))
    eng = mvs.Engine(mvs.Options(mode=mvs.MODE_PLANE, best_k=3, device=0))
    ray, _ = eng.stage_run(*args)
    pln, _ = eng.stage_run(*args, plane_normals=True)
    eng.close()
    np.testing.assert_array_equal(pln.keys, ray.keys)
    np.testing.assert_array_equal(pln.positions, ray.positions)
    p = pln.positions
    table = (np.abs(p[:, 2]) < 0.001) & (np.hypot(p[:, 0], p[:, 1]) > 0.14)
    ang = lambda n: np.degrees(np.arccos(np.clip(n[table] @ np.array([0.0, 0.0, 1.0]), -1, 1)))
    a_pln, a_ray = np.median(ang(pln.normals)), np.median(ang(ray.normals))
    print("table points", table.sum(), "median angle to +z: plane", a_pln, "ray", a_ray)
    assert table.sum() > 100
    assert a_pln < 5.0 and a_pln < 0.5 * a_ray


def test_bgra_frames(mvs, orc, capture):
    """BgraToGray on the device is bit-identical to the oracle's restatement
    of orchestrator.cpp:53-67 (padded rows included), and a job staged from
    BGRA frames equals the job staged from the host-converted gray images."""
    rng = np.random.default_rng(5)
    frame = rng.integers(0, 256, (37, 53, 4), dtype=np.uint8)
    padded = np.zeros((37, 60, 4), np.uint8)
    padded[:, :53] = frame
    assert np.array_equal(mvs.BgraToGray(padded[:, :53]), orc.bgra_to_gray(padded[:, :53]))
    assert np.array_equal(mvs.BgraToGray(frame), orc.bgra_to_gray(frame))

    cams = [v.camera for v in capture.views]
    # colour frames whose gray image is exactly the capture's image
    bgra = []
    for v in capture.views:
        g = v.image.astype(np.int32)
        f = np.stack([g, g, g, np.full_like(g, 255)], -1).astype(np.uint8)
        assert np.array_equal(orc.bgra_to_gray(f), (g * 256 >> 8).astype(np.uint8))
        bgra.append(f)
    cfg = cfg_of(mvs, capture)
    opts = mvs.Options(mode=mvs.MODE_PLANE, best_k=3, device=0)
    maps = []
    for use_bgra in (False, True):
        eng = mvs.Engine(opts)
        ids = [eng.stage_image_bgra(f, c.intrinsics_array()) if use_bgra else
               eng.stage_image(orc.bgra_to_gray(f), c.intrinsics_array()) for f, c in zip(bgra, cams)]
        j = eng.stage_images(ids[0], ids[1:], cams[0].pose_array(), [c.pose_array() for c in cams[1:]], cfg)
        eng.run(j)
        maps.append(eng.download(j))
        eng.close()
    np.testing.assert_array_equal(maps[0].depth, maps[1].depth)
    np.testing.assert_array_equal(maps[0].cost, maps[1].cost)


def test_stage_run_device_cloud(mvs, capture):
    """recon_mvs_stage_run_device keeps the fused cloud in device memory for
    the next stage on the GPU: downloaded, it equals recon_mvs_stage_run's
    cloud bit for bit; its Poisson weights are max(0, confidence)
    (UnifiedPointCloud::ToOrientedCloud), its colours zero and its bounds the
    positions' min / max (PointCloudBounds); torch reads its arrays in place."""
    import torch

    cams = [v.camera for v in capture.views]
    imgs = [v.image for v in capture.views]
    poses = [c.pose_array() for c in cams]
    intr = [c.intrinsics_array() for c in cams]
    cfg = cfg_of(mvs, capture)
    eng = mvs.Engine(mvs.Options(mode=mvs.MODE_PLANE, best_k=3, device=0))
    try:
        want, n_want = eng.stage_run(imgs, poses, intr, cfg, consistency_views=2, plane_normals=True)
        dc, n_got = eng.stage_run_device(imgs, poses, intr, cfg, consistency_views=2, plane_normals=True)
        assert n_got == n_want and dc.count == want.size() > 1000 and dc.c.device == 0
        got = dc.download()
        for name in ("positions", "normals", "confidences", "keys", "counts", "colors"):
            np.testing.assert_array_equal(getattr(got, name), getattr(want, name), err_msg=name)
        pos = torch.as_tensor(dc.array("positions"), device="cuda")
        conf = torch.as_tensor(dc.array("confidences"), device="cuda")
        w = torch.as_tensor(dc.array("weights"), device="cuda")
        col = torch.as_tensor(dc.array("colors"), device="cuda")
        assert pos.shape == (dc.count, 3) and pos.dtype == torch.float64
        np.testing.assert_array_equal(pos.cpu().numpy(), want.positions)
        np.testing.assert_array_equal(w.cpu().numpy(), np.maximum(0.0, want.confidences))
        assert torch.equal(w, torch.clamp(conf, min=0.0))
        assert int(torch.count_nonzero(col)) == 0
        lo, hi = dc.bounds
        np.testing.assert_array_equal(lo, want.positions.min(0))
        np.testing.assert_array_equal(hi, want.positions.max(0))
        dc.free()
        assert dc.c.impl is None and dc.count == 0
    finally:
        eng.close()
