"""GPU: storage precision (FP32 / FP16 / BF16 source textures) against the
FP64 oracle run of the same search.

The scene has Brown-Conrady distortion, so the engine undistorts on the
device and the textures hold fractional intensities: FP16 (11-bit mantissa)
and BF16 (8-bit) storage then round them.  The oracle runs the same
plane-mode search (same random streams, same schedule) with FP64 costs on
the same undistorted intensities (orc_undistort is bit-identical to the
device remap).  Reported per form: median / P95 relative depth difference
and normal angle to the FP64 run, and the error against analytic truth.

Bounds (interior pixels valid in both runs):
  * FP32:  median relative depth difference <= 2e-5, normal angle <= 0.05 deg
  * FP16:  median <= 5e-5;  BF16 (an ablation): median <= 1e-3
  * 8-bit (the bandwidth floor: undistorted intensities rounded to 8 bits):
    median <= 1e-3, error vs truth within 25 % of the FP64 run's
  * every other form's median error vs truth within 10 % of the FP64 run's.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

BORDER = 8


@pytest.fixture(scope="module")
def mvs():
    import recon_mvs

    recon_mvs.load_library()
    return recon_mvs


@pytest.fixture(scope="module")
def scene():
    import synthetic as S

    return S.tabletop(width=240, height=180, f=1450.0 * 240 / 1920, num_sources=8, seed=5, baseline=(0.04, 0.16))


def cfg_kw(sc):
    return dict(min_depth_m=sc.min_depth, max_depth_m=sc.max_depth, iterations=4, patch_size=11,
                subpixel_iterations=4)


@pytest.fixture(scope="module")
def fp64_run(orc, scene):
    import oracle as O

    cams = scene.cameras
    imgs = [scene.ref.image] + [s.image for s in scene.sources]
    und = [orc.undistort(im, c.intrinsics_array()) for im, c in zip(imgs, cams)]
    pin = [c.undistorted() for c in cams]
    vs = O.ViewSet(und[0], und[1:], pin[0], pin[1:])
    cfg = O.make_config(num_threads=0, **cfg_kw(scene))
    filled, depth, normal, cost = orc.plane_patchmatch(vs, cfg, best_k=4, seed=0x5DEECE66D, refine=1)
    assert filled > 0.8 * depth.size
    return depth, normal


def gpu_run(mvs, scene, storage, interp=0):
    cams = scene.cameras
    imgs = [scene.ref.image] + [s.image for s in scene.sources]
    views = mvs.ViewArgs.from_cameras(imgs[0], imgs[1:], cams[0], cams[1:])
    opts = mvs.Options(mode=mvs.MODE_PLANE, best_k=4, storage=storage, interp=interp, device=0)
    eng = mvs.Engine(opts)
    try:
        job = eng.stage(views, mvs.MvsConfig(**cfg_kw(scene)), undistort=True)
        eng.run(job)
        return eng.download(job)
    finally:
        eng.close()


def compare(dm, fp64, truth, label):
    d64, n64 = fp64
    sl = np.s_[BORDER:-BORDER, BORDER:-BORDER]
    a, b, t = dm.depth[sl].astype(np.float64), d64[sl].astype(np.float64), truth[sl]
    ok = np.isfinite(a) & np.isfinite(b) & np.isfinite(t)
    rel = np.abs(a[ok] - b[ok]) / b[ok]
    na, nb = dm.normal[sl][ok].astype(np.float64), n64[sl][ok].astype(np.float64)
    cosang = np.clip(np.sum(na * nb, -1) / (np.linalg.norm(na, axis=-1) * np.linalg.norm(nb, axis=-1)), -1, 1)
    ang = np.degrees(np.arccos(cosang))
    err_g = np.abs(a[ok] - t[ok]) / t[ok]
    err_o = np.abs(b[ok] - t[ok]) / t[ok]
    stats = dict(median_rel=float(np.median(rel)), p95_rel=float(np.quantile(rel, 0.95)),
                 same=float(np.mean(rel < 1e-6)), median_deg=float(np.median(ang)),
                 p95_deg=float(np.quantile(ang, 0.95)), truth_median=float(np.median(err_g)),
                 fp64_truth_median=float(np.median(err_o)), n=int(ok.sum()))
    print(label, stats)
    return stats


def test_fp32_tracks_fp64_run(mvs, scene, fp64_run):
    s = compare(gpu_run(mvs, scene, mvs.STORAGE_FP32), fp64_run, scene.ref.depth, "fp32")
    assert s["n"] > 0.8 * (scene.ref.depth.size)
    assert s["median_rel"] <= 2e-5
    assert s["median_deg"] <= 0.05
    assert s["truth_median"] <= 1.1 * s["fp64_truth_median"]


@pytest.mark.parametrize("form", ["fp16", "bf16", "fp16_texinterp", "u8", "u8_texinterp"])
def test_reduced_storage_vs_fp64_run(mvs, scene, fp64_run, form):
    storage = {"fp16": mvs.STORAGE_FP16, "bf16": mvs.STORAGE_BF16, "fp16_texinterp": mvs.STORAGE_FP16,
               "u8": mvs.STORAGE_U8, "u8_texinterp": mvs.STORAGE_U8}[form]
    s = compare(gpu_run(mvs, scene, storage, interp=int(form.endswith("texinterp"))), fp64_run, scene.ref.depth, form)
    # 8-bit storage rounds the undistorted intensities: the bandwidth floor,
    # not a precision form
    bound = {"fp16": 5e-5, "bf16": 1e-3, "fp16_texinterp": 2e-4, "u8": 1e-3, "u8_texinterp": 1e-3}[form]
    assert s["median_rel"] <= bound
    assert s["truth_median"] <= (1.25 if form.startswith("u8") else 1.1) * s["fp64_truth_median"]


def test_bf16_rejects_texture_interpolation(mvs):
    with pytest.raises(mvs.MvsError):
        mvs.Engine(mvs.Options(mode=mvs.MODE_PLANE, storage=mvs.STORAGE_BF16, interp=1, device=0))


def test_u8_needs_plane_mode(mvs):
    with pytest.raises(mvs.MvsError):
        mvs.Engine(mvs.Options(mode=mvs.MODE_COMPAT, storage=mvs.STORAGE_U8, device=0))
