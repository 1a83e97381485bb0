"""GPU parity: the CUDA engine through its C ABI against the reference's
golden vectors and the CPU oracle.

Tolerances (stated per test):
  * integer/index/byte work and the FP64 paths -- bit-exact;
  * FP32 window costs vs the reference's FP64 -- |dc| <= 1e-5 * |c| + 2e-6
    for at least 99.9 % of hypotheses (the absolute floor covers costs near
    0, where the relative bound is meaningless), and never above 1e-3;
  * whole depth maps (order-dependent searches) -- statistics vs truth.
"""
import numpy as np
import pytest

import golden_io as G
import oracle as O

pytestmark = pytest.mark.gpu

REL, ABS = 1e-5, 2e-6


@pytest.fixture(scope="module")
def mvs():
    import recon_mvs

    recon_mvs.load_library()
    return recon_mvs


def gpu_views(mvs, d, prefix=""):
    return mvs.ViewArgs(d[prefix + "ref"], list(d[prefix + "srcs"]), d[prefix + "ref_pose"], list(d[prefix + "poses"]),
                        d[prefix + "ref_intr"], list(d[prefix + "intr"]), list(d[prefix + "source_indices"]))


def gpu_config(mvs, d):
    return mvs.MvsConfig(**G.config(d))


def assert_costs_close(got, want, label):
    got = np.asarray(got, np.float64)
    want = np.asarray(want, np.float64)
    inf_w = want >= 1e29
    inf_g = got >= 1e29
    mism = (inf_w != inf_g).mean()
    both = ~inf_w & ~inf_g
    err = np.abs(got[both] - want[both])
    ok = err <= REL * np.abs(want[both]) + ABS
    print(f"{label}: n={both.sum()} inf-mismatch={mism:.4%} ok={ok.mean():.5%} "
          f"max|d|={err.max() if err.size else 0:.3e} p99|d|={np.quantile(err, 0.99) if err.size else 0:.3e}")
    assert mism <= 1e-3
    assert ok.mean() >= 0.999
    assert err.max() <= 1e-3


@pytest.mark.parametrize("name", ["eval_plane.npz", "eval_distort.npz"])
def test_compat_cost_matches_reference(mvs, name):
    """EvaluateCandidate (patchmatch_stereo.cpp:344-418) on the reference's
    own hypotheses: translated windows, distortion, both index forms."""
    d = G.load(name)
    cost, sup = mvs.Evaluate(gpu_views(mvs, d), gpu_config(mvs, d), mvs.Options(mode=mvs.MODE_COMPAT),
                             d["px"], d["py"], d["inv"])
    assert_costs_close(cost, d["cost"], name)
    valid = d["cost"] < 1e29
    assert (sup[valid] == d["valid_views"][valid]).mean() >= 0.999


def test_compute_ncc_bit_exact(mvs):
    d = G.load("ncc_known.npz")
    imgs = [d["a"], d["brighter"], d["flat"]]
    for i, ((ri, si), c) in enumerate(zip(d["which"], d["coords"])):
        r = mvs.ComputeNcc(imgs[ri], imgs[si], *c, patch_size=11)
        assert r.valid == d["valid"][i] and r.ncc == d["ncc"][i]
        assert r.weak_texture == d["weak"][i] and r.valid_samples == d["samples"][i]


def plane_hypotheses(sc, n, seed):
    """Seeded plane hypotheses around the analytic truth plus random ones."""
    rng = np.random.default_rng(seed)
    h, w = sc.ref.depth.shape
    px = rng.integers(0, w, n)
    py = rng.integers(0, h, n)
    td = sc.ref.depth[py, px]
    tn = sc.ref.normal[py, px]
    inv = np.where(np.isfinite(td), 1.0 / np.where(np.isfinite(td), td, 1.0), 0.0)
    inv = inv * (1.0 + rng.normal(0, 0.01, n))
    rand = rng.random(n) < 0.3
    inv[rand] = rng.uniform(1 / sc.max_depth, 1 / sc.min_depth, rand.sum())
    nrm = tn + rng.normal(0, 0.1, (n, 3))
    nrm[~np.isfinite(nrm).all(1)] = [0.0, 0.0, -1.0]
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    bad = ~np.isfinite(td)
    inv[bad] = rng.uniform(1 / sc.max_depth, 1 / sc.min_depth, bad.sum())
    return px, py, inv, nrm


def test_plane_cost_matches_fp64_oracle(mvs, orc):
    """Plane-induced homography cost vs the FP64 oracle restatement on
    identical hypotheses (FP32, FP16 and 8-bit storage all hold the 8-bit
    texels exactly; the 8-bit texture reads I / 255, a scale NCC ignores)."""
    import synthetic as S

    sc = S.sphere_on_backdrop(width=160, height=120, f=150.0, num_sources=4, seed=3)
    cams = [sc.ref.camera] + [s.camera for s in sc.sources]
    imgs = [sc.ref.image] + [s.image for s in sc.sources]
    px, py, inv, nrm = plane_hypotheses(sc, 4000, 7)
    cfg_d = dict(min_depth_m=sc.min_depth, max_depth_m=sc.max_depth, patch_size=11)
    vs_o = O.ViewSet(imgs[0], imgs[1:], cams[0], cams[1:])
    for best_k, sampling in ((0, 0), (2, 0), (2, 1)):
        want, want_sup, want_view = orc.plane_costs(vs_o, O.make_config(**cfg_d), best_k, px, py, inv, nrm,
                                                    half_pixel=sampling)
        for storage in (mvs.STORAGE_FP32, mvs.STORAGE_FP16, mvs.STORAGE_U8):
            opts = mvs.Options(mode=mvs.MODE_PLANE, best_k=best_k, storage=storage, sampling=sampling)
            va = mvs.ViewArgs.from_cameras(imgs[0], imgs[1:], cams[0], cams[1:])
            got, sup, view = mvs.Evaluate(va, mvs.MvsConfig(**cfg_d), opts, px, py, inv, nrm.astype(np.float32),
                                          per_view=True)
            assert_costs_close(got, want, f"plane best_k={best_k} storage={storage} sampling={sampling}")
            assert_costs_close(view.ravel(), want_view.ravel(), "per-view")


def test_compat_single_sweep_matches_reference(mvs, orc):
    """One COMPAT direction sweep (iterations = 1, one direction) from the
    reference's own random initialisation: every pixel evaluates the same
    candidates with the same draws, so the GPU map equals the reference's
    (the oracle, bit-exact with it) except where FP32 and FP64 costs order
    two candidates within rounding of each other."""
    d = G.load("pm_plane.npz")
    for dirs, it in ((1, 1), (4, 1)):
        cfg_d = {**G.config(d), "iterations": it, "propagation_directions": dirs}
        want = orc.patchmatch_stereo(G.viewset(d), O.make_config(**cfg_d))
        dm = mvs.PatchMatchStereo(gpu_views(mvs, d), mvs.MvsConfig(**cfg_d), options=mvs.Options(mode=mvs.MODE_COMPAT))
        both = np.isfinite(want.depth) & np.isfinite(dm.depth)
        same = (dm.depth[both] == want.depth[both]).mean()
        print(f"dirs={dirs}: filled {dm.filled} vs {want.filled}, identical {same:.5f}")
        assert abs(dm.filled - want.filled) <= 0.002 * want.filled
        assert same >= (0.995 if dirs == 1 else 0.98)


def test_compat_patchmatch_on_reference_scene(mvs):
    """COMPAT PatchMatchStereo on the reference unit test's plane scene
    against the reference's golden map (2 iterations x 4 directions, 4 row
    blocks): near-ties flipped by FP32 rounding propagate through later
    sweeps, so agreement is statistical; the refined map passes the unit
    test's accuracy gates (test_mvs.cpp:337-466)."""
    d = G.load("pm_plane.npz")
    vs = gpu_views(mvs, d)
    cfg = gpu_config(mvs, d)
    dm = mvs.PatchMatchStereo(vs, cfg, options=mvs.Options(mode=mvs.MODE_COMPAT))
    ref = d["depth"]
    both = np.isfinite(ref) & np.isfinite(dm.depth)
    rel = np.abs(dm.depth[both] - ref[both]) / ref[both]
    print("filled", dm.filled, int(d["filled"]), "identical", (rel == 0).mean(), "within 1%", (rel <= 0.01).mean())
    assert abs(dm.filled - int(d["filled"])) <= 0.01 * d["filled"]
    assert (rel == 0).mean() >= 0.85
    assert (rel <= 0.01).mean() >= 0.97
    n = mvs.RefineSubpixel(vs, cfg, dm, options=mvs.Options(mode=mvs.MODE_COMPAT))
    truth = d["truth"]
    err = (np.abs(dm.depth - truth) * 1000.0)[20:-20, 20:-20]
    err = np.sort(err[np.isfinite(err)])
    med, p95 = err[len(err) // 2], err[int(len(err) * 0.95)]
    gold = (np.abs(d["rdepth"] - truth) * 1000.0)[20:-20, 20:-20]
    gold = np.sort(gold[np.isfinite(gold)])
    print("refined", n, "median mm", med, "p95 mm", p95, "reference", gold[len(gold) // 2],
          gold[int(len(gold) * 0.95)])
    assert med <= 19.1 * 0.15 * 1.5 and p95 <= 19.1 * 0.15 * 3.0


def err_stats(depth, truth, margin):
    e = np.abs(depth.astype(np.float64) - truth)[margin:-margin, margin:-margin]
    t = truth[margin:-margin, margin:-margin]
    rel = (e / t)[np.isfinite(e)]
    return float(np.median(rel)), float(np.quantile(rel, 0.95)), float(np.isfinite(e).mean())


@pytest.mark.parametrize("scene", ["sphere", "plane"])
def test_plane_mode_no_worse_than_reference(mvs, orc, scene):
    """Statistical parity (the depth maps come from different search orders):
    plane mode's median and 95th-percentile depth error vs analytic truth are
    no worse than the reference's own PatchMatchStereo + RefineSubpixel map
    on the same inputs."""
    import synthetic as S

    if scene == "sphere":
        sc = S.sphere_on_backdrop(width=160, height=120, f=150.0, num_sources=4, seed=21)
        cams = [sc.ref.camera] + [s.camera for s in sc.sources]
        imgs = [sc.ref.image] + [s.image for s in sc.sources]
        truth, lo, hi = sc.ref.depth, sc.min_depth, sc.max_depth
        cfg_d = dict(min_depth_m=lo, max_depth_m=hi, iterations=6, patch_size=11, num_threads=4)
    else:
        imgs, cams, truth = S.plane_test_scene()
        truth = truth.astype(np.float64)
        cfg_d = dict(min_depth_m=0.15, max_depth_m=0.80, iterations=3, patch_size=11, num_threads=4,
                     random_search_radius_ratio=0.35, subpixel_iterations=5)
    vs_o = O.ViewSet(imgs[0], imgs[1:], cams[0], cams[1:])
    ocfg = O.make_config(**cfg_d)
    ref_map = orc.refine_subpixel(vs_o, ocfg, orc.patchmatch_stereo(vs_o, ocfg))
    va = mvs.ViewArgs.from_cameras(imgs[0], imgs[1:], cams[0], cams[1:])
    # The reference test's plane texture is aliased (a hash pattern finer than
    # a pixel).  The reference samples both images at half-pixel offsets -- an
    # implicit 2x2 blur; plane mode, which samples pixel centres, is given the
    # engine's symmetric shift-free 3x3 binomial pre-filter for that scene.
    opts = mvs.Options(mode=mvs.MODE_PLANE, best_k=3, prefilter=1 if scene == "plane" else 0)
    dm = mvs.PatchMatchStereo(va, mvs.MvsConfig(**cfg_d), options=opts)
    margin = 12
    r_med, r_p95, r_fill = err_stats(ref_map.depth, truth, margin)
    g_med, g_p95, g_fill = err_stats(dm.depth, truth, margin)
    print(f"{scene}: reference median {r_med:.2e} p95 {r_p95:.2e} fill {r_fill:.3f} | "
          f"plane median {g_med:.2e} p95 {g_p95:.2e} fill {g_fill:.3f}")
    assert g_med <= r_med and g_p95 <= r_p95
    assert g_fill >= r_fill - 0.02


def test_plane_mode_deterministic_and_storage_exact(mvs):
    """Same seed -> identical maps; 8-bit texels are exact in FP16, so FP16
    and FP32 storage give identical maps."""
    import synthetic as S

    sc = S.sphere_on_backdrop(width=128, height=96, f=120.0, num_sources=3, seed=4)
    cams = [sc.ref.camera] + [s.camera for s in sc.sources]
    imgs = [sc.ref.image] + [s.image for s in sc.sources]
    va = mvs.ViewArgs.from_cameras(imgs[0], imgs[1:], cams[0], cams[1:])
    cfg = mvs.MvsConfig(min_depth_m=sc.min_depth, max_depth_m=sc.max_depth, iterations=3)
    a = mvs.PatchMatchStereo(va, cfg, options=mvs.Options(mode=mvs.MODE_PLANE, seed=7))
    b = mvs.PatchMatchStereo(va, cfg, options=mvs.Options(mode=mvs.MODE_PLANE, seed=7))
    c = mvs.PatchMatchStereo(va, cfg, options=mvs.Options(mode=mvs.MODE_PLANE, seed=7, storage=mvs.STORAGE_FP16))
    for x in (b, c):
        assert np.array_equal(a.depth, x.depth, equal_nan=True)
        assert np.array_equal(a.normal, x.normal) and np.array_equal(a.support_count, x.support_count)
    e = mvs.PatchMatchStereo(va, cfg, options=mvs.Options(mode=mvs.MODE_PLANE, seed=8))
    assert not np.array_equal(a.depth, e.depth, equal_nan=True)


def test_compat_refine_matches_reference(mvs, orc):
    """RefineSubpixel on the reference's own PatchMatch output: each pixel
    is independent, so the refined inverse depth must match the reference
    per pixel to within the final golden-section bracket."""
    d = G.load("pm_plane.npz")
    vs = gpu_views(mvs, d)
    cfg = gpu_config(mvs, d)
    dm = mvs.DepthMap(d["depth"].copy(), d["support"].copy(), d["conf"].copy())
    n = mvs.RefineSubpixel(vs, cfg, dm, options=mvs.Options(mode=mvs.MODE_COMPAT))
    assert abs(n - int(d["refined"])) <= 0.001 * d["refined"]
    ref = d["rdepth"]
    both = np.isfinite(ref) & np.isfinite(dm.depth)
    rel = np.abs(dm.depth[both] - ref[both]) / ref[both]
    print("refine: identical", (rel <= 1e-6).mean(), "within 0.5%", (rel <= 5e-3).mean())
    assert (rel <= 1e-6).mean() >= 0.97
    assert (rel <= 5e-3).mean() >= 0.999


def test_fuse_bit_exact(mvs):
    """FuseDepthMaps on the reference's refined maps: the fused cloud is
    bit-identical to the reference's (compared sorted by position)."""
    for name in ("pm_plane.npz", "pm_sphere.npz"):
        d = G.load(name)
        cfg = gpu_config(mvs, d)
        maps = [mvs.DepthMap(d["rdepth"], d["support"], d["rconf"])]
        poses, intr = [d["ref_pose"]], [d["ref_intr"]]
        if "b_depth" in d:
            maps.append(mvs.DepthMap(d["b_depth"], d["b_support"], d["b_conf"]))
            poses.append(d["b_ref_pose"])
            intr.append(d["b_ref_intr"])
        pc = mvs.FuseDepthMaps(maps, poses, intr, cfg)
        order = np.lexsort((pc.positions[:, 2], pc.positions[:, 1], pc.positions[:, 0]))
        pos, nrm, conf = pc.positions[order], pc.normals[order], pc.confidences[order]
        assert len(pos) == int(d["fcount"])
        assert G.digest(pos, nrm, conf) == str(d["fdigest"]), name
        assert pc.counts.sum() > 0


def consistency_maps(sc_views):
    """Truth-derived depth maps with holes and outliers, for consistency tests."""
    rng = np.random.default_rng(5)
    maps = []
    for v in sc_views:
        dd = v.depth.astype(np.float32).copy()
        dd[rng.random(dd.shape) < 0.05] = np.nan
        bad = rng.random(dd.shape) < 0.05
        dd[bad] *= rng.uniform(0.9, 1.1, bad.sum()).astype(np.float32)
        maps.append(dd)
    return maps


def test_geometric_consistency_bit_exact(mvs):
    import synthetic as S

    sc = S.sphere_on_backdrop(width=120, height=90, f=110.0, num_sources=4, seed=8)
    views = [sc.ref] + sc.sources
    depths = consistency_maps(views)
    poses = [v.camera.pose_array() for v in views]
    intr = [v.camera.intrinsics_array() for v in views]
    oracle_maps = [(dd, np.ones(dd.shape, np.uint8), np.ones(dd.shape, np.float32)) for dd in depths]
    gpu_maps = [mvs.DepthMap(dd, np.ones(dd.shape, np.uint8), np.ones(dd.shape, np.float32)) for dd in depths]
    for r in range(len(views)):
        want_c, want_k = O.geo_consistency(oracle_maps, poses, intr, r, 0.01, 1.0, 3)
        got_c, got_k = mvs.GeometricConsistency(gpu_maps, poses, intr, r, 0.01, 1.0, 3)
        assert np.array_equal(got_c, want_c) and np.array_equal(got_k, want_k)
        assert want_k.mean() > 0.3


def test_undistort_bit_exact(mvs, orc):
    import synthetic as S

    sc = S.tabletop(width=192, height=144, f=145.0, num_sources=1, seed=4)
    k = sc.ref.camera.intrinsics_array()
    want = orc.undistort(sc.ref.image, k)
    got = mvs.Undistort(sc.ref.image, k)
    assert np.array_equal(got, want)
    assert np.abs(got - sc.ref.image).mean() > 0.1  # the remap moved pixels


def test_contract_violations(mvs):
    d = G.load("eval_plane.npz")
    cfg = gpu_config(mvs, d)
    bad = mvs.ViewArgs(d["ref"], list(d["srcs"]), d["ref_pose"], list(d["poses"]), d["ref_intr"], list(d["intr"]),
                       [1, 2, 3, 9])
    with pytest.raises(mvs.MvsError) as e:
        mvs.PatchMatchStereo(bad, cfg)
    assert e.value.status == mvs.RECON_ERR_INVALID_ARGUMENT
    bad2 = mvs.ViewArgs(d["ref"], list(d["srcs"]), d["ref_pose"], list(d["poses"]), d["ref_intr"],
                        list(d["intr"])[:3], [1, 2, 3, 4])
    with pytest.raises(mvs.MvsError):
        mvs.PatchMatchStereo(bad2, cfg)
    # images beyond the 32768-pixel side (the texture-gather limit, which
    # also keeps pixel indices in 32 bits) are refused before any device work
    wide = np.zeros((1, 40000), np.uint8)
    bad3 = mvs.ViewArgs(wide, [wide], d["ref_pose"], [d["poses"][1]], d["ref_intr"], [d["intr"][1]], [0])
    with pytest.raises(mvs.MvsError) as e:
        mvs.PatchMatchStereo(bad3, cfg)
    assert e.value.status == mvs.RECON_ERR_INVALID_ARGUMENT
    eng = mvs.Engine(mvs.Options(mode=mvs.MODE_PLANE, device=0))
    with pytest.raises(mvs.MvsError) as e:
        eng.stage_image(wide, d["ref_intr"])
    assert e.value.status == mvs.RECON_ERR_INVALID_ARGUMENT
    eng.close()
    # empty depth range: RECON_OK, nothing filled (patchmatch_stereo.cpp:485)
    cfg2 = gpu_config(mvs, d)
    cfg2.min_depth_m, cfg2.max_depth_m = 0.9, 0.5
    dm = mvs.PatchMatchStereo(gpu_views(mvs, d), cfg2)
    assert dm.filled == 0 and np.isnan(dm.depth).all()


@pytest.mark.parametrize("patch", [11, 7, 9])
def test_sweep_costs_match_independent_evaluation(mvs, patch):
    """The red-black sweep reads the reference window from its shared-memory
    tile (window sizes 7 and 11) or from global memory (other sizes); the
    cost it stores for each pixel must equal an independent evaluation of the
    pixel's final hypothesis through recon_mvs_evaluate."""
    import synthetic as S

    sc = S.sphere_on_backdrop(width=200, height=150, f=190.0, num_sources=4, seed=12)
    cams = [sc.ref.camera] + [s.camera for s in sc.sources]
    imgs = [sc.ref.image] + [s.image for s in sc.sources]
    va = mvs.ViewArgs.from_cameras(imgs[0], imgs[1:], cams[0], cams[1:])
    cfg = mvs.MvsConfig(min_depth_m=sc.min_depth, max_depth_m=sc.max_depth, iterations=2, patch_size=patch)
    opts = mvs.Options(mode=mvs.MODE_PLANE, refine=0, best_k=3)
    dm = mvs.PatchMatchStereo(va, cfg, options=opts)
    ok = np.isfinite(dm.depth) & (dm.cost < 1e29)
    ys, xs = np.nonzero(ok)
    rng = np.random.default_rng(1)
    pick = rng.choice(len(xs), 3000, replace=False)
    px, py = xs[pick], ys[pick]
    inv = 1.0 / dm.depth[py, px].astype(np.float64)
    cost, _ = mvs.Evaluate(va, cfg, opts, px, py, inv, dm.normal[py, px])
    d = np.abs(cost.astype(np.float64) - dm.cost[py, px])
    print(f"patch {patch}: max |d| {d.max():.2e}, p99 {np.quantile(d, 0.99):.2e}")
    assert np.quantile(d, 0.99) < 2e-5 and d.max() < 1e-3


def test_texture_unit_interpolation_cost_error(mvs, orc):
    """interp = 1 trades exact FP32 bilinear weights for the texture unit's
    8-bit fixed-point weights.  Its stated error against the FP64 oracle on
    identical hypotheses: |dc| <= 2e-3 for 99 % of hypotheses, <= 1e-2 for
    all, and no view changes validity beyond 0.1 %."""
    import synthetic as S

    sc = S.sphere_on_backdrop(width=160, height=120, f=150.0, num_sources=4, seed=3)
    cams = [sc.ref.camera] + [s.camera for s in sc.sources]
    imgs = [sc.ref.image] + [s.image for s in sc.sources]
    px, py, inv, nrm = plane_hypotheses(sc, 4000, 9)
    cfg_d = dict(min_depth_m=sc.min_depth, max_depth_m=sc.max_depth, patch_size=11)
    vs_o = O.ViewSet(imgs[0], imgs[1:], cams[0], cams[1:])
    want, _, _ = orc.plane_costs(vs_o, O.make_config(**cfg_d), 0, px, py, inv, nrm)
    va = mvs.ViewArgs.from_cameras(imgs[0], imgs[1:], cams[0], cams[1:])
    for storage in (mvs.STORAGE_FP32, mvs.STORAGE_FP16):
        got, _ = mvs.Evaluate(va, mvs.MvsConfig(**cfg_d), mvs.Options(mode=mvs.MODE_PLANE, best_k=0, interp=1,
                                                                     storage=storage), px, py, inv,
                              nrm.astype(np.float32))
        both = (want < 1e29) & (got < 1e29)
        assert ((want < 1e29) != (got < 1e29)).mean() <= 1e-3
        d = np.abs(got[both] - want[both])
        print(f"interp=1 storage={storage}: p99 |d| {np.quantile(d, 0.99):.2e} max {d.max():.2e}")
        assert np.quantile(d, 0.99) <= 2e-3 and d.max() <= 1e-2
