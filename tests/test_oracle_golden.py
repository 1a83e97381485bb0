"""Pin the CPU oracle (oracle/mvs_oracle.c) to the reference.

The golden vectors in tests/golden were produced by the reference's own
sources (tests/golden/make_golden.py).  The restatement must reproduce them
bit for bit: it keeps the reference's FP64 evaluation order.  Mirrors the
reference unit test (tests/unit/test_mvs.cpp) case by case.
"""
import numpy as np
import pytest

import golden_io as G
import oracle as O


def test_ncc_known_answers(orc):
    """ComputeNcc: identical windows -> 1, +40 brightness -> 1 (zero mean),
    flat window -> weak texture (test_mvs.cpp:259-293), then 60 random
    sub-pixel windows, all bit-exact with the reference."""
    d = G.load("ncc_known.npz")
    imgs = [d["a"], d["brighter"], d["flat"]]
    for i, ((ri, si), (ru, rv, su, sv)) in enumerate(zip(d["which"], d["coords"])):
        r = orc.compute_ncc(imgs[ri], imgs[si], ru, rv, su, sv, 11)
        assert r.valid == d["valid"][i]
        assert r.ncc == d["ncc"][i]
        assert r.weak_texture == d["weak"][i]
        assert r.valid_samples == d["samples"][i]
    same = orc.compute_ncc(imgs[0], imgs[0], 32.0, 32.0, 32.0, 32.0, 11)
    assert same.valid and abs(same.ncc - 1.0) < 1e-6 and not same.weak_texture
    shifted = orc.compute_ncc(imgs[0], imgs[1], 32.0, 32.0, 32.0, 32.0, 11)
    assert shifted.valid and abs(shifted.ncc - 1.0) < 1e-6
    assert orc.compute_ncc(imgs[2], imgs[0], 32.0, 32.0, 32.0, 32.0, 11).weak_texture


def test_camera_round_trip(orc):
    """Distortion round trip < 1e-6 px and the reference's exact rays and
    projections (test_mvs.cpp:210-253)."""
    d = G.load("camera.npz")
    worst = 0.0
    for (u, v), ray, proj in zip(d["uv"], d["rays"], d["proj"]):
        r = orc.pixel_to_ray(d["intr"], u, v)
        assert np.array_equal(r, ray)
        ok, u2, v2 = orc.project_point(d["intr"], r)
        assert ok and u2 == proj[0] and v2 == proj[1]
        worst = max(worst, float(np.hypot(u2 - u, v2 - v)))
    assert worst < 1e-6
    assert not orc.project_point(d["intr"], np.array([0.0, 0.0, -1.0]))[0]


@pytest.mark.parametrize("name", ["eval_plane.npz", "eval_distort.npz"])
def test_evaluate_candidate_bit_exact(orc, name):
    d = G.load(name)
    vs = G.viewset(d)
    cfg = O.make_config(**G.config(d))
    cost, vv = orc.evaluate_candidates(vs, cfg, d["px"], d["py"], d["inv"])
    assert np.array_equal(cost, d["cost"])
    assert np.array_equal(vv, d["valid_views"])
    assert (cost < 1e29).sum() > len(cost) // 4


def test_patchmatch_refine_fuse_plane(orc):
    """PatchMatchStereo (2 iterations x 4 directions, 4 row blocks),
    RefineSubpixel and FuseDepthMaps on the unit test's plane scene."""
    d = G.load("pm_plane.npz")
    vs = G.viewset(d)
    cfg = O.make_config(**G.config(d))
    pm = orc.patchmatch_stereo(vs, cfg)
    assert pm.filled == d["filled"]
    assert np.array_equal(pm.depth, d["depth"], equal_nan=True)
    assert np.array_equal(pm.support, d["support"])
    assert np.array_equal(pm.confidence, d["conf"])
    rf = orc.refine_subpixel(vs, cfg, pm)
    assert rf.filled == d["refined"]
    assert np.array_equal(rf.depth, d["rdepth"], equal_nan=True)
    assert np.array_equal(rf.confidence, d["rconf"])
    pos, nrm, conf = O.fuse_depth_maps("oracle", [(rf.depth, rf.support, rf.confidence)], [d["ref_pose"]],
                                       [d["ref_intr"]], cfg)
    assert len(pos) == d["fcount"] and G.digest(pos, nrm, conf) == str(d["fdigest"])
    # the reference test's accuracy gates (test_mvs.cpp:337-466)
    truth = d["truth"]
    err = (np.abs(rf.depth - truth) * 1000.0)[20:-20, 20:-20]
    err = np.sort(err[np.isfinite(err)])
    assert pm.filled > truth.size * 0.5
    assert err[len(err) // 2] <= 19.1 * 0.15 * 1.5
    assert err[int(len(err) * 0.95)] <= 19.1 * 0.15 * 3.0
    assert len(pos) > 1000


def test_patchmatch_seeded_two_map_fusion(orc):
    """Sparse seeding, 7x7 window, restart ratio 0.2, 3 row blocks, the
    relative-intrinsics and global-intrinsics index forms, two-map fusion
    with the photometric filter."""
    d = G.load("pm_sphere.npz")
    cfg = O.make_config(**G.config(d))
    vs = G.viewset(d)
    pm = orc.patchmatch_stereo(vs, cfg, seeds=d["seeds"])
    assert pm.filled == d["filled"]
    assert np.array_equal(pm.depth, d["depth"], equal_nan=True)
    assert np.array_equal(pm.support, d["support"])
    assert np.array_equal(pm.confidence, d["conf"])
    rf = orc.refine_subpixel(vs, cfg, pm)
    assert rf.filled == d["refined"]
    assert np.array_equal(rf.depth, d["rdepth"], equal_nan=True)
    assert np.array_equal(rf.confidence, d["rconf"])
    vsb = G.viewset(d, prefix="b_")
    pmb = orc.patchmatch_stereo(vsb, cfg)
    assert pmb.filled == d["b_filled"]
    assert np.array_equal(pmb.depth, d["b_depth"], equal_nan=True)
    pos, nrm, conf = O.fuse_depth_maps(
        "oracle", [(rf.depth, rf.support, rf.confidence), (pmb.depth, pmb.support, pmb.confidence)],
        [d["ref_pose"], d["b_ref_pose"]], [d["ref_intr"], d["b_ref_intr"]], cfg)
    assert len(pos) == d["fcount"] and G.digest(pos, nrm, conf) == str(d["fdigest"])


def test_select_source_views(orc):
    d = G.load("select.npz")
    import ast

    cfgs = [ast.literal_eval(c) for c in d["cfgs"]]
    k = 0
    for pose_set, set_cfgs in ((d["poses"], cfgs[:3]), (d["ring"], cfgs[3:])):
        for cd in set_cfgs:
            sel = orc.select_source_views(pose_set[0], list(pose_set),
                                          np.array([400.0, 400, 80, 60, 0, 0, 0, 0, 0, 160, 120]), O.make_config(**cd))
            want = [int(i) for i in d["sel"][k] if i >= 0]
            assert sel == want
            assert len(sel) <= cd["num_views"]
            assert len(set(sel)) == len(sel)  # no duplicates (test_mvs.cpp:489-495)
            assert 0 not in sel  # never the reference itself
            k += 1


def test_contract_violations_return_zero(orc):
    """Index-contract violations return 0 (patchmatch_stereo.cpp:434-468)."""
    d = G.load("eval_plane.npz")
    cfg = O.make_config(**G.config(d))
    vs = O.ViewSet(d["ref"], list(d["srcs"]), G._Cam(d["ref_intr"], d["ref_pose"]), None,
                   source_indices=[1, 2, 3, 9], all_poses=list(d["poses"]), intrinsics=list(d["intr"]))
    assert orc.patchmatch_stereo(vs, cfg).filled == 0
    vs = O.ViewSet(d["ref"], list(d["srcs"]), G._Cam(d["ref_intr"], d["ref_pose"]), None,
                   source_indices=[1, 2, 3, 4], all_poses=list(d["poses"]), intrinsics=list(d["intr"])[:3])
    assert orc.patchmatch_stereo(vs, cfg).filled == 0
    bad = O.make_config(**{**G.config(d), "min_depth_m": 0.9, "max_depth_m": 0.5})
    vs = G.viewset(d)
    assert orc.patchmatch_stereo(vs, bad).filled == 0


def test_oracle_matches_live_reference(orc, ref_lib):
    """Where the reference tree is present: fresh random hypotheses on a
    distorted scene, oracle vs the reference library, bit-exact."""
    import synthetic as S

    sc = S.sphere_on_backdrop(width=80, height=60, f=75.0, num_sources=3, seed=9)
    cams = [sc.ref.camera] + [s.camera for s in sc.sources]
    for c in cams:
        c.k1, c.k2, c.p2 = -0.03, 0.005, 1e-4
    vs = O.ViewSet(sc.ref.image, [s.image for s in sc.sources], cams[0], cams[1:])
    cfg = O.make_config(min_depth_m=0.25, max_depth_m=0.55, num_threads=2, iterations=1, patch_size=9)
    rng = np.random.default_rng(3)
    px, py, inv = rng.integers(0, 80, 400), rng.integers(0, 60, 400), rng.uniform(1.8, 4.0, 400)
    a = orc.evaluate_candidates(vs, cfg, px, py, inv)
    b = ref_lib.evaluate_candidates(vs, cfg, px, py, inv)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    pa, pb = orc.patchmatch_stereo(vs, cfg), ref_lib.patchmatch_stereo(vs, cfg)
    assert pa.filled == pb.filled and np.array_equal(pa.depth, pb.depth, equal_nan=True)
