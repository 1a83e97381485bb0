"""Generate the golden vectors that pin the CPU oracle to the reference.

Run in a checkout where the reference tree is present:

    python tests/golden/make_golden.py

It compiles the reference's own MVS sources (oracle/Makefile `ref` target ->
oracle/_ref/libref_mvs.so) and records their outputs on small seeded scenes
into tests/golden/*.npz, inputs included, so the checks run anywhere
without the reference tree:

  ncc_known.npz      ComputeNcc on the reference unit test's windows
                     (identical, +40 brightness, flat)  test_mvs.cpp:259-293
  camera.npz         PixelToRay / ProjectPoint with the unit test's
                     Brown-Conrady camera                 test_mvs.cpp:210-253
  eval_plane.npz     EvaluateCandidate on 3000 seeded hypotheses of the
                     unit test's plane scene (global intrinsics)
  eval_distort.npz   the same on a small distorted sphere scene
  pm_plane.npz       PatchMatchStereo + RefineSubpixel + FuseDepthMaps on
                     the plane scene (2 iterations, 4 directions, 4 threads)
  pm_sphere.npz      the same on a 96x72 sphere scene with sparse seeds
  select.npz         SelectSourceViews on the unit test's poses and on a
                     20-pose ring
  tsdf.npz           TsdfVolume::IntegrateDepthFrame + ExtractPoints (the
                     reference's tsdf_fusion.cpp, oracle/_ref/libref_tsdf.so)
                     on the reference TSDF test's tilted wall (3 frames) and
                     on a 320x240 sphere capture with holes and
                     low-confidence pixels (4 frames); grids and points
                     recorded as digests

`python tests/golden/make_golden.py tsdf` writes tsdf.npz alone.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "recon-scanner_gb300"))

import oracle as O  # noqa: E402
import synthetic as S  # noqa: E402

CFG_PLANE = dict(num_views=4, num_threads=4, patch_size=11, iterations=2, random_search_count=5,
                 random_search_radius_ratio=0.35, subpixel_iterations=5, min_depth_m=0.15,
                 max_depth_m=0.80, fusion_voxel_size_m=0.0005)


def digest(*arrays):
    """sha256 over the raw bytes of arrays (bit-exact comparisons of large
    outputs without storing them)."""
    import hashlib
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def cloud_fields(prefix, pos, nrm, conf):
    return {prefix + "count": len(pos), prefix + "digest": digest(pos, nrm, conf),
            prefix + "pos_head": pos[:200], prefix + "nrm_head": nrm[:200], prefix + "conf_head": conf[:200]}


def cfg_array(d):
    return np.array([[k, repr(v)] for k, v in d.items()])


def plane_views():
    imgs, cams, truth = S.plane_test_scene()
    return imgs, cams, truth


def views_arrays(ref_img, srcs, ref_cam, src_cams, poses, source_indices, intr):
    return dict(ref=ref_img, srcs=np.stack(srcs), ref_intr=ref_cam.intrinsics_array(),
                ref_pose=ref_cam.pose_array(), poses=np.stack(poses), source_indices=np.asarray(source_indices),
                intr=np.stack(intr))


def viewset_from(d):
    class _C:
        def __init__(self, k, p):
            self._k, self._p = k, p

        def intrinsics_array(self):
            return self._k

        def pose_array(self):
            return self._p

    ref_cam = _C(d["ref_intr"], d["ref_pose"])
    srcs = list(d["srcs"])
    return O.ViewSet(d["ref"], srcs, ref_cam, None, source_indices=list(d["source_indices"]),
                     all_poses=list(d["poses"]), intrinsics=list(d["intr"]))


def small_sphere(distort: bool):
    sc = S.sphere_on_backdrop(width=96, height=72, f=90.0, num_sources=4, seed=5)
    cams = [sc.ref.camera] + [s.camera for s in sc.sources]
    imgs = [sc.ref.image] + [s.image for s in sc.sources]
    if distort:
        for c in cams:
            c.k1, c.k2, c.p1 = 0.04, -0.01, 2e-4
    return imgs, cams, sc


def main():
    O.build_oracle(ref=True)
    ref = O.load("reference")
    out = {}

    # ---- ComputeNcc known answers (test_mvs.cpp:259-293) ----
    w = h = 64
    ys, xs = np.mgrid[0:h, 0:w]
    uu, vv = xs * 0.08, ys * 0.11
    val = 128.0 + 60.0 * np.sin(uu) * np.cos(vv * 1.3) + 30.0 * np.sin(uu * 2.7 + vv * 0.4) + 18.0 * np.cos(uu * 4.1 - vv * 3.3)
    hsh = (xs.astype(np.uint32) * np.uint32(73856093)) ^ (ys.astype(np.uint32) * np.uint32(19349663))
    val += (hsh & 0xFF).astype(np.float64) * 0.15 - 19.0
    a = np.clip(val, 0, 255).astype(np.uint8)
    brighter = np.minimum(255.0, a.astype(np.float64) + 40.0).astype(np.uint8)
    flat = np.full((h, w), 128, np.uint8)
    rng = np.random.default_rng(11)
    cases = [(a, a, 32.0, 32.0, 32.0, 32.0), (a, brighter, 32.0, 32.0, 32.0, 32.0), (flat, a, 32.0, 32.0, 32.0, 32.0)]
    for _ in range(60):
        cases.append((a, brighter, *rng.uniform(-4, 68, 4)))
    res = [ref.compute_ncc(c[0], c[1], *c[2:], 11) for c in cases]
    np.savez_compressed(os.path.join(HERE, "ncc_known.npz"), a=a, brighter=brighter, flat=flat,
                        which=np.array([[0, 0], [0, 1], [2, 0]] + [[0, 1]] * 60),
                        coords=np.array([c[2:] for c in cases]),
                        valid=np.array([r.valid for r in res]), ncc=np.array([r.ncc for r in res]),
                        weak=np.array([r.weak_texture for r in res]), samples=np.array([r.valid_samples for r in res]))

    # ---- camera model (test_mvs.cpp:210-253) ----
    intr = np.array([1250.0, 1250.0, 960.0, 540.0, -0.22, 0.06, -0.005, 0.0008, -0.0006, 1920, 1080])
    uv = np.array([[40.0 + i * 9.0, 30.0 + i * 5.0] for i in range(200) if 40 + i * 9 < 1910 and 30 + i * 5 < 1070])
    rays = np.array([ref.pixel_to_ray(intr, u, v) for u, v in uv])
    proj = np.array([ref.project_point(intr, r)[1:] for r in rays])
    np.savez_compressed(os.path.join(HERE, "camera.npz"), intr=intr, uv=uv, rays=rays, proj=proj)

    # ---- EvaluateCandidate ----
    imgs, cams, truth = plane_views()
    d = views_arrays(imgs[0], imgs[1:], cams[0], cams[1:], [c.pose_array() for c in cams], [1, 2, 3, 4],
                     [c.intrinsics_array() for c in cams])
    vs = viewset_from(d)
    cfg = O.make_config(**CFG_PLANE)
    rng = np.random.default_rng(21)
    n = 3000
    px, py = rng.integers(0, 160, n), rng.integers(0, 120, n)
    inv = rng.uniform(1 / 0.85, 1 / 0.14, n)
    cost, nv = ref.evaluate_candidates(vs, cfg, px, py, inv)
    np.savez_compressed(os.path.join(HERE, "eval_plane.npz"), **d, cfg=cfg_array(CFG_PLANE), px=px, py=py,
                        inv=inv, cost=cost, valid_views=nv)

    imgs2, cams2, _ = small_sphere(distort=True)
    d2 = views_arrays(imgs2[0], imgs2[1:], cams2[0], cams2[1:], [c.pose_array() for c in cams2[1:]], [0, 1, 2, 3],
                      [c.intrinsics_array() for c in cams2[1:]])
    vs2 = viewset_from(d2)
    cfg2d = dict(num_threads=2, min_depth_m=0.25, max_depth_m=0.55, iterations=1)
    cfg2 = O.make_config(**cfg2d)
    px, py = rng.integers(0, 96, 1500), rng.integers(0, 72, 1500)
    inv = rng.uniform(1 / 0.6, 1 / 0.24, 1500)
    cost, nv = ref.evaluate_candidates(vs2, cfg2, px, py, inv)
    np.savez_compressed(os.path.join(HERE, "eval_distort.npz"), **d2, cfg=cfg_array(cfg2d), px=px, py=py,
                        inv=inv, cost=cost, valid_views=nv)

    # ---- PatchMatch + refine + fuse on the plane scene ----
    pm = ref.patchmatch_stereo(vs, cfg)
    rf = ref.refine_subpixel(vs, cfg, pm)
    fpos, fnrm, fconf = O.fuse_depth_maps("reference", [(rf.depth, rf.support, rf.confidence)],
                                          [cams[0].pose_array()], [cams[0].intrinsics_array()], cfg)
    np.savez_compressed(os.path.join(HERE, "pm_plane.npz"), **d, cfg=cfg_array(CFG_PLANE), truth=truth,
                        filled=pm.filled, depth=pm.depth, support=pm.support, conf=pm.confidence,
                        refined=rf.filled, rdepth=rf.depth, rconf=rf.confidence,
                        **cloud_fields("f", fpos, fnrm, fconf))

    # ---- a small sphere scene with sparse seeds, 3 threads ----
    imgs3, cams3, sc3 = small_sphere(distort=False)
    d3 = views_arrays(imgs3[0], imgs3[1:], cams3[0], cams3[1:], [c.pose_array() for c in cams3], [1, 2, 3, 4],
                      [c.intrinsics_array() for c in cams3[1:]])
    vs3 = viewset_from(d3)
    cfg3d = dict(num_threads=3, min_depth_m=0.25, max_depth_m=0.55, iterations=2, patch_size=7,
                 random_search_count=4, restart_ratio=0.2, subpixel_iterations=3, min_view_consistency=1,
                 photo_threshold=0.5)
    cfg3 = O.make_config(**cfg3d)
    seeds = []
    for _ in range(40):
        x, y = rng.uniform(0, 96), rng.uniform(0, 72)
        dd = sc3.ref.depth[int(y), int(x)]
        if np.isfinite(dd):
            seeds.append([x, y, dd * rng.uniform(0.97, 1.03)])
    seeds = np.array(seeds)
    pm3 = ref.patchmatch_stereo(vs3, cfg3, seeds=seeds)
    rf3 = ref.refine_subpixel(vs3, cfg3, pm3)
    # a second map from source 0's viewpoint for a two-map fusion
    d3b = views_arrays(imgs3[1], [imgs3[0], imgs3[2]], cams3[1], [cams3[0], cams3[2]],
                       [c.pose_array() for c in cams3], [0, 2], [c.intrinsics_array() for c in cams3])
    vs3b = viewset_from(d3b)
    pm3b = ref.patchmatch_stereo(vs3b, cfg3)
    fpos3, fnrm3, fconf3 = O.fuse_depth_maps(
        "reference", [(rf3.depth, rf3.support, rf3.confidence), (pm3b.depth, pm3b.support, pm3b.confidence)],
        [cams3[0].pose_array(), cams3[1].pose_array()], [cams3[0].intrinsics_array(), cams3[1].intrinsics_array()], cfg3)
    np.savez_compressed(os.path.join(HERE, "pm_sphere.npz"), **d3, cfg=cfg_array(cfg3d), seeds=seeds,
                        filled=pm3.filled, depth=pm3.depth, support=pm3.support, conf=pm3.confidence,
                        refined=rf3.filled, rdepth=rf3.depth, rconf=rf3.confidence,
                        b_ref=imgs3[1], b_srcs=np.stack([imgs3[0], imgs3[2]]), b_ref_pose=cams3[1].pose_array(),
                        b_ref_intr=cams3[1].intrinsics_array(), b_source_indices=np.array([0, 2]),
                        b_poses=np.stack([c.pose_array() for c in cams3]),
                        b_intr=np.stack([c.intrinsics_array() for c in cams3]), b_filled=pm3b.filled, b_depth=pm3b.depth,
                        b_support=pm3b.support, b_conf=pm3b.confidence,
                        **cloud_fields("f", fpos3, fnrm3, fconf3))

    # ---- SelectSourceViews ----
    poses = []
    for i in range(5):  # test_mvs.cpp:469-500
        ang = i * 0.15
        c, s = np.cos(ang), np.sin(ang)
        R = np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]])
        poses.append(np.concatenate([R.reshape(-1), [-0.03 * i, 0.0, 0.0], [0.0]]))
    # 20 poses, 19 candidates: more than libstdc++'s 16-element insertion-sort
    # threshold, so std::sort runs its introsort there; the scores are kept
    # distinct (a tie order beyond 16 candidates is implementation-defined).
    ring = [np.concatenate([np.eye(3).reshape(-1), np.zeros(3), [0.0]])]
    for i in range(1, 20):
        th, ph = np.radians(3.0 + 2.5 * i), 1.1 * i
        center = 0.05 * np.array([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)])
        R, t = S.look_at(center, (0.0, 0.0, 0.4), up=(0.0, -1.0, 0.0))
        ring.append(np.concatenate([R.reshape(-1), t, [0.0]]))
    sel_cfgs = {0: [dict(num_views=3), dict(num_views=6, ref_view_index=0), dict(num_views=25, ideal_angle_min_deg=1.0)],
                1: [dict(num_views=6, ideal_angle_min_deg=55.0, ideal_angle_max_deg=60.0),
                    dict(num_views=25, ideal_angle_min_deg=55.0, ideal_angle_max_deg=60.0, ref_view_index=0),
                    dict(num_views=10, ideal_angle_min_deg=20.0, ideal_angle_max_deg=21.0, reference_depth_m=0.5)]}
    sels, cfg_list = [], []
    for si, pose_set in enumerate((poses, ring)):
        for cd in sel_cfgs[si]:
            sel = ref.select_source_views(pose_set[0], pose_set, np.array([400.0, 400, 80, 60, 0, 0, 0, 0, 0, 160, 120]),
                                          O.make_config(**cd))
            sels.append(sel + [-1] * (25 - len(sel)))
            cfg_list.append(repr(cd))
    np.savez_compressed(os.path.join(HERE, "select.npz"), poses=np.stack(poses), ring=np.stack(ring),
                        cfgs=np.array(cfg_list), sel=np.array(sels))
    print("golden vectors written to", HERE)


def make_tsdf():
    scenes = {"wall": S.tilted_wall_frames(), "capture": S.tsdf_capture()}
    out = {}
    for name, (cfgd, frames) in scenes.items():
        cfg = O.tsdf_config(**cfgd)
        r = O.tsdf_reference(cfg, frames)
        out[name + "_cfg"] = np.array([[k, repr(v)] for k, v in cfgd.items()])
        out[name + "_depth"] = np.stack([f[0] for f in frames])
        out[name + "_conf"] = np.stack([f[1] for f in frames])
        out[name + "_w2c"] = np.stack([np.asarray(f[2], np.float64) for f in frames])
        out[name + "_unc"] = np.asarray([f[3] for f in frames], np.float32)
        out[name + "_integrated"] = np.asarray(r["integrated"], np.int64)
        out[name + "_grid_digest"] = digest(r["tsdf"], r["weight"])
        out[name + "_fused_voxels"] = int((r["weight"] > 0).sum())
        out.update(cloud_fields(name + "_", r["positions"], r["normals"], r["confidences"]))
    np.savez_compressed(os.path.join(HERE, "tsdf.npz"), **out)


if __name__ == "__main__":
    if sys.argv[1:] == ["tsdf"]:
        make_tsdf()
        print("tsdf.npz written to", HERE)
        sys.exit(0)
    main()
    make_tsdf()
