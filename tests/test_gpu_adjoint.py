"""GPU: the differentiation form -- the hand-written adjoint of the aggregated
plane cost, Gauss-Newton refinement and pose recovery.

Gradient check: 10^4 seeded hypotheses near the analytic surface of the
tabletop views (distorted cameras, undistorted on the device; the oracle
reads the same undistorted intensities, orc_undistort being bit-identical to
the device remap).  The GPU adjoint (FP32) is compared with FP64 central
differences of the oracle's plane cost (orc_plane_cost) in the pixel
parameters (depth, theta, phi) and in every source's 6-DoF pose.  The
criterion is the relative error of the gradient vector, with the depth
derivative scaled by the depth (log-depth) and the translation derivatives by
the scene depth so that components share units: <= 1e-3 for at least 99 % of
hypotheses (pixel parameters) and 97 % of (hypothesis, source) pairs (pose).
The rest are hypotheses where a window sample sits on a texel edge
(bilinear interpolation is not differentiable there) or a best-k tie.
"""
import copy

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N_HYP = 10_000
SCENE_DEPTH = 0.4


def sph(ang):
    t, p = ang[:, 0], ang[:, 1]
    return np.stack([np.sin(t) * np.cos(p), np.sin(t) * np.sin(p), np.cos(t)], -1)


def so3_exp(w):
    th = np.linalg.norm(w)
    K = np.array([[0, -w[2], w[1]], [w[2], 0, -w[0]], [-w[1], w[0], 0]])
    if th < 1e-12:
        return np.eye(3) + K + 0.5 * K @ K
    return np.eye(3) + np.sin(th) / th * K + (1 - np.cos(th)) / th ** 2 * K @ K


def perturbed(cam, w, tau):
    c = copy.deepcopy(cam)
    E = so3_exp(np.asarray(w, np.float64))
    c.R = E @ cam.R
    c.t = E @ cam.t + np.asarray(tau, np.float64)
    return c


@pytest.fixture(scope="module")
def mvs():
    import recon_mvs

    recon_mvs.load_library()
    return recon_mvs


@pytest.fixture(scope="module")
def setup(orc):
    import synthetic as S

    sc = S.tabletop(width=640, height=480, f=1450.0 * 640 / 1920, num_sources=8, seed=4)
    cams = sc.cameras
    imgs = [sc.ref.image] + [s.image for s in sc.sources]
    und = [orc.undistort(im, c.intrinsics_array()) for im, c in zip(imgs, cams)]
    pin = [c.undistorted() for c in cams]
    rng = np.random.default_rng(7)
    h, w = sc.ref.depth.shape
    ys, xs = np.nonzero(np.isfinite(sc.ref.depth[8:-8, 8:-8]))
    pick = rng.choice(len(xs), N_HYP, replace=False)
    px, py = xs[pick] + 8, ys[pick] + 8
    d_true = sc.ref.depth[py, px]
    n_true = sc.ref.normal[py, px]
    depth = d_true * (1.0 + rng.uniform(-0.005, 0.005, N_HYP))
    theta = np.arccos(np.clip(n_true[:, 2], -1, 1)) + rng.uniform(-0.05, 0.05, N_HYP)
    phi = np.arctan2(n_true[:, 1], n_true[:, 0]) + rng.uniform(-0.05, 0.05, N_HYP)
    return dict(sc=sc, cams=cams, imgs=imgs, und=und, pin=pin, px=px.astype(np.int32), py=py.astype(np.int32),
                depth=depth, ang=np.stack([theta, phi], -1))


def cfg_kw(sc):
    return dict(min_depth_m=sc.min_depth, max_depth_m=sc.max_depth, patch_size=11, iterations=4,
                subpixel_iterations=4)


def oracle_cost(orc, vs, cfg, S, depth, ang):
    cost, _, _ = orc.plane_costs(vs, cfg, 4, S["px"], S["py"], 1.0 / depth, sph(ang))
    return cost


@pytest.fixture(scope="module")
def gpu_adjoint(mvs, setup):
    S = setup
    sc = S["sc"]
    views = mvs.ViewArgs.from_cameras(S["imgs"][0], S["imgs"][1:], S["cams"][0], S["cams"][1:])
    eng = mvs.Engine(mvs.Options(mode=mvs.MODE_PLANE, best_k=4, device=0))
    job = eng.stage(views, mvs.MvsConfig(**cfg_kw(sc)), undistort=True)
    out = eng.adjoint(job, S["px"], S["py"], S["depth"], S["ang"], gn=True, pose=True)
    eng.close()
    return out


def rel_err(got, want):
    return np.linalg.norm(got - want, axis=-1) / np.maximum(np.linalg.norm(want, axis=-1), 1e-30)


def test_adjoint_cost_matches_oracle(orc, setup, gpu_adjoint):
    import oracle as O

    S = setup
    vs = O.ViewSet(S["und"][0], S["und"][1:], S["pin"][0], S["pin"][1:])
    cfg = O.make_config(num_threads=0, **cfg_kw(S["sc"]))
    want = oracle_cost(orc, vs, cfg, S, S["depth"], S["ang"])
    cost = gpu_adjoint[0]
    ok = (want < 1e29) & (cost < 1e29)
    print("valid", ok.mean(), "max |dc|", np.abs(cost[ok] - want[ok]).max())
    assert ok.mean() > 0.95
    assert np.mean(np.abs(cost[ok] - want[ok]) <= 1e-4) >= 0.999


def test_pixel_gradient_vs_fp64_central_differences(orc, setup, gpu_adjoint):
    import oracle as O

    S = setup
    vs = O.ViewSet(S["und"][0], S["und"][1:], S["pin"][0], S["pin"][1:])
    cfg = O.make_config(num_threads=0, **cfg_kw(S["sc"]))
    d, ang = S["depth"], S["ang"]
    base = oracle_cost(orc, vs, cfg, S, d, ang)
    fd = np.zeros((N_HYP, 3))
    hd = 1e-8 * d
    fd[:, 0] = (oracle_cost(orc, vs, cfg, S, d + hd, ang) - oracle_cost(orc, vs, cfg, S, d - hd, ang)) / (2 * hd)
    for j in (0, 1):
        e = np.zeros_like(ang)
        e[:, j] = 1e-8
        fd[:, 1 + j] = (oracle_cost(orc, vs, cfg, S, d, ang + e) - oracle_cost(orc, vs, cfg, S, d, ang - e)) / 2e-8
    cost, grad = gpu_adjoint[0], gpu_adjoint[1].astype(np.float64)
    ok = (base < 1e29) & (cost < 1e29) & np.all(np.isfinite(fd), -1)
    scale = np.array([1.0, 1.0, 1.0])
    g = grad[ok] * scale
    f = fd[ok] * scale
    g[:, 0] *= d[ok]
    f[:, 0] *= d[ok]
    r = rel_err(g, f)
    print(f"pixel gradient: n={ok.sum()} rel err median {np.median(r):.2e} p99 {np.quantile(r, 0.99):.2e} "
          f"<=1e-3: {np.mean(r <= 1e-3):.4f}")
    assert np.mean(r <= 1e-3) >= 0.99


def test_pose_gradient_vs_fp64_central_differences(orc, setup, gpu_adjoint):
    import oracle as O

    S = setup
    pin = S["pin"]
    cfg = O.make_config(num_threads=0, **cfg_kw(S["sc"]))
    d, ang = S["depth"], S["ang"]
    pose_grad = gpu_adjoint[3].astype(np.float64)  # n x S x 6
    ns = pose_grad.shape[1]
    fd = np.zeros((N_HYP, ns, 6))
    steps = [1e-8] * 3 + [1e-9] * 3
    for s in range(ns):
        for j in range(6):
            w, tau = np.zeros(3), np.zeros(3)
            (w if j < 3 else tau)[j % 3] = steps[j]
            c = []
            for sign in (1, -1):
                cams = list(pin)
                cams[1 + s] = perturbed(pin[1 + s], sign * w, sign * tau)
                vs = O.ViewSet(S["und"][0], S["und"][1:], cams[0], cams[1:])
                c.append(oracle_cost(orc, vs, cfg, S, d, ang))
            fd[:, s, j] = (c[0] - c[1]) / (2 * steps[j])
    cost = gpu_adjoint[0]
    sel = np.any(pose_grad != 0, -1) & (cost < 1e29)[:, None] & np.all(np.isfinite(fd), -1)
    g = pose_grad[sel]
    f = fd[sel]
    g[:, 3:] *= SCENE_DEPTH
    f[:, 3:] *= SCENE_DEPTH
    r = rel_err(g, f)
    print(f"pose gradient: n={sel.sum()} rel err median {np.median(r):.2e} p99 {np.quantile(r, 0.99):.2e} "
          f"<=1e-3: {np.mean(r <= 1e-3):.4f}")
    assert np.mean(r <= 1e-3) >= 0.97


def run_pm(mvs, S, refine, cams=None):
    sc = S["sc"]
    cams = cams or S["cams"]
    views = mvs.ViewArgs.from_cameras(S["imgs"][0], S["imgs"][1:], cams[0], cams[1:])
    eng = mvs.Engine(mvs.Options(mode=mvs.MODE_PLANE, best_k=4, device=0, refine=refine))
    try:
        job = eng.stage(views, mvs.MvsConfig(**cfg_kw(sc)), undistort=True)
        eng.run(job)
        return eng.download(job)
    finally:
        eng.close()


def median_rel(dm, truth):
    e = np.abs(dm.depth[8:-8, 8:-8].astype(np.float64) - truth[8:-8, 8:-8]) / truth[8:-8, 8:-8]
    return float(np.nanmedian(e))


def test_gauss_newton_refinement_beats_golden_section(mvs, setup):
    S = setup
    truth = S["sc"].ref.depth
    e0 = median_rel(run_pm(mvs, S, 0), truth)
    e1 = median_rel(run_pm(mvs, S, 1), truth)
    e2 = median_rel(run_pm(mvs, S, 2), truth)
    print(f"median rel depth error: no refine {e0:.3e}, golden section {e1:.3e}, Gauss-Newton {e2:.3e}")
    assert e2 < e1


def perturbed_cameras(S, seed=11):
    """Sources perturbed by a seeded 0.2 deg rotation and 0.5 mm translation."""
    rng = np.random.default_rng(seed)
    cams = list(S["cams"])
    out = [cams[0]]
    for c in cams[1:]:
        axis = rng.normal(size=3)
        axis /= np.linalg.norm(axis)
        tdir = rng.normal(size=3)
        tdir /= np.linalg.norm(tdir)
        out.append(perturbed(c, np.radians(0.2) * axis, 0.0005 * tdir))
    return out


def pose_errors(poses, truth):
    """Rotation error (deg) and camera-centre error (mm) per source; poses
    are Camera objects or rows [R (9), t (3)]."""
    rot, ctr = [], []
    for c, t in zip(poses, truth):
        R = c[:9].reshape(3, 3) if isinstance(c, np.ndarray) else c.R
        tt = c[9:12] if isinstance(c, np.ndarray) else c.t
        dR = R @ t.R.T
        rot.append(np.degrees(np.arccos(np.clip((np.trace(dR) - 1) / 2, -1, 1))))
        ctr.append(np.linalg.norm(-R.T @ tt + t.R.T @ t.t) * 1e3)
    return np.array(rot), np.array(ctr)


def recover(mvs, S, cams, depth_map, normal_map, iterations=15, stride=2):
    views = mvs.ViewArgs.from_cameras(S["imgs"][0], S["imgs"][1:], cams[0], cams[1:])
    eng = mvs.Engine(mvs.Options(mode=mvs.MODE_PLANE, best_k=4, device=0))
    try:
        job = eng.stage(views, mvs.MvsConfig(**cfg_kw(S["sc"])), undistort=True)
        ys, xs = np.nonzero(np.isfinite(depth_map[8:-8:stride, 8:-8:stride]))
        px, py = (xs * stride + 8).astype(np.int32), (ys * stride + 8).astype(np.int32)
        n = normal_map[py, px].astype(np.float64)
        ang = np.stack([np.arccos(np.clip(n[:, 2], -1, 1)), np.arctan2(n[:, 1], n[:, 0])], -1)
        return eng.recover_poses(job, px, py, depth_map[py, px].astype(np.float64), ang, iterations=iterations)
    finally:
        eng.close()


def with_poses(cams, rows):
    out = [cams[0]]
    for c, p in zip(cams[1:], rows):
        c = copy.deepcopy(c)
        c.R = p[:9].reshape(3, 3).copy()
        c.t = p[9:12].copy()
        out.append(c)
    return out


def test_pose_recovery_on_true_surface(mvs, setup):
    """With the analytic surface as the hypotheses, pose recovery returns
    the true poses up to the image noise: the solver and the pose adjoint
    are right."""
    S = setup
    pert = perturbed_cameras(S)
    poses, hist = recover(mvs, S, pert, S["sc"].ref.depth, S["sc"].ref.normal)
    r0, c0 = pose_errors(pert[1:], S["cams"][1:])
    r1, c1 = pose_errors(list(poses), S["cams"][1:])
    print("true surface: cost", hist[0], "->", hist[-1], "rotation deg", r0.max(), "->", r1.round(4),
          "centre mm", c0.max(), "->", c1.round(4))
    assert hist[-1] < hist[0]
    # image noise and 8-bit intensities bound the recovery: every source's
    # rotation error falls from 0.2 deg to < 0.04 deg, its centre error from
    # 0.5 mm to < 0.3 mm
    assert r1.max() < 0.04 and c1.max() < 0.3


def test_pose_recovery_from_patchmatch(mvs, setup):
    """PatchMatch on the perturbed poses, pose recovery from its own map,
    PatchMatch again on the recovered poses: the map improves."""
    S = setup
    truth = S["sc"].ref.depth
    pert = perturbed_cameras(S)
    dm0 = run_pm(mvs, S, 1, pert)
    poses, hist = recover(mvs, S, pert, dm0.depth, dm0.normal)
    cams1 = with_poses(pert, poses)
    dm1 = run_pm(mvs, S, 1, cams1)
    r0, c0 = pose_errors(pert[1:], S["cams"][1:])
    r1, c1 = pose_errors(cams1[1:], S["cams"][1:])
    e_true = median_rel(run_pm(mvs, S, 1), truth)
    e0, e1 = median_rel(dm0, truth), median_rel(dm1, truth)
    print("from PatchMatch: cost", hist[0], "->", hist[-1])
    print("rotation error deg", r0.round(3), "->", r1.round(3))
    print("centre error mm", c0.round(3), "->", c1.round(3))
    print(f"median rel depth error: true poses {e_true:.3e}, perturbed {e0:.3e}, recovered {e1:.3e}")
    assert hist[-1] < hist[0]
    assert np.median(r1) < 0.75 * np.median(r0)
    assert e1 < e0
