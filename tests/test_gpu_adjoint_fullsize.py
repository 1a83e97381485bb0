"""GPU: the adjoint's pixel gradient at the differentiation workload's own
size -- the 1920x1440 tabletop views with every source pose perturbed by a
seeded 0.2 deg rotation and 0.5 mm translation (distorted cameras,
undistorted on the device; the oracle reads the same undistorted
intensities) -- at 10^4 seeded hypotheses near the analytic surface, against
FP64 central differences (step 1e-8, relative in depth) of the oracle's
plane cost.

Criterion: the relative error of the gradient vector (the depth derivative
scaled by the depth) is <= 1e-3 for >= 99.9 % of hypotheses, outside three
named classes where a relative 1e-3 comparison does not measure the adjoint:

  * texel edge -- a window sample of an averaged view lies within 3e-5 texel
    of a source texel edge (the oracle reports the distance).  Bilinear
    interpolation has a kink there, and the FP32 sample positions of the
    device (accurate to ~1e-5 texel) and the FP64 ones of the oracle can fall
    on opposite sides: both costs agree, but they differentiate different
    interpolation cells;
  * kink inside the step -- the forward and backward FP64 differences
    disagree by more than 1e-3 relative: a sample crosses a texel edge within
    the finite-difference step, so the central difference is no derivative;
  * near-stationary -- the gradient norm is below 5 % of the set's median:
    the adjoint's FP32 per-view sums carry an absolute error of ~2e-4, which
    is more than 1e-3 of such a gradient.
The test prints each class's share; together they hold a few per cent of the
hypotheses.
"""
import copy

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

W, H, F = 1920, 1440, 1450.0
N_HYP = 10_000


def so3_exp(w):
    th = np.linalg.norm(w)
    K = np.array([[0, -w[2], w[1]], [w[2], 0, -w[0]], [-w[1], w[0], 0]])
    if th < 1e-12:
        return np.eye(3) + K
    return np.eye(3) + np.sin(th) / th * K + (1 - np.cos(th)) / th ** 2 * K @ K


def sph(ang):
    t, p = ang[:, 0], ang[:, 1]
    return np.stack([np.sin(t) * np.cos(p), np.sin(t) * np.sin(p), np.cos(t)], -1)


def test_pixel_gradient_full_size(orc):
    import recon_mvs as M
    import synthetic as S

    M.load_library()
    sc = S.tabletop(width=W, height=H, f=F, num_sources=8, seed=2, device="cuda:0")
    cams = sc.cameras
    imgs = [v.image for v in sc.views]
    rng = np.random.default_rng(17)
    pert = [cams[0]]
    for c in cams[1:]:
        a = rng.normal(size=3)
        tdir = rng.normal(size=3)
        e = so3_exp(np.radians(0.2) * a / np.linalg.norm(a))
        p = copy.deepcopy(c)
        p.R, p.t = e @ c.R, e @ c.t + 0.0005 * tdir / np.linalg.norm(tdir)
        pert.append(p)
    cfg_kw = dict(min_depth_m=sc.min_depth, max_depth_m=sc.max_depth, iterations=8, patch_size=11,
                  subpixel_iterations=4)
    ys, xs = np.nonzero(np.isfinite(sc.ref.depth[8:-8, 8:-8]))
    pick = rng.choice(len(xs), N_HYP, replace=False)
    px, py = (xs[pick] + 8).astype(np.int32), (ys[pick] + 8).astype(np.int32)
    nt = sc.ref.normal[py, px]
    depth = sc.ref.depth[py, px] * (1 + rng.uniform(-0.005, 0.005, N_HYP))
    ang = np.stack([np.arccos(np.clip(nt[:, 2], -1, 1)) + rng.uniform(-0.05, 0.05, N_HYP),
                    np.arctan2(nt[:, 1], nt[:, 0]) + rng.uniform(-0.05, 0.05, N_HYP)], -1)
    eng = M.Engine(M.Options(mode=M.MODE_PLANE, best_k=4, device=0))
    try:
        job = eng.stage(M.ViewArgs.from_cameras(imgs[0], imgs[1:], pert[0], pert[1:]), M.MvsConfig(**cfg_kw),
                        undistort=True)
        cost, grad, _, _ = eng.adjoint(job, px, py, depth, ang)
    finally:
        eng.close()
    und = [orc.undistort(im, c.intrinsics_array()) for im, c in zip(imgs, pert)]
    pin = [c.undistorted() for c in pert]
    vs = O.ViewSet(und[0], und[1:], pin[0], pin[1:])
    ocfg = O.make_config(num_threads=0, **cfg_kw)
    oc = lambda d_, a_: orc.plane_costs(vs, ocfg, 4, px, py, 1.0 / d_, sph(a_))[0]
    base = oc(depth, ang)
    h = 1e-8
    fwd, bwd = np.zeros((N_HYP, 3)), np.zeros((N_HYP, 3))
    hd = h * depth
    fwd[:, 0] = (oc(depth + hd, ang) - base) / hd * depth
    bwd[:, 0] = (base - oc(depth - hd, ang)) / hd * depth
    for j in (0, 1):
        e = np.zeros_like(ang)
        e[:, j] = h
        fwd[:, 1 + j] = (oc(depth, ang + e) - base) / h
        bwd[:, 1 + j] = (base - oc(depth, ang - e)) / h
    cen = 0.5 * (fwd + bwd)
    g = grad.astype(np.float64)
    g[:, 0] *= depth
    ok = (cost < 1e29) & (base < 1e29) & np.all(np.isfinite(cen), -1)
    fn = np.linalg.norm(cen, axis=-1)
    with np.errstate(invalid="ignore", divide="ignore"):
        rel = np.linalg.norm(g - cen, axis=-1) / fn
        kink = np.linalg.norm(fwd - bwd, axis=-1) / fn
    edge = orc.plane_edge_distance(vs, ocfg, 4, px, py, 1.0 / depth, sph(ang))
    classes = {"texel edge": edge < 3e-5, "kink inside the step": kink > 1e-3,
               "near-stationary": fn < 0.05 * np.median(fn[ok])}
    excluded = np.zeros(N_HYP, bool)
    for name, c in classes.items():
        print(f"{name}: {np.mean(c[ok]):.4f} of the hypotheses")
        excluded |= c
    kept = ok & ~excluded
    frac = float(np.mean(rel[kept] <= 1e-3))
    print(f"pixel gradient, 1920x1440: n={ok.sum()}, all: {np.mean(rel[ok] <= 1e-3):.4f} within 1e-3 "
          f"(median {np.median(rel[ok]):.2e}); outside the classes ({kept.sum()}): {frac:.5f}")
    assert ok.mean() > 0.98
    assert kept.sum() >= 0.9 * ok.sum()
    assert frac >= 0.999
