"""Seeded synthetic multi-view scenes with analytic depth and normals.

The reference measures its MVS accuracy on a rendered synthetic plane
(tests/unit/test_mvs.cpp:56-204); there is no public dataset on this path.
These generators render the workloads the engine is measured on -- a sphere
in front of a backdrop plane (640x480, 4 sources), a sphere / box / three
cylinders resting on a tilted plane (1920x1440, 8 sources, Brown-Conrady
distortion), and orbit captures of the same scene -- by ray casting analytic
primitives with a solid (3-D) value-noise albedo, so that one surface point
has one intensity in every view.

Everything is plain torch tensor arithmetic so the same code renders small
scenes on the CPU (tests) and full-size scenes on the GPU (bench).  Cameras
follow the reference convention: R, t map world -> camera, pixel centres at
index + 0.5, y down.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np
import torch


# ----------------------------------------------------------------------------
# cameras
# ----------------------------------------------------------------------------

@dataclass
class Camera:
    """Pinhole + Brown-Conrady camera, world -> camera pose (R, t)."""

    fx: float
    fy: float
    cx: float
    cy: float
    width: int
    height: int
    R: np.ndarray  # 3x3 float64, world -> camera
    t: np.ndarray  # 3 float64
    k1: float = 0.0
    k2: float = 0.0
    k3: float = 0.0
    p1: float = 0.0
    p2: float = 0.0

    def intrinsics_array(self) -> np.ndarray:
        """The 11 doubles of recon_camera_intrinsics, in struct order."""
        return np.array([self.fx, self.fy, self.cx, self.cy, self.k1, self.k2, self.k3,
                         self.p1, self.p2, float(self.width), float(self.height)], np.float64)

    def pose_array(self) -> np.ndarray:
        """The 13 doubles of recon_pose: r[9] row-major, t[3], timestamp."""
        return np.concatenate([self.R.reshape(-1), self.t, [0.0]]).astype(np.float64)

    def center(self) -> np.ndarray:
        return -(self.R.T @ self.t)

    def undistorted(self) -> "Camera":
        c = Camera(**{k: getattr(self, k) for k in self.__dataclass_fields__})
        c.k1 = c.k2 = c.k3 = c.p1 = c.p2 = 0.0
        return c


def look_at(center, target, up=(0.0, 0.0, 1.0)) -> tuple[np.ndarray, np.ndarray]:
    """World->camera (R, t) for a camera at `center` looking at `target`;
    image y points along -up (downwards)."""
    center = np.asarray(center, np.float64)
    fwd = np.asarray(target, np.float64) - center
    fwd /= np.linalg.norm(fwd)
    up = np.asarray(up, np.float64)
    right = np.cross(fwd, -up)
    if np.linalg.norm(right) < 1e-9:
        right = np.cross(fwd, np.array([0.0, 1.0, 0.0]))
    right /= np.linalg.norm(right)
    down = np.cross(fwd, right)
    R = np.stack([right, down, fwd])
    return R, -(R @ center)


# ----------------------------------------------------------------------------
# scene primitives
# ----------------------------------------------------------------------------

@dataclass
class Scene:
    planes: list = field(default_factory=list)     # (point, unit normal, disk radius or None)
    spheres: list = field(default_factory=list)    # (center, radius)
    boxes: list = field(default_factory=list)      # (center, R_box (3x3 local->world), half extents)
    cylinders: list = field(default_factory=list)  # (base center, unit axis, radius, height)
    noise_scale: float = 0.005                     # lattice spacing of the albedo noise, metres
    weak_regions: list = field(default_factory=list)  # (center, radius): low-contrast balls
    contrast: tuple = (0.2, 0.9)
    weak_contrast: float = 0.02


def _hash3(ix, iy, iz, salt):
    h = (ix * 73856093) ^ (iy * 19349663) ^ (iz * 83492791) ^ salt
    h = h & 0xFFFFFFFF
    h = ((h >> 16) ^ h) * 0x45D9F3B & 0xFFFFFFFF
    h = ((h >> 16) ^ h) * 0x45D9F3B & 0xFFFFFFFF
    h = (h >> 16) ^ h
    return h.to(torch.float64) / 4294967296.0


def value_noise(p: torch.Tensor, scale: float, salt: int) -> torch.Tensor:
    """Trilinear value noise in [0, 1) with lattice spacing `scale` (metres)."""
    q = p / scale
    f = torch.floor(q)
    w = q - f
    w = w * w * (3.0 - 2.0 * w)  # smoothstep fade
    i = f.to(torch.int64)
    out = torch.zeros(p.shape[:-1], dtype=torch.float64, device=p.device)
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                h = _hash3(i[..., 0] + dx, i[..., 1] + dy, i[..., 2] + dz, salt)
                wx = w[..., 0] if dx else 1.0 - w[..., 0]
                wy = w[..., 1] if dy else 1.0 - w[..., 1]
                wz = w[..., 2] if dz else 1.0 - w[..., 2]
                out = out + h * wx * wy * wz
    return out


def albedo(scene: Scene, p: torch.Tensor) -> torch.Tensor:
    n = 0.65 * value_noise(p, scene.noise_scale, 0x1234) + 0.35 * value_noise(p, scene.noise_scale * 0.5, 0x9876)
    # value noise concentrates near 0.5; stretch to use the contrast range
    n = torch.clamp((n - 0.5) * 2.2 + 0.5, 0.0, 1.0)
    lo, hi = scene.contrast
    a = lo + (hi - lo) * n
    if scene.weak_regions:
        weak = torch.zeros(p.shape[:-1], dtype=torch.bool, device=p.device)
        for c, r in scene.weak_regions:
            c = torch.as_tensor(c, dtype=torch.float64, device=p.device)
            weak |= ((p - c) ** 2).sum(-1) < r * r
        mid = 0.5 * (lo + hi)
        a = torch.where(weak, mid + scene.weak_contrast * (n - 0.5), a)
    return a


def _intersect(scene: Scene, o: torch.Tensor, d: torch.Tensor):
    """Nearest hit of rays o + t d (t > 0).  Returns t and the world normal."""
    dev = d.device
    inf = torch.full(d.shape[:-1], math.inf, dtype=torch.float64, device=dev)
    best_t = inf.clone()
    best_n = torch.zeros_like(d)

    def take(t, nrm):
        nonlocal best_t, best_n
        ok = (t > 1e-9) & (t < best_t)
        best_t = torch.where(ok, t, best_t)
        best_n = torch.where(ok[..., None], nrm, best_n)

    for p0, nv, radius in scene.planes:
        p0 = torch.as_tensor(p0, dtype=torch.float64, device=dev)
        nv = torch.as_tensor(nv, dtype=torch.float64, device=dev)
        den = (d * nv).sum(-1)
        t = ((p0 - o) * nv).sum(-1) / torch.where(den.abs() < 1e-12, torch.full_like(den, 1e-12), den)
        if radius is not None:
            hit = o + t[..., None] * d
            t = torch.where(((hit - p0) ** 2).sum(-1) <= radius * radius, t, inf)
        take(t, nv.expand_as(d))

    for c, r in scene.spheres:
        c = torch.as_tensor(c, dtype=torch.float64, device=dev)
        oc = o - c
        b = (oc * d).sum(-1)
        a = (d * d).sum(-1)
        cc = (oc * oc).sum(-1) - r * r
        disc = b * b - a * cc
        sq = torch.sqrt(torch.clamp(disc, min=0.0))
        t = torch.where(disc >= 0, (-b - sq) / a, inf)
        hit = o + t[..., None] * d
        take(t, (hit - c) / r)

    for c, Rb, half in scene.boxes:
        c = torch.as_tensor(c, dtype=torch.float64, device=dev)
        Rb = torch.as_tensor(Rb, dtype=torch.float64, device=dev)
        half = torch.as_tensor(half, dtype=torch.float64, device=dev)
        ol = (o - c) @ Rb  # world -> box local (Rb columns are the box axes)
        dl = d @ Rb
        dl_safe = torch.where(dl.abs() < 1e-15, torch.full_like(dl, 1e-15), dl)
        t1 = (-half - ol) / dl_safe
        t2 = (half - ol) / dl_safe
        tmin = torch.minimum(t1, t2)
        tmax = torch.maximum(t1, t2)
        tn, axis = tmin.max(-1)
        tf = tmax.min(-1).values
        t = torch.where((tn <= tf) & (tf > 0), tn, inf)
        sign = -torch.sign(torch.gather(dl, -1, axis[..., None]))[..., 0]
        nl = torch.zeros_like(dl)
        nl.scatter_(-1, axis[..., None], sign[..., None])
        take(t, nl @ Rb.T)

    for base, axis, r, h in scene.cylinders:
        base = torch.as_tensor(base, dtype=torch.float64, device=dev)
        ax = torch.as_tensor(axis, dtype=torch.float64, device=dev)
        ob = o - base
        d_par = (d * ax).sum(-1)
        o_par = (ob * ax).sum(-1)
        d_perp = d - d_par[..., None] * ax
        o_perp = ob - o_par[..., None] * ax
        a = (d_perp * d_perp).sum(-1)
        b = (o_perp * d_perp).sum(-1)
        cc = (o_perp * o_perp).sum(-1) - r * r
        disc = b * b - a * cc
        a_safe = torch.where(a < 1e-15, torch.full_like(a, 1e-15), a)
        t = torch.where(disc >= 0, (-b - torch.sqrt(torch.clamp(disc, min=0.0))) / a_safe, inf)
        s = o_par + t * d_par
        t = torch.where((s >= 0) & (s <= h), t, inf)
        hit = ob + t[..., None] * d
        radial = hit - ((hit * ax).sum(-1))[..., None] * ax
        take(t, radial / r)
        # top cap
        d_par_safe = torch.where(d_par.abs() < 1e-15, torch.full_like(d_par, 1e-15), d_par)
        tc = (h - o_par) / d_par_safe
        hitc = ob + tc[..., None] * d
        rc = hitc - ((hitc * ax).sum(-1))[..., None] * ax
        tc = torch.where((rc * rc).sum(-1) <= r * r, tc, inf)
        take(tc, ax.expand_as(d))

    return best_t, best_n


def _undistort_normalized(xd, yd, cam: Camera, iters: int = 20):
    """Newton inverse of the Brown-Conrady model (vectorised; rendering only)."""
    x, y = xd.clone(), yd.clone()
    k1, k2, k3, p1, p2 = cam.k1, cam.k2, cam.k3, cam.p1, cam.p2
    for _ in range(iters):
        r2 = x * x + y * y
        radial = 1 + k1 * r2 + k2 * r2 * r2 + k3 * r2 * r2 * r2
        fx_ = x * radial + 2 * p1 * x * y + p2 * (r2 + 2 * x * x) - xd
        fy_ = y * radial + p1 * (r2 + 2 * y * y) + 2 * p2 * x * y - yd
        dr = k1 + 2 * k2 * r2 + 3 * k3 * r2 * r2
        j00 = radial + 2 * x * x * dr + 2 * p1 * y + 6 * p2 * x
        j01 = 2 * x * y * dr + 2 * p1 * x + 2 * p2 * y
        j10 = 2 * x * y * dr + 2 * p1 * x + 2 * p2 * y
        j11 = radial + 2 * y * y * dr + 6 * p1 * y + 2 * p2 * x
        det = j00 * j11 - j01 * j10
        x = x - (j11 * fx_ - j01 * fy_) / det
        y = y - (-j10 * fx_ + j00 * fy_) / det
    return x, y


@dataclass
class RenderedView:
    camera: Camera
    image: np.ndarray           # uint8 (H, W), as captured (distorted when the camera is)
    depth: np.ndarray | None    # float64 (H, W) axial depth of the undistorted camera, NaN = miss
    normal: np.ndarray | None   # float64 (H, W, 3) camera-frame unit normals, facing the camera


def render(scene: Scene, cam: Camera, noise_sigma: float, seed: int, device="cpu",
           truth: bool = True) -> RenderedView:
    dev = torch.device(device)
    W, H = cam.width, cam.height
    u = torch.arange(W, dtype=torch.float64, device=dev) + 0.5
    v = torch.arange(H, dtype=torch.float64, device=dev) + 0.5
    vv, uu = torch.meshgrid(v, u, indexing="ij")
    R = torch.as_tensor(cam.R, dtype=torch.float64, device=dev)
    center = torch.as_tensor(cam.center(), dtype=torch.float64, device=dev)

    def cast(xn, yn):
        dc = torch.stack([xn, yn, torch.ones_like(xn)], -1)  # camera-frame ray, z = 1
        dw = dc @ R  # R^T dc for each ray
        t, nw = _intersect(scene, center.expand_as(dw), dw)
        return dc, dw, t, nw

    xd = (uu - cam.cx) / cam.fx
    yd = (vv - cam.cy) / cam.fy
    distorted = any(abs(k) > 0 for k in (cam.k1, cam.k2, cam.k3, cam.p1, cam.p2))
    xn, yn = _undistort_normalized(xd, yd, cam) if distorted else (xd, yd)
    _, dw, t, _ = cast(xn, yn)
    hit = center + t[..., None] * dw
    ok = torch.isfinite(t)
    a = albedo(scene, torch.where(ok[..., None], hit, torch.zeros_like(hit)))
    img = torch.where(ok, a * 255.0, torch.zeros_like(a))
    g = torch.Generator(device="cpu").manual_seed(seed)
    noise = torch.randn((H, W), generator=g, dtype=torch.float64).to(dev)
    img = torch.clamp(torch.round(img + noise * (noise_sigma * 255.0)), 0, 255).to(torch.uint8)

    depth = normal = None
    if truth:
        dc, _, t2, nw2 = cast(xd, yd) if distorted else cast(xn, yn)
        z = t2 * dc[..., 2]
        depth = torch.where(torch.isfinite(t2), z, torch.full_like(z, float("nan")))
        nc = nw2 @ R.T
        flip = (nc * dc).sum(-1) > 0
        nc = torch.where(flip[..., None], -nc, nc)
        depth = depth.cpu().numpy()
        normal = nc.cpu().numpy()
    return RenderedView(cam, img.cpu().numpy(), depth, normal)


# ----------------------------------------------------------------------------
# the measured workloads
# ----------------------------------------------------------------------------

@dataclass
class MvsScene:
    """A reference view plus its sources, ready for PatchMatchStereo."""

    name: str
    ref: RenderedView
    sources: list
    min_depth: float
    max_depth: float
    seed: int
    extra: dict = field(default_factory=dict)

    @property
    def cameras(self):
        return [self.ref.camera] + [s.camera for s in self.sources]

    @property
    def views(self):
        return [self.ref] + list(self.sources)


def as_reference(sc: MvsScene, k: int) -> MvsScene:
    """The same capture with view k as the reference and every other view as
    a source (view k's truth depth must have been rendered)."""
    v = sc.views
    return MvsScene(f"{sc.name}[{k}]", v[k], v[:k] + v[k + 1:], sc.min_depth, sc.max_depth, sc.seed, sc.extra)


def sphere_on_backdrop(width=640, height=480, f=600.0, num_sources=4, baseline=0.10,
                       seed=1, device="cpu", noise_sigma=1.0 / 255.0) -> MvsScene:
    """Sphere r = 50 mm centred 0.35 m in front of the reference camera, a
    backdrop plane at 0.45 m, sources on a baseline-radius circle around the
    reference, all aimed at the sphere centre; value-noise albedo with an
    ~8 px feature size and contrast 0.2-0.9, Gaussian pixel noise."""
    scale = f / 600.0
    sc = Scene(planes=[((0.0, 0.0, 0.45), (0.0, 0.0, -1.0), None)],
               spheres=[((0.0, 0.0, 0.35), 0.05)],
               noise_scale=8.0 * 0.4 / f)
    # the reference camera frame is the world frame
    R0, t0 = np.eye(3), np.zeros(3)
    cams = [Camera(f, f, width / 2.0, height / 2.0, width, height, R0, t0)]
    rng = np.random.default_rng(seed)
    phase = rng.uniform(0, 2 * math.pi)
    for i in range(num_sources):
        ang = phase + 2 * math.pi * i / num_sources
        c = np.array([baseline * math.cos(ang), baseline * math.sin(ang), 0.0])
        R, t = look_at(c, (0.0, 0.0, 0.35), up=(0.0, -1.0, 0.0))
        cams.append(Camera(f, f, width / 2.0, height / 2.0, width, height, R, t))
    views = [render(sc, cam, noise_sigma, seed * 1000 + i, device) for i, cam in enumerate(cams)]
    del scale
    return MvsScene("sphere_on_backdrop", views[0], views[1:], 0.25, 0.55, seed)


def tabletop_scene(seed: int = 2) -> Scene:
    """World frame: a plane z = 0 (up = +z) with a sphere r = 50 mm, a box
    60 x 40 x 30 mm and three cylinders r = 10 / 15 / 20 mm resting on it;
    10 % of the visible area in low-contrast (0.02) patches."""
    rng = np.random.default_rng(seed)
    a = math.radians(rng.uniform(0, 90))
    Rb = np.array([[math.cos(a), -math.sin(a), 0.0], [math.sin(a), math.cos(a), 0.0], [0.0, 0.0, 1.0]])
    cyl = []
    for (x, y), r, h in zip([(-0.085, 0.045), (-0.04, -0.095), (0.075, -0.085)], (0.010, 0.015, 0.020),
                            (0.060, 0.045, 0.035)):
        cyl.append(((x, y, 0.0), (0.0, 0.0, 1.0), r, h))
    weak = []
    for _ in range(7):
        weak.append(((rng.uniform(-0.16, 0.16), rng.uniform(-0.16, 0.16), 0.0), rng.uniform(0.02, 0.035)))
    return Scene(planes=[((0.0, 0.0, 0.0), (0.0, 0.0, 1.0), 0.32)],
                 spheres=[((0.0, 0.0, 0.05), 0.05)],
                 boxes=[((0.085, 0.05, 0.015), Rb, (0.030, 0.020, 0.015))],
                 cylinders=cyl, noise_scale=8.0 * 0.4 / 1450.0, weak_regions=weak)


def tabletop(width=1920, height=1440, f=1450.0, num_sources=8, k1=0.05, k2=-0.01,
             seed=2, device="cpu", noise_sigma=1.0 / 255.0, baseline=(0.08, 0.12),
             arc_deg=240.0, depth_range=(0.25, 0.70)) -> MvsScene:
    """The full-resolution workload: the tabletop scene seen from 0.375 m
    with the plane spanning about 0.3-0.5 m of depth, 8 sources on a seeded
    80-120 mm baseline arc around the reference, all with Brown-Conrady
    distortion (k1, k2); images are rendered distorted and must be
    undistorted before matching.  Truth depth refers to the undistorted
    reference camera.  The search range covers what every view of the
    capture sees (0.30-0.63 m): used as references, the views on the far
    side of the arc see the table up to 0.63 m."""
    sc = tabletop_scene(seed)
    rng = np.random.default_rng(seed + 17)
    tilt = math.radians(26.7)  # plane normal vs optical axis
    target = np.array([0.0, 0.0, 0.03])
    dist = 0.375
    ref_c = target + dist * np.array([0.0, -math.sin(tilt), math.cos(tilt)])
    R0, t0 = look_at(ref_c, target)
    cx, cy = width / 2.0, height / 2.0
    cams = [Camera(f, f, cx, cy, width, height, R0, t0, k1=k1, k2=k2)]
    right, down = R0[0], R0[1]
    start = rng.uniform(0, 2 * math.pi)
    for i in range(num_sources):
        ang = start + math.radians(arc_deg) * i / max(1, num_sources - 1) + rng.normal(0, 0.05)
        b = rng.uniform(*baseline)
        c = ref_c + b * (math.cos(ang) * right + math.sin(ang) * down)
        R, t = look_at(c, target)
        cams.append(Camera(f, f, cx, cy, width, height, R, t, k1=k1, k2=k2))
    views = [render(sc, cam, noise_sigma, seed * 1000 + i, device) for i, cam in enumerate(cams)]
    return MvsScene("tabletop", views[0], views[1:], depth_range[0], depth_range[1], seed)


def orbit_cameras(n_frames=120, seed=3, resolutions=((640, 480), (1280, 960), (1920, 1440)),
                  f_at_1920=1450.0):
    """A seeded orbit capture of the tabletop scene: radius 0.30-0.45 m,
    elevation 10-60 degrees, each frame at a seeded resolution (focal length
    scaled with the width)."""
    rng = np.random.default_rng(seed)
    cams = []
    for i in range(n_frames):
        az = 2 * math.pi * i / n_frames + rng.normal(0, 0.01)
        el = math.radians(10 + 50 * (0.5 + 0.5 * math.sin(3 * az + rng.normal(0, 0.05))))
        rad = rng.uniform(0.30, 0.45)
        c = np.array([rad * math.cos(el) * math.cos(az), rad * math.cos(el) * math.sin(az), rad * math.sin(el)])
        R, t = look_at(c, (0.0, 0.0, 0.03))
        w, h = resolutions[rng.integers(0, len(resolutions))]
        f = f_at_1920 * w / 1920.0
        cams.append(Camera(f, f, w / 2.0, h / 2.0, w, h, R, t))
    return cams


def orbit_capture(n_frames=120, n_refs=48, seed=3, src_range=(6, 10), min_baseline=0.015, device="cpu",
                  noise_sigma=1.0 / 255.0, resolutions=((640, 480), (1280, 960), (1920, 1440))) -> list:
    """The batched workload: n_refs reference views drawn (seeded) from an
    orbit capture of the tabletop scene (orbit_cameras: radius 0.30-0.45 m,
    elevation 10-60 degrees, a seeded mix of resolutions), each with a seeded
    6-10 sources -- the nearest frames by camera centre at least
    min_baseline away.  Pinhole cameras.  Returns one MvsScene per reference
    (frames shared between scenes are rendered once)."""
    cams = orbit_cameras(n_frames, seed, resolutions)
    scene = tabletop_scene(2)
    rng = np.random.default_rng(seed + 5)
    refs = sorted(int(r) for r in rng.choice(n_frames, n_refs, replace=False))
    centers = np.stack([c.center() for c in cams])
    plan = []
    for r in refs:
        ns = int(rng.integers(src_range[0], src_range[1] + 1))
        d = np.linalg.norm(centers - centers[r], axis=1)
        order = [int(i) for i in np.argsort(d, kind="stable") if i != r and d[i] >= min_baseline]
        plan.append((r, order[:ns]))
    need = sorted({r for r, _ in plan} | {i for _, src in plan for i in src})
    ref_set = {r for r, _ in plan}
    frames = {i: render(scene, cams[i], noise_sigma, seed * 1000 + i, device, truth=i in ref_set) for i in need}
    return [MvsScene(f"orbit[{r}]", frames[r], [frames[i] for i in src], 0.10, 0.90, seed, {"frame": r,
                     "sources": src}) for r, src in plan]


def plane_test_scene(width=160, height=120, f=400.0, num_views=5, baseline=0.016, depth=0.35):
    """The reference unit test's own scene (tests/unit/test_mvs.cpp:56-204):
    a fronto-parallel plane at 0.35 m with the deterministic sinusoid + hash
    texture, sources on an X baseline aimed at the plane centre.  Rendered
    by forward scattering with world-coordinate texture lookups.  Returns
    (images list uint8, cameras, truth depth)."""
    cams = [Camera(f, f, width / 2.0, height / 2.0, width, height, np.eye(3), np.zeros(3))]
    for i in range(1, num_views):
        frac = i / (num_views - 1)
        dx = (frac * 2.0 - 1.0) * baseline
        center = np.array([dx, 0.0, 0.0])
        fwd = np.array([0.0, 0.0, depth]) - center
        fwd /= np.linalg.norm(fwd)
        right = np.cross(fwd, np.array([0.0, -1.0, 0.0]))
        right /= np.linalg.norm(right)
        down = np.cross(fwd, right)
        R = np.stack([right, down, fwd])
        cams.append(Camera(f, f, width / 2.0, height / 2.0, width, height, R, -(R @ center)))

    def texture(tx, ty):
        uu = tx.astype(np.float64) * 0.08
        vv = ty.astype(np.float64) * 0.11
        val = (128.0 + 60.0 * np.sin(uu) * np.cos(vv * 1.3) + 30.0 * np.sin(uu * 2.7 + vv * 0.4)
               + 18.0 * np.cos(uu * 4.1 - vv * 3.3))
        h = ((tx.astype(np.uint32) * np.uint32(73856093)) ^ (ty.astype(np.uint32) * np.uint32(19349663)))
        val += (h & 0xFF).astype(np.float64) * 0.15 - 19.0
        return np.clip(val, 0.0, 255.0).astype(np.uint8)

    images = []
    truth = None
    ys, xs = np.mgrid[0:height, 0:width]
    for vi, cam in enumerate(cams):
        ray = np.stack([(xs + 0.5 - cam.cx) / cam.fx, (ys + 0.5 - cam.cy) / cam.fy, np.ones_like(xs, np.float64)], -1)
        dw = ray @ cam.R
        o = cam.center()
        t = (depth - o[2]) / dw[..., 2]
        p = o + t[..., None] * dw
        if vi == 0:
            truth = p[..., 2].astype(np.float32)
        # std::lround: halves round away from zero
        lround = lambda a: (np.sign(a) * np.floor(np.abs(a) + 0.5)).astype(np.int64)
        tx = lround(p[..., 0] * 1500.0) + 512
        ty = lround(p[..., 1] * 1500.0) + 512
        images.append(texture(tx, ty))
    return images, cams, truth


# ----------------------------------------------------------------------------
# RGBD depth frames for TSDF fusion
# ----------------------------------------------------------------------------

def tsdf_pose(tx: float, ty: float, tz: float, yaw: float) -> np.ndarray:
    """4x4 world -> camera transform: a rotation about y by `yaw` and a
    translation (the reference TSDF test's pose family,
    tests/unit/test_tsdf_tiled.cpp:82-90)."""
    c, s = math.cos(yaw), math.sin(yaw)
    m = np.eye(4)
    m[0, 0], m[0, 2], m[2, 0], m[2, 2] = c, s, -s, c
    m[:3, 3] = (tx, ty, tz)
    return m


def tilted_wall_frames():
    """The reference TSDF test's scene (tests/unit/test_tsdf_tiled.cpp:38-60,
    62-80, 134-138): a 160 x 160 depth frame of the plane
    z = 0.5 + 0.05 x_norm, confidence 220, fused from three poses; its
    TsdfConfig as a dict."""
    w = h = 160
    u = np.arange(w)
    x_norm = (2.0 * u / (w - 1)) - 1.0
    z = 0.5 + 0.05 * x_norm
    row = np.floor(z * 1000.0 + 0.5).astype(np.uint16)  # lround of positive values
    depth = np.tile(row, (h, 1))
    conf = np.full((h, w), 220, np.uint8)
    poses = [tsdf_pose(0.0, 0.0, 0.0, 0.0), tsdf_pose(0.03, 0.01, 0.0, 0.05), tsdf_pose(-0.02, 0.0, 0.0, -0.04)]
    cfg = dict(voxel_size_m=0.004, truncation_m=0.02, min_depth_m=0.05, max_depth_m=2.0, fx=180.0, fy=180.0, cx=80.0,
               cy=80.0, origin_x=-0.30, origin_y=-0.20, origin_z=0.30, bbox_max_x=0.30, bbox_max_y=0.20,
               bbox_max_z=0.70, min_confidence=30)
    return cfg, [(depth, conf, p, 0.004) for p in poses]


def tsdf_capture(width=320, height=240, f=300.0, n_frames=4, seed=0, voxel=0.002, truncation=0.008,
                 holes=0.02, low_confidence=0.05):
    """Depth frames of a sphere (r = 50 mm, centre 0.35 m ahead) in front of
    a wall at 0.45 m, as an RGBD sensor reports them: uint16 millimetres of
    axial depth for the TSDF convention (pixel index = image coordinate, ray
    ((u - cx) / fx, (v - cy) / fy, 1)), Gaussian depth noise growing with
    depth, a seeded share of holes (0) and of confidences below the default
    threshold of 30; poses from tsdf_pose around the first camera; each frame
    with its own depth uncertainty.  Returns (TsdfConfig dict covering the
    scene, frames)."""
    rng = np.random.default_rng(seed)
    cx, cy = width / 2.0, height / 2.0
    v, u = np.mgrid[0:height, 0:width].astype(np.float64)
    dcam = np.stack([(u - cx) / f, (v - cy) / f, np.ones_like(u)], -1)
    frames = []
    for i in range(n_frames):
        yaw = rng.uniform(-0.08, 0.08)
        w2c = tsdf_pose(rng.uniform(-0.02, 0.02), rng.uniform(-0.015, 0.015), rng.uniform(-0.01, 0.01), yaw)
        R, t = w2c[:3, :3], w2c[:3, 3]
        cen = -R.T @ t
        dw = dcam @ R  # R^T d per pixel
        tz = (0.45 - cen[2]) / dw[..., 2]
        oc = cen - np.array([0.0, 0.0, 0.35])
        b = dw @ oc
        a = (dw * dw).sum(-1)
        cc = oc @ oc - 0.05 ** 2
        disc = b * b - a * cc
        ts = np.where(disc >= 0, (-b - np.sqrt(np.maximum(disc, 0.0))) / a, np.inf)
        z = np.where((ts > 0) & (ts < tz), ts, tz)  # camera z = t for d_z = 1
        z = z * (1.0 + rng.normal(0.0, 0.0005, z.shape))
        depth = np.clip(np.floor(z * 1000.0 + 0.5), 0, 65535).astype(np.uint16)
        depth[rng.random(depth.shape) < holes] = 0
        conf = rng.integers(30, 256, depth.shape).astype(np.uint8)
        low = rng.random(depth.shape) < low_confidence
        conf[low] = rng.integers(0, 30, int(low.sum())).astype(np.uint8)
        frames.append((depth, conf, w2c, float(rng.uniform(0.002, 0.006))))
    cfg = dict(voxel_size_m=voxel, truncation_m=truncation, min_depth_m=0.05, max_depth_m=2.0, fx=f, fy=f, cx=cx,
               cy=cy, origin_x=-0.20, origin_y=-0.16, origin_z=0.26, bbox_max_x=0.20, bbox_max_y=0.16,
               bbox_max_z=0.50, min_confidence=30)
    return cfg, frames
