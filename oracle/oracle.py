"""ctypes loader for the CPU checkers (TEST INFRASTRUCTURE ONLY).

Two libraries share one ABI (oracle/mvs_oracle.h):
  * liboracle.so        -- the C restatement of the reference MVS path
                           (oracle/mvs_oracle.c), built here and on any host;
  * _ref/libref_mvs.so  -- the reference's own sources compiled as they are
                           (oracle/ref_wrapper.cpp), where the reference tree
                           or its staged copy (oracle/_ref/tree) is present.

Only tests/, __graft_entry__.smoke() and bench.py (CPU baseline and the
reference arm) may import this module.  The GPU engine never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass, fields

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libref_mvs.so")
REF_RELEASE_SO = os.path.join(HERE, "_ref", "libref_mvs_release.so")
# The reference project's tree: $RECON_REFERENCE_TREE when set, else the
# staged copy of the few files this path needs (`make -C oracle stage`, made
# where the reference exists; git-ignored, it travels with the working tree).
STAGED_TREE = os.path.join(HERE, "_ref", "tree")


def reference_tree() -> str | None:
    env = os.environ.get("RECON_REFERENCE_TREE")
    if env and os.path.isdir(env):
        return env
    if os.path.isfile(os.path.join(STAGED_TREE, "core", "src", "mvs", "patchmatch_stereo.cpp")):
        return STAGED_TREE
    return None


class Intrinsics(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("fx", "fy", "cx", "cy", "k1", "k2", "k3", "p1", "p2", "width", "height")]


class Pose(C.Structure):
    _fields_ = [("r", C.c_double * 9), ("t", C.c_double * 3), ("timestamp_ns", C.c_double)]


# recon::MvsConfig (core/include/recon/mvs.h:24-67), defaults included.
_CONFIG_FIELDS = [
    ("num_views", C.c_int32, 7), ("ref_view_index", C.c_int32, -1),
    ("ideal_angle_min_deg", C.c_double, 8.0), ("ideal_angle_max_deg", C.c_double, 35.0),
    ("max_view_scale_mismatch", C.c_double, 0.15), ("view_angle_weight", C.c_double, 1.0),
    ("view_texture_weight", C.c_double, 0.8), ("view_spread_weight", C.c_double, 0.6),
    ("view_scale_weight", C.c_double, 0.4), ("reference_depth_m", C.c_double, 0.40),
    ("patch_size", C.c_int32, 11), ("iterations", C.c_int32, 4), ("random_search_count", C.c_int32, 5),
    ("random_search_radius_ratio", C.c_double, 0.30), ("restart_ratio", C.c_double, 0.05),
    ("propagation_directions", C.c_int32, 4), ("propagation_enabled", C.c_int32, 1),
    ("num_threads", C.c_int32, 0), ("photo_threshold", C.c_double, 1.0),
    ("depth_regularization", C.c_double, 0.02), ("geo_consistency_threshold", C.c_double, 0.02),
    ("weak_texture_variance", C.c_double, 12.0), ("subpixel_iterations", C.c_int32, 4),
    ("subpixel_fit_points", C.c_int32, 5), ("subpixel_window_ratio", C.c_double, 0.005),
    ("min_depth_m", C.c_double, 0.10), ("max_depth_m", C.c_double, 1.50),
    ("min_view_consistency", C.c_int32, 2), ("fusion_voxel_size_m", C.c_double, 0.001),
]
CONFIG_DEFAULTS = {n: d for n, _, d in _CONFIG_FIELDS}


class Config(C.Structure):
    _fields_ = [(n, t) for n, t, _ in _CONFIG_FIELDS]


def make_config(**overrides) -> Config:
    c = Config()
    for n, _, d in _CONFIG_FIELDS:
        setattr(c, n, overrides.get(n, d))
    unknown = set(overrides) - set(CONFIG_DEFAULTS)
    if unknown:
        raise KeyError(f"unknown MvsConfig fields: {sorted(unknown)}")
    return c


class Views(C.Structure):
    _fields_ = [
        ("ref", C.POINTER(C.c_uint8)), ("ref_w", C.c_int32), ("ref_h", C.c_int32),
        ("num_src", C.c_int32), ("src", C.POINTER(C.POINTER(C.c_uint8))),
        ("src_w", C.POINTER(C.c_int32)), ("src_h", C.POINTER(C.c_int32)),
        ("ref_pose", C.POINTER(Pose)), ("src_poses", C.POINTER(Pose)), ("num_src_poses", C.c_int32),
        ("ref_intr", C.POINTER(Intrinsics)), ("src_intr", C.POINTER(Intrinsics)), ("num_src_intr", C.c_int32),
        ("source_indices", C.POINTER(C.c_int32)),
        ("ref_f", C.POINTER(C.c_float)), ("src_f", C.POINTER(C.POINTER(C.c_float))),
    ]


class NccResult(C.Structure):
    _fields_ = [("valid", C.c_int32), ("ncc", C.c_double), ("weak_texture", C.c_int32), ("valid_samples", C.c_int32)]


class DepthMapC(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("depth", C.POINTER(C.c_float)),
                ("support_count", C.POINTER(C.c_uint8)), ("confidence", C.POINTER(C.c_float))]


class ConsistencyParams(C.Structure):
    _fields_ = [("rel_depth_max", C.c_float), ("reproj_px_max", C.c_float), ("min_views", C.c_int32)]


def intrinsics_from(arr) -> Intrinsics:
    a = np.asarray(arr, np.float64)
    return Intrinsics(*a.tolist())


def pose_from(arr) -> Pose:
    a = np.asarray(arr, np.float64)
    p = Pose()
    for i in range(9):
        p.r[i] = a[i]
    for i in range(3):
        p.t[i] = a[9 + i]
    p.timestamp_ns = a[12] if a.size > 12 else 0.0
    return p


def _ptr(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


class ViewSet:
    """Keeps the numpy buffers of one PatchMatchStereo call alive and exposes
    them as an orc_views struct.  `cams` are synthetic.Camera objects (or any
    object with intrinsics_array()/pose_array()); poses are passed as a
    global array with intrinsics in relative form by default."""

    def __init__(self, ref_img, src_imgs, ref_cam, src_cams, source_indices=None,
                 all_poses=None, intrinsics="relative"):
        # FP32 images (e.g. undistorted intensities) are kept for the plane
        # cost and the plane search; the 8-bit copies are their rounding
        self.is_float = np.issubdtype(np.asarray(ref_img).dtype, np.floating)
        if self.is_float:
            self.ref_f = np.ascontiguousarray(ref_img, np.float32)
            self.srcs_f = [np.ascontiguousarray(s, np.float32) for s in src_imgs]
            ref_img = np.clip(np.round(self.ref_f), 0, 255)
            src_imgs = [np.clip(np.round(s), 0, 255) for s in self.srcs_f]
        self.ref = np.ascontiguousarray(ref_img, np.uint8)
        self.srcs = [np.ascontiguousarray(s, np.uint8) for s in src_imgs]
        n = len(self.srcs)
        if all_poses is None:
            all_poses = [c.pose_array() for c in src_cams]
            source_indices = list(range(n)) if source_indices is None else source_indices
        self.source_indices = np.asarray(source_indices, np.int32)
        self.poses = (Pose * len(all_poses))(*[pose_from(p) for p in all_poses])
        if intrinsics == "relative":
            intr = [c.intrinsics_array() for c in src_cams]
        else:
            intr = intrinsics
        self.intr = (Intrinsics * len(intr))(*[intrinsics_from(k) for k in intr])
        self.ref_pose = pose_from(ref_cam.pose_array())
        self.ref_intr = intrinsics_from(ref_cam.intrinsics_array())
        self.src_ptrs = (C.POINTER(C.c_uint8) * n)(*[_ptr(s, C.c_uint8) for s in self.srcs])
        self.src_w = np.asarray([s.shape[1] for s in self.srcs], np.int32)
        self.src_h = np.asarray([s.shape[0] for s in self.srcs], np.int32)
        self.struct = Views(
            _ptr(self.ref, C.c_uint8), self.ref.shape[1], self.ref.shape[0], n,
            C.cast(self.src_ptrs, C.POINTER(C.POINTER(C.c_uint8))),
            _ptr(self.src_w, C.c_int32), _ptr(self.src_h, C.c_int32),
            C.pointer(self.ref_pose), C.cast(self.poses, C.POINTER(Pose)), len(all_poses),
            C.pointer(self.ref_intr), C.cast(self.intr, C.POINTER(Intrinsics)), len(intr),
            _ptr(self.source_indices, C.c_int32))
        if self.is_float:
            self.src_f_ptrs = (C.POINTER(C.c_float) * n)(*[_ptr(s, C.c_float) for s in self.srcs_f])
            self.struct.ref_f = _ptr(self.ref_f, C.c_float)
            self.struct.src_f = C.cast(self.src_f_ptrs, C.POINTER(C.POINTER(C.c_float)))

    @property
    def shape(self):
        return self.ref.shape


def build_oracle(ref: bool | None = None, quiet=True) -> None:
    """Compile liboracle.so (and the reference library when the reference
    tree exists and `ref` is not False)."""
    targets = ["all"]
    if os.environ.get("RECON_REFERENCE_TREE"):
        targets.append("stage")
    if ref or (ref is None and reference_tree() is not None):
        targets.append("ref")
    subprocess.run(["make", "-s", "-C", HERE, *targets], check=True,
                   stdout=subprocess.DEVNULL if quiet else None)


_LIBS: dict = {}


def _bind(lib: C.CDLL, prefix: str):
    V, P = C.POINTER(Views), C.POINTER(Config)
    f = lambda name: getattr(lib, prefix + name)
    f("compute_ncc").restype = NccResult
    f("compute_ncc").argtypes = [C.POINTER(C.c_uint8), C.c_int32, C.c_int32, C.POINTER(C.c_uint8), C.c_int32,
                                 C.c_int32, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int32]
    f("evaluate_candidates").argtypes = [V, P, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                         C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_int32)]
    f("patchmatch_stereo").restype = C.c_uint32
    f("patchmatch_stereo").argtypes = [V, P, C.POINTER(C.c_double), C.c_int32, C.POINTER(C.c_float),
                                       C.POINTER(C.c_uint8), C.POINTER(C.c_float)]
    f("refine_subpixel").restype = C.c_uint32
    f("refine_subpixel").argtypes = [V, P, C.POINTER(C.c_float), C.POINTER(C.c_uint8), C.POINTER(C.c_float)]
    f("select_source_views").restype = C.c_int32
    f("select_source_views").argtypes = [C.POINTER(Pose), C.POINTER(Pose), C.c_int32, C.POINTER(Intrinsics), P,
                                         C.POINTER(C.c_int32)]
    f("pixel_to_ray").argtypes = [C.POINTER(Intrinsics), C.c_double, C.c_double, C.POINTER(C.c_double)]
    f("project_point").restype = C.c_int32
    f("project_point").argtypes = [C.POINTER(Intrinsics), C.POINTER(C.c_double), C.POINTER(C.c_double),
                                   C.POINTER(C.c_double)]


def load(which: str = "oracle") -> "Checker":
    """which = 'oracle' (the C restatement), 'reference' (the reference's
    own sources, built to pin the restatement bit for bit) or
    'reference_release' (the same sources with the reference's release
    flags: what the CPU baseline times)."""
    if which in _LIBS:
        return _LIBS[which]
    path = {"oracle": ORACLE_SO, "reference": REF_SO, "reference_release": REF_RELEASE_SO}[which]
    if not os.path.exists(path):
        build_oracle(ref=(which != "oracle"))
    lib = C.CDLL(path)
    prefix = "orc_" if which == "oracle" else "ref_"
    _bind(lib, prefix)
    if which == "oracle":
        d = C.POINTER(C.c_double)
        i32 = C.POINTER(C.c_int32)
        V, P = C.POINTER(Views), C.POINTER(Config)
        lib.orc_pm_init.argtypes = [V, P, d, C.c_int32, d, d, i32]
        lib.orc_pm_sweep.argtypes = [V, P, C.c_int32, C.c_int32, d, d, i32, d, d, i32]
        lib.orc_pm_output.restype = C.c_uint32
        lib.orc_pm_output.argtypes = [V, P, d, d, i32, C.POINTER(C.c_float), C.POINTER(C.c_uint8),
                                      C.POINTER(C.c_float)]
        lib.orc_pm_prepare.restype = C.c_int32
        lib.orc_pm_prepare.argtypes = [V, P, d, d, d]
        lib.orc_refine_pixels.argtypes = [V, P, C.POINTER(C.c_float), C.c_int32, i32, i32, d, d, i32]
        lib.orc_fuse_depth_maps.restype = C.c_int64
        lib.orc_fuse_depth_maps.argtypes = [C.POINTER(DepthMapC), C.c_int32, C.POINTER(Pose), C.POINTER(Intrinsics),
                                            P, C.c_int64, C.POINTER(C.c_int64), d, d, C.POINTER(C.c_float),
                                            C.POINTER(C.c_uint32)]
        lib.orc_plane_costs.argtypes = [V, P, C.c_int32, C.c_int32, i32, i32, d, d, d, i32, d, C.c_int32]
        lib.orc_plane_edge_distance.argtypes = [V, P, C.c_int32, C.c_int32, i32, i32, d, d, d]
        lib.orc_geo_consistency.argtypes = [C.POINTER(DepthMapC), C.c_int32, C.POINTER(Pose), C.POINTER(Intrinsics),
                                            C.c_int32, C.POINTER(ConsistencyParams), C.POINTER(C.c_uint8),
                                            C.POINTER(C.c_uint8)]
        lib.orc_relative_transform_f32.argtypes = [C.POINTER(Pose), C.POINTER(Pose), C.POINTER(C.c_float),
                                                   C.POINTER(C.c_float)]
        lib.orc_undistort.argtypes = [C.POINTER(C.c_uint8), C.c_int32, C.c_int32, C.POINTER(Intrinsics),
                                      C.POINTER(C.c_float)]
        lib.orc_plane_patchmatch.restype = C.c_uint32
        lib.orc_plane_patchmatch.argtypes = [V, P, C.c_int32, C.c_uint64, C.c_int32, C.POINTER(C.c_float),
                                             C.POINTER(C.c_float), C.POINTER(C.c_float)]
        lib.orc_plane_patchmatch_ex.restype = C.c_uint32
        lib.orc_plane_patchmatch_ex.argtypes = [V, P, C.c_int32, C.c_uint64, C.c_int32, C.c_int32,
                                                C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float)]
        lib.orc_plane_patchmatch_ex2.restype = C.c_uint32
        lib.orc_plane_patchmatch_ex2.argtypes = [V, P, C.c_int32, C.c_uint64, C.c_int32, C.c_int32, C.c_int32,
                                                 C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float)]
        lib.orc_tsdf_dims.argtypes = [C.POINTER(TsdfConfig), C.POINTER(C.c_int32)]
        lib.orc_tsdf_integrate.restype = C.c_uint32
        lib.orc_tsdf_integrate.argtypes = [C.POINTER(TsdfConfig), C.POINTER(C.c_float), C.POINTER(C.c_float),
                                           C.POINTER(C.c_uint16), C.POINTER(C.c_uint8), C.c_int32, C.c_int32,
                                           C.POINTER(C.c_double), C.c_float]
        lib.orc_tsdf_extract.restype = C.c_int64
        lib.orc_tsdf_extract.argtypes = [C.POINTER(TsdfConfig), C.POINTER(C.c_float), C.POINTER(C.c_float),
                                         C.c_int64, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                         C.POINTER(C.c_float), C.POINTER(C.c_int64)]
        lib.orc_bgra_to_gray.argtypes = [C.POINTER(C.c_uint8), C.c_int32, C.c_int32, C.c_int32,
                                         C.POINTER(C.c_uint8)]
        lib.orc_xorshift_next.restype = C.c_uint32
        lib.orc_xorshift_next.argtypes = [C.POINTER(C.c_uint64)]
        lib.orc_apply_distortion.argtypes = [C.POINTER(Intrinsics), C.c_double, C.c_double, d, d]
    else:
        lib.ref_fuse_depth_maps.restype = C.c_int64
        lib.ref_fuse_depth_maps.argtypes = [C.POINTER(DepthMapC), C.c_int32, C.POINTER(Pose), C.POINTER(Intrinsics),
                                            C.POINTER(Config), C.c_int64, C.POINTER(C.c_double),
                                            C.POINTER(C.c_double), C.POINTER(C.c_float)]
    chk = Checker(lib, prefix)
    _LIBS[which] = chk
    return chk


# ---- TSDF fusion (core/src/rgbd/tsdf_fusion.cpp) ----
REF_TSDF_SO = os.path.join(HERE, "_ref", "libref_tsdf.so")

# TsdfConfig (core/include/recon/tsdf_fusion.h:17-39), defaults included.
_TSDF_FIELDS = [("voxel_size_m", C.c_double, 0.001), ("truncation_m", C.c_double, 0.008),
                ("min_depth_m", C.c_double, 0.05), ("max_depth_m", C.c_double, 3.0), ("fx", C.c_double, 1.0),
                ("fy", C.c_double, 1.0), ("cx", C.c_double, 0.0), ("cy", C.c_double, 0.0),
                ("origin_x", C.c_double, 0.0), ("origin_y", C.c_double, 0.0), ("origin_z", C.c_double, 0.0),
                ("bbox_max_x", C.c_double, 1.0), ("bbox_max_y", C.c_double, 1.0), ("bbox_max_z", C.c_double, 1.0),
                ("min_confidence", C.c_int32, 30)]
TSDF_DEFAULTS = {n: d for n, _, d in _TSDF_FIELDS}


class TsdfConfig(C.Structure):
    _fields_ = [(n, t) for n, t, _ in _TSDF_FIELDS]


def tsdf_config(**overrides) -> TsdfConfig:
    unknown = set(overrides) - set(TSDF_DEFAULTS)
    if unknown:
        raise KeyError(f"unknown TsdfConfig fields: {sorted(unknown)}")
    c = TsdfConfig()
    for n, _, d in _TSDF_FIELDS:
        setattr(c, n, overrides.get(n, d))
    return c


def _tsdf_frames(frames):
    """frames: list of (depth uint16 HxW, confidence uint8 HxW or None, w2c
    4x4, depth uncertainty) -> stacked arrays."""
    depth = np.ascontiguousarray(np.stack([f[0] for f in frames]), np.uint16)
    has_conf = frames[0][1] is not None
    conf = np.ascontiguousarray(np.stack([f[1] for f in frames]), np.uint8) if has_conf else None
    w2c = np.ascontiguousarray(np.stack([np.asarray(f[2], np.float64).reshape(4, 4) for f in frames]), np.float64)
    unc = np.ascontiguousarray([f[3] for f in frames], np.float32)
    return depth, conf, w2c, unc


def tsdf_dims(cfg: TsdfConfig):
    lib = load("oracle").lib
    d = (C.c_int32 * 3)()
    lib.orc_tsdf_dims(C.byref(cfg), d)
    return tuple(int(v) for v in d)


def tsdf_fuse(cfg: TsdfConfig, frames):
    """The oracle: TsdfVolume::IntegrateDepthFrame over the frames, then
    ExtractPoints.  Returns dict(tsdf, weight (nz, ny, nx), integrated,
    positions, normals, confidences, voxel_index)."""
    lib = load("oracle").lib
    nx, ny, nz = tsdf_dims(cfg)
    tsdf = np.ones((nz, ny, nx), np.float32)
    weight = np.zeros((nz, ny, nx), np.float32)
    integ = []
    for dep, cf_, m, u in frames:  # frame by frame: a frame may have no confidence map
        dep = np.ascontiguousarray(dep, np.uint16)
        cf_ = None if cf_ is None else np.ascontiguousarray(cf_, np.uint8)
        m = np.ascontiguousarray(np.asarray(m, np.float64).reshape(4, 4))
        h, w = dep.shape
        integ.append(int(lib.orc_tsdf_integrate(C.byref(cfg), _ptr(tsdf, C.c_float), _ptr(weight, C.c_float),
                                                _ptr(dep, C.c_uint16), _ptr(cf_, C.c_uint8) if cf_ is not None else None,
                                                w, h, _ptr(m, C.c_double), float(u))))
    n = int(lib.orc_tsdf_extract(C.byref(cfg), _ptr(tsdf, C.c_float), _ptr(weight, C.c_float), 0, None, None, None,
                                 None))
    pos = np.zeros((max(n, 1), 3))
    nrm = np.zeros((max(n, 1), 3))
    cf = np.zeros(max(n, 1), np.float32)
    vi = np.zeros(max(n, 1), np.int64)
    lib.orc_tsdf_extract(C.byref(cfg), _ptr(tsdf, C.c_float), _ptr(weight, C.c_float), n, _ptr(pos, C.c_double),
                         _ptr(nrm, C.c_double), _ptr(cf, C.c_float), _ptr(vi, C.c_int64))
    return dict(tsdf=tsdf, weight=weight, integrated=integ, positions=pos[:n], normals=nrm[:n], confidences=cf[:n],
                voxel_index=vi[:n])


def tsdf_reference(cfg: TsdfConfig, frames):
    """The reference's own TSDF code (libref_tsdf.so): dict(tsdf, weight,
    integrated, positions, normals, confidences)."""
    if not os.path.exists(REF_TSDF_SO):
        build_oracle(ref=True)
    lib = C.CDLL(REF_TSDF_SO)
    nx, ny, nz = tsdf_dims(cfg)
    depth, conf, w2c, unc = _tsdf_frames(frames)
    nf, h, w = depth.shape
    tsdf = np.ones((nz, ny, nx), np.float32)
    weight = np.zeros((nz, ny, nx), np.float32)
    cptr = _ptr(conf, C.c_uint8) if conf is not None else None
    lib.ref_tsdf_grid.argtypes = [C.POINTER(TsdfConfig), C.c_int32, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32,
                                  C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.ref_tsdf_grid(C.byref(cfg), nf, depth.ctypes.data, conf.ctypes.data if conf is not None else None, w, h,
                      w2c.ctypes.data, unc.ctypes.data, tsdf.ctypes.data, weight.ctypes.data)
    cap = nx * ny * nz
    pos = np.zeros((cap, 3))
    nrm = np.zeros((cap, 3))
    cf = np.zeros(cap, np.float32)
    integ = np.zeros(nf, np.uint32)
    lib.ref_tsdf_run.restype = C.c_int64
    lib.ref_tsdf_run.argtypes = [C.POINTER(TsdfConfig), C.c_int32, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32,
                                 C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]
    n = int(lib.ref_tsdf_run(C.byref(cfg), nf, depth.ctypes.data, conf.ctypes.data if conf is not None else None, w,
                             h, w2c.ctypes.data, unc.ctypes.data, integ.ctypes.data, cap, pos.ctypes.data,
                             nrm.ctypes.data, cf.ctypes.data))
    del cptr
    return dict(tsdf=tsdf, weight=weight, integrated=[int(v) for v in integ], positions=pos[:n], normals=nrm[:n],
                confidences=cf[:n])


def reference_available() -> bool:
    return os.path.exists(REF_SO) or reference_tree() is not None


@dataclass
class PmOutput:
    filled: int
    depth: np.ndarray
    support: np.ndarray
    confidence: np.ndarray


class Checker:
    """Python face of one checker library; method names follow the
    reference functions they restate."""

    def __init__(self, lib, prefix):
        self.lib = lib
        self.prefix = prefix

    def _f(self, name):
        return getattr(self.lib, self.prefix + name)

    def compute_ncc(self, ref, src, ref_u, ref_v, src_u, src_v, patch_size=11):
        ref = np.ascontiguousarray(ref, np.uint8)
        src = np.ascontiguousarray(src, np.uint8)
        return self._f("compute_ncc")(_ptr(ref, C.c_uint8), ref.shape[1], ref.shape[0], _ptr(src, C.c_uint8),
                                      src.shape[1], src.shape[0], ref_u, ref_v, src_u, src_v, patch_size)

    def evaluate_candidates(self, vs: ViewSet, cfg: Config, px, py, inv):
        px = np.ascontiguousarray(px, np.int32)
        py = np.ascontiguousarray(py, np.int32)
        inv = np.ascontiguousarray(inv, np.float64)
        cost = np.zeros(len(px), np.float64)
        vv = np.zeros(len(px), np.int32)
        self._f("evaluate_candidates")(C.byref(vs.struct), C.byref(cfg), len(px), _ptr(px, C.c_int32),
                                       _ptr(py, C.c_int32), _ptr(inv, C.c_double), _ptr(cost, C.c_double),
                                       _ptr(vv, C.c_int32))
        return cost, vv

    def patchmatch_stereo(self, vs: ViewSet, cfg: Config, seeds=None) -> PmOutput:
        h, w = vs.shape
        depth = np.full((h, w), np.nan, np.float32)
        sup = np.zeros((h, w), np.uint8)
        conf = np.zeros((h, w), np.float32)
        if seeds is not None and len(seeds):
            s = np.ascontiguousarray(seeds, np.float64).reshape(-1, 3)
            sp, ns = _ptr(s, C.c_double), len(s)
        else:
            sp, ns = None, 0
        filled = self._f("patchmatch_stereo")(C.byref(vs.struct), C.byref(cfg), sp, ns, _ptr(depth, C.c_float),
                                              _ptr(sup, C.c_uint8), _ptr(conf, C.c_float))
        return PmOutput(int(filled), depth, sup, conf)

    def refine_subpixel(self, vs: ViewSet, cfg: Config, pm: PmOutput) -> PmOutput:
        depth = pm.depth.copy()
        sup = pm.support.copy()
        conf = pm.confidence.copy()
        n = self._f("refine_subpixel")(C.byref(vs.struct), C.byref(cfg), _ptr(depth, C.c_float),
                                       _ptr(sup, C.c_uint8), _ptr(conf, C.c_float))
        return PmOutput(int(n), depth, sup, conf)

    def select_source_views(self, ref_pose, poses, intr, cfg: Config):
        ps = (Pose * len(poses))(*[pose_from(p) for p in poses])
        out = np.zeros(max(1, len(poses)), np.int32)
        rp = pose_from(ref_pose)
        k = intrinsics_from(intr)
        n = self._f("select_source_views")(C.byref(rp), C.cast(ps, C.POINTER(Pose)), len(poses), C.byref(k),
                                           C.byref(cfg), _ptr(out, C.c_int32))
        return out[:n].tolist()

    def pixel_to_ray(self, intr, u, v):
        k = intrinsics_from(intr)
        ray = np.zeros(3, np.float64)
        self._f("pixel_to_ray")(C.byref(k), u, v, _ptr(ray, C.c_double))
        return ray

    def project_point(self, intr, p):
        k = intrinsics_from(intr)
        p = np.ascontiguousarray(p, np.float64)
        u, v = C.c_double(), C.c_double()
        ok = self._f("project_point")(C.byref(k), _ptr(p, C.c_double), C.byref(u), C.byref(v))
        return bool(ok), u.value, v.value

    # ---- restatement-only entry points ----
    def pm_init(self, vs: ViewSet, cfg: Config, seeds=None):
        h, w = vs.shape
        inv = np.zeros(h * w, np.float64)
        cost = np.zeros(h * w, np.float64)
        sup = np.zeros(h * w, np.int32)
        if seeds is not None and len(seeds):
            s = np.ascontiguousarray(seeds, np.float64).reshape(-1, 3)
            sp, ns = _ptr(s, C.c_double), len(s)
        else:
            sp, ns = None, 0
        self.lib.orc_pm_init(C.byref(vs.struct), C.byref(cfg), sp, ns, _ptr(inv, C.c_double),
                             _ptr(cost, C.c_double), _ptr(sup, C.c_int32))
        return inv, cost, sup

    def pm_sweep(self, vs: ViewSet, cfg: Config, it, direction, inv, cost, sup):
        inv = np.ascontiguousarray(inv, np.float64)
        cost = np.ascontiguousarray(cost, np.float64)
        sup = np.ascontiguousarray(sup, np.int32)
        oi, oc, os_ = np.empty_like(inv), np.empty_like(cost), np.empty_like(sup)
        self.lib.orc_pm_sweep(C.byref(vs.struct), C.byref(cfg), it, direction, _ptr(inv, C.c_double),
                              _ptr(cost, C.c_double), _ptr(sup, C.c_int32), _ptr(oi, C.c_double),
                              _ptr(oc, C.c_double), _ptr(os_, C.c_int32))
        return oi, oc, os_

    def pm_prepare(self, vs: ViewSet, cfg: Config):
        a, b, c = C.c_double(), C.c_double(), C.c_double()
        ok = self.lib.orc_pm_prepare(C.byref(vs.struct), C.byref(cfg), C.byref(a), C.byref(b), C.byref(c))
        return bool(ok), a.value, b.value, c.value

    def refine_pixels(self, vs: ViewSet, cfg: Config, depth, px, py):
        depth = np.ascontiguousarray(depth, np.float32)
        px = np.ascontiguousarray(px, np.int32)
        py = np.ascontiguousarray(py, np.int32)
        bi = np.zeros(len(px), np.float64)
        bc = np.zeros(len(px), np.float64)
        wr = np.zeros(len(px), np.int32)
        self.lib.orc_refine_pixels(C.byref(vs.struct), C.byref(cfg), _ptr(depth, C.c_float), len(px),
                                   _ptr(px, C.c_int32), _ptr(py, C.c_int32), _ptr(bi, C.c_double),
                                   _ptr(bc, C.c_double), _ptr(wr, C.c_int32))
        return bi, bc, wr

    def plane_edge_distance(self, vs: ViewSet, cfg: Config, best_k, px, py, inv, normals):
        """Per hypothesis, the smallest distance (texels) from a sample of
        its averaged views' windows to a source texel edge."""
        px = np.ascontiguousarray(px, np.int32)
        py = np.ascontiguousarray(py, np.int32)
        inv = np.ascontiguousarray(inv, np.float64)
        nrm = np.ascontiguousarray(normals, np.float64).reshape(-1, 3)
        out = np.zeros(len(px), np.float64)
        self.lib.orc_plane_edge_distance(C.byref(vs.struct), C.byref(cfg), best_k, len(px), _ptr(px, C.c_int32),
                                         _ptr(py, C.c_int32), _ptr(inv, C.c_double), _ptr(nrm, C.c_double),
                                         _ptr(out, C.c_double))
        return out

    def plane_costs(self, vs: ViewSet, cfg: Config, best_k, px, py, inv, normals, half_pixel=0):
        px = np.ascontiguousarray(px, np.int32)
        py = np.ascontiguousarray(py, np.int32)
        inv = np.ascontiguousarray(inv, np.float64)
        nrm = np.ascontiguousarray(normals, np.float64).reshape(-1, 3)
        n = len(px)
        cost = np.zeros(n, np.float64)
        vv = np.zeros(n, np.int32)
        view_cost = np.zeros((n, len(vs.srcs)), np.float64)
        self.lib.orc_plane_costs(C.byref(vs.struct), C.byref(cfg), best_k, n, _ptr(px, C.c_int32),
                                 _ptr(py, C.c_int32), _ptr(inv, C.c_double), _ptr(nrm, C.c_double),
                                 _ptr(cost, C.c_double), _ptr(vv, C.c_int32), _ptr(view_cost, C.c_double),
                                 int(half_pixel))
        return cost, vv, view_cost

    def plane_patchmatch(self, vs: ViewSet, cfg: Config, best_k=4, seed=0x5DEECE66D, refine=1, prune=False,
                         explore=0):
        """The plane-mode search with FP64 costs (prune: with the engine's
        exact shortcuts; explore: the engine's exploration schedule, 0 =
        every iteration).  Returns (filled, depth, normal HxWx3, cost)."""
        h, w = vs.ref.shape
        depth = np.zeros((h, w), np.float32)
        normal = np.zeros((h, w, 3), np.float32)
        cost = np.zeros((h, w), np.float32)
        filled = self.lib.orc_plane_patchmatch_ex2(C.byref(vs.struct), C.byref(cfg), int(best_k), int(seed),
                                                   int(refine), int(bool(prune)), int(explore),
                                                   _ptr(depth, C.c_float), _ptr(normal, C.c_float),
                                                   _ptr(cost, C.c_float))
        return int(filled), depth, normal, cost

    def bgra_to_gray(self, bgra):
        b = np.ascontiguousarray(bgra, np.uint8)
        h, w = b.shape[0], b.shape[1]
        out = np.zeros((h, w), np.uint8)
        self.lib.orc_bgra_to_gray(_ptr(b, C.c_uint8), w, h, b.strides[0], _ptr(out, C.c_uint8))
        return out

    def undistort(self, img, intr):
        img = np.ascontiguousarray(img, np.uint8)
        out = np.zeros(img.shape, np.float32)
        k = intrinsics_from(intr)
        self.lib.orc_undistort(_ptr(img, C.c_uint8), img.shape[1], img.shape[0], C.byref(k), _ptr(out, C.c_float))
        return out


def depth_maps_struct(maps):
    """maps: list of (depth float32 HxW, support uint8, confidence float32)."""
    keep = []
    arr = (DepthMapC * len(maps))()
    for i, (d, s, c) in enumerate(maps):
        d = np.ascontiguousarray(d, np.float32)
        s = np.ascontiguousarray(s, np.uint8)
        c = np.ascontiguousarray(c, np.float32)
        keep += [d, s, c]
        arr[i] = DepthMapC(d.shape[1], d.shape[0], _ptr(d, C.c_float), _ptr(s, C.c_uint8), _ptr(c, C.c_float))
    return arr, keep


def fuse_depth_maps(which: str, maps, poses, intrinsics, cfg: Config):
    """Returns positions (N,3), normals (N,3), confidences (N,), sorted
    lexicographically by position (the reference emits unordered_map
    order)."""
    chk = load(which)
    arr, keep = depth_maps_struct(maps)
    ps = (Pose * len(poses))(*[pose_from(p) for p in poses])
    ks = (Intrinsics * len(intrinsics))(*[intrinsics_from(k) for k in intrinsics])
    cap = int(sum(m[0].size for m in maps)) + 1
    pos = np.zeros((cap, 3), np.float64)
    nrm = np.zeros((cap, 3), np.float64)
    conf = np.zeros(cap, np.float32)
    if which == "oracle":
        keys = np.zeros(cap, np.int64)
        cnt = np.zeros(cap, np.uint32)
        n = chk.lib.orc_fuse_depth_maps(arr, len(maps), C.cast(ps, C.POINTER(Pose)), C.cast(ks, C.POINTER(Intrinsics)),
                                        C.byref(cfg), cap, _ptr(keys, C.c_int64), _ptr(pos, C.c_double),
                                        _ptr(nrm, C.c_double), _ptr(conf, C.c_float), _ptr(cnt, C.c_uint32))
    else:
        n = chk.lib.ref_fuse_depth_maps(arr, len(maps), C.cast(ps, C.POINTER(Pose)), C.cast(ks, C.POINTER(Intrinsics)),
                                        C.byref(cfg), cap, _ptr(pos, C.c_double), _ptr(nrm, C.c_double),
                                        _ptr(conf, C.c_float))
    del keep
    pos, nrm, conf = pos[:n], nrm[:n], conf[:n]
    order = np.lexsort((pos[:, 2], pos[:, 1], pos[:, 0]))
    return pos[order], nrm[order], conf[order]


def geo_consistency(maps, poses, intrinsics, ref_index, rel_depth_max, reproj_px_max, min_views):
    chk = load("oracle")
    arr, keep = depth_maps_struct(maps)
    ps = (Pose * len(poses))(*[pose_from(p) for p in poses])
    ks = (Intrinsics * len(intrinsics))(*[intrinsics_from(k) for k in intrinsics])
    prm = ConsistencyParams(rel_depth_max, reproj_px_max, min_views)
    h, w = maps[ref_index][0].shape
    cnt = np.zeros((h, w), np.uint8)
    kp = np.zeros((h, w), np.uint8)
    chk.lib.orc_geo_consistency(arr, len(maps), C.cast(ps, C.POINTER(Pose)), C.cast(ks, C.POINTER(Intrinsics)),
                                ref_index, C.byref(prm), _ptr(cnt, C.c_uint8), _ptr(kp, C.c_uint8))
    del keep
    return cnt, kp


def config_fields():
    return [f[0] for f in _CONFIG_FIELDS]


__all__ = ["load", "make_config", "ViewSet", "Config", "CONFIG_DEFAULTS", "fuse_depth_maps",
           "geo_consistency", "reference_available", "build_oracle", "fields"]
