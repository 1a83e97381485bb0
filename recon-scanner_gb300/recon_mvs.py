"""Python face of the GB300 MVS engine (ctypes over librecon_mvs_gb300.so).

Mirrors the reference's MVS interface (core/include/recon/mvs.h:133-214):
SelectSourceViews, ComputeNcc, PatchMatchStereo, RefineSubpixel and
FuseDepthMaps keep their names, argument meaning and index contract;
MvsConfig keeps its fields and defaults.  The engine-level extras (plane
mode, device-resident jobs, geometric consistency, undistortion, hypothesis
evaluation) sit beside them.

There is no CPU fallback: loading fails loudly when the CUDA library is
missing or cannot be built.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "librecon_mvs_gb300.so")

RECON_OK = 0
RECON_ERR_INVALID_ARGUMENT = 1
RECON_ERR_OUT_OF_MEMORY = 2
RECON_ERR_MVS_GPU_FAILURE = 502

MODE_COMPAT = 0
MODE_PLANE = 1
STORAGE_FP32 = 0
STORAGE_FP16 = 1
STORAGE_BF16 = 2
STORAGE_U8 = 3


class Intrinsics(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("fx", "fy", "cx", "cy", "k1", "k2", "k3", "p1", "p2", "width", "height")]


class Pose(C.Structure):
    _fields_ = [("r", C.c_double * 9), ("t", C.c_double * 3), ("timestamp_ns", C.c_double)]


_CFG = [
    ("num_views", C.c_int32), ("ref_view_index", C.c_int32), ("ideal_angle_min_deg", C.c_double),
    ("ideal_angle_max_deg", C.c_double), ("max_view_scale_mismatch", C.c_double), ("view_angle_weight", C.c_double),
    ("view_texture_weight", C.c_double), ("view_spread_weight", C.c_double), ("view_scale_weight", C.c_double),
    ("reference_depth_m", C.c_double), ("patch_size", C.c_int32), ("iterations", C.c_int32),
    ("random_search_count", C.c_int32), ("random_search_radius_ratio", C.c_double), ("restart_ratio", C.c_double),
    ("propagation_directions", C.c_int32), ("propagation_enabled", C.c_int32), ("num_threads", C.c_int32),
    ("photo_threshold", C.c_double), ("depth_regularization", C.c_double), ("geo_consistency_threshold", C.c_double),
    ("weak_texture_variance", C.c_double), ("subpixel_iterations", C.c_int32), ("subpixel_fit_points", C.c_int32),
    ("subpixel_window_ratio", C.c_double), ("min_depth_m", C.c_double), ("max_depth_m", C.c_double),
    ("min_view_consistency", C.c_int32), ("fusion_voxel_size_m", C.c_double),
]


class MvsConfig(C.Structure):
    """recon::MvsConfig (mvs.h:24-67); MvsConfig() has the reference defaults."""

    _fields_ = _CFG

    def __init__(self, **kw):
        super().__init__()
        _lib().recon_mvs_config_default(C.byref(self))
        for k, v in kw.items():
            if k not in dict(_CFG):
                raise KeyError(k)
            setattr(self, k, v)

    def set_param(self, key: str, value):
        """recon_set_param semantics for the mvs_* keys (see the C header)."""
        st = _lib().recon_mvs_config_set_param(C.byref(self), key.encode(), int(round(value)) if isinstance(value, (int, np.integer)) else int(value),
                                               float(value))
        _check(st)

    def apply_preset(self, preset: int):
        _check(_lib().recon_mvs_config_apply_preset(C.byref(self), preset))


class Options(C.Structure):
    _fields_ = [("mode", C.c_int32), ("storage", C.c_int32), ("best_k", C.c_int32), ("refine", C.c_int32),
                ("seed", C.c_uint64), ("device", C.c_int32), ("sampling", C.c_int32), ("prefilter", C.c_int32),
                ("interp", C.c_int32), ("tile_rows", C.c_int32), ("per_view", C.c_int32),
                ("exhaustive", C.c_int32), ("coarse_iterations", C.c_int32), ("window_staging", C.c_int32),
                ("exploration_iterations", C.c_int32)]

    def __init__(self, **kw):
        super().__init__()
        _lib().recon_mvs_options_default(C.byref(self))
        for k, v in kw.items():
            setattr(self, k, v)


class Views(C.Structure):
    _fields_ = [
        ("ref_gray", C.POINTER(C.c_uint8)), ("ref_w", C.c_int32), ("ref_h", C.c_int32), ("num_src", C.c_int32),
        ("src_gray", C.POINTER(C.POINTER(C.c_uint8))), ("src_w", C.POINTER(C.c_int32)),
        ("src_h", C.POINTER(C.c_int32)), ("ref_pose", C.POINTER(Pose)), ("src_poses", C.POINTER(Pose)),
        ("num_src_poses", C.c_int32), ("ref_intr", C.POINTER(Intrinsics)),
        ("src_intrinsics", C.POINTER(Intrinsics)), ("num_src_intrinsics", C.c_int32),
        ("source_indices", C.POINTER(C.c_int32)),
    ]


class DepthMapC(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("depth", C.POINTER(C.c_float)),
                ("support_count", C.POINTER(C.c_uint8)), ("confidence", C.POINTER(C.c_float)),
                ("normal", C.POINTER(C.c_float)), ("cost", C.POINTER(C.c_float))]


class NccResult(C.Structure):
    _fields_ = [("valid", C.c_int32), ("ncc", C.c_double), ("weak_texture", C.c_int32), ("valid_samples", C.c_int32)]


class PointCloudC(C.Structure):
    _fields_ = [("count", C.c_int64), ("positions", C.POINTER(C.c_double)), ("normals", C.POINTER(C.c_double)),
                ("colors", C.POINTER(C.c_float)), ("confidences", C.POINTER(C.c_float)),
                ("keys", C.POINTER(C.c_int64)), ("counts", C.POINTER(C.c_uint32))]


class DeviceCloudC(C.Structure):
    _fields_ = [("count", C.c_int64), ("positions", C.c_void_p), ("normals", C.c_void_p), ("colors", C.c_void_p),
                ("confidences", C.c_void_p), ("weights", C.c_void_p), ("keys", C.c_void_p), ("counts", C.c_void_p),
                ("bounds_lo", C.c_double * 3), ("bounds_hi", C.c_double * 3), ("device", C.c_int32),
                ("impl", C.c_void_p)]


class TsdfConfig(C.Structure):
    """recon::TsdfConfig (tsdf_fusion.h:17-39); TsdfConfig() has the reference defaults."""

    _fields_ = [("voxel_size_m", C.c_double), ("truncation_m", C.c_double), ("min_depth_m", C.c_double),
                ("max_depth_m", C.c_double), ("fx", C.c_double), ("fy", C.c_double), ("cx", C.c_double),
                ("cy", C.c_double), ("origin_x", C.c_double), ("origin_y", C.c_double), ("origin_z", C.c_double),
                ("bbox_max_x", C.c_double), ("bbox_max_y", C.c_double), ("bbox_max_z", C.c_double),
                ("min_confidence", C.c_int32)]

    def __init__(self, **kw):
        super().__init__()
        _lib().recon_tsdf_config_default(C.byref(self))
        for k, v in kw.items():
            setattr(self, k, v)


class Stats(C.Structure):
    _fields_ = [("hypotheses_evaluated", C.c_uint64), ("last_run_ms", C.c_double), ("last_sweep_ms", C.c_double),
                ("last_sweep_launches", C.c_int32), ("tile_rows", C.c_int32), ("ctas_per_sm", C.c_int32),
                ("graph_launches", C.c_int32), ("tune_trials", C.c_int32), ("window_staging", C.c_int32),
                ("windows_evaluated", C.c_uint64), ("windows_staged", C.c_uint64)]


CANCEL_FN = C.CFUNCTYPE(C.c_int32, C.c_void_p)
PROGRESS_FN = C.CFUNCTYPE(None, C.c_void_p, C.c_double)


class StageParams(C.Structure):
    _fields_ = [("undistort", C.c_int32), ("batch_size", C.c_int32), ("consistency_views", C.c_int32),
                ("plane_normals", C.c_int32), ("consistency_rel_depth", C.c_float),
                ("consistency_reproj_px", C.c_float),
                ("cancel", CANCEL_FN), ("progress", PROGRESS_FN), ("user", C.c_void_p)]


class MvsError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"recon_status {status}: {msg}")
        self.status = status


_LIB = None

# every C symbol the header declares, with its ctypes signature
_SIGS = {
    "recon_mvs_abi_version": (C.c_uint32, []),
    "recon_mvs_last_error": (C.c_char_p, []),
    "recon_mvs_config_default": (None, [C.POINTER(MvsConfig)]),
    "recon_mvs_options_default": (None, [C.POINTER(Options)]),
    "recon_mvs_config_set_param": (C.c_int, [C.POINTER(MvsConfig), C.c_char_p, C.c_int32, C.c_double]),
    "recon_mvs_config_apply_preset": (C.c_int, [C.POINTER(MvsConfig), C.c_int32]),
    "recon_mvs_select_source_views": (C.c_int, [C.POINTER(Pose), C.POINTER(Pose), C.c_int32, C.POINTER(Intrinsics),
                                                C.POINTER(MvsConfig), C.POINTER(C.c_int32), C.c_int32,
                                                C.POINTER(C.c_int32)]),
    "recon_mvs_compute_ncc": (C.c_int, [C.POINTER(C.c_uint8), C.c_int32, C.c_int32, C.POINTER(C.c_uint8), C.c_int32,
                                        C.c_int32, C.POINTER(C.c_double), C.c_int32, C.c_int32,
                                        C.POINTER(NccResult)]),
    "recon_mvs_evaluate": (C.c_int, [C.POINTER(Views), C.POINTER(MvsConfig), C.POINTER(Options), C.c_int32,
                                     C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_double),
                                     C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_int32),
                                     C.POINTER(C.c_float)]),
    "recon_mvs_patchmatch": (C.c_int, [C.POINTER(Views), C.POINTER(MvsConfig), C.POINTER(Options),
                                       C.POINTER(C.c_double), C.c_int32, C.POINTER(DepthMapC),
                                       C.POINTER(C.c_uint32)]),
    "recon_mvs_refine_subpixel": (C.c_int, [C.POINTER(Views), C.POINTER(MvsConfig), C.POINTER(Options),
                                            C.POINTER(DepthMapC), C.POINTER(C.c_uint32)]),
    "recon_mvs_geometric_consistency": (C.c_int, [C.POINTER(DepthMapC), C.POINTER(Pose), C.POINTER(Intrinsics),
                                                  C.c_int32, C.c_int32, C.c_float, C.c_float, C.c_int32,
                                                  C.POINTER(C.c_uint8), C.POINTER(C.c_uint8)]),
    "recon_mvs_geometric_consistency_noalloc": (C.c_int, [C.POINTER(DepthMapC), C.POINTER(Pose),
                                                          C.POINTER(Intrinsics), C.c_int32, C.c_int32, C.c_float,
                                                          C.c_float, C.c_int32, C.c_void_p, C.c_void_p,
                                                          C.c_void_p]),
    "recon_mvs_fuse": (C.c_int, [C.POINTER(DepthMapC), C.POINTER(Pose), C.POINTER(Intrinsics), C.c_int32,
                                 C.POINTER(MvsConfig), C.POINTER(C.POINTER(C.c_uint8)), C.POINTER(PointCloudC)]),
    "recon_mvs_point_cloud_free": (None, [C.POINTER(PointCloudC)]),
    "recon_mvs_undistort": (C.c_int, [C.POINTER(C.c_uint8), C.c_int32, C.c_int32, C.POINTER(Intrinsics),
                                      C.POINTER(C.c_float)]),
    "recon_mvs_context_create": (C.c_int, [C.POINTER(Options), C.POINTER(C.c_void_p)]),
    "recon_mvs_context_destroy": (None, [C.c_void_p]),
    "recon_mvs_job_stage": (C.c_int, [C.c_void_p, C.POINTER(Views), C.POINTER(MvsConfig), C.c_int32,
                                      C.POINTER(C.c_int32)]),
    "recon_mvs_job_run": (C.c_int, [C.c_void_p, C.c_int32]),
    "recon_mvs_jobs_run": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.c_int32]),
    "recon_mvs_job_download": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(DepthMapC), C.POINTER(C.c_uint32)]),
    "recon_mvs_image_stage": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint8), C.c_int32, C.c_int32,
                                        C.POINTER(Intrinsics), C.c_int32, C.POINTER(C.c_int32)]),
    "recon_mvs_image_release": (C.c_int, [C.c_void_p, C.c_int32]),
    "recon_mvs_image_stage_bgra": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint8), C.c_int32, C.c_int32, C.c_int32,
                                             C.POINTER(Intrinsics), C.c_int32, C.POINTER(C.c_int32)]),
    "recon_mvs_bgra_to_gray": (C.c_int, [C.POINTER(C.c_uint8), C.c_int32, C.c_int32, C.c_int32,
                                         C.POINTER(C.c_uint8)]),
    "recon_mvs_job_stage_images": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.POINTER(C.c_int32),
                                             C.POINTER(Pose), C.POINTER(Pose), C.POINTER(MvsConfig),
                                             C.POINTER(C.c_int32)]),
    "recon_mvs_stage_run": (C.c_int, [C.c_void_p, C.POINTER(C.POINTER(C.c_uint8)), C.POINTER(C.c_int32),
                                      C.POINTER(C.c_int32), C.POINTER(Pose), C.POINTER(Intrinsics), C.c_int32,
                                      C.POINTER(MvsConfig), C.POINTER(StageParams), C.POINTER(PointCloudC),
                                      C.POINTER(C.c_int32)]),
    "recon_mvs_stage_run_device": (C.c_int, [C.c_void_p, C.POINTER(C.POINTER(C.c_uint8)), C.POINTER(C.c_int32),
                                             C.POINTER(C.c_int32), C.POINTER(Pose), C.POINTER(Intrinsics), C.c_int32,
                                             C.POINTER(MvsConfig), C.POINTER(StageParams), C.POINTER(DeviceCloudC),
                                             C.POINTER(C.c_int32)]),
    "recon_mvs_device_cloud_download": (C.c_int, [C.c_void_p, C.POINTER(DeviceCloudC), C.POINTER(PointCloudC)]),
    "recon_mvs_device_cloud_free": (None, [C.POINTER(DeviceCloudC)]),
    "recon_mvs_test_inject_tma_timeout": (C.c_int, [C.c_void_p]),
    "recon_tsdf_config_default": (C.c_int, [C.c_void_p]),
    "recon_tsdf_create": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_void_p)]),
    "recon_tsdf_integrate": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint16), C.POINTER(C.c_uint8), C.c_int32,
                                       C.c_int32, C.POINTER(C.c_double), C.c_float, C.POINTER(C.c_uint32)]),
    "recon_tsdf_extract_points": (C.c_int, [C.c_void_p, C.POINTER(PointCloudC)]),
    "recon_tsdf_dims": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    "recon_tsdf_memory_usage": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint64)]),
    "recon_tsdf_read_grid": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "recon_tsdf_destroy": (None, [C.c_void_p]),
    "recon_mvs_job_adjoint": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.POINTER(C.c_int32),
                                        C.POINTER(C.c_int32), C.POINTER(C.c_double), C.POINTER(C.c_double),
                                        C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float),
                                        C.POINTER(C.c_float)]),
    "recon_mvs_job_recover_poses": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.POINTER(C.c_int32),
                                              C.POINTER(C.c_int32), C.POINTER(C.c_double), C.POINTER(C.c_double),
                                              C.c_int32, C.POINTER(Pose), C.POINTER(C.c_double)]),
    "recon_mvs_job_release": (C.c_int, [C.c_void_p, C.c_int32]),
    "recon_mvs_synchronize": (C.c_int, [C.c_void_p]),
    "recon_mvs_context_stats": (C.c_int, [C.c_void_p, C.POINTER(Stats)]),
}


def load_library(path: str = LIB_PATH, build_if_missing: bool = True) -> C.CDLL:
    """Load (building first if needed) the CUDA library and bind every
    symbol.  Raises when it cannot: there is no other implementation."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise OSError(f"{path} missing; build it with recon-scanner_gb300/build.py")
        import importlib.util

        spec = importlib.util.spec_from_file_location("recon_mvs_build", os.path.join(HERE, "build.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build()
    lib = C.CDLL(path)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


_lib = load_library


def _check(st):
    if st != RECON_OK:
        raise MvsError(st, _lib().recon_mvs_last_error().decode(errors="replace"))


def _ptr(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


def intrinsics(arr) -> Intrinsics:
    return Intrinsics(*np.asarray(arr, np.float64).tolist())


def pose(arr) -> Pose:
    a = np.asarray(arr, np.float64)
    p = Pose()
    for i in range(9):
        p.r[i] = a[i]
    for i in range(3):
        p.t[i] = a[9 + i]
    return p


class ViewArgs:
    """Arguments of one PatchMatchStereo call, kept alive for the ABI.

    ref_gray: uint8 HxW; src_gray: list of uint8 images (relative index k);
    poses: the global pose array (13 doubles each, recon_pose order);
    source_indices: global indices of the sources; intrinsics: list of 11
    doubles, global (len == len(poses)) or relative (len == len(src_gray)).
    """

    def __init__(self, ref_gray, src_gray, ref_pose, poses, ref_intr, src_intrinsics, source_indices):
        self.ref = np.ascontiguousarray(ref_gray, np.uint8)
        self.srcs = [np.ascontiguousarray(s, np.uint8) for s in src_gray]
        n = len(self.srcs)
        self.src_ptrs = (C.POINTER(C.c_uint8) * max(1, n))(*[_ptr(s, C.c_uint8) for s in self.srcs])
        self.src_w = np.asarray([s.shape[1] for s in self.srcs] or [0], np.int32)
        self.src_h = np.asarray([s.shape[0] for s in self.srcs] or [0], np.int32)
        self.ref_pose = pose(ref_pose)
        self.poses = (Pose * max(1, len(poses)))(*[pose(p) for p in poses])
        self.ref_intr = intrinsics(ref_intr)
        self.intr = (Intrinsics * max(1, len(src_intrinsics)))(*[intrinsics(k) for k in src_intrinsics])
        self.idx = np.asarray(source_indices, np.int32)
        self.struct = Views(_ptr(self.ref, C.c_uint8), self.ref.shape[1], self.ref.shape[0], n,
                            C.cast(self.src_ptrs, C.POINTER(C.POINTER(C.c_uint8))), _ptr(self.src_w, C.c_int32),
                            _ptr(self.src_h, C.c_int32), C.pointer(self.ref_pose),
                            C.cast(self.poses, C.POINTER(Pose)), len(poses), C.pointer(self.ref_intr),
                            C.cast(self.intr, C.POINTER(Intrinsics)), len(src_intrinsics),
                            _ptr(self.idx, C.c_int32))

    @classmethod
    def from_cameras(cls, ref_img, src_imgs, ref_cam, src_cams):
        """Convenience: cameras with intrinsics_array()/pose_array(); the
        global pose array is the sources' own, intrinsics relative."""
        poses = [c.pose_array() for c in src_cams]
        return cls(ref_img, src_imgs, ref_cam.pose_array(), poses, ref_cam.intrinsics_array(),
                   [c.intrinsics_array() for c in src_cams], list(range(len(src_cams))))

    @property
    def shape(self):
        return self.ref.shape


@dataclass
class DepthMap:
    """recon::DepthMap (mvs.h:85-109) plus the engine's normal and cost maps."""

    depth: np.ndarray
    support_count: np.ndarray
    confidence: np.ndarray
    normal: np.ndarray | None = None
    cost: np.ndarray | None = None
    filled: int = 0

    @classmethod
    def allocate(cls, w, h, with_normal=True):
        return cls(np.full((h, w), np.nan, np.float32), np.zeros((h, w), np.uint8), np.zeros((h, w), np.float32),
                   np.zeros((h, w, 3), np.float32) if with_normal else None, np.zeros((h, w), np.float32))

    @property
    def width(self):
        return self.depth.shape[1]

    @property
    def height(self):
        return self.depth.shape[0]

    def struct(self):
        return DepthMapC(self.width, self.height, _ptr(self.depth, C.c_float), _ptr(self.support_count, C.c_uint8),
                         _ptr(self.confidence, C.c_float),
                         _ptr(self.normal, C.c_float) if self.normal is not None else None,
                         _ptr(self.cost, C.c_float) if self.cost is not None else None)


@dataclass
class PointCloud:
    positions: np.ndarray
    normals: np.ndarray
    colors: np.ndarray
    confidences: np.ndarray
    keys: np.ndarray
    counts: np.ndarray

    def size(self):
        return len(self.positions)


class _DeviceArray:
    """A device array of a DeviceCloud seen through __cuda_array_interface__
    (torch.as_tensor(view, device="cuda") wraps it without a copy)."""

    def __init__(self, ptr, shape, typestr, owner):
        self._owner = owner  # keeps the cloud alive while the view is used
        self.__cuda_array_interface__ = {"shape": shape, "typestr": typestr, "data": (int(ptr or 0), False),
                                         "version": 3}


class DeviceCloud:
    """A fused cloud left in device memory (recon_mvs_device_cloud): one
    record per voxel; .array(name) views a field on the device, .download()
    copies the cloud to the host, .free() releases it."""

    _FIELDS = {"positions": (3, "<f8"), "normals": (3, "<f8"), "colors": (3, "<f4"), "confidences": (1, "<f4"),
               "weights": (1, "<f4"), "keys": (1, "<i8"), "counts": (1, "<u4")}

    def __init__(self, engine, c: DeviceCloudC):
        self.engine = engine
        self.c = c

    @property
    def count(self):
        return int(self.c.count)

    @property
    def bounds(self):
        return np.array(list(self.c.bounds_lo)), np.array(list(self.c.bounds_hi))

    def array(self, name):
        k, t = self._FIELDS[name]
        shape = (self.count, k) if k > 1 else (self.count,)
        return _DeviceArray(getattr(self.c, name), shape, t, self)

    def download(self) -> "PointCloud":
        pc = PointCloudC()
        _check(_lib().recon_mvs_device_cloud_download(self.engine.ctx, C.byref(self.c), C.byref(pc)))
        return _take_cloud(pc)

    def free(self):
        if self.c.impl:
            _lib().recon_mvs_device_cloud_free(C.byref(self.c))

    def __del__(self):
        try:
            self.free()
        except Exception:  # noqa: BLE001 -- interpreter shutdown
            pass


# ----------------------------------------------------------------------------
# the reference's functions
# ----------------------------------------------------------------------------

def SelectSourceViews(ref_pose, poses, intrinsics_, config: MvsConfig):
    out = np.zeros(max(1, len(poses)), np.int32)
    n = C.c_int32()
    ps = (Pose * max(1, len(poses)))(*[pose(p) for p in poses])
    rp, k = pose(ref_pose), intrinsics(intrinsics_)
    _check(_lib().recon_mvs_select_source_views(C.byref(rp), C.cast(ps, C.POINTER(Pose)), len(poses), C.byref(k),
                                                C.byref(config), _ptr(out, C.c_int32), len(out), C.byref(n)))
    return out[: n.value].tolist()


def ComputeNcc(ref_img, src_img, ref_u, ref_v, src_u, src_v, patch_size=11) -> NccResult:
    return ComputeNccBatch(ref_img, src_img, np.array([[ref_u, ref_v, src_u, src_v]]), patch_size)[0]


def ComputeNccBatch(ref_img, src_img, coords, patch_size=11):
    ref_img = np.ascontiguousarray(ref_img, np.uint8)
    src_img = np.ascontiguousarray(src_img, np.uint8)
    coords = np.ascontiguousarray(coords, np.float64).reshape(-1, 4)
    out = (NccResult * max(1, len(coords)))()
    _check(_lib().recon_mvs_compute_ncc(_ptr(ref_img, C.c_uint8), ref_img.shape[1], ref_img.shape[0],
                                        _ptr(src_img, C.c_uint8), src_img.shape[1], src_img.shape[0],
                                        _ptr(coords, C.c_double), len(coords), patch_size, out))
    return [out[i] for i in range(len(coords))]


def PatchMatchStereo(views: ViewArgs, config: MvsConfig, seed_points=None, options: Options | None = None) -> DepthMap:
    """recon::PatchMatchStereo.  Returns the depth map; .filled is the
    reference's return value."""
    options = options or Options()
    h, w = views.shape
    dm = DepthMap.allocate(w, h)
    filled = C.c_uint32()
    if seed_points is not None and len(seed_points):
        s = np.ascontiguousarray(seed_points, np.float64).reshape(-1, 3)
        sp, ns = _ptr(s, C.c_double), len(s)
    else:
        sp, ns = None, 0
    st = dm.struct()
    _check(_lib().recon_mvs_patchmatch(C.byref(views.struct), C.byref(config), C.byref(options), sp, ns, C.byref(st),
                                       C.byref(filled)))
    dm.filled = int(filled.value)
    return dm


def RefineSubpixel(views: ViewArgs, config: MvsConfig, depth: DepthMap, options: Options | None = None) -> int:
    """recon::RefineSubpixel, in place; returns the refined-pixel count."""
    n = C.c_uint32()
    st = depth.struct()
    _check(_lib().recon_mvs_refine_subpixel(C.byref(views.struct), C.byref(config),
                                            C.byref(options) if options else None, C.byref(st), C.byref(n)))
    return int(n.value)


def FuseDepthMaps(depth_maps, poses, intrinsics_list, config: MvsConfig, keep_masks=None) -> PointCloud:
    """recon::FuseDepthMaps; depth_maps is a list of DepthMap."""
    n = len(depth_maps)
    arr = (DepthMapC * max(1, n))(*[d.struct() for d in depth_maps])
    ps = (Pose * max(1, n))(*[pose(p) for p in poses])
    ks = (Intrinsics * max(1, n))(*[intrinsics(k) for k in intrinsics_list])
    keep_ptrs = None
    keeps = None
    if keep_masks is not None:
        keeps = [None if k is None else np.ascontiguousarray(k, np.uint8) for k in keep_masks]
        keep_ptrs = (C.POINTER(C.c_uint8) * n)(*[None if k is None else _ptr(k, C.c_uint8) for k in keeps])
    pc = PointCloudC()
    _check(_lib().recon_mvs_fuse(arr, C.cast(ps, C.POINTER(Pose)), C.cast(ks, C.POINTER(Intrinsics)), n,
                                 C.byref(config), keep_ptrs, C.byref(pc)))
    del keeps  # the masks had to outlive the call
    return _take_cloud(pc)


def _take_cloud(pc: PointCloudC) -> PointCloud:
    """Copy a library-allocated cloud into numpy arrays and free it."""
    try:
        m = int(pc.count)
        if m == 0:
            z = np.zeros((0, 3))
            return PointCloud(z, z.copy(), np.zeros(0, np.float32), np.zeros(0, np.float32), np.zeros(0, np.int64),
                              np.zeros(0, np.uint32))
        cp = lambda p, k, dt: np.ctypeslib.as_array(p, shape=(m * k,)).astype(dt).copy()
        return PointCloud(cp(pc.positions, 3, np.float64).reshape(m, 3), cp(pc.normals, 3, np.float64).reshape(m, 3),
                          cp(pc.colors, 3, np.float32), cp(pc.confidences, 1, np.float32),
                          cp(pc.keys, 1, np.int64), cp(pc.counts, 1, np.uint32))
    finally:
        _lib().recon_mvs_point_cloud_free(C.byref(pc))


# ----------------------------------------------------------------------------
# engine extras
# ----------------------------------------------------------------------------

def Evaluate(views: ViewArgs, config: MvsConfig, options: Options, px, py, inv_depth, normals=None, per_view=False):
    px = np.ascontiguousarray(px, np.int32)
    py = np.ascontiguousarray(py, np.int32)
    inv = np.ascontiguousarray(inv_depth, np.float64)
    n = len(px)
    nrm = None if normals is None else np.ascontiguousarray(normals, np.float32).reshape(-1, 3)
    cost = np.zeros(n, np.float32)
    sup = np.zeros(n, np.int32)
    vc = np.zeros((n, len(views.srcs)), np.float32) if per_view else None
    _check(_lib().recon_mvs_evaluate(C.byref(views.struct), C.byref(config), C.byref(options), n,
                                     _ptr(px, C.c_int32), _ptr(py, C.c_int32), _ptr(inv, C.c_double),
                                     _ptr(nrm, C.c_float) if nrm is not None else None, _ptr(cost, C.c_float),
                                     _ptr(sup, C.c_int32), _ptr(vc, C.c_float) if vc is not None else None))
    return (cost, sup, vc) if per_view else (cost, sup)


def GeometricConsistency(depth_maps, poses, intrinsics_list, ref_index, rel_depth_max, reproj_px_max, min_views):
    n = len(depth_maps)
    arr = (DepthMapC * n)(*[d.struct() for d in depth_maps])
    ps = (Pose * n)(*[pose(p) for p in poses])
    ks = (Intrinsics * n)(*[intrinsics(k) for k in intrinsics_list])
    h, w = depth_maps[ref_index].depth.shape
    cnt = np.zeros((h, w), np.uint8)
    keep = np.zeros((h, w), np.uint8)
    _check(_lib().recon_mvs_geometric_consistency(arr, C.cast(ps, C.POINTER(Pose)), C.cast(ks, C.POINTER(Intrinsics)),
                                                  n, ref_index, rel_depth_max, reproj_px_max, min_views,
                                                  _ptr(cnt, C.c_uint8), _ptr(keep, C.c_uint8)))
    return cnt, keep


def BgraToGray(bgra):
    """BgraToGray (orchestrator.cpp:53-67) on the device: H x W x 4 -> H x W."""
    b = np.ascontiguousarray(bgra, np.uint8)
    h, w = b.shape[0], b.shape[1]
    out = np.zeros((h, w), np.uint8)
    _check(_lib().recon_mvs_bgra_to_gray(_ptr(b, C.c_uint8), w, h, b.strides[0], _ptr(out, C.c_uint8)))
    return out


def Undistort(img, intrinsics_):
    img = np.ascontiguousarray(img, np.uint8)
    out = np.zeros(img.shape, np.float32)
    k = intrinsics(intrinsics_)
    _check(_lib().recon_mvs_undistort(_ptr(img, C.c_uint8), img.shape[1], img.shape[0], C.byref(k),
                                      _ptr(out, C.c_float)))
    return out


class Engine:
    """A context with device-resident jobs (one reference view each)."""

    def __init__(self, options: Options | None = None):
        self.options = options or Options()
        self.ctx = C.c_void_p()
        _check(_lib().recon_mvs_context_create(C.byref(self.options), C.byref(self.ctx)))
        self._keep = {}
        self._nsrc = {}
        self._img_shape = {}

    def stage(self, views: ViewArgs, config: MvsConfig, undistort=False) -> int:
        job = C.c_int32()
        _check(_lib().recon_mvs_job_stage(self.ctx, C.byref(views.struct), C.byref(config), int(undistort),
                                          C.byref(job)))
        self._keep[job.value] = views.shape
        self._nsrc[job.value] = len(views.srcs)
        return job.value

    def run(self, job: int):
        _check(_lib().recon_mvs_job_run(self.ctx, job))

    def run_many(self, jobs):
        arr = np.ascontiguousarray(jobs, np.int32)
        _check(_lib().recon_mvs_jobs_run(self.ctx, _ptr(arr, C.c_int32), len(arr)))

    def download(self, job: int, dm: DepthMap | None = None) -> DepthMap:
        h, w = self._keep[job]
        dm = dm or DepthMap.allocate(w, h)
        f = C.c_uint32()
        st = dm.struct()
        _check(_lib().recon_mvs_job_download(self.ctx, job, C.byref(st), C.byref(f)))
        dm.filled = int(f.value)
        return dm

    def stage_image(self, gray, intr, undistort=False) -> int:
        """Upload one image once for any number of jobs (intr: 11 values or
        Intrinsics)."""
        g = np.ascontiguousarray(gray, np.uint8)
        k = intrinsics(intr)
        out = C.c_int32()
        _check(_lib().recon_mvs_image_stage(self.ctx, _ptr(g, C.c_uint8), g.shape[1], g.shape[0], C.byref(k),
                                            int(undistort), C.byref(out)))
        self._img_shape[out.value] = g.shape
        return out.value

    def stage_image_bgra(self, bgra, intr, undistort=False) -> int:
        """Upload a BGRA8 frame (H x W x 4, or H x stride rows); gray on the device."""
        b = np.ascontiguousarray(bgra, np.uint8)
        h, w = b.shape[0], b.shape[1]
        stride = b.strides[0]
        k = intrinsics(intr)
        out = C.c_int32()
        _check(_lib().recon_mvs_image_stage_bgra(self.ctx, _ptr(b, C.c_uint8), w, h, stride, C.byref(k),
                                                 int(undistort), C.byref(out)))
        self._img_shape[out.value] = (h, w)
        return out.value

    def release_image(self, image: int):
        _check(_lib().recon_mvs_image_release(self.ctx, image))

    def stage_images(self, ref_image: int, src_images, ref_pose, src_poses, config: MvsConfig) -> int:
        """A job from staged images (poses: 13 values or Pose each)."""
        ids = np.ascontiguousarray(src_images, np.int32)
        ps = (Pose * len(ids))(*[pose(p) for p in src_poses])
        rp = pose(ref_pose)
        job = C.c_int32()
        _check(_lib().recon_mvs_job_stage_images(self.ctx, ref_image, len(ids), _ptr(ids, C.c_int32), C.byref(rp),
                                                 C.cast(ps, C.POINTER(Pose)), C.byref(config), C.byref(job)))
        self._keep[job.value] = self._img_shape[ref_image]
        self._nsrc[job.value] = len(ids)
        return job.value

    def adjoint(self, job: int, px, py, depth, angles, gn=False, pose=False):
        """The adjoint at hypotheses (pixel, depth, theta/phi).  Returns
        (cost n, grad n x 3, gn n x 6 or None, pose_grad n x S x 6 or None)."""
        px = np.ascontiguousarray(px, np.int32)
        py = np.ascontiguousarray(py, np.int32)
        depth = np.ascontiguousarray(depth, np.float64)
        angles = np.ascontiguousarray(angles, np.float64).reshape(-1, 2)
        n = len(px)
        cost = np.zeros(n, np.float32)
        grad = np.zeros((n, 3), np.float32)
        H = np.zeros((n, 6), np.float32) if gn else None
        ns = self._nsrc[job]
        pg = np.zeros((n, ns, 6), np.float32) if pose else None
        _check(_lib().recon_mvs_job_adjoint(self.ctx, job, n, _ptr(px, C.c_int32), _ptr(py, C.c_int32),
                                            _ptr(depth, C.c_double), _ptr(angles, C.c_double),
                                            _ptr(cost, C.c_float), _ptr(grad, C.c_float),
                                            _ptr(H, C.c_float) if gn else None,
                                            _ptr(pg, C.c_float) if pose else None))
        return cost, grad, H, pg

    def recover_poses(self, job: int, px, py, depth, angles, iterations=10):
        """Pose recovery on the job's sources.  Returns (poses num_src x 12
        [R row-major, t], cost history)."""
        px = np.ascontiguousarray(px, np.int32)
        py = np.ascontiguousarray(py, np.int32)
        depth = np.ascontiguousarray(depth, np.float64)
        angles = np.ascontiguousarray(angles, np.float64).reshape(-1, 2)
        ns = self._nsrc[job]
        poses = (Pose * ns)()
        hist = np.zeros(iterations + 1, np.float64)
        _check(_lib().recon_mvs_job_recover_poses(self.ctx, job, len(px), _ptr(px, C.c_int32), _ptr(py, C.c_int32),
                                                  _ptr(depth, C.c_double), _ptr(angles, C.c_double), iterations,
                                                  poses, _ptr(hist, C.c_double)))
        out = np.array([[*p.r, *p.t] for p in poses], np.float64)
        return out, hist

    def stage_run(self, images, poses, intrinsics_list, config: MvsConfig, undistort=False, batch_size=0,
                  consistency_views=0, rel_depth=0.01, reproj_px=1.0, cancel=None, progress=None,
                  plane_normals=False):
        """Orchestrator::StageMvs on the batched engine: keyframe images (None
        = no image), poses and intrinsics -> (PointCloud, maps fused).
        cancel() -> bool and progress(fraction) are optional callables."""
        n = len(images)
        imgs = [None if im is None else np.ascontiguousarray(im, np.uint8) for im in images]
        ptrs = (C.POINTER(C.c_uint8) * max(1, n))(*[None if im is None else _ptr(im, C.c_uint8) for im in imgs])
        w = np.asarray([0 if im is None else im.shape[1] for im in imgs] or [0], np.int32)
        h = np.asarray([0 if im is None else im.shape[0] for im in imgs] or [0], np.int32)
        ps = (Pose * max(1, n))(*[pose(p) for p in poses])
        ks = (Intrinsics * max(1, n))(*[intrinsics(k) for k in intrinsics_list])
        cb_cancel = CANCEL_FN((lambda _u: 1 if cancel() else 0) if cancel else 0)
        cb_progress = PROGRESS_FN((lambda _u, f: progress(f)) if progress else 0)
        prm = StageParams(int(undistort), int(batch_size), int(consistency_views), int(plane_normals), rel_depth,
                          reproj_px, cb_cancel, cb_progress, None)
        pc = PointCloudC()
        maps = C.c_int32()
        _check(_lib().recon_mvs_stage_run(self.ctx, C.cast(ptrs, C.POINTER(C.POINTER(C.c_uint8))),
                                          _ptr(w, C.c_int32), _ptr(h, C.c_int32), C.cast(ps, C.POINTER(Pose)),
                                          C.cast(ks, C.POINTER(Intrinsics)), n, C.byref(config), C.byref(prm),
                                          C.byref(pc), C.byref(maps)))
        return _take_cloud(pc), maps.value

    def stage_run_device(self, images, poses, intrinsics_list, config: MvsConfig, undistort=False, batch_size=0,
                         consistency_views=0, rel_depth=0.01, reproj_px=1.0, plane_normals=False):
        """stage_run with the fused cloud kept in device memory -> (DeviceCloud,
        maps fused)."""
        n = len(images)
        imgs = [None if im is None else np.ascontiguousarray(im, np.uint8) for im in images]
        ptrs = (C.POINTER(C.c_uint8) * max(1, n))(*[None if im is None else _ptr(im, C.c_uint8) for im in imgs])
        w = np.asarray([0 if im is None else im.shape[1] for im in imgs] or [0], np.int32)
        h = np.asarray([0 if im is None else im.shape[0] for im in imgs] or [0], np.int32)
        ps = (Pose * max(1, n))(*[pose(p) for p in poses])
        ks = (Intrinsics * max(1, n))(*[intrinsics(k) for k in intrinsics_list])
        prm = StageParams(int(undistort), int(batch_size), int(consistency_views), int(plane_normals), rel_depth,
                          reproj_px, CANCEL_FN(0), PROGRESS_FN(0), None)
        dc = DeviceCloudC()
        maps = C.c_int32()
        _check(_lib().recon_mvs_stage_run_device(self.ctx, C.cast(ptrs, C.POINTER(C.POINTER(C.c_uint8))),
                                                 _ptr(w, C.c_int32), _ptr(h, C.c_int32), C.cast(ps, C.POINTER(Pose)),
                                                 C.cast(ks, C.POINTER(Intrinsics)), n, C.byref(config), C.byref(prm),
                                                 C.byref(dc), C.byref(maps)))
        return DeviceCloud(self, dc), maps.value

    def release(self, job: int):
        _check(_lib().recon_mvs_job_release(self.ctx, job))
        self._keep.pop(job, None)

    def synchronize(self):
        _check(_lib().recon_mvs_synchronize(self.ctx))

    def stats(self) -> Stats:
        s = Stats()
        _check(_lib().recon_mvs_context_stats(self.ctx, C.byref(s)))
        return s

    def close(self):
        if self.ctx:
            _lib().recon_mvs_context_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def exported_symbols():
    return list(_SIGS)


class TsdfVolume:
    """recon::TsdfVolume (tsdf_fusion.h:42-98) with its grid in device memory."""

    def __init__(self, config: TsdfConfig, device: int = 0):
        self.ptr = C.c_void_p()
        _check(_lib().recon_tsdf_create(C.byref(config), device, C.byref(self.ptr)))

    def IntegrateDepthFrame(self, depth_mm, confidence, world_to_camera, depth_uncertainty_m) -> int:
        d = np.ascontiguousarray(depth_mm, np.uint16)
        c = None if confidence is None else np.ascontiguousarray(confidence, np.uint8)
        m = np.ascontiguousarray(np.asarray(world_to_camera, np.float64).reshape(4, 4))
        n = C.c_uint32()
        _check(_lib().recon_tsdf_integrate(self.ptr, _ptr(d, C.c_uint16), _ptr(c, C.c_uint8) if c is not None else None,
                                           d.shape[1], d.shape[0], _ptr(m, C.c_double), float(depth_uncertainty_m),
                                           C.byref(n)))
        return int(n.value)

    def ExtractPoints(self) -> "PointCloud":
        pc = PointCloudC()
        _check(_lib().recon_tsdf_extract_points(self.ptr, C.byref(pc)))
        return _take_cloud(pc)

    def dims(self):
        d = (C.c_int32 * 3)()
        _check(_lib().recon_tsdf_dims(self.ptr, d))
        return tuple(int(v) for v in d)

    def MemoryUsageBytes(self) -> int:
        b = C.c_uint64()
        _check(_lib().recon_tsdf_memory_usage(self.ptr, C.byref(b)))
        return int(b.value)

    def grid(self):
        """(tsdf, weight) as (nz, ny, nx) FP32 host arrays."""
        nx, ny, nz = self.dims()
        t = np.zeros((nz, ny, nx), np.float32)
        w = np.zeros((nz, ny, nx), np.float32)
        _check(_lib().recon_tsdf_read_grid(self.ptr, _ptr(t, C.c_float), _ptr(w, C.c_float)))
        return t, w

    def close(self):
        if self.ptr:
            _lib().recon_tsdf_destroy(self.ptr)
            self.ptr = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001 -- interpreter shutdown
            pass
