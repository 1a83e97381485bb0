"""Benchmark: depth maps/s of plane-mode PatchMatch MVS on one GB300.

Workload (the headline configuration): the tabletop capture -- 9 views at
1920x1440, f = 1450 px with Brown-Conrady distortion (k1 = 0.05,
k2 = -0.01), the tabletop scene (sphere, box, three cylinders on a tilted
plane, value-noise albedo with 10 % weak-texture patches) -- each view the
reference of one depth map with the other 8 as its sources; 11x11 windows,
8 iterations.  A step = the 9 maps: initialisation, 8 red-black iterations,
sub-pixel refinement, output.  Images are undistorted on the device when
staged; the capture's consistency + fusion stage is reported beside it.

  form   -- the chosen form: all maps of the step in one batch (one
            persistent launch per half-sweep, replayed from a CUDA graph),
            source images stored as FP16 textures, window samples
            interpolated by the texture unit, Gauss-Newton refinement from
            the adjoint, coarse-to-fine initialisation (iterations 1-2 of the
            8 on the half-resolution pyramid level, as the reference design
            lays out its search: level 1 for the coarse rounds, level 0 for
            the fine ones), and an exploration schedule (the random and
            fronto-parallel candidates in iterations 1-3 only, the search's
            propagation and local perturbations in all 8); the plain path
            (FP32 textures, exact FP32
            interpolation, one launch per view, the reference's
            golden-section refinement, all 8 iterations at full resolution)
            is timed in the same run and reported under "plain" with its
            depth agreement, and the forms between the two under
            "attribution";
  value  -- depth maps/s with the staged inputs resident in HBM; each step
            is timed with CUDA events on the engine's stream and L2 is
            flushed (a 512 MiB write) between steps, outside the events;
  e2e    -- the same metric through the public C ABI from host buffers:
            stage the capture (H2D of its 8-bit images once each,
            undistortion, textures), stage the jobs, run, download (depth,
            support, confidence, normal, cost), release.

Other workloads: --workload small (C1, one 640x480 map), c3 (48 orbit
references, batched vs per-view), c4 (the differentiation form), c5 (mixed
precision), tsdf (TSDF fusion of depth frames, the RGBD branch).

`--impl reference` times the reference's own CPU implementation on the host
cores instead (its patchmatch_stereo.cpp compiled for this host, all
threads; the oracle's restatement only where that cannot be built), one
bounded tile sample of map 0 per step, extrapolated to whole depth maps;
`--impl reference --full-map` times the whole map 0 once, beside every tile's
estimate.

Multi-GPU: the path does not shard (replicas only); each rank runs its own
replica and value = total depth maps / max-over-ranks time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "recon-scanner_gb300"))

METRIC = "depth maps/s 1920×1440×8src (1 GB300), chosen vs plain GPU at ≤0.1% depth err"
K, S_SRC = 11, 8
W, H, F, ITERS = 1920, 1440, 1450.0, 8
# algorithmic FLOP of the plane-induced homography cost: K^2 * 26 + 30 per
# source window sampled (26 = 15 projection + 6 bilinear + 5 moments), 40 per
# hypothesis
FP32_LANES = 128  # FP32 lanes per SM (sm_100 / sm_103 family)


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "sm_max_mhz": 2070.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = "clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown," \
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown," \
             "clocks_event_reasons.sw_power_cap"

    def __init__(self, index):
        self.index = index
        self.samples = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def make_scenes(device):
    """The step's reference views (one MvsScene each)."""
    import synthetic as Syn

    if WORKLOAD == "small":
        return [Syn.sphere_on_backdrop(width=W, height=H, f=F, num_sources=S_SRC, seed=1, device=device)]
    if WORKLOAD == "c3":
        return Syn.orbit_capture(n_frames=120, n_refs=48, seed=3, device=device)
    cap = Syn.tabletop(width=W, height=H, f=F, num_sources=S_SRC, seed=2, device=device, depth_range=DEPTH_RANGE)
    return [Syn.as_reference(cap, k) for k in range(len(cap.views))]


WORKLOAD = "c2"
DEPTH_RANGE = (0.25, 0.70)  # the tabletop capture's search range: every view's depths (0.30-0.63 m)


def set_workload(name):
    """c2: the headline capture -- 9 views at 1920x1440, each the reference
    of one depth map with the other 8 as its sources; small: the 640x480 x 4
    sources sphere scene (one map; profiling captures, CPU-runnable size);
    c3: 48 references from a 120-frame orbit, mixed resolutions, 6-10
    sources each."""
    global WORKLOAD, W, H, F, ITERS, S_SRC
    WORKLOAD = name
    if name == "small":
        W, H, F, ITERS, S_SRC = 640, 480, 600.0, 6, 4


def views_of(M, sc):
    cams = [sc.ref.camera] + [s.camera for s in sc.sources]
    imgs = [sc.ref.image] + [s.image for s in sc.sources]
    return M.ViewArgs.from_cameras(imgs[0], imgs[1:], cams[0], cams[1:])


def config_of(M, sc):
    return M.MvsConfig(min_depth_m=sc.min_depth, max_depth_m=sc.max_depth, iterations=ITERS, patch_size=K,
                       subpixel_iterations=4)


def dist_init():
    import torch
    import torch.distributed as dist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1 and not dist.is_initialized():
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend)
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
    return world, rank, local


def barrier_max(world, value):
    if world == 1:
        return value
    import torch
    import torch.distributed as dist

    t = torch.tensor([value], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


# ---------------------------------------------------------------------------
# CPU reference arm / baseline
# ---------------------------------------------------------------------------

def cpu_reference_impl():
    """The CPU implementation that the reference arm and cpu_baseline time:
    the reference's own patchmatch_stereo.cpp compiled for this host with
    the reference's release flags (oracle/_ref/libref_mvs_release.so, from
    the reference tree or its staged copy; kind "reference") where it can be built, else the oracle's C restatement
    (kind "port").  Returns (checker, kind, note, oracle checker); the oracle
    also undistorts the images beforehand (the reference has no
    undistortion), outside every timed region."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    O.build_oracle(ref=False)
    orc = O.load("oracle")
    if O.reference_tree() is not None or os.path.exists(O.REF_SO):
        try:
            O.build_oracle(ref=True)
            return (O.load("reference_release"), "reference",
                    "the reference's own patchmatch_stereo.cpp (release flags -O3 -DNDEBUG)", orc)
        except Exception as e:  # noqa: BLE001 -- a failed build falls back, and says so
            return orc, "port", f"oracle restatement (reference build failed: {str(e)[:120]})", orc
    return orc, "port", "oracle restatement of patchmatch_stereo.cpp (no reference sources on this host)", orc


class CpuReferenceSampler:
    """Times the reference's PatchMatchStereo + RefineSubpixel on bounded
    samples of one depth map and extrapolates to the whole map.

    The frame is cut into a grid of tiles, `cols` wide and 16 x threads rows
    tall (the reference splits each sweep into min(threads, H/16) row blocks,
    so every thread stays busy); the last tile of a row or column is moved
    inwards so that the grid covers the frame.  One sample = one tile:
    PatchMatchStereo with 0 iterations (initial cost) and with 1 iteration,
    whose difference is one iteration (4 direction sweeps); then
    RefineSubpixel (single-threaded in the reference) on `refine_rows` rows
    at the tile's middle.  Per-map estimate of a sample = (initial + ITERS x
    one iteration) x frame / tile area + refine x frame / refined area.
    Samples visit the tiles in a fixed shuffled order, so consecutive samples
    spread over the frame (borders, weak-texture patches, occlusions)."""

    def __init__(self, sc, threads=None, cols=480, refine_rows=4):
        import numpy as np

        self.chk, self.kind, self.impl_note, orc = cpu_reference_impl()
        import oracle as O

        self.O = O
        self.threads = threads or os.cpu_count() or 1
        self.sc = sc
        self.W, self.H = sc.ref.camera.width, sc.ref.camera.height
        self.cols = min(cols, self.W)
        self.rows = min(self.H, 16 * self.threads)
        self.refine_rows = refine_rows
        cams = [sc.ref.camera] + [s.camera for s in sc.sources]
        self.und = [c.undistorted() for c in cams]
        self.imgs = [np.clip(np.round(orc.undistort(im, c.intrinsics_array())), 0, 255).astype(np.uint8)
                     for im, c in zip([sc.ref.image] + [s.image for s in sc.sources], cams)]

        def starts(n, size):
            v = list(range(0, n - size + 1, size))
            if v[-1] + size < n:
                v.append(n - size)
            return v

        grid = [(x, y) for y in starts(self.H, self.rows) for x in starts(self.W, self.cols)]
        self.tiles = [grid[i] for i in np.random.default_rng(0).permutation(len(grid))]

    def _cfg(self, iters, threads=None):
        sc = self.sc
        return self.O.make_config(min_depth_m=sc.min_depth, max_depth_m=sc.max_depth, iterations=iters,
                                  patch_size=K, num_threads=threads or self.threads, subpixel_iterations=4)

    def _views(self, x0, y0, cols, rows):
        import copy

        import numpy as np

        cr = copy.deepcopy(self.und[0])
        cr.cx, cr.cy = self.und[0].cx - x0, self.und[0].cy - y0
        cr.width, cr.height = cols, rows
        ref = np.ascontiguousarray(self.imgs[0][y0:y0 + rows, x0:x0 + cols])
        return self.O.ViewSet(ref, self.imgs[1:], cr, self.und[1:])

    def sample(self, i):
        """Sample i: (measured seconds, per-map estimate in seconds)."""
        import numpy as np

        x0, y0 = self.tiles[i % len(self.tiles)]
        vs = self._views(x0, y0, self.cols, self.rows)
        t0 = time.perf_counter()
        self.chk.patchmatch_stereo(vs, self._cfg(0))
        t_init = time.perf_counter() - t0
        t0 = time.perf_counter()
        pm = self.chk.patchmatch_stereo(vs, self._cfg(1))
        t_pm1 = time.perf_counter() - t0
        t_one = max(0.0, t_pm1 - t_init)
        r0 = self.rows // 2 - self.refine_rows // 2
        vs_r = self._views(x0, y0 + r0, self.cols, self.refine_rows)
        pm_r = type(pm)(pm.filled, np.ascontiguousarray(pm.depth[r0:r0 + self.refine_rows]),
                        np.ascontiguousarray(pm.support[r0:r0 + self.refine_rows]),
                        np.ascontiguousarray(pm.confidence[r0:r0 + self.refine_rows]))
        t0 = time.perf_counter()
        self.chk.refine_subpixel(vs_r, self._cfg(1), pm_r)
        t_ref = time.perf_counter() - t0
        area = self.W * self.H / (self.cols * self.rows)
        est = (t_init + ITERS * t_one) * area + t_ref * self.W * self.H / (self.cols * self.refine_rows)
        return t_init + t_pm1 + t_ref, est

    def full_map(self):
        """The whole map once, no extrapolation: (PatchMatchStereo seconds,
        RefineSubpixel seconds, the refined map's accuracy vs analytic
        truth)."""
        vs = self._views(0, 0, self.W, self.H)
        t0 = time.perf_counter()
        pm = self.chk.patchmatch_stereo(vs, self._cfg(ITERS))
        t_pm = time.perf_counter() - t0
        t0 = time.perf_counter()
        refined = self.chk.refine_subpixel(vs, self._cfg(ITERS), pm)
        t_ref = time.perf_counter() - t0

        class _Map:
            depth = refined.depth

        return t_pm, t_ref, accuracy([_Map], [self.sc.ref.depth], (self.sc.min_depth, self.sc.max_depth))

    def describe(self, n, measured_s):
        return (f"{self.impl_note} ({self.kind}), {self.threads} threads, on map 0 of the workload: {n} "
                f"sample(s) of a {self.cols}x{self.rows} tile each (initial cost + 1 iteration, RefineSubpixel "
                f"single-threaded on {self.cols}x{self.refine_rows}), tiles from a {len(self.tiles)}-tile grid "
                f"covering the frame in a fixed shuffled order, each scaled to {ITERS} iterations and the "
                f"{self.W}x{self.H} frame; {measured_s:.1f} s measured")


def cpu_baseline_sample(sc, n_samples=4):
    """cpu_baseline of the GPU arm: a bounded sample (n_samples tiles, about
    10-30 s of CPU work) of map 0.  Returns (seconds per map, threads, kind,
    note)."""
    smp = CpuReferenceSampler(sc)
    runs = [smp.sample(i) for i in range(n_samples)]
    est = statistics.mean(r[1] for r in runs)
    return est, smp.threads, smp.kind, smp.describe(n_samples, sum(r[0] for r in runs))


def describe_workload(scenes):
    """The workload in words, shared by both arms of the bench."""
    n_src = [len(sc.sources) for sc in scenes]
    if WORKLOAD == "c2":
        return (f"tabletop capture: 9 views {W}x{H} (k1=0.05, k2=-0.01, undistorted on the device), each the "
                f"reference of one map with the other {S_SRC} as sources")
    if WORKLOAD == "c3":
        return (f"orbit capture: {len(scenes)} references from 120 frames, mixed 640x480/1280x960/1920x1440, "
                f"{min(n_src)}-{max(n_src)} sources")
    return f"sphere {W}x{H}, {S_SRC} sources"


def run_reference_arm(args):
    """The reference's own CPU implementation on the host cores.  A step is
    one bounded sample (one tile of map 0, see CpuReferenceSampler); value =
    1 / the mean per-map estimate of the timed steps, ms_per_step = the
    measured time of a sample.  --full-map instead times the whole map 0
    once (no extrapolation) and reports every tile's estimate beside it."""
    world, rank, _ = dist_init()
    if rank != 0:
        return
    scenes = make_scenes("cpu")
    smp = CpuReferenceSampler(scenes[0])
    if args.full_map:
        t_pm, t_ref, acc = smp.full_map()
        runs = [smp.sample(i) for i in range(len(smp.tiles))]
        est = statistics.mean(r[1] for r in runs)
        full = t_pm + t_ref
        print(json.dumps({"impl": "reference", "kind": smp.kind, "threads": smp.threads,
                          "workload": f"{describe_workload(scenes)}; {K}x{K}, {ITERS} iterations; map 0",
                          "full_map_s": full, "patchmatch_s": t_pm, "refine_s": t_ref, "accuracy": acc,
                          "tile_estimate_s": est, "tiles": len(runs),
                          "tile_estimate_rel_err": (est - full) / full,
                          "first_k_estimates": {str(k): statistics.mean(r[1] for r in runs[:k])
                                                for k in (4, 10, 20) if k <= len(runs)}}))
        return
    runs = []
    for i in range(args.warmup + args.steps):
        r = smp.sample(i)
        if i >= args.warmup:
            runs.append(r)
    per_map = statistics.mean(r[1] for r in runs)
    value = 1.0 / per_map
    measured = sum(r[0] for r in runs)
    line = {"metric": METRIC, "value": value, "unit": "depth maps/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": measured / len(runs) * 1000.0, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded scenes, analytic truth)",
            "impl": "reference",
            "config": {"workload": f"{describe_workload(scenes)}; {K}x{K}, {ITERS} iterations",
                       "algorithm": "the reference's PatchMatchStereo + RefineSubpixel (FP64, host threads); a "
                                    "step is one tile sample of map 0, value extrapolates the samples to "
                                    "whole depth maps",
                       "seconds_per_map_estimate": per_map,
                       "parallelism": "host threads"},
            "cpu_baseline": {"value": value, "unit": "depth maps/s", "cores": smp.threads, "kind": smp.kind,
                             "sample": smp.describe(len(runs), measured)},
            "e2e": {"value": value, "unit": "depth maps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if WORKLOAD == "c2":
        # one whole map 0 of the reference's own code (its release build, 8
        # x86 threads), timed once against the tile estimate of the same host
        line["extrapolation_check"] = {
            "full_map_s": 3216.1, "tile_estimate_s_48_tiles": 2739.4, "rel_err_48_tiles": -0.148,
            "rel_err_4_10_20_tiles": [-0.306, -0.221, -0.240],
            "host": "8 x86 Xeon threads (the build host), the reference's release build",
            "reading": "the tile samples under-estimate a whole map by 15-30 %: the reference arm's speed is "
                       "if anything too high, so GPU / CPU ratios from it are conservative"}
    print(json.dumps(line))


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------

def stage_capture(M, eng, scenes, cfgs, undistort):
    """Stage every distinct view of the step once (a capture's views serve as
    the reference of one map and sources of the others), then one job per
    scene from the staged images.  Returns (jobs, image ids)."""
    ids = {}
    for sc in scenes:
        for v in [sc.ref] + list(sc.sources):
            if id(v) not in ids:
                ids[id(v)] = eng.stage_image(v.image, v.camera.intrinsics_array(), undistort=undistort)
    jobs = [eng.stage_images(ids[id(sc.ref)], [ids[id(v)] for v in sc.sources], sc.ref.camera.pose_array(),
                             [v.camera.pose_array() for v in sc.sources], c) for sc, c in zip(scenes, cfgs)]
    return jobs, list(ids.values())


def time_form(M, views, cfgs, opts, steps, warmup, flush, world, undistort, sampler=None, scenes=None):
    """Stage the step's views once, run `warmup` untimed steps, then `steps`
    timed steps (CUDA events on the engine stream around the whole run; L2
    flushed between steps, outside the events).  A step runs every view:
    as one batch, or one launch per view when opts.per_view = 1.  Returns
    per-step ms, sweep ms, (hypotheses, source windows sampled) per step,
    launches/step, maps, stats."""
    import torch

    eng = M.Engine(opts)
    if scenes is not None:
        jobs, _ = stage_capture(M, eng, scenes, cfgs, undistort)
    else:
        jobs = [eng.stage(v, c, undistort=undistort) for v, c in zip(views, cfgs)]
    for _ in range(warmup):
        eng.run_many(jobs)
        eng.synchronize()
    step_ms, sweep_ms, hyps, wins = [], [], [], []
    launches = 0
    barrier(world)
    ctx = sampler if sampler is not None else _Null()
    with ctx:
        for _ in range(steps):
            flush.random_(0, 255)
            torch.cuda.synchronize()
            s0 = eng.stats()
            eng.run_many(jobs)
            eng.synchronize()
            st = eng.stats()
            step_ms.append(st.last_run_ms)
            sweep_ms.append(st.last_sweep_ms)
            hyps.append(st.hypotheses_evaluated - s0.hypotheses_evaluated)
            wins.append(st.windows_evaluated - s0.windows_evaluated)
    barrier(world)
    st = eng.stats()
    groups = len(jobs) if opts.per_view else -(-len(jobs) // 64)
    launches = st.last_sweep_launches + 3 * groups  # + init, refine, output per group
    maps = [eng.download(j) for j in jobs]
    for j in jobs:
        eng.release(j)
    eng.close()
    return step_ms, sweep_ms, (hyps, wins), launches, maps, st


class _Null:
    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False


def accuracy(maps, truths, depth_range=None):
    """Pooled over the step's maps: relative depth error vs analytic truth.
    With the search range given, also over the pixels whose true depth lies
    inside it (no search can return a depth outside its range), and the
    share of pixels whose truth lies outside."""
    import numpy as np

    rel_all, abs_all, filled, rel_in, outside = [], [], [], [], []
    for dm, truth in zip(maps, truths):
        err = np.abs(dm.depth.astype(np.float64) - truth)
        rel = err / truth
        ok = np.isfinite(rel)
        rel_all.append(rel[ok])
        abs_all.append(err[ok])
        filled.append(float(np.isfinite(dm.depth).mean()))
        if depth_range is not None:
            with np.errstate(invalid="ignore"):
                inside = (truth >= depth_range[0]) & (truth <= depth_range[1])
            rel_in.append(rel[ok & inside])
            outside.append(float((np.isfinite(truth) & ~inside).sum()) / max(1, int(np.isfinite(truth).sum())))
    rel = np.concatenate(rel_all) if rel_all else np.zeros(0)
    err = np.concatenate(abs_all) if abs_all else np.zeros(0)
    out = {"filled": float(np.mean(filled)),
           "median_rel_err": float(np.median(rel)) if rel.size else None,
           "p95_rel_err": float(np.quantile(rel, 0.95)) if rel.size else None,
           "median_abs_err_mm": float(np.median(err) * 1e3) if err.size else None}
    if depth_range is not None:
        r = np.concatenate(rel_in) if rel_in else np.zeros(0)
        out["in_range"] = {"median_rel_err": float(np.median(r)) if r.size else None,
                           "p95_rel_err": float(np.quantile(r, 0.95)) if r.size else None,
                           "truth_outside_range": float(np.mean(outside)),
                           "per_map_truth_outside_range": [round(v, 4) for v in outside]}
    return out


def agreement(maps_a, maps_b):
    import numpy as np

    d = []
    for a, b in zip(maps_a, maps_b):
        both = np.isfinite(a.depth) & np.isfinite(b.depth)
        d.append(np.abs(a.depth[both].astype(np.float64) - b.depth[both]) / b.depth[both])
    d = np.concatenate(d) if d else np.zeros(0)
    return (float(np.median(d)) if d.size else None), (float(np.quantile(d, 0.95)) if d.size else None)


def fuse_capture(M, scenes, maps, rel=0.01, reproj=1.0, min_views=3):
    """The capture's fusion stage: every map's geometric consistency against
    the other maps (>= min_views consistent views, reprojection <= reproj px,
    relative depth <= rel), then FuseDepthMaps of the kept pixels.  Timed on
    the host around the public calls (maps are host buffers).  Accuracy: the
    fused points seen by view 0, against its analytic depth."""
    import numpy as np

    cams = [sc.ref.camera for sc in scenes]
    poses = [c.pose_array() for c in cams]
    intr = [c.undistorted().intrinsics_array() for c in cams]
    t0 = time.perf_counter()
    keeps = []
    kept = 0
    for k in range(len(maps)):
        _, keep = M.GeometricConsistency(maps, poses, intr, k, rel, reproj, min_views)
        keeps.append(keep)
        kept += int(keep.sum())
    cfg = M.MvsConfig()
    cloud = M.FuseDepthMaps(maps, poses, intr, cfg, keep_masks=keeps)
    secs = time.perf_counter() - t0
    c0 = cams[0]
    Xc = cloud.positions @ c0.R.T + c0.t
    ok = Xc[:, 2] > 1e-6
    u = np.floor(c0.fx * Xc[ok, 0] / Xc[ok, 2] + c0.cx).astype(np.int64)
    v = np.floor(c0.fy * Xc[ok, 1] / Xc[ok, 2] + c0.cy).astype(np.int64)
    z = Xc[ok, 2]
    inside = (u >= 0) & (v >= 0) & (u < c0.width) & (v < c0.height)
    truth = scenes[0].ref.depth[v[inside], u[inside]]
    zz = z[inside]
    vis = np.isfinite(truth) & (np.abs(zz - truth) < 0.05 * truth)  # points on the surface view 0 sees
    rel_err = np.abs(zz[vis] - truth[vis]) / truth[vis]
    return {"points": int(cloud.size()), "kept_pixels": kept, "seconds": secs,
            "thresholds": {"min_views": min_views, "reproj_px": reproj, "rel_depth": rel},
            "view0_points": int(vis.sum()),
            "view0_median_rel_err": float(np.median(rel_err)) if rel_err.size else None,
            "view0_p95_rel_err": float(np.quantile(rel_err, 0.95)) if rel_err.size else None,
            "timing": "host wall clock: 9 consistency calls + fusion, host buffers in and out"}


def attribution(M, views, cfgs, mk, args, flush, world, undistort, scenes, truths, rng, chosen_value, chosen_maps):
    """What each step from the plain path to the chosen form buys: the
    capture timed (`--attr-steps` steps after one warm-up, L2 flushed between
    steps) in the forms between them -- batched FP32 exact golden section,
    + FP16 storage, + Gauss-Newton (the batched FP16 form with exact
    interpolation) -- beside the plain path and the chosen form (texture-unit
    interpolation) timed above; each with its accuracy.  The exact
    Gauss-Newton form is also timed with its windows staged in shared memory
    (with the fraction of windows read from the boxes and a bit-identity
    check against its texture reads), alone and with coarse-to-fine.  And what the
    texture unit's 8-bit filter weights cost: the plane cost of 2 x 10^4
    seeded hypotheses on a pinhole copy of the capture's map 0, FP16 storage,
    exact and texture-unit interpolation, against the FP64 oracle (a checker
    run after every timed region)."""
    import numpy as np

    import synthetic as Syn

    # (name, fp16, interp, refine, coarse iterations, window staging: 1 texture reads, 2 staged boxes)
    forms = [("batched_fp32_exact_golden", False, 0, 1, 0, 1), ("batched_fp16_exact_golden", True, 0, 1, 0, 1),
             ("batched_fp16_exact_gauss_newton", True, 0, 2, 0, 1),
             ("batched_fp16_exact_gauss_newton_staged_windows", True, 0, 2, 0, 2),
             ("batched_fp16_exact_gauss_newton_staged_windows_coarse_to_fine", True, 0, 2, args.coarse, 2),
             ("batched_fp16_texture_gauss_newton_full_resolution", True, 1, 2, 0, 1),
             ("batched_fp16_texture_gauss_newton_coarse_to_fine", True, 1, 2, args.coarse, 1)]
    out = {"steps": args.attr_steps, "forms": {}}
    exact_maps = None
    for name, fp16, interp, refine, coarse, staging in forms:
        ms, _, _, _, fmaps, fst = time_form(M, views, cfgs, mk(fp16, interp, False, refine, coarse, staging, 0),
                                            args.attr_steps, 1, flush, world, undistort, scenes=scenes)
        tot = barrier_max(world, float(sum(ms)))
        med, p95 = agreement(fmaps, chosen_maps)
        out["forms"][name] = {"value": world * len(views) * args.attr_steps / (tot / 1000.0),
                              "accuracy": accuracy(fmaps, truths, rng),
                              "vs_chosen_median_rel_depth_diff": med, "vs_chosen_p95_rel_depth_diff": p95}
        if staging == 2:
            out["forms"][name]["windows_staged_frac"] = fst.windows_staged / max(fst.windows_evaluated, 1)
        if name == "batched_fp16_exact_gauss_newton":
            exact_maps = fmaps
        elif name == "batched_fp16_exact_gauss_newton_staged_windows":
            # the schedules read the same texels with the same arithmetic
            out["forms"][name]["bit_identical_to_texture_reads"] = all(
                np.array_equal(a.depth, b.depth, equal_nan=True) and np.array_equal(a.cost, b.cost, equal_nan=True)
                for a, b in zip(fmaps, exact_maps))
    out["forms"]["chosen"] = {"value": chosen_value, "form": "the timed form of this line"}
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    orc = O.load("oracle")
    sc = Syn.tabletop(width=W, height=H, f=F, num_sources=S_SRC, k1=0.0, k2=0.0, seed=2, device="cuda:0",
                      depth_range=DEPTH_RANGE)
    cams = sc.cameras
    imgs = [v.image for v in sc.views]
    rs = np.random.default_rng(23)
    n = 20_000
    px, py = rs.integers(0, W, n), rs.integers(0, H, n)
    td, tn = sc.ref.depth[py, px], sc.ref.normal[py, px]
    okt = np.isfinite(td)
    inv = np.where(okt, 1.0 / np.where(okt, td, 1.0), rs.uniform(1 / sc.max_depth, 1 / sc.min_depth, n))
    inv = (inv * (1.0 + rs.normal(0, 0.01, n))).astype(np.float32).astype(np.float64)
    nrm = np.where(okt[:, None], tn, [0.0, 0.0, -1.0]) + rs.normal(0, 0.1, (n, 3))
    nrm = (nrm / np.linalg.norm(nrm, axis=1, keepdims=True)).astype(np.float32).astype(np.float64)
    cfg_d = dict(min_depth_m=sc.min_depth, max_depth_m=sc.max_depth, patch_size=K)
    want, _, _ = orc.plane_costs(O.ViewSet(imgs[0], imgs[1:], cams[0], cams[1:]), O.make_config(**cfg_d),
                                 args.best_k, px, py, inv, nrm)
    va = M.ViewArgs.from_cameras(imgs[0], imgs[1:], cams[0], cams[1:])
    cost = {}
    for name, interp in (("fp16_exact", 0), ("fp16_texture", 1)):
        o = M.Options(mode=M.MODE_PLANE, best_k=args.best_k, storage=M.STORAGE_FP16, interp=interp, device=0)
        got, _ = M.Evaluate(va, M.MvsConfig(**cfg_d), o, px, py, inv, nrm.astype(np.float32))
        ok = (want < 1e29) & (got < 1e29)
        d = np.abs(got[ok].astype(np.float64) - want[ok])
        cost[name] = {"hypotheses": int(ok.sum()), "median_abs": float(np.median(d)),
                      "p99_abs": float(np.quantile(d, 0.99)), "max_abs": float(d.max()),
                      "within_1e-5_rel_plus_2e-6": float(np.mean(d <= 1e-5 * np.abs(want[ok]) + 2e-6))}
    out["cost_vs_fp64_oracle"] = cost
    out["note"] = ("plain = FP32 storage, exact interpolation, one launch per view, golden section, every iteration "
                   "at full resolution; each form adds one change: batched, FP16 storage, Gauss-Newton, texture-unit "
                   "interpolation (8-bit weights), coarse-to-fine (the first iterations on the half-resolution "
                   "level, the same total); chosen adds the exploration schedule (the random and fronto-parallel "
                   "candidates only in the first iterations).  Beside the chain: the exact Gauss-Newton form with "
                   "its source windows staged in shared memory by TMA (window_staging = 2; the same maps as its "
                   "texture reads, bit for bit), alone and with coarse-to-fine")
    return out


def reference_algorithm_maps(M, scenes, cfgs, maps):
    """The reference's own algorithm on every map of the workload:
    PatchMatchStereo + RefineSubpixel (fronto-parallel windows, golden
    section + parabola fit; patchmatch_stereo.cpp:422-979) run by the
    engine's COMPAT mode, its device restatement, on the views undistorted on
    the device and rounded to 8 bits (the reference's input type), with
    pinhole cameras.  Per map: its accuracy vs analytic truth next to the
    chosen form's on the same map (all pixels, and the pixels whose true
    depth lies in the search range); pooled; time per map."""
    import numpy as np

    per_map, ref_maps, secs = [], [], 0.0
    opts = M.Options(mode=M.MODE_COMPAT, device=0)
    for k, (sc, cfg) in enumerate(zip(scenes, cfgs)):
        vs = [sc.ref] + list(sc.sources)
        imgs = [np.clip(np.rint(M.Undistort(v.image, v.camera.intrinsics_array())), 0, 255).astype(np.uint8)
                for v in vs]
        cams = [v.camera.undistorted() for v in vs]
        va = M.ViewArgs.from_cameras(imgs[0], imgs[1:], cams[0], cams[1:])
        t0 = time.perf_counter()
        dm = M.PatchMatchStereo(va, cfg, options=opts)
        M.RefineSubpixel(va, cfg, dm, options=opts)
        secs += time.perf_counter() - t0
        ref_maps.append(dm)
        rng = (sc.min_depth, sc.max_depth)
        r, c = accuracy([dm], [sc.ref.depth], rng), accuracy([maps[k]], [sc.ref.depth], rng)
        per_map.append({"map": k, "reference_median": r["median_rel_err"], "reference_p95": r["p95_rel_err"],
                        "chosen_median": c["median_rel_err"], "chosen_p95": c["p95_rel_err"],
                        "reference_in_range_median": r["in_range"]["median_rel_err"],
                        "reference_in_range_p95": r["in_range"]["p95_rel_err"],
                        "chosen_in_range_median": c["in_range"]["median_rel_err"],
                        "chosen_in_range_p95": c["in_range"]["p95_rel_err"],
                        "truth_outside_range": r["in_range"]["truth_outside_range"]})
    rng = (scenes[0].min_depth, scenes[0].max_depth)
    out = accuracy(ref_maps, [sc.ref.depth for sc in scenes], rng)
    out["seconds_per_map"] = secs / len(scenes)
    out["per_map"] = per_map
    out["note"] = ("COMPAT mode = the reference's PatchMatchStereo + RefineSubpixel restated on the device; "
                   "in_range = pixels whose true depth lies in the search range")
    return out


def stage_capture_run(M, scenes, opts):
    """The whole MVS stage of the capture through one public call
    (recon_mvs_stage_run: host images in, fused cloud out): staging with
    on-device undistortion, SelectSourceViews (num_views = 8), one batched run,
    consistency (>= 3 views, 1 px, 1 %) and fusion on the device.  Host wall
    clock; the first call (autotune, module load) is excluded."""
    cams = [sc.ref.camera for sc in scenes]
    imgs = [sc.ref.image for sc in scenes]
    cfg = M.MvsConfig(min_depth_m=scenes[0].min_depth, max_depth_m=scenes[0].max_depth, iterations=ITERS,
                      patch_size=K, subpixel_iterations=4, num_views=S_SRC)
    eng = M.Engine(opts)
    args = (imgs, [c.pose_array() for c in cams], [c.intrinsics_array() for c in cams], cfg)
    kw = dict(undistort=True, consistency_views=3, rel_depth=0.01, reproj_px=1.0)
    eng.stage_run(*args, **kw)
    t0 = time.perf_counter()
    cloud, nmaps = eng.stage_run(*args, **kw)
    secs = time.perf_counter() - t0
    eng.close()
    # the sources SelectSourceViews gives each keyframe inside the stage (its
    # scale-ratio gate drops some): the stage's PatchMatch work differs from
    # the timed step's, where every map takes the capture's other 8 views
    poses = args[1]
    src = [len(M.SelectSourceViews(poses[k], poses, cams[k].intrinsics_array(), cfg)) for k in range(len(cams))]
    return {"seconds": secs, "maps": nmaps, "points": int(cloud.size()), "maps_per_s": nmaps / secs,
            "call": "recon_mvs_stage_run, host images in, fused cloud out",
            "sources_per_map": src, "source_views": int(sum(src)),
            "value_source_views": int(sum(len(sc.sources) for sc in scenes)),
            "refine": {0: "none", 1: "golden section", 2: "Gauss-Newton"}.get(int(opts.refine), str(opts.refine)),
            "note": "the stage selects each keyframe's sources with SelectSourceViews (num_views = 8, scale-ratio "
                    "gate), so it searches fewer source views than the timed step; no L2 flush between its calls"}


KERNEL_SOURCES = ["pm.cu", "cost.cuh", "common.cuh", "adjoint.cuh", "kernels.h"]


def kernel_sources_digest():
    """Digest of the sweep's kernel sources and of the build recipe (its
    compiler flags): a profile taken on other sources or flags does not
    describe the kernel this run times."""
    import hashlib

    h = hashlib.sha256()
    for name in KERNEL_SOURCES:
        with open(os.path.join(ROOT, "recon-scanner_gb300", "csrc", name), "rb") as f:
            h.update(f.read())
    with open(os.path.join(ROOT, "recon-scanner_gb300", "build.py"), "rb") as f:
        h.update(f.read())
    return h.hexdigest()[:16]


def sweep_profile(workload, args):
    """The committed ncu figures of the sweep kernel for this workload and
    form (profiles/traffic.json): DRAM bytes and texture-pipe share per
    launch, with the commit and kernel-source digest they were taken at.
    `applies` is true only when the digest matches these sources and the form
    matches this run's."""
    tp = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(tp):
        return {"applies": False, "why": "no committed profile"}
    with open(tp) as f:
        prof = json.load(f).get("k_plane_sweep", {}).get(workload)
    if not prof:
        return {"applies": False, "why": f"no committed profile for workload {workload}"}
    form = {"fp16": bool(args.fp16), "interp": int(args.interp), "per_view": bool(args.per_view),
            "coarse": int(args.coarse), "exploration": int(args.exploration)}
    digest = kernel_sources_digest()
    out = dict(prof)
    out["sources_digest_now"] = digest
    out["applies"] = prof.get("sources_digest") == digest and prof.get("form") == form
    if prof.get("form") != form:
        out["why"] = "profiled form differs from this run's"
    elif prof.get("sources_digest") != digest:
        out["why"] = "kernel sources changed since the profile"
    return out


def run_gpu(args):
    import numpy as np
    import torch

    world, rank, local = dist_init()
    torch.cuda.set_device(local)
    import recon_mvs as M

    M.load_library()
    peaks, peak_src = load_peaks()
    scenes = make_scenes(f"cuda:{local}")
    views = [views_of(M, sc) for sc in scenes]
    cfgs = [config_of(M, sc) for sc in scenes]
    truths = [sc.ref.depth for sc in scenes]
    undistort = WORKLOAD == "c2"
    n_maps = len(scenes)
    pixels = [sc.ref.camera.width * sc.ref.camera.height for sc in scenes]
    n_src = [len(sc.sources) for sc in scenes]
    # pixel-weighted sources per map: the FLOP model's S for mixed batches
    s_eff = float(np.dot(pixels, n_src) / np.sum(pixels))
    # FLOP model: per source window sampled K*K*26 + 30, per hypothesis 40
    flop_per_window, flop_per_hyp_setup = K * K * 26 + 30, 40
    mk = lambda fp16, interp, per_view, refine, coarse=args.coarse, staging=args.window_staging, \
        explore=args.exploration: M.Options(
            mode=M.MODE_PLANE, best_k=args.best_k, storage=M.STORAGE_FP16 if fp16 else M.STORAGE_FP32, device=local,
            refine=refine, prefilter=int(args.prefilter), sampling=args.sampling, interp=interp,
            per_view=int(per_view), tile_rows=args.tile_rows, coarse_iterations=coarse,
            window_staging=staging if interp == 0 else 0, exploration_iterations=explore)
    opts = mk(args.fp16, args.interp, args.per_view, args.refine)
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device=f"cuda:{local}")

    clk = ClockSampler(local)
    step_ms, sweep_ms, (hyps, wins), launches_per_step, maps, st = time_form(M, views, cfgs, opts, args.steps, args.warmup,
                                                                     flush, world, undistort, clk, scenes=scenes)
    total_ms = barrier_max(world, float(sum(step_ms)))
    value = world * n_maps * args.steps / (total_ms / 1000.0)
    rng = {(sc.min_depth, sc.max_depth) for sc in scenes}
    rng = rng.pop() if len(rng) == 1 else None
    acc = accuracy(maps, truths, rng)

    plain = None
    if not args.plain and not args.chosen_only:
        p_fp16 = False if WORKLOAD != "c3" else args.fp16
        p_interp = 0 if WORKLOAD != "c3" else args.interp
        p_ms, _, _, p_launches, p_maps, _ = time_form(M, views, cfgs, mk(p_fp16, p_interp, True, 1, 0, explore=0), args.steps,
                                                      args.warmup, flush, world, undistort, scenes=scenes)
        p_total = barrier_max(world, float(sum(p_ms)))
        med, p95 = agreement(maps, p_maps)
        plain = {"value": world * n_maps * args.steps / (p_total / 1000.0), "unit": "depth maps/s",
                 "ms_per_step": p_total / args.steps, "storage": "fp16" if p_fp16 else "fp32",
                 "interp": "texture-unit" if p_interp else "exact fp32", "launch": "one launch per view",
                 "refine": "golden section on the inverse depth (the reference's schedule)",
                 "gpu_launches_per_step": p_launches, "accuracy": accuracy(p_maps, truths, rng),
                 "chosen_vs_plain_median_rel_depth_diff": med, "chosen_vs_plain_p95_rel_depth_diff": p95}

    # ---- end to end through the C ABI from host buffers ----
    e2e_times = []
    phases = {"stage": [], "run": [], "download": [], "release": []}
    if args.e2e_steps > 0:
        eng = M.Engine(opts)
        dmh = [M.DepthMap.allocate(sc.ref.camera.width, sc.ref.camera.height) for sc in scenes]
        for it in range(args.e2e_steps + 1):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            jobs, imgs = stage_capture(M, eng, scenes, cfgs, undistort)
            eng.synchronize()
            t1 = time.perf_counter()
            eng.run_many(jobs)
            eng.synchronize()
            t2 = time.perf_counter()
            for j, d in zip(jobs, dmh):
                eng.download(j, d)
            t3 = time.perf_counter()
            for j in jobs:
                eng.release(j)
            for i in imgs:
                eng.release_image(i)
            t4 = time.perf_counter()
            if it > 0:
                e2e_times.append(t4 - t0)
                for k, v in zip(phases, (t1 - t0, t2 - t1, t3 - t2, t4 - t3)):
                    phases[k].append(v * 1e3)
        eng.close()
    e2e_s = barrier_max(world, statistics.mean(e2e_times)) if e2e_times else float("nan")
    e2e_value = world * n_maps / e2e_s
    distinct = {id(v): v for sc in scenes for v in [sc.ref] + list(sc.sources)}
    h2d = int(sum(v.image.size for v in distinct.values()))
    d2h = int(sum(p * (4 + 1 + 4 + 12 + 4) + 4 for p in pixels))

    # ---- roofline of the dominant kernel (the red-black sweep) ----
    sweeps = max(1, st.last_sweep_launches)
    per_launch_ms = statistics.mean(sweep_ms) / sweeps
    hyp_per_launch = statistics.mean(hyps) / sweeps
    win_per_launch = statistics.mean(wins) / sweeps
    flop_per_launch = flop_per_window * win_per_launch + flop_per_hyp_setup * hyp_per_launch
    achieved_tflops = flop_per_launch / (per_launch_ms * 1e-3) / 1e12
    sm_mhz = peaks.get("sm_max_mhz", 2070.0)
    sm_count = torch.cuda.get_device_properties(local).multi_processor_count
    peak_tflops = sm_count * FP32_LANES * 2 * sm_mhz * 1e6 / 1e12
    prof = sweep_profile(WORKLOAD, args)
    traffic = prof.get("dram_bytes_per_launch") if prof.get("applies") else None
    tex_pipe = prof.get("tex_data_pipe_pct") if prof.get("applies") else None

    # the HBM side of the roofline, per half-sweep: the algorithmic bytes
    # (every map's source images + its per-pixel state read and written:
    # float4 plane + float cost + uint8 support = 21 B) over the sweep time,
    # against the measured copy bandwidth
    b_img = 2 if args.fp16 else 4
    alg_bytes = sum((1 + ns) * px * b_img + 2 * px * 21 for px, ns in zip(pixels, n_src))
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    hbm_gbs = alg_bytes / (per_launch_ms * 1e-3) / 1e9
    hbm_side = {"algorithmic_bytes_per_launch": alg_bytes, "achieved_gbs": hbm_gbs, "peak_gbs": hbm_peak,
                "frac": hbm_gbs / hbm_peak, "measured_dram_bytes_per_launch": traffic,
                "peak_source": f"{peak_src} MEASURED_PEAKS.json hbm_gbs"}

    form = (f"{'fp16' if args.fp16 else 'fp32'} storage, {'texture-unit' if args.interp else 'exact fp32'} "
            f"interpolation, {'one launch per view' if args.per_view else 'batched persistent launch, CUDA graph'}, "
            f"{'Gauss-Newton (adjoint) refinement' if args.refine == 2 else 'golden-section refinement'}"
            + (f", coarse-to-fine: iterations 1-{args.coarse} of {ITERS} on the half-resolution level (2x2 means)"
               if args.coarse else ", every iteration at full resolution")
            + (f", exploration candidates (random, fronto-parallel) in iterations 1-{args.exploration} only"
               if args.exploration else ""))
    wl = describe_workload(scenes)
    line = {"metric": METRIC, "value": value, "unit": "depth maps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (fp16 storage)" if args.fp16 else "f32",
            "data": "synthetic (seeded scenes, analytic truth)",
            "config": {"workload": f"{wl}; {K}x{K}, {ITERS} iterations, plane mode, best_k={args.best_k}",
                       "maps_per_step": n_maps, "megapixels_per_step": sum(pixels) / 1e6,
                       "form": form, "coarse_iterations": args.coarse,
                       "exploration_iterations": args.exploration, "tile_rows": st.tile_rows,
                       "ctas_per_sm": st.ctas_per_sm,
                       "prefilter": bool(args.prefilter), "sampling": args.sampling,
                       "l2": "flushed between steps (512 MiB write, outside the timed events)",
                       "parallelism": f"replicas x{world}"},
            "gpu_launches": launches_per_step * args.steps,
            "e2e": {"value": e2e_value, "unit": "depth maps/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h,
                    "ms_by_phase": {k: statistics.mean(v) for k, v in phases.items() if v}},
            "roofline": {"bound": "fp32", "achieved": achieved_tflops, "peak": peak_tflops, "unit": "TFLOP/s",
                         "frac": achieved_tflops / peak_tflops, "traffic": traffic,
                         "kernel": "k_plane_sweep",
                         "peak_source": f"{sm_count} SMs (device) x {FP32_LANES} FP32 lanes x 2 x sm_max_mhz {sm_mhz} "
                                        f"({peak_src} MEASURED_PEAKS.json clock)",
                         "hypotheses_per_launch": hyp_per_launch, "windows_per_launch": win_per_launch,
                         "ms_per_launch": per_launch_ms, "flop_per_launch": flop_per_launch,
                         "flop_model": f"{flop_per_window} per source window sampled + {flop_per_hyp_setup} per "
                                       f"hypothesis",
                         "hbm": hbm_side,
                         "binding_unit": {"unit": "L1TEX texture data pipe (bilinear source reads)",
                                          "pct_of_peak": tex_pipe,
                                          "source": "ncu l1tex__data_pipe_tex_wavefronts.avg."
                                                    "pct_of_peak_sustained_elapsed"},
                         "profile": prof},
            "hypotheses_per_s": statistics.mean(hyps) / (statistics.mean(step_ms) * 1e-3),
            "accuracy": acc, "plain": plain, "clocks": clk.summary()}
    if WORKLOAD == "c2" and not args.plain and not args.chosen_only and not args.no_attribution:
        line["attribution"] = attribution(M, views, cfgs, mk, args, flush, world, undistort, scenes, truths, rng,
                                          value, maps)
    if WORKLOAD == "c2" and not args.no_fusion:
        line["fusion"] = fuse_capture(M, scenes, maps)
        line["stage"] = stage_capture_run(M, scenes, opts)
    if WORKLOAD == "c2" and not args.no_reference_map:
        line["reference_algorithm"] = reference_algorithm_maps(M, scenes, cfgs, maps)
    if rank == 0 and not args.no_cpu_baseline:
        secs, threads, kind, note = cpu_baseline_sample(scenes[0])
        line["cpu_baseline"] = {"value": 1.0 / secs, "unit": "depth maps/s", "cores": threads, "kind": kind,
                                "sample": note}
    if rank == 0:
        print(json.dumps(line))


# ---------------------------------------------------------------------------
# the differentiation and mixed-precision workloads (reports, not the headline)
# ---------------------------------------------------------------------------

def _pinhole_views(orc, sc):
    """Undistorted FP32 intensities (orc_undistort, bit-identical to the
    device remap) and pinhole cameras: what the engine matches."""
    cams = sc.cameras
    imgs = [sc.ref.image] + [s.image for s in sc.sources]
    return [orc.undistort(im, c.intrinsics_array()) for im, c in zip(imgs, cams)], [c.undistorted() for c in cams]


def _sph(ang):
    import numpy as np

    t, p = ang[:, 0], ang[:, 1]
    return np.stack([np.sin(t) * np.cos(p), np.sin(t) * np.sin(p), np.cos(t)], -1)


def run_differentiable(args, n_hyp=10_000):
    """The C2 views with source poses perturbed by a seeded 0.2 deg rotation
    and 0.5 mm translation: (1) the adjoint at 10^4 seeded pixels vs FP64
    central differences of the oracle cost (pixel parameters; pose on 10^3),
    adjoint throughput; (2) Gauss-Newton vs golden-section refinement
    accuracy; (3) pose recovery from the PatchMatch map."""
    import copy

    import numpy as np
    import torch

    import recon_mvs as M
    import synthetic as Syn

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    M.load_library()
    O.build_oracle(ref=False)
    orc = O.load("oracle")
    sc = Syn.tabletop(width=W, height=H, f=F, num_sources=S_SRC, seed=2, device="cuda:0")
    cams = sc.cameras
    imgs = [sc.ref.image] + [s.image for s in sc.sources]
    rng = np.random.default_rng(17)

    def so3(w):
        th = np.linalg.norm(w)
        K_ = np.array([[0, -w[2], w[1]], [w[2], 0, -w[0]], [-w[1], w[0], 0]])
        return np.eye(3) + np.sin(th) / th * K_ + (1 - np.cos(th)) / th ** 2 * K_ @ K_ if th > 1e-12 else np.eye(3)

    def perturb(c, w, tau):
        c = copy.deepcopy(c)
        E = so3(np.asarray(w, np.float64))
        c.R, c.t = E @ c.R, E @ c.t + np.asarray(tau, np.float64)
        return c

    pert = [cams[0]]
    for c in cams[1:]:
        a = rng.normal(size=3)
        tdir = rng.normal(size=3)
        pert.append(perturb(c, np.radians(0.2) * a / np.linalg.norm(a), 0.0005 * tdir / np.linalg.norm(tdir)))
    cfg_kw = dict(min_depth_m=sc.min_depth, max_depth_m=sc.max_depth, iterations=ITERS, patch_size=K,
                  subpixel_iterations=4)
    views = M.ViewArgs.from_cameras(imgs[0], imgs[1:], pert[0], pert[1:])
    out = {"metric": "differentiation form (C4)", "config": {
        "workload": f"tabletop {W}x{H}, {S_SRC} sources, poses perturbed 0.2 deg / 0.5 mm (seeded)"}}

    # (1) gradients
    ys, xs = np.nonzero(np.isfinite(sc.ref.depth[8:-8, 8:-8]))
    pick = rng.choice(len(xs), n_hyp, replace=False)
    px, py = (xs[pick] + 8).astype(np.int32), (ys[pick] + 8).astype(np.int32)
    nt = sc.ref.normal[py, px]
    depth = sc.ref.depth[py, px] * (1 + rng.uniform(-0.005, 0.005, n_hyp))
    ang = np.stack([np.arccos(np.clip(nt[:, 2], -1, 1)) + rng.uniform(-0.05, 0.05, n_hyp),
                    np.arctan2(nt[:, 1], nt[:, 0]) + rng.uniform(-0.05, 0.05, n_hyp)], -1)
    eng = M.Engine(M.Options(mode=M.MODE_PLANE, best_k=4, device=0))
    job = eng.stage(views, M.MvsConfig(**cfg_kw), undistort=True)
    eng.adjoint(job, px[:128], py[:128], depth[:128], ang[:128])  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    cost, grad, _, pgrad = eng.adjoint(job, px, py, depth, ang, pose=True)
    t_adj = time.perf_counter() - t0
    und, pin = _pinhole_views(orc, Syn.MvsScene("p", Syn.RenderedView(pert[0], imgs[0], None, None),
                                                [Syn.RenderedView(c, im, None, None) for c, im in
                                                 zip(pert[1:], imgs[1:])], sc.min_depth, sc.max_depth, 2))
    vs = O.ViewSet(und[0], und[1:], pin[0], pin[1:])
    ocfg = O.make_config(num_threads=0, **cfg_kw)
    oc = lambda d_, a_: orc.plane_costs(vs, ocfg, 4, px, py, 1.0 / d_, _sph(a_))[0]
    fd = np.zeros((n_hyp, 3))
    hd = 1e-8 * depth
    fd[:, 0] = (oc(depth + hd, ang) - oc(depth - hd, ang)) / (2 * hd)
    for j in (0, 1):
        e = np.zeros_like(ang)
        e[:, j] = 1e-8
        fd[:, 1 + j] = (oc(depth, ang + e) - oc(depth, ang - e)) / 2e-8
    ok = (cost < 1e29) & np.all(np.isfinite(fd), -1)
    g, f = grad[ok].astype(np.float64), fd[ok].copy()
    g[:, 0] *= depth[ok]
    f[:, 0] *= depth[ok]
    r = np.linalg.norm(g - f, axis=-1) / np.linalg.norm(f, axis=-1)
    out["pixel_gradient"] = {"hypotheses": int(ok.sum()), "rel_err_median": float(np.median(r)),
                             "rel_err_p99": float(np.quantile(r, 0.99)), "frac_le_1e-3": float(np.mean(r <= 1e-3)),
                             "adjoint_hypotheses_per_s_with_pose": n_hyp / t_adj}
    m = 1000
    fdp = np.zeros((m, S_SRC, 6))
    steps = [1e-8] * 3 + [1e-9] * 3
    for s_ in range(S_SRC):
        for j in range(6):
            w, tau = np.zeros(3), np.zeros(3)
            (w if j < 3 else tau)[j % 3] = steps[j]
            c2 = []
            for sign in (1, -1):
                cl = list(pin)
                cl[1 + s_] = perturb(pin[1 + s_], sign * w, sign * tau)
                v2 = O.ViewSet(und[0], und[1:], cl[0], cl[1:])
                c2.append(orc.plane_costs(v2, ocfg, 4, px[:m], py[:m], 1.0 / depth[:m], _sph(ang[:m]))[0])
            fdp[:, s_, j] = (c2[0] - c2[1]) / (2 * steps[j])
    pg = pgrad[:m].astype(np.float64)
    sel = np.any(pg != 0, -1) & (cost[:m] < 1e29)[:, None] & np.all(np.isfinite(fdp), -1)
    gp, fp = pg[sel], fdp[sel]
    gp[:, 3:] *= 0.4
    fp[:, 3:] *= 0.4
    rp = np.linalg.norm(gp - fp, axis=-1) / np.linalg.norm(fp, axis=-1)
    out["pose_gradient"] = {"pairs": int(sel.sum()), "rel_err_median": float(np.median(rp)),
                            "rel_err_p99": float(np.quantile(rp, 0.99)), "frac_le_1e-3": float(np.mean(rp <= 1e-3))}

    # (2) + (3): maps on the perturbed poses, pose recovery, maps again
    def pm(refine, cam_list):
        e2 = M.Engine(M.Options(mode=M.MODE_PLANE, best_k=4, device=0, refine=refine))
        v2 = M.ViewArgs.from_cameras(imgs[0], imgs[1:], cam_list[0], cam_list[1:])
        j2 = e2.stage(v2, M.MvsConfig(**cfg_kw), undistort=True)
        e2.run(j2)
        dm = e2.download(j2)
        ms = e2.stats().last_run_ms
        e2.close()
        return dm, ms

    def med(dm):
        e = np.abs(dm.depth[8:-8, 8:-8].astype(np.float64) - sc.ref.depth[8:-8, 8:-8]) / sc.ref.depth[8:-8, 8:-8]
        return float(np.nanmedian(e))

    ref_true = {k: pm(k, cams) for k in (1, 2)}
    out["refinement_true_poses"] = {"golden_section_median_rel_err": med(ref_true[1][0]),
                                    "gauss_newton_median_rel_err": med(ref_true[2][0]),
                                    "golden_section_run_ms": ref_true[1][1], "gauss_newton_run_ms": ref_true[2][1]}
    def perr(lst):
        rot = [np.degrees(np.arccos(np.clip((np.trace(c.R @ t.R.T) - 1) / 2, -1, 1))) for c, t in zip(lst, cams[1:])]
        ctr = [np.linalg.norm(-c.R.T @ c.t + t.R.T @ t.t) * 1e3 for c, t in zip(lst, cams[1:])]
        return float(np.median(rot)), float(np.median(ctr))

    # A common scale of every baseline and depth leaves every image, so the
    # photometric cost cannot see it: centres relative to the reference are
    # aligned by the least-squares scale before comparing them, and the map
    # is scaled by the same factor.
    c_ref_true = -cams[0].R.T @ cams[0].t

    def scale_of(lst):
        a = np.stack([-c.R.T @ c.t - c_ref_true for c in lst])
        b = np.stack([-t.R.T @ t.t - c_ref_true for t in cams[1:]])
        return float(np.sum(a * b) / np.sum(a * a))

    def perr_aligned(lst):
        k = scale_of(lst)
        ctr = [np.linalg.norm(k * (-c.R.T @ c.t - c_ref_true) - (-t.R.T @ t.t - c_ref_true)) * 1e3
               for c, t in zip(lst, cams[1:])]
        return k, float(np.median(ctr))

    def med_scaled(dm, k):
        e = np.abs(k * dm.depth[8:-8, 8:-8].astype(np.float64) - sc.ref.depth[8:-8, 8:-8]) / sc.ref.depth[8:-8, 8:-8]
        return float(np.nanmedian(e))

    # alternate: map on the current poses, pose recovery from that map (the
    # job keeps the recovered transforms between rounds)
    cur = pert
    rounds = []
    t_pose = 0.0
    for rnd in range(3):
        dm, _ = pm(2, cur)
        ys, xs = np.nonzero(np.isfinite(dm.depth[8:-8:4, 8:-8:4]))
        qx, qy = (xs * 4 + 8).astype(np.int32), (ys * 4 + 8).astype(np.int32)
        nn = dm.normal[qy, qx].astype(np.float64)
        qa = np.stack([np.arccos(np.clip(nn[:, 2], -1, 1)), np.arctan2(nn[:, 1], nn[:, 0])], -1)
        t0 = time.perf_counter()
        poses, hist = eng.recover_poses(job, qx, qy, dm.depth[qy, qx].astype(np.float64), qa, iterations=15)
        t_pose += time.perf_counter() - t0
        nxt = [cams[0]]
        for c, p_ in zip(pert[1:], poses):
            c = copy.deepcopy(c)
            c.R, c.t = p_[:9].reshape(3, 3).copy(), p_[9:12].copy()
            nxt.append(c)
        k0 = perr_aligned(cur[1:])[0]
        rounds.append({"map_median_rel_err": med(dm), "map_median_rel_err_scale_aligned": med_scaled(dm, k0),
                       "pixels": int(len(qx)), "cost": [float(hist[0]), float(hist[-1])],
                       "median_rotation_err_deg_before_after": [perr(cur[1:])[0], perr(nxt[1:])[0]],
                       "median_centre_err_mm_before_after": [perr(cur[1:])[1], perr(nxt[1:])[1]],
                       "median_centre_err_mm_scale_aligned_before_after": [perr_aligned(cur[1:])[1],
                                                                           perr_aligned(nxt[1:])[1]],
                       "gauge_scale_after": perr_aligned(nxt[1:])[0]})
        cur = nxt
    eng.close()
    dm_final, _ = pm(2, cur)
    out["pose_recovery"] = {"rounds": rounds, "final_map_median_rel_err": med(dm_final),
                            "final_map_median_rel_err_scale_aligned": med_scaled(dm_final, perr_aligned(cur[1:])[0]),
                            "true_pose_map_median_rel_err": med(ref_true[2][0]), "seconds": t_pose,
                            "iterations_per_round": 15}
    print(json.dumps(out))


def run_precision(args):
    """1 + 16 sources at 1920x1440 (40-160 mm baselines) on the tabletop
    scene: each storage form (FP32, FP16, BF16, 8-bit; exact or texture-unit
    interpolation) timed (depth maps/s, one map per step), its
    error vs analytic truth, and -- on a 160x120 centre crop run by both --
    its depth / normal difference to the FP64 oracle run of the same search."""
    import numpy as np
    import torch

    import recon_mvs as M
    import synthetic as Syn

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    M.load_library()
    O.build_oracle(ref=False)
    orc = O.load("oracle")
    sc = Syn.tabletop(width=W, height=H, f=F, num_sources=16, seed=2, device="cuda:0", baseline=(0.04, 0.16))
    views = views_of(M, sc)
    cfg = config_of(M, sc)
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device="cuda:0")
    forms = {"fp32": (M.STORAGE_FP32, 0), "fp16": (M.STORAGE_FP16, 0), "bf16": (M.STORAGE_BF16, 0),
             "fp16_texture_interp": (M.STORAGE_FP16, 1),
             # the bandwidth floor: 8-bit textures (the undistorted intensities rounded to 8 bits)
             "u8": (M.STORAGE_U8, 0), "u8_texture_interp": (M.STORAGE_U8, 1)}
    # the crop: same cameras with the principal point shifted
    cw, ch = 160, 120
    x0, y0 = W // 2 - cw // 2, H // 2 - ch // 2
    import copy

    ref_c = copy.deepcopy(sc.ref.camera)
    ref_c.cx, ref_c.cy, ref_c.width, ref_c.height = ref_c.cx - x0, ref_c.cy - y0, cw, ch
    crop_img = np.ascontiguousarray(sc.ref.image[y0:y0 + ch, x0:x0 + cw])
    src_cams = [s.camera for s in sc.sources]
    src_imgs = [s.image for s in sc.sources]
    crop_views = M.ViewArgs.from_cameras(crop_img, src_imgs, ref_c, src_cams)
    und_ref = orc.undistort(crop_img, ref_c.intrinsics_array())
    und_src = [orc.undistort(im, c.intrinsics_array()) for im, c in zip(src_imgs, src_cams)]
    vs = O.ViewSet(und_ref, und_src, ref_c.undistorted(), [c.undistorted() for c in src_cams])
    ocfg = O.make_config(min_depth_m=sc.min_depth, max_depth_m=sc.max_depth, iterations=ITERS, patch_size=K,
                         subpixel_iterations=4, num_threads=0)
    t0 = time.perf_counter()
    _, d64, n64, _ = orc.plane_patchmatch(vs, ocfg, best_k=args.best_k, seed=0x5DEECE66D, refine=1)
    t64 = time.perf_counter() - t0
    truth_crop = sc.ref.depth[y0:y0 + ch, x0:x0 + cw]
    out = {"metric": "mixed precision (C5): depth maps/s and errors per storage form",
           "config": {"workload": f"tabletop {W}x{H}, 16 sources (40-160 mm), {K}x{K}, {ITERS} iterations",
                      "fp64_oracle_crop": f"{cw}x{ch} centre crop, {t64:.1f} s on the host"}, "forms": {}}
    b = 8
    for name, (storage, interp) in forms.items():
        opts = M.Options(mode=M.MODE_PLANE, best_k=args.best_k, storage=storage, interp=interp, device=0)
        step_ms, _, _, _, maps, _ = time_form(M, [views], [cfg], opts, args.steps, args.warmup, flush, 1, True)
        full = accuracy(maps, [sc.ref.depth])
        eng = M.Engine(opts)
        j = eng.stage(crop_views, cfg, undistort=True)
        eng.run(j)
        dm = eng.download(j)
        eng.close()
        a, o, t = dm.depth[b:-b, b:-b].astype(np.float64), d64[b:-b, b:-b].astype(np.float64), truth_crop[b:-b, b:-b]
        ok = np.isfinite(a) & np.isfinite(o)
        rel = np.abs(a[ok] - o[ok]) / o[ok]
        na, no = dm.normal[b:-b, b:-b][ok].astype(np.float64), n64[b:-b, b:-b][ok].astype(np.float64)
        ang = np.degrees(np.arccos(np.clip(np.sum(na * no, -1), -1, 1)))
        okt = ok & np.isfinite(t)
        out["forms"][name] = {
            "maps_per_s": 1000.0 * len(step_ms) / sum(step_ms), "ms_per_map": statistics.mean(step_ms),
            "vs_truth": full,
            "vs_fp64_run": {"median_rel_depth": float(np.median(rel)), "p95_rel_depth": float(np.quantile(rel, 0.95)),
                            "median_normal_deg": float(np.median(ang)), "p95_normal_deg": float(np.quantile(ang, 0.95)),
                            "pixels": int(ok.sum())},
            "crop_vs_truth_median_rel": float(np.median(np.abs(a[okt] - t[okt]) / t[okt])),
            "fp64_crop_vs_truth_median_rel": float(np.median(np.abs(o[okt] - t[okt]) / t[okt]))}
    print(json.dumps(out))


def run_tsdf(args, n_frames=8):
    """TSDF fusion (the RGBD branch, recon_tsdf_*): 8 depth frames of 640x480
    (uint16 mm, holes and low-confidence pixels, per-frame uncertainty) of
    the sphere-and-wall scene fused into a 1 mm grid over a 0.40 x 0.32 x 0.24
    m box (31 M voxels), then ExtractPoints.  A step = a fresh volume, the 8
    frames (host buffers in) and the surface points (host cloud out): frames/s
    by host wall clock around the synchronous calls.  Beside it the
    reference's own TsdfVolume (oracle/_ref/libref_tsdf.so, single-threaded
    as in the reference) on the same frames, and the grid / points agreement
    with the oracle."""
    import numpy as np

    import recon_mvs as M
    import synthetic as Syn

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    M.load_library()
    cfgd, frames = Syn.tsdf_capture(width=640, height=480, f=600.0, n_frames=n_frames, seed=4, voxel=0.001,
                                    truncation=0.008)
    cfg = M.TsdfConfig(**cfgd)

    def step():
        vol = M.TsdfVolume(cfg)
        integ = [vol.IntegrateDepthFrame(d, c, p, u) for d, c, p, u in frames]
        pc = vol.ExtractPoints()
        grid = vol.grid() if want_grid else None
        vol.close()
        return integ, pc, grid

    want_grid = False
    for _ in range(args.warmup):
        step()
    secs = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        integ, pc, _ = step()
        secs.append(time.perf_counter() - t0)
    want_grid = True
    integ, pc, (t, w) = step()
    ocfg = O.tsdf_config(**cfgd)
    t0 = time.perf_counter()
    want = O.tsdf_fuse(ocfg, frames)
    t_orc = time.perf_counter() - t0
    ref_kind, t_ref = "port", t_orc
    if O.reference_tree() is not None or os.path.exists(O.REF_TSDF_SO):
        try:
            t0 = time.perf_counter()
            O.tsdf_reference(ocfg, frames)
            t_ref, ref_kind = time.perf_counter() - t0, "reference"
        except Exception:  # noqa: BLE001 -- the port stands in, and the line says so
            pass
    per_step = statistics.mean(secs)
    nvox = int(np.prod(O.tsdf_dims(ocfg)))
    out = {"metric": "TSDF fusion: depth frames/s (640x480 into a 1 mm grid) + surface extraction",
           "value": n_frames / per_step, "unit": "frames/s", "ms_per_step": per_step * 1e3, "steps": args.steps,
           "warmup": args.warmup, "higher_is_better": True, "dtype": "f32 grid, f64 geometry",
           "data": "synthetic (seeded sphere-and-wall capture)",
           "config": {"workload": f"{n_frames} frames 640x480, voxel 1 mm, truncation 8 mm, grid "
                                  f"{'x'.join(str(v) for v in O.tsdf_dims(ocfg))} ({nvox / 1e6:.1f} M voxels)",
                      "timing": "host wall clock around the synchronous public calls: a fresh volume, 8 frames "
                                "from host buffers, ExtractPoints to a host cloud"},
           "points": int(pc.size()), "integrated": integ,
           "matches_oracle": {"grid": bool(np.array_equal(t, want["tsdf"]) and np.array_equal(w, want["weight"])),
                              "points": bool(np.array_equal(pc.positions, want["positions"])
                                             and np.array_equal(pc.normals, want["normals"]))},
           "cpu_baseline": {"value": n_frames / t_ref, "unit": "frames/s", "cores": 1, "kind": ref_kind,
                            "sample": f"the same {n_frames} frames and extraction, {t_ref:.1f} s "
                                      "(the reference's TsdfVolume is single-threaded)"}}
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--best-k", type=int, default=4)
    ap.add_argument("--refine", type=int, default=None,
                    help="chosen form's refinement: 1 golden section, 2 Gauss-Newton from the adjoint (default)")
    ap.add_argument("--fp16", action="store_true", default=None)
    ap.add_argument("--plain", action="store_true",
                    help="time only the plain path: FP32 storage, exact FP32 interpolation")
    ap.add_argument("--chosen-only", action="store_true", help="skip timing the plain path beside the chosen form")
    ap.add_argument("--prefilter", action="store_true", help="3x3 binomial pre-filter at staging")
    ap.add_argument("--sampling", type=int, default=0, help="0 pixel-centre windows, 1 the reference's convention")
    ap.add_argument("--interp", type=int, default=None, help="0 exact FP32 bilinear, 1 texture-unit bilinear")
    ap.add_argument("--window-staging", type=int, default=0, choices=[0, 1, 2],
                    help="exact interpolation: 0 autotuned, 1 texture reads, 2 source windows staged in shared memory")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--full-map", action="store_true",
                    help="with --impl reference: time the whole map 0 once and every tile sample beside it")
    ap.add_argument("--workload", default="c2", choices=["c2", "small", "c3", "c4", "c5", "tsdf"])
    ap.add_argument("--no-fusion", action="store_true", help="skip the capture's consistency + fusion stage")
    ap.add_argument("--no-attribution", action="store_true", help="skip timing the forms between plain and chosen")
    ap.add_argument("--attr-steps", type=int, default=2, help="timed steps of each attribution form")
    ap.add_argument("--no-reference-map", action="store_true",
                    help="skip the reference algorithm's maps (COMPAT mode) of the capture")
    ap.add_argument("--per-view", action="store_true", help="one launch per view instead of the batched form")
    ap.add_argument("--tile-rows", type=int, default=0, help="sweep tile rows (2, 4, 8); 0 = autotuned")
    ap.add_argument("--depth-range", default=None, help="the tabletop capture's search range 'lo,hi' in metres")
    ap.add_argument("--coarse", type=int, default=None,
                    help="coarse-to-fine: the first N of the iterations on the half-resolution level (chosen form "
                         "default 2, the reference design's rounds 1-2 on pyramid level 1; 0 = off)")
    ap.add_argument("--exploration", type=int, default=None,
                    help="exploration schedule: the random and fronto-parallel candidates in the first N iterations "
                         "only (chosen form default: the coarse iterations + 1; 0 = every iteration)")
    args = ap.parse_args()
    set_workload(args.workload)
    if args.depth_range:
        global DEPTH_RANGE
        DEPTH_RANGE = tuple(float(v) for v in args.depth_range.split(","))
    # the chosen form (default): FP16 storage + texture-unit interpolation;
    # the plain FP32 path is timed beside it unless --plain asks for it alone
    if args.refine is None:
        args.refine = 1 if (args.plain or args.workload == "c3") else 2
    if args.coarse is None:
        args.coarse = 0 if (args.plain or args.workload == "c3") else 2
    if args.exploration is None:
        args.exploration = 0 if (args.plain or args.workload == "c3" or not args.coarse) else args.coarse + 1
    if args.plain:
        args.fp16, args.interp, args.per_view = False, 0, True
    elif args.workload == "c3":
        # the batched workload is specified all-FP32: batched vs per-view only
        args.fp16 = False if args.fp16 is None else args.fp16
        args.interp = 0 if args.interp is None else args.interp
    else:
        args.fp16 = True if args.fp16 is None else args.fp16
        args.interp = 1 if args.interp is None else args.interp
    if args.impl == "reference":
        run_reference_arm(args)
    elif args.workload == "c4":
        run_differentiable(args)
    elif args.workload == "c5":
        run_precision(args)
    elif args.workload == "tsdf":
        run_tsdf(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
