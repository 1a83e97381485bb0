"""Benchmark: depth maps/s of plane-mode PatchMatch MVS on one GB300.

Workload (the headline configuration): one reference view + 8 sources at
1920x1440, f = 1450 px with Brown-Conrady distortion (k1 = 0.05,
k2 = -0.01), the tabletop scene (sphere, box, three cylinders on a tilted
plane, value-noise albedo with 10 % weak-texture patches), 11x11 windows,
8 iterations, FP32.  A step = one depth map: initialisation, 8 red-black
iterations, sub-pixel refinement, output.  Images are undistorted on the
device when staged.

  form   -- the chosen form: source images stored as FP16 textures, window
            samples interpolated by the texture unit; the plain FP32 path
            (FP32 textures, exact FP32 interpolation) is timed in the same
            run and reported under "plain_fp32" with its depth agreement;
  value  -- depth maps/s with the staged inputs resident in HBM; each step
            is timed with CUDA events on the engine's stream and L2 is
            flushed (a 512 MiB write) between steps, outside the events;
  e2e    -- the same metric through the public C ABI from host buffers:
            stage (H2D of 9 8-bit images + undistortion + textures),
            run, download (depth, support, confidence, normal, cost), release.

`--impl reference` times the reference algorithm on the host cores instead
(the CPU oracle restatement of patchmatch_stereo.cpp, all threads) on a
bounded sample of the same workload, extrapolated to one depth map.

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
# per pixel-hypothesis algorithmic FLOP, plane-induced homography mode:
# S * (K^2 * 26 + 30) + 40  (26 = 15 projection + 6 bilinear + 5 moments)
FLOP_PER_HYP = S_SRC * (K * K * 26 + 30) + 40
SM_COUNT, FP32_LANES = 152, 128


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
    cap = Syn.tabletop(width=W, height=H, f=F, num_sources=S_SRC, seed=2, device=device)
    return [Syn.as_reference(cap, k) for k in range(len(cap.views))]


WORKLOAD = "c2"


def set_workload(name):
    """c2: the headline capture -- 9 views at 1920x1440, each the reference
    of one depth map with the other 8 as its sources; small: the 640x480 x 4
    sources sphere scene (one map; profiling captures, CPU-runnable size);
    c3: 48 references from a 120-frame orbit, mixed resolutions, 6-10
    sources each."""
    global WORKLOAD, W, H, F, ITERS, S_SRC, FLOP_PER_HYP
    WORKLOAD = name
    if name == "small":
        W, H, F, ITERS, S_SRC = 640, 480, 600.0, 6, 4
    FLOP_PER_HYP = S_SRC * (K * K * 26 + 30) + 40


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

def cpu_reference_sample(sc, cols=480, refine_rows=4, threads=None):
    """Time the reference algorithm (the oracle's restatement of
    patchmatch_stereo.cpp) on a crop of the workload and extrapolate to one
    depth map.  The crop is 16 x threads rows tall -- the reference splits
    its sweeps into min(threads, H/16) row blocks, so this keeps every
    thread busy -- and `cols` wide, centred.  PatchMatch: initial cost + one
    iteration (4 direction sweeps), scaled to ITERS iterations and the full
    frame; RefineSubpixel (single-threaded in the reference) on
    `refine_rows` rows, scaled to the frame.
    Returns (seconds per depth map, threads, note)."""
    import copy

    import numpy as np

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    O.build_oracle(ref=False)
    orc = O.load("oracle")
    threads = threads or os.cpu_count() or 1
    W, H = sc.ref.camera.width, sc.ref.camera.height
    cols = min(cols, W)
    rows = min(H, 16 * threads)
    cams = [sc.ref.camera] + [s.camera for s in sc.sources]
    und = [c.undistorted() for c in cams]
    imgs = [np.clip(np.round(orc.undistort(im, c.intrinsics_array())), 0, 255).astype(np.uint8)
            for im, c in zip([sc.ref.image] + [s.image for s in sc.sources], cams)]
    x0 = W // 2 - cols // 2

    def crop(nrows):
        y0 = H // 2 - nrows // 2
        cr = copy.deepcopy(und[0])
        cr.cx, cr.cy = und[0].cx - x0, und[0].cy - y0
        cr.width, cr.height = cols, nrows
        ref = np.ascontiguousarray(imgs[0][y0:y0 + nrows, x0:x0 + cols])
        return O.ViewSet(ref, imgs[1:], cr, und[1:])

    def cfg(iters):
        return O.make_config(min_depth_m=sc.min_depth, max_depth_m=sc.max_depth, iterations=iters, patch_size=K,
                             num_threads=threads, subpixel_iterations=4)

    vs = crop(rows)
    t0 = time.perf_counter()
    orc.patchmatch_stereo(vs, cfg(0))
    t_init = time.perf_counter() - t0
    t0 = time.perf_counter()
    pm = orc.patchmatch_stereo(vs, cfg(1))
    t_one = max(0.0, time.perf_counter() - t0 - t_init)
    vs_r = crop(refine_rows)
    r0 = rows // 2 - refine_rows // 2
    pm_r = type(pm)(pm.filled, np.ascontiguousarray(pm.depth[r0:r0 + refine_rows]),
                    np.ascontiguousarray(pm.support[r0:r0 + refine_rows]),
                    np.ascontiguousarray(pm.confidence[r0:r0 + refine_rows]))
    t0 = time.perf_counter()
    orc.refine_subpixel(vs_r, cfg(1), pm_r)
    t_ref = time.perf_counter() - t0
    area = (W * H) / (cols * rows)
    total = (t_init + ITERS * t_one) * area + t_ref * (W * H) / (cols * refine_rows)
    note = (f"reference algorithm (oracle restatement of patchmatch_stereo.cpp), {threads} threads: initial cost + "
            f"1 iteration on a centred {cols}x{rows} crop, scaled x{ITERS} iterations and x{area:.1f} to the frame; "
            f"single-threaded RefineSubpixel on {cols}x{refine_rows}, scaled to the frame; "
            f"{t_init + t_one + t_ref:.1f} s measured")
    return total, threads, note


def run_reference_arm(args):
    world, rank, _ = dist_init()
    if rank != 0:
        return
    sc = make_scenes("cpu")[0]
    secs = []
    threads = os.cpu_count() or 1
    note = ""
    for i in range(args.warmup + args.steps):
        t, threads, note = cpu_reference_sample(sc)
        if i >= args.warmup:
            secs.append(t)
    per_map = statistics.mean(secs)
    value = 1.0 / per_map
    line = {"metric": METRIC, "value": value, "unit": "depth maps/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": per_map * 1000.0, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded tabletop scene, analytic truth)",
            "impl": "reference",
            "config": {"workload": f"tabletop {W}x{H}, {S_SRC} sources, {K}x{K}, {ITERS} iterations",
                       "parallelism": "host threads"},
            "cpu_baseline": {"value": value, "unit": "depth maps/s", "cores": threads, "kind": "port",
                             "sample": note},
            "e2e": {"value": value, "unit": "depth maps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------

def time_form(M, views, cfgs, opts, steps, warmup, flush, world, undistort, sampler=None):
    """Stage the step's views once, run `warmup` untimed steps, then `steps`
    timed steps (CUDA events on the engine stream around the whole run; L2
    flushed between steps, outside the events).  A step runs every view:
    as one batch, or one launch per view when opts.per_view = 1.  Returns
    per-step ms, sweep ms, hypotheses, launches/step, maps, stats."""
    import torch

    eng = M.Engine(opts)
    jobs = [eng.stage(v, c, undistort=undistort) for v, c in zip(views, cfgs)]
    for _ in range(warmup):
        eng.run_many(jobs)
        eng.synchronize()
    step_ms, sweep_ms, hyps = [], [], []
    launches = 0
    barrier(world)
    ctx = sampler if sampler is not None else _Null()
    with ctx:
        for _ in range(steps):
            flush.random_(0, 255)
            torch.cuda.synchronize()
            h0 = eng.stats().hypotheses_evaluated
            eng.run_many(jobs)
            eng.synchronize()
            st = eng.stats()
            step_ms.append(st.last_run_ms)
            sweep_ms.append(st.last_sweep_ms)
            hyps.append(st.hypotheses_evaluated - h0)
    barrier(world)
    st = eng.stats()
    groups = len(jobs) if opts.per_view else -(-len(jobs) // 64)
    launches = st.last_sweep_launches + 3 * groups  # + init, refine, output per group
    maps = [eng.download(j) for j in jobs]
    for j in jobs:
        eng.release(j)
    eng.close()
    return step_ms, sweep_ms, hyps, launches, maps, st


class _Null:
    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False


def accuracy(maps, truths):
    """Pooled over the step's maps: relative depth error vs analytic truth."""
    import numpy as np

    rel_all, abs_all, filled = [], [], []
    for dm, truth in zip(maps, truths):
        err = np.abs(dm.depth.astype(np.float64) - truth)
        rel = err / truth
        ok = np.isfinite(rel)
        rel_all.append(rel[ok])
        abs_all.append(err[ok])
        filled.append(float(np.isfinite(dm.depth).mean()))
    rel = np.concatenate(rel_all) if rel_all else np.zeros(0)
    err = np.concatenate(abs_all) if abs_all else np.zeros(0)
    return {"filled": float(np.mean(filled)),
            "median_rel_err": float(np.median(rel)) if rel.size else None,
            "p95_rel_err": float(np.quantile(rel, 0.95)) if rel.size else None,
            "median_abs_err_mm": float(np.median(err) * 1e3) if err.size else None}


def agreement(maps_a, maps_b):
    import numpy as np

    d = []
    for a, b in zip(maps_a, maps_b):
        both = np.isfinite(a.depth) & np.isfinite(b.depth)
        d.append(np.abs(a.depth[both].astype(np.float64) - b.depth[both]) / b.depth[both])
    d = np.concatenate(d) if d else np.zeros(0)
    return (float(np.median(d)) if d.size else None), (float(np.quantile(d, 0.95)) if d.size else None)


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
    flop_per_hyp = s_eff * (K * K * 26 + 30) + 40
    mk = lambda fp16, interp, per_view: M.Options(
        mode=M.MODE_PLANE, best_k=args.best_k, storage=M.STORAGE_FP16 if fp16 else M.STORAGE_FP32, device=local,
        refine=1, prefilter=int(args.prefilter), sampling=args.sampling, interp=interp, per_view=int(per_view),
        tile_rows=args.tile_rows)
    opts = mk(args.fp16, args.interp, args.per_view)
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device=f"cuda:{local}")

    clk = ClockSampler(local)
    step_ms, sweep_ms, hyps, launches_per_step, maps, st = time_form(M, views, cfgs, opts, args.steps, args.warmup,
                                                                     flush, world, undistort, clk)
    total_ms = barrier_max(world, float(sum(step_ms)))
    value = world * n_maps * args.steps / (total_ms / 1000.0)
    acc = accuracy(maps, truths)

    plain = None
    if not args.plain and not args.chosen_only:
        p_fp16 = False if WORKLOAD != "c3" else args.fp16
        p_interp = 0 if WORKLOAD != "c3" else args.interp
        p_ms, _, _, p_launches, p_maps, _ = time_form(M, views, cfgs, mk(p_fp16, p_interp, True), args.steps,
                                                      args.warmup, flush, world, undistort)
        p_total = barrier_max(world, float(sum(p_ms)))
        med, p95 = agreement(maps, p_maps)
        plain = {"value": world * n_maps * args.steps / (p_total / 1000.0), "unit": "depth maps/s",
                 "ms_per_step": p_total / args.steps, "storage": "fp16" if p_fp16 else "fp32",
                 "interp": "texture-unit" if p_interp else "exact fp32", "launch": "one launch per view",
                 "gpu_launches_per_step": p_launches, "accuracy": accuracy(p_maps, truths),
                 "chosen_vs_plain_median_rel_depth_diff": med, "chosen_vs_plain_p95_rel_depth_diff": p95}

    # ---- end to end through the C ABI from host buffers ----
    e2e_times = []
    if args.e2e_steps > 0:
        eng = M.Engine(opts)
        dmh = [M.DepthMap.allocate(sc.ref.camera.width, sc.ref.camera.height) for sc in scenes]
        for i in range(args.e2e_steps + 1):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            jobs = [eng.stage(v, c, undistort=undistort) for v, c in zip(views, cfgs)]
            eng.run_many(jobs)
            for j, d in zip(jobs, dmh):
                eng.download(j, d)
            for j in jobs:
                eng.release(j)
            t1 = time.perf_counter()
            if i > 0:
                e2e_times.append(t1 - t0)
        eng.close()
    e2e_s = barrier_max(world, statistics.mean(e2e_times)) if e2e_times else float("nan")
    e2e_value = world * n_maps / e2e_s
    h2d = int(sum(sc.ref.image.size + sum(s.image.size for s in sc.sources) for sc in scenes))
    d2h = int(sum(p * (4 + 1 + 4 + 12 + 4) + 4 for p in pixels))

    # ---- roofline of the dominant kernel (the red-black sweep) ----
    sweeps = max(1, st.last_sweep_launches)
    per_launch_ms = statistics.mean(sweep_ms) / sweeps
    hyp_per_launch = statistics.mean(hyps) / sweeps
    achieved_tflops = flop_per_hyp * hyp_per_launch / (per_launch_ms * 1e-3) / 1e12
    sm_mhz = peaks.get("sm_max_mhz", 2070.0)
    peak_tflops = SM_COUNT * FP32_LANES * 2 * sm_mhz * 1e6 / 1e12
    traffic = None
    tp = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tp):
        with open(tp) as f:
            traffic = json.load(f).get("plane_sweep_bytes_per_launch", {}).get(
                f"{WORKLOAD}{'_per_view' if args.per_view else ''}")

    form = (f"{'fp16' if args.fp16 else 'fp32'} storage, {'texture-unit' if args.interp else 'exact fp32'} "
            f"interpolation, {'one launch per view' if args.per_view else 'batched persistent launch, CUDA graph'}")
    if WORKLOAD == "c2":
        wl = (f"tabletop capture: 9 views {W}x{H} (k1=0.05, k2=-0.01, undistorted on the device), each the "
              f"reference of one map with the other {S_SRC} as sources")
    elif WORKLOAD == "c3":
        wl = (f"orbit capture: {n_maps} references from 120 frames, mixed 640x480/1280x960/1920x1440, "
              f"{min(n_src)}-{max(n_src)} sources")
    else:
        wl = f"sphere {W}x{H}, {S_SRC} sources"
    line = {"metric": METRIC, "value": value, "unit": "depth maps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (fp16 storage)" if args.fp16 else "f32",
            "data": "synthetic (seeded scenes, analytic truth)",
            "config": {"workload": f"{wl}; {K}x{K}, {ITERS} iterations, plane mode, best_k={args.best_k}, "
                                   f"golden-section refine",
                       "maps_per_step": n_maps, "megapixels_per_step": sum(pixels) / 1e6,
                       "form": form, "tile_rows": st.tile_rows, "ctas_per_sm": st.ctas_per_sm,
                       "prefilter": bool(args.prefilter), "sampling": args.sampling,
                       "l2": "flushed between steps (512 MiB write, outside the timed events)",
                       "parallelism": f"replicas x{world}"},
            "gpu_launches": launches_per_step * args.steps,
            "e2e": {"value": e2e_value, "unit": "depth maps/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "roofline": {"bound": "fp32", "achieved": achieved_tflops, "peak": peak_tflops, "unit": "TFLOP/s",
                         "frac": achieved_tflops / peak_tflops, "traffic": traffic,
                         "kernel": "k_plane_sweep",
                         "peak_source": f"{SM_COUNT} SMs x {FP32_LANES} FP32 lanes x 2 x sm_max_mhz {sm_mhz} "
                                        f"({peak_src} MEASURED_PEAKS.json clock)",
                         "hypotheses_per_launch": hyp_per_launch, "ms_per_launch": per_launch_ms,
                         "flop_per_hypothesis": flop_per_hyp},
            "hypotheses_per_s": statistics.mean(hyps) / (statistics.mean(step_ms) * 1e-3),
            "accuracy": acc, "plain": plain, "clocks": clk.summary()}
    if rank == 0 and not args.no_cpu_baseline:
        secs, threads, note = cpu_reference_sample(scenes[0])
        line["cpu_baseline"] = {"value": 1.0 / secs, "unit": "depth maps/s", "cores": threads, "kind": "port",
                                "sample": note}
    if rank == 0:
        print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--best-k", type=int, default=4)
    ap.add_argument("--fp16", action="store_true", default=None)
    ap.add_argument("--plain", action="store_true",
                    help="time only the plain path: FP32 storage, exact FP32 interpolation")
    ap.add_argument("--chosen-only", action="store_true", help="skip timing the plain path beside the chosen form")
    ap.add_argument("--prefilter", action="store_true", help="3x3 binomial pre-filter at staging")
    ap.add_argument("--sampling", type=int, default=0, help="0 pixel-centre windows, 1 the reference's convention")
    ap.add_argument("--interp", type=int, default=None, help="0 exact FP32 bilinear, 1 texture-unit bilinear")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="c2", choices=["c2", "small", "c3"])
    ap.add_argument("--per-view", action="store_true", help="one launch per view instead of the batched form")
    ap.add_argument("--tile-rows", type=int, default=0, help="sweep tile rows (2, 4, 8); 0 = autotuned")
    args = ap.parse_args()
    set_workload(args.workload)
    # the chosen form (default): FP16 storage + texture-unit interpolation;
    # the plain FP32 path is timed beside it unless --plain asks for it alone
    if args.plain:
        args.fp16, args.interp, args.per_view = False, 0, True
    else:
        args.fp16 = True if args.fp16 is None else args.fp16
        args.interp = 1 if args.interp is None else args.interp
    if args.impl == "reference":
        run_reference_arm(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
