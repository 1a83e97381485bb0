"""Build librecon_mvs_gb300.so in-tree with nvcc for sm_103a.

Each .cu translation unit is compiled in parallel, then linked with a static
CUDA runtime into recon-scanner_gb300/librecon_mvs_gb300.so.  Host code is
compiled with -ffp-contract=off: a few host-side FP64 compositions feed
kernels whose outputs are compared bit-exactly with the CPU oracle, on x86
and on aarch64 (where gcc would otherwise fuse multiply-adds).  Device code
is compiled with -fmad=false: a multiply-add is fused only where the source
says fmaf, so the same expression rounds the same way wherever it is inlined
-- the sweep's window schedules, tile shapes and batch forms give the same
maps bit for bit by construction, not by the compiler's choice at each site.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "librecon_mvs_gb300.so")
SOURCES = ["engine.cu", "pm.cu", "fusion.cu", "noalloc.cu", "adjoint.cu", "tsdf.cu"]
HEADERS = ["common.cuh", "cost.cuh", "kernels.h"]
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc() -> str:
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the GB300 MVS engine has no CPU build")
    return cand


def _flags(extra=()):
    return [ARCH, "-O3", "-std=c++17", "-lineinfo", "-fmad=false",
            "-Xcompiler", "-fPIC,-ffp-contract=off,-fvisibility=hidden",
            "-I" + os.path.join(ROOT, "include"), "-I" + CSRC, *extra]


def _stale(target, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, ptxas_verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(ROOT, "include", "recon_mvs_gb300.h")]
    objs = []
    jobs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s, *hdrs, __file__]):
            extra = ["-Xptxas", "-v"] if ptxas_verbose else []
            jobs.append([nvcc(), *_flags(extra), "-c", s, "-o", o])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            futs = [ex.submit(subprocess.run, cmd, capture_output=True, text=True) for cmd in jobs]
            for cmd, fut in zip(jobs, futs):
                r = fut.result()
                if verbose or r.returncode != 0 or ptxas_verbose:
                    sys.stderr.write(r.stdout + r.stderr)
                if r.returncode != 0:
                    raise RuntimeError("nvcc failed: " + " ".join(cmd))
    if force or jobs or _stale(LIB, objs):
        cmd = [nvcc(), ARCH, "-shared", "-cudart", "static", "-o", LIB, *objs, "-Xcompiler", "-fPIC", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError("link failed: " + " ".join(cmd))
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True, ptxas_verbose="--ptxas" in sys.argv)
    print(LIB)
