"""The allocation-free geometric-consistency entry point.

recon_mvs_geometric_consistency_noalloc serves callers that keep all their
device memory in their own pools and cannot let a library call cudaMalloc
(a streaming loop with pre-sized buffers, a process with a rationed GPU
budget).  They pass device pointers for the depth maps and the outputs; the
only other device memory the kernel uses is a fixed array inside the
library.  Its results must equal those of recon_mvs_geometric_consistency
bit for bit (integer counts and flags), on consecutive calls that reuse the
shared array with different inputs, and it must refuse more source maps than
the array holds.

Device buffers come from torch; the entry point is called through the C ABI.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def make_maps(seed, n_src, w=120, h=90):
    import synthetic as S

    sc = S.sphere_on_backdrop(width=w, height=h, f=w * 110.0 / 120.0, num_sources=n_src, seed=seed)
    views = [sc.ref] + sc.sources
    rng = np.random.default_rng(seed)
    depths = []
    for v in views:
        d = v.depth.astype(np.float32).copy()
        d[rng.random(d.shape) < 0.05] = np.nan
        bad = rng.random(d.shape) < 0.05
        d[bad] *= rng.uniform(0.9, 1.1, bad.sum()).astype(np.float32)
        depths.append(d)
    poses = [v.camera.pose_array() for v in views]
    intr = [v.camera.intrinsics_array() for v in views]
    return depths, poses, intr


def run_both(M, torch, depths, poses, intr, ref_index):
    n = len(depths)
    host_maps = [M.DepthMap(d, np.ones(d.shape, np.uint8), np.ones(d.shape, np.float32)) for d in depths]
    want_c, want_k = M.GeometricConsistency(host_maps, poses, intr, ref_index, 0.01, 1.0, 2)

    dev = [torch.from_numpy(d).cuda() for d in depths]
    arr = (M.DepthMapC * n)()
    for i, (d, t) in enumerate(zip(depths, dev)):
        arr[i].width, arr[i].height = d.shape[1], d.shape[0]
        arr[i].depth = C.cast(C.c_void_p(t.data_ptr()), C.POINTER(C.c_float))
    ps = (M.Pose * n)(*[M.pose(p) for p in poses])
    ks = (M.Intrinsics * n)(*[M.intrinsics(k) for k in intr])
    h, w = depths[ref_index].shape
    out_c = torch.full((h, w), 255, dtype=torch.uint8, device="cuda")
    out_k = torch.full((h, w), 255, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    st = M.load_library().recon_mvs_geometric_consistency_noalloc(
        arr, C.cast(ps, C.POINTER(M.Pose)), C.cast(ks, C.POINTER(M.Intrinsics)), n, ref_index, 0.01, 1.0, 2,
        C.c_void_p(out_c.data_ptr()), C.c_void_p(out_k.data_ptr()), C.c_void_p(stream))
    assert st == M.RECON_OK, M.load_library().recon_mvs_last_error()
    torch.cuda.synchronize()
    return (want_c, want_k), (out_c.cpu().numpy(), out_k.cpu().numpy())


def test_noalloc_consistency_matches_allocating_entry_point():
    torch = pytest.importorskip("torch")
    import recon_mvs as M

    M.load_library()
    # two calls in a row with different inputs, sizes and source counts:
    # the second reuses the shared descriptor array left by the first
    for seed, n_src, ref_index, size in ((31, 4, 0, (120, 90)), (32, 6, 3, (96, 72))):
        depths, poses, intr = make_maps(seed, n_src, *size)
        (wc, wk), (gc, gk) = run_both(M, torch, depths, poses, intr, ref_index)
        assert np.array_equal(gc, wc) and np.array_equal(gk, wk)
        assert wk.mean() > 0.2 and wc.max() >= 2


def test_noalloc_rejects_more_sources_than_the_array_holds():
    torch = pytest.importorskip("torch")
    import recon_mvs as M

    lib = M.load_library()
    depths, poses, intr = make_maps(33, 1, 40, 30)
    n = 66  # 65 source maps: one more than the fixed array holds
    dev = torch.from_numpy(depths[0]).cuda()
    arr = (M.DepthMapC * n)()
    for i in range(n):
        arr[i].width, arr[i].height = 40, 30
        arr[i].depth = C.cast(C.c_void_p(dev.data_ptr()), C.POINTER(C.c_float))
    ps = (M.Pose * n)(*[M.pose(poses[i % 2]) for i in range(n)])
    ks = (M.Intrinsics * n)(*[M.intrinsics(intr[i % 2]) for i in range(n)])
    out = torch.zeros((30, 40), dtype=torch.uint8, device="cuda")
    st = lib.recon_mvs_geometric_consistency_noalloc(arr, C.cast(ps, C.POINTER(M.Pose)),
                                                     C.cast(ks, C.POINTER(M.Intrinsics)), n, 0, 0.01, 1.0, 2,
                                                     C.c_void_p(out.data_ptr()), C.c_void_p(out.data_ptr()), None)
    assert st == M.RECON_ERR_INVALID_ARGUMENT
    assert b"64" in lib.recon_mvs_last_error()
