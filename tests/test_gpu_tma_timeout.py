"""GPU: the failure path of the sweep's bounded waits for its reference-tile
copies (TMA, completion on an mbarrier polled a bounded number of times).

recon_mvs_test_inject_tma_timeout makes the next run issue no tile copy and
poll only 4096 times, so every wait runs out -- a flag that nothing sets, no
fault: the blocks record the failure in the context's error flag and leave.
The run's download must report RECON_ERR_MVS_GPU_FAILURE, and the same
context must then run the same job normally, to the map an untouched
context produces."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RECON_ERR_MVS_GPU_FAILURE = 502


def test_tma_wait_timeout_reports_failure_and_context_recovers():
    import recon_mvs as mvs
    import synthetic as S

    mvs.load_library()
    sc = S.sphere_on_backdrop(width=160, height=120, f=150.0, num_sources=3, seed=31)
    views = mvs.ViewArgs.from_cameras(sc.ref.image, [s.image for s in sc.sources], sc.ref.camera,
                                      [s.camera for s in sc.sources])
    cfg = mvs.MvsConfig(min_depth_m=sc.min_depth, max_depth_m=sc.max_depth, iterations=3, patch_size=11)
    opts = mvs.Options(mode=mvs.MODE_PLANE, best_k=3, device=0)
    eng = mvs.Engine(opts)
    try:
        j = eng.stage(views, cfg)
        eng.run(j)
        first = eng.download(j)
        assert first.filled > 0.9 * first.depth.size
        mvs._check(mvs._lib().recon_mvs_test_inject_tma_timeout(eng.ctx))
        eng.run(j)
        with pytest.raises(mvs.MvsError) as err:
            eng.download(j)
        assert err.value.status == RECON_ERR_MVS_GPU_FAILURE
        eng.run(j)
        again = eng.download(j)
        np.testing.assert_array_equal(again.depth, first.depth)
        np.testing.assert_array_equal(again.cost, first.cost)
    finally:
        eng.close()
