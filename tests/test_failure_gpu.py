"""Failure detection on the GPU, in the forms that fault or hang nothing.

* A bounded device wait that runs out: mds_test_inject arms a fault in which
  the next tensor-core screen launch withholds its end-of-work marker (a flag
  that nothing then sets). Its MMA and epilogue roles give up after their
  one-second limit, release their resources, and the call returns
  MDS_ERR_TIMEOUT; the same context then computes the same result as
  before. Both the pivot pass (a set large enough for tile skipping) and
  the main screen (a small set) are covered.
* Non-finite input coordinates: the prep kernels record the frame and the
  call returns MDS_ERR_ARG naming it (the reference passes them on to
  GROMACS and std::sort, which leaves the result undefined).
* An HBM budget too small for the problem: MDS_ERR_NOMEM, no allocation.
* Serving: a request larger than max_batch_frames is refused at submission.
"""
import time

import numpy as np
import pytest

from mdsctk_gb300 import _lib as L
from mdsctk_gb300 import synth


@pytest.mark.gpu
@pytest.mark.parametrize("n", [200, 2000])
def test_screen_stall_times_out_and_context_recovers(ctx, n):
    x = synth.trajectory(n, 96, seed=90 + n, basins=2, dwell=100)
    m = synth.uniform_masses(96)
    d0, i0 = ctx.knn_rms(x, None, m, 10, precision="bf16x3")
    L.check(ctx.h, ctx._lib.mds_test_inject(ctx.h, L.MDS_INJECT_SCREEN_STALL))
    t0 = time.time()
    with pytest.raises(L.MdsError) as e:
        ctx.knn_rms(x, None, m, 10, precision="bf16x3")
    assert e.value.code == L.MDS_ERR_TIMEOUT, e.value
    assert time.time() - t0 < 30
    d1, i1 = ctx.knn_rms(x, None, m, 10, precision="bf16x3")
    assert np.array_equal(d0, d1) and np.array_equal(i0, i1)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "bf16x3"])
def test_non_finite_coordinates_rejected(ctx, precision):
    x = synth.trajectory(400, 64, seed=91)
    m = synth.uniform_masses(64)
    bad = x.copy()
    bad[123, 5, 1] = np.nan
    with pytest.raises(L.MdsError) as e:
        ctx.knn_rms(bad, None, m, 10, precision=precision)
    assert e.value.code == L.MDS_ERR_ARG and "123" in str(e.value)
    fit = x[:50].copy()
    fit[7, 0, 2] = np.inf
    with pytest.raises(L.MdsError) as e:
        ctx.knn_rms(x, fit, m, 10, precision=precision)
    assert e.value.code == L.MDS_ERR_ARG and "fit frame 7" in str(e.value)
    with pytest.raises(L.MdsError) as e:
        ctx.knn_rms(bad[:40], bad[100:140], m, 0, sort=False)
    assert e.value.code == L.MDS_ERR_ARG
    d, i = ctx.knn_rms(x, None, m, 10, precision=precision)  # still usable
    assert np.all(np.isfinite(d))


@pytest.mark.gpu
def test_hbm_budget_too_small():
    from mdsctk_gb300 import Context

    x = synth.trajectory(3000, 304, seed=92)
    with Context(0, hbm_budget=4 << 20) as c:
        with pytest.raises(L.MdsError) as e:
            c.knn_rms(x, None, None, 20, precision="bf16x3")
        assert e.value.code == L.MDS_ERR_NOMEM
        assert "budget" in str(e.value)


@pytest.mark.gpu
def test_serving_refuses_oversized_request():
    from mdsctk_gb300.serve import Server

    land = synth.trajectory(400, 48, seed=93, basins=2, dwell=100)
    with Server(land, None, k=8, sigma=1.0, nev=3, max_batch_frames=64, slots=1) as srv:
        with pytest.raises(L.MdsError) as e:
            srv.submit(synth.trajectory(65, 48, seed=94))
        assert e.value.code == L.MDS_ERR_ARG
        ext, d, i, info = srv.wait(srv.submit(synth.trajectory(64, 48, seed=95)))
        assert d.shape == (64, 8)
