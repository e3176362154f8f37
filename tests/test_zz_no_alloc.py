"""GPU test of mds_knn_data_noalloc, the allocation-free knn_data entry point.

It serves callers that cannot allocate device memory where they call, such
as a plugin inside another framework whose caching allocator has reserved
the device memory. The entry point is called through the C ABI with device
buffers the test owns, and its output must equal mds_knn_data's on the same
inputs (distances bit-identical by construction, as for knn_data itself):
  * on two calls in a row with different data, since the fixed scratch
    array keeps the previous call's contents;
  * for k large enough that the screen's candidate pools cannot hold
    K' >= k + 17, where every row is rechecked exactly;
  * on vectors repeated many times, so that rows fail the guard check and
    take the exact fallback, the one part of the call that differs from the
    shared path.
This file sorts last so that a run stopping at the first failure has
already run every other test."""
import ctypes

import numpy as np
import pytest

from mdsctk_gb300 import _lib as L
from mdsctk_gb300 import synth


def _call_noalloc(ctx, ref, fit, k, corr):
    import torch

    dev = torch.device("cuda", 0)
    r = torch.from_numpy(ref).to(dev)
    f = None if fit is None else torch.from_numpy(fit).to(dev)
    n_fit = ref.shape[0] if fit is None else fit.shape[0]
    kk = min(k, ref.shape[0] - 1)
    d = torch.empty((n_fit, kk), dtype=torch.float64, device=dev)
    i = torch.empty((n_fit, kk), dtype=torch.int32, device=dev)
    torch.cuda.synchronize()
    ku = ctypes.c_int(0)
    rc = ctx._lib.mds_knn_data_noalloc(ctx.h, ctypes.c_void_p(r.data_ptr()), ref.shape[0],
                                       None if f is None else ctypes.c_void_p(f.data_ptr()),
                                       0 if fit is None else n_fit, ref.shape[1], k,
                                       L.MDS_CORRELATION if corr else 0, ctypes.c_void_p(d.data_ptr()),
                                       ctypes.c_void_p(i.data_ptr()), ctypes.byref(ku))
    L.check(ctx.h, rc)
    assert ku.value == kk
    return d.cpu().numpy(), i.cpu().numpy()


def _same_as_knn_data(ctx, ref, fit, k, corr):
    d, i = _call_noalloc(ctx, ref, fit, k, corr)
    st = ctx.stats()
    od, oi = ctx.knn_data(ref, fit, k, correlation=corr)
    assert np.array_equal(d, od)
    bad = np.argwhere(i != oi)
    for r, c in bad:  # index order may differ only among exactly equal distances
        assert np.sum(od[r] == od[r, c]) >= 2
    return st


@pytest.mark.gpu
@pytest.mark.parametrize("corr", [False, True])
def test_noalloc_matches_knn_data_twice(ctx, corr):
    x1 = synth.dihedral_vectors(1500, 32, seed=41).astype(np.float64)
    x2 = synth.dihedral_vectors(900, 32, seed=42).astype(np.float64)
    q2 = synth.dihedral_vectors(300, 32, seed=43).astype(np.float64)
    # first call: all pairs of x1; second call: other data, fit != ref
    for ref, fit, k in ((x1, None, 24), (x2, q2, 17)):
        _same_as_knn_data(ctx, ref, fit, k, corr)


@pytest.mark.gpu
@pytest.mark.parametrize("k", [150, 300])
def test_noalloc_large_k(ctx, k):
    # k = 150: K' = 192 still leaves 16 spare candidates; k = 300: rows exact
    x = synth.dihedral_vectors(1200, 24, seed=44).astype(np.float64)
    st = _same_as_knn_data(ctx, x, None, k, False)
    if k == 300:
        assert st["kprime"] == 0


@pytest.mark.gpu
def test_noalloc_guard_fallback(ctx):
    # 20 distinct vectors, each repeated 100 times: a row's K' = 64 best keys
    # are all copies of itself, so the (k+1)-th exact distance is not below
    # the K'-th bound and every row takes the exact fallback
    base = synth.dihedral_vectors(20, 16, seed=45).astype(np.float64)
    x = np.repeat(base, 100, axis=0)
    st = _same_as_knn_data(ctx, x, None, 24, False)
    assert st["rows_flagged"] > 0
    # and the next call, on data that flags nothing, is unaffected
    y = synth.dihedral_vectors(700, 16, seed=46).astype(np.float64)
    st2 = _same_as_knn_data(ctx, y, None, 12, False)
    assert st2["rows_flagged"] == 0


@pytest.mark.gpu
def test_noalloc_rejects_oversized(ctx):
    x = np.zeros((120000, 64))
    with pytest.raises(L.MdsError) as e:
        _call_noalloc(ctx, x, None, 30, False)
    assert e.value.code == L.MDS_ERR_UNSUPPORTED
