"""The oracle's restatements against the reference's own functions, on CPU.

oracle/ref_build.py compiles, from the reference checkout, the functions of
mdsctk.cpp the hot path uses (euclidean_distance, correlation_distance,
euclidean_distance_sparse, sp_dsymv, sp_dgemv, entropic_affinity_sigma(s)),
mdsctk.h's permutation::sort and decomp_sparse.cpp's affinity block. Where
they are present the oracle must agree with them bit for bit; the GPU tests
hold the GPU path to the oracle, so these rows of the path are pinned on
reference code. Skipped where no reference checkout exists."""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")


@pytest.fixture(scope="module")
def ref(oracle):
    if oracle.ref_lib() is None:
        pytest.skip("no reference checkout to build oracle/_ref from")
    return oracle


def _pts(name, dim):
    return np.fromfile(os.path.join(GOLD, name + ".pts"), np.float64).reshape(-1, dim)


def _same_knn(d, i, rd, ri):
    assert np.array_equal(d, rd)
    for r, c in np.argwhere(i != ri):  # the reference's partial_sort leaves tie order open
        assert np.sum(rd[r] == rd[r, c]) >= 2


@pytest.mark.parametrize("case", ["rings", "swissroll", "swissroll_corr", "dihedral_corr", "dihedral_fit"])
def test_knn_data_pinned(ref, case):
    from mdsctk_gb300 import synth

    fit, corr, k = None, case.endswith("corr"), 12
    if case.startswith("rings"):
        x = _pts("rings", 2)
    elif case.startswith("swissroll"):
        x = _pts("swissroll", 3)
    else:
        x = synth.dihedral_vectors(700, 16, seed=3).astype(np.float64)
        if case == "dihedral_fit":
            fit = synth.dihedral_vectors(90, 16, seed=4).astype(np.float64)
    d, i = ref.knn_data(x, fit, k, correlation=corr)
    rd, ri = ref.ref_knn_data(x, fit, k, correlation=corr)
    _same_knn(d, i, rd, ri)
    # full rows (-s false): the distances in reference order
    d, _ = ref.knn_data(x[:50], None if fit is None else fit[:20], 0, correlation=corr, sort=False)
    rd, _ = ref.ref_knn_data(x[:50], None if fit is None else fit[:20], 0, correlation=corr, sort=False)
    assert np.array_equal(d, rd)


def test_knn_data_golden_fixture_pinned(ref):
    # the committed regression vectors are the reference's own output too
    g = np.load(os.path.join(GOLD, "knn_data_swissroll.npz"))
    x = _pts("swissroll", 3)
    rd, ri = ref.ref_knn_data(x, None, 12)
    _same_knn(g["d"], g["i"], rd, ri)
    rdc, ric = ref.ref_knn_data(x, None, 12, correlation=True)
    _same_knn(g["dc"], g["ic"], rdc, ric)


def test_knn_data_sparse_pinned(ref):
    rng = np.random.default_rng(11)
    vecs = []
    for r in range(300):
        nnz = int(rng.integers(0, 40))
        idx = rng.integers(0, 120, nnz)
        if r % 3 == 0:
            idx = np.sort(idx)  # sorted; others unsorted with repeats: the same walk
        val = np.round(rng.normal(size=nnz), 3)
        vecs.append((idx, val))
    X = ref.csr(vecs)
    d, i = ref.knn_data_sparse(X, None, 9)
    rd, ri = ref.ref_knn_data_sparse(X, None, 9)
    _same_knn(d, i, rd, ri)


def _graph(ref, diag=False, keep=10):
    x = _pts("rings", 2)
    d, i = ref.knn_data(x, None, 15)
    n, pcol, irow, val = ref.sysparse(d, i, keep)
    if diag:
        # a diagonal entry at the head of some columns (sp_dsymv's special case)
        pc, ir, va = [0], [], []
        for c in range(n):
            if c % 4 == 0:
                ir.append(c)
                va.append(0.5 + c * 1e-3)
            ir += list(irow[pcol[c]:pcol[c + 1]])
            va += list(val[pcol[c]:pcol[c + 1]])
            pc.append(len(ir))
        pcol, irow, val = np.array(pc, np.int32), np.array(ir, np.int32), np.array(va)
    return n, pcol, irow, val


@pytest.mark.parametrize("diag", [False, True])
def test_spmv_and_affinity_pinned(ref, diag):
    n, pcol, irow, val = _graph(ref, diag)
    sigma = float(np.median(val))
    A, dinv = ref.affinity(n, pcol, irow, val, sigma)
    rA = np.array(val, np.float64)
    rdinv = np.zeros(n)
    ref.ref_lib().ref_affinity(n, pcol.astype(np.int32), irow.astype(np.int32), rA, sigma, rdinv)
    assert np.array_equal(A, rA) and np.array_equal(dinv, rdinv)
    v = np.random.default_rng(2).normal(size=n)
    w = ref.sp_dsymv(n, pcol, irow, A, v)
    rw = np.zeros(n)
    ref.ref_lib().ref_sp_dsymv(n, irow.astype(np.int32), pcol.astype(np.int32), A, v, rw)
    assert np.array_equal(w, rw)
    w = ref.sp_dgemv(n, pcol, irow, A, v)
    ref.ref_lib().ref_sp_dgemv(n, irow.astype(np.int32), pcol.astype(np.int32), A, v, rw)
    assert np.array_equal(w, rw)


@pytest.mark.parametrize("ka,K", [(10, 5.0), (12, 7.5), (12, 12.0)])
def test_entropic_sigmas_pinned(ref, ka, K):
    n, pcol, irow, val = _graph(ref, keep=15)
    # the lists auto_decomp_sparse hands to entropic_affinity_sigmas: stored
    # distances in neighbour-index order, cut to ka, then sorted
    L = [[] for _ in range(n)]
    for c in range(n):
        for y in range(pcol[c], pcol[c + 1]):
            L[c].append(val[y])
            L[irow[y]].append(val[y])
    assert min(len(l) for l in L) >= ka
    lists = np.array([sorted(l[:ka]) for l in L], np.float64)
    s = ref.auto_sigmas(n, pcol, irow, val, ka, perplexity=K)
    rs = np.zeros(n)
    ref.ref_lib().ref_entropic_sigmas(n, ka, K, np.ascontiguousarray(lists), rs)
    assert np.array_equal(s, rs)
