"""CPU oracle for the MDSCTK hot path -- TEST INFRASTRUCTURE ONLY.

Loads ``oracle/_build/libmds_oracle.so`` (built from ``mds_oracle.cpp`` by
``oracle/Makefile``) and adds the eigensolve step in Python. Only the tests,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` import
this module; the product library never does.

Pinned on the reference's own code (ref_build.py compiles its functions
from the checkout into _ref/, where one is present): euclidean_distance,
correlation_distance, euclidean_distance_sparse with permutation::sort in
the kNN loops, sp_dsymv, sp_dgemv, decomp_sparse's affinity block and
entropic_affinity_sigmas; tests/test_ref_pin.py checks the restatements
below against them bit for bit.

Parity status: **parity unpinned** for the RMSD values (GROMACS do_fit /
rmsdev / reset_x are third-party and absent; the reference cannot be built
here and ships no golden outputs). The eigensolve is anchored on ARPACK, the
reference's own solver dependency, through scipy's ``eigsh`` wrapper with the
reference's parameters (decomp_sparse.cpp:185-237): which='LA',
ncv=min(10*nev+1, n), tol=0, maxiter=100*nev.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libmds_oracle.so")
_lib = None

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")


def build() -> str:
    """Compile the oracle library with the committed Makefile."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        c_int, c_dbl = ctypes.c_int, ctypes.c_double
        L.orc_center.argtypes = [_f32p, c_int, c_int, _f32p]
        L.orc_center.restype = None
        L.orc_rmsd.argtypes = [_f32p, _f32p, c_int, _f32p, c_int]
        L.orc_rmsd.restype = c_dbl
        L.orc_rmsd_port.argtypes = [_f32p, _f32p, c_int, _f32p, c_int]
        L.orc_rmsd_port.restype = c_dbl
        L.orc_knn_rms.argtypes = [_f32p, c_int, _f32p, c_int, c_int, _f32p, c_int, c_int,
                                  c_int, c_int, _f64p, _i32p]
        L.orc_knn_rms.restype = c_int
        L.orc_knn_rms_port.argtypes = [_f32p, c_int, _f32p, c_int, c_int, _f32p, c_int, c_int,
                                       c_int, c_int, _f64p, _i32p]
        L.orc_knn_rms_port.restype = c_int
        L.orc_knn_data.argtypes = [_f64p, c_int, _f64p, c_int, c_int, c_int, c_int, c_int,
                                   c_int, _f64p, _i32p]
        L.orc_knn_data.restype = c_int
        _i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
        L.orc_knn_data_sparse.argtypes = [_i64p, _i32p, _f64p, c_int, _i64p, _i32p, _f64p, c_int, c_int,
                                          c_int, c_int, _f64p, _i32p]
        L.orc_knn_data_sparse.restype = c_int
        L.orc_contact_profile.argtypes = [_f32p, c_int, c_int, _i32p, c_int, _i32p, c_int, c_dbl, _i64p,
                                          ctypes.c_void_p]
        L.orc_contact_profile.restype = None
        L.orc_sysparse.argtypes = [_f64p, _i32p, c_int, c_int, c_int, _i32p, _i32p, _f64p]
        L.orc_sysparse.restype = ctypes.c_int64
        L.orc_gesparse.argtypes = [_f64p, _i32p, c_int, c_int, c_int, c_int, _i32p, _i32p, _f64p]
        L.orc_gesparse.restype = ctypes.c_int64
        L.orc_affinity.argtypes = [c_int, _i32p, _i32p, _f64p, c_dbl, _f64p]
        L.orc_affinity.restype = None
        L.orc_affinity_nystrom.argtypes = [c_int, _i32p, _i32p, _f64p, c_dbl, _f64p]
        L.orc_affinity_nystrom.restype = None
        L.orc_auto_sigmas.argtypes = [c_int, _i32p, _i32p, _f64p, c_int, c_dbl, c_int, _f64p]
        L.orc_auto_sigmas.restype = c_int
        L.orc_affinity_auto.argtypes = [c_int, _i32p, _i32p, _f64p, _f64p, _f64p]
        L.orc_affinity_auto.restype = None
        L.orc_affinity_nystrom_auto.argtypes = [c_int, _i32p, _i32p, _f64p, _f64p, _f64p]
        L.orc_affinity_nystrom_auto.restype = None
        L.orc_xtc_decode.argtypes = [ctypes.c_void_p, ctypes.c_size_t, c_int, _i32p, ctypes.c_void_p,
                                     ctypes.c_void_p, ctypes.c_void_p]
        L.orc_xtc_decode.restype = c_int
        L.orc_sp_dsymv.argtypes = [c_int, _i32p, _i32p, _f64p, _f64p, _f64p]
        L.orc_sp_dsymv.restype = None
        L.orc_sp_dgemv.argtypes = [c_int, _i32p, _i32p, _f64p, _f64p, _f64p]
        L.orc_sp_dgemv.restype = None
        L.orc_num_threads.argtypes = []
        L.orc_num_threads.restype = c_int
        _lib = L
    return _lib


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def center(xyz, mass):
    """reset_x on every frame; returns a centred copy [n, natoms, 3] f32."""
    x = _c(xyz, np.float32).copy()
    n, na = x.shape[0], x.shape[1]
    lib().orc_center(x.reshape(-1), n, na, _c(mass, np.float32))
    return x


def rmsd(x, y, mass, nofit=False):
    """FP64 minimum RMSD (nm) between two centred frames."""
    return lib().orc_rmsd(_c(x, np.float32).reshape(-1), _c(y, np.float32).reshape(-1),
                          int(np.asarray(x).shape[0]), _c(mass, np.float32), int(nofit))


def rmsd_port(ref, fit, mass, nofit=False):
    """RMSD (nm) by the reference's do_fit + rmsdev procedure."""
    return lib().orc_rmsd_port(_c(ref, np.float32).reshape(-1), _c(fit, np.float32).reshape(-1),
                               int(np.asarray(ref).shape[0]), _c(mass, np.float32), int(nofit))


def knn_rms(ref, fit, mass, k, nofit=False, sort=True, threads=0):
    """knn_rms oracle (FP64). Returns (distances [nfit,k] in Angstrom, indices)."""
    ref = _c(ref, np.float32)
    fit = ref if fit is None else _c(fit, np.float32)
    nref, na = ref.shape[0], ref.shape[1]
    nfit = fit.shape[0]
    kk = min(k, nref - 1)
    width = kk if sort else nref
    d = np.zeros(nfit * width, np.float64)
    i = np.zeros(nfit * width, np.int32)
    lib().orc_knn_rms(ref.reshape(-1), nref, fit.reshape(-1), nfit, na, _c(mass, np.float32),
                      int(k), int(nofit), int(sort), int(threads), d, i)
    return d.reshape(nfit, width), i.reshape(nfit, width)


def knn_rms_port(ref, fit, mass, k, nofit=False, blksize=128, threads=0):
    """The reference's CPU loop restated (the timed CPU baseline)."""
    ref = _c(ref, np.float32)
    fit = ref if fit is None else _c(fit, np.float32)
    nref, na = ref.shape[0], ref.shape[1]
    nfit = fit.shape[0]
    kk = min(k, nref - 1)
    d = np.zeros(nfit * kk, np.float64)
    i = np.zeros(nfit * kk, np.int32)
    lib().orc_knn_rms_port(ref.reshape(-1), nref, fit.reshape(-1), nfit, na,
                           _c(mass, np.float32), int(k), int(nofit), int(blksize), int(threads),
                           d, i)
    return d.reshape(nfit, kk), i.reshape(nfit, kk)


def knn_data(ref, fit, k, correlation=False, sort=True, threads=0):
    """knn_data oracle (bit-exact FP64 restatement)."""
    ref = _c(ref, np.float64)
    fit = ref if fit is None else _c(fit, np.float64)
    nref, dim = ref.shape
    nfit = fit.shape[0]
    kk = min(k, nref - 1)
    width = kk if sort else nref
    d = np.zeros(nfit * width, np.float64)
    i = np.zeros(nfit * width, np.int32)
    lib().orc_knn_data(ref.reshape(-1), nref, fit.reshape(-1), nfit, dim, int(k),
                       int(correlation), int(sort), int(threads), d, i)
    return d.reshape(nfit, width), i.reshape(nfit, width)


def csr(vectors):
    """Sparse vectors [(indices, values), ...] -> (off int64[n+1], idx int32, val f64)."""
    off = np.zeros(len(vectors) + 1, np.int64)
    for r, (ii, _) in enumerate(vectors):
        off[r + 1] = off[r] + len(ii)
    idx = np.concatenate([np.asarray(ii, np.int32) for ii, _ in vectors]) if vectors else np.zeros(0, np.int32)
    val = np.concatenate([np.asarray(vv, np.float64) for _, vv in vectors]) if vectors else np.zeros(0)
    return off, np.ascontiguousarray(idx, np.int32), np.ascontiguousarray(val, np.float64)


def knn_data_sparse(ref, fit, k, sort=True, threads=0):
    """knn_data_sparse oracle (bit-exact FP64 restatement). ref/fit: CSR
    triplets (off, idx, val) as made by csr(); fit None = ref."""
    ro, ri, rv = ref
    fo, fi, fv = ref if fit is None else fit
    nref, nfit = len(ro) - 1, len(fo) - 1
    kk = min(k, nref - 1)
    width = kk if sort else nref
    d = np.zeros(max(1, nfit * width), np.float64)
    i = np.zeros(max(1, nfit * width), np.int32)
    c = lambda a, t: np.ascontiguousarray(a, t)
    lib().orc_knn_data_sparse(c(ro, np.int64), c(ri, np.int32), c(rv, np.float64), nref, c(fo, np.int64),
                              c(fi, np.int32), c(fv, np.float64), nfit, int(k), int(sort), int(threads), d, i)
    return d[:nfit * width].reshape(nfit, width), i[:nfit * width].reshape(nfit, width)


def contact_profile(xyz, g1, g2, eps=9.0):
    """contact_profile oracle: xyz [nframes, natoms, 3] float32 nm; g1, g2
    0-based atom indices. Returns (offsets int64[nframes+1], idx int32)."""
    xyz = _c(xyz, np.float32)
    nframes, natoms = xyz.shape[0], xyz.shape[1]
    g1 = _c(g1, np.int32)
    g2 = _c(g2, np.int32)
    off = np.zeros(nframes + 1, np.int64)
    lib().orc_contact_profile(xyz.reshape(-1), nframes, natoms, g1, len(g1), g2, len(g2), float(eps), off, None)
    idx = np.zeros(max(1, int(off[-1])), np.int32)
    lib().orc_contact_profile(xyz.reshape(-1), nframes, natoms, g1, len(g1), g2, len(g2), float(eps), off,
                              idx.ctypes.data_as(ctypes.c_void_p))
    return off, idx[:int(off[-1])]


def sysparse(dist, idx, k=None):
    """make_sysparse oracle. dist/idx: [nrows, maxk]. Returns (n, pcol, irow, val)."""
    dist = _c(dist, np.float64)
    idx = _c(idx, np.int32)
    nrows, maxk = dist.shape
    k = maxk if k is None else k
    pcol = np.zeros(nrows + 1, np.int32)
    cap = max(1, nrows * k)
    irow = np.zeros(cap, np.int32)
    val = np.zeros(cap, np.float64)
    nnz = lib().orc_sysparse(dist.reshape(-1), idx.reshape(-1), nrows, maxk, k, pcol, irow, val)
    return nrows, pcol, irow[:nnz].copy(), val[:nnz].copy()


def gesparse(dist, idx, k=None, symmetric=False):
    """make_gesparse oracle. Returns (m, pcol, irow, val)."""
    dist = _c(dist, np.float64)
    idx = _c(idx, np.int32)
    nrows, maxk = dist.shape
    k = maxk if k is None else k
    pcol = np.zeros(nrows + 1, np.int32)
    cap = max(1, nrows * k * (2 if symmetric else 1))
    irow = np.zeros(cap, np.int32)
    val = np.zeros(cap, np.float64)
    nnz = lib().orc_gesparse(dist.reshape(-1), idx.reshape(-1), nrows, maxk, k, int(symmetric),
                             pcol, irow, val)
    return nrows, pcol, irow[:nnz].copy(), val[:nnz].copy()


def affinity(n, pcol, irow, val, sigma):
    """Normalised Gaussian affinity (decomp_sparse.cpp:158-178). Returns (val, d^-1/2)."""
    v = _c(val, np.float64).copy()
    d = np.zeros(n, np.float64)
    lib().orc_affinity(n, _c(pcol, np.int32), _c(irow, np.int32), v, float(sigma), d)
    return v, d


def affinity_nystrom(m, pcolB, irowB, valB, sigma, d_a):
    v = _c(valB, np.float64).copy()
    lib().orc_affinity_nystrom(m, _c(pcolB, np.int32), _c(irowB, np.int32), v, float(sigma),
                               _c(d_a, np.float64))
    return v


def sp_dsymv(n, pcol, irow, A, v):
    w = np.zeros(n, np.float64)
    lib().orc_sp_dsymv(n, _c(irow, np.int32), _c(pcol, np.int32), _c(A, np.float64),
                       _c(v, np.float64), w)
    return w


def sp_dgemv(n, pcol, irow, A, v):
    w = np.zeros(n, np.float64)
    lib().orc_sp_dgemv(n, _c(irow, np.int32), _c(pcol, np.int32), _c(A, np.float64),
                       _c(v, np.float64), w)
    return w


def sym_operator(n, pcol, irow, A):
    """scipy LinearOperator applying sp_dsymv semantics."""
    from scipy.sparse.linalg import LinearOperator

    pcol = _c(pcol, np.int32)
    irow = _c(irow, np.int32)
    A = _c(A, np.float64)
    return LinearOperator((n, n), matvec=lambda v: sp_dsymv(n, pcol, irow, A, np.ravel(v)),
                          dtype=np.float64)


def decomp_sparse(n, pcol, irow, dist, sigma, nev, ncv=None, tol=0.0, maxiter=None, v0=None):
    """decomp_sparse oracle: affinity, normalisation, ARPACK 'LA' eigenpairs.

    Returns (evals descending [nev], evecs [nev, n], residuals [nev]) in the
    reference's output order (decomp_sparse.cpp:242-270).
    """
    from scipy.sparse.linalg import eigsh

    A, _ = affinity(n, pcol, irow, dist, sigma)
    op = sym_operator(n, pcol, irow, A)
    if ncv is None:
        ncv = min(10 * nev + 1, n)
    if maxiter is None:
        maxiter = 100 * nev
    w, V = eigsh(op, k=nev, which="LA", ncv=ncv, tol=tol, maxiter=maxiter, v0=v0)
    order = np.argsort(w)[::-1]
    w = w[order]
    V = V[:, order].T.copy()
    res = np.array([np.linalg.norm(sp_dsymv(n, pcol, irow, A, V[x]) - w[x] * V[x]) / abs(w[x])
                    for x in range(nev)])
    return w, V, res


def auto_sigmas(n, pcol, irow, dist, k_sigma, perplexity=None):
    """Per-landmark sigmas of auto_decomp_sparse (auto_decomp_sparse.cpp:153-178,
    mdsctk.cpp:388-565); perplexity None = the k-sigma means only."""
    sig = np.zeros(n, np.float64)
    rc = lib().orc_auto_sigmas(n, _c(pcol, np.int32), _c(irow, np.int32), _c(dist, np.float64), int(k_sigma),
                               float(perplexity or 0.0), int(perplexity is not None), sig)
    if rc != 0:
        raise ValueError("entropic sigmas need every landmark list to hold k-sigma >= ceil(K) entries")
    return sig


def affinity_auto(n, pcol, irow, val, sig):
    v = _c(val, np.float64).copy()
    d = np.zeros(n, np.float64)
    lib().orc_affinity_auto(n, _c(pcol, np.int32), _c(irow, np.int32), v, _c(sig, np.float64), d)
    return v, d


def affinity_nystrom_auto(m, pcolB, irowB, valB, sig, d_a):
    v = _c(valB, np.float64).copy()
    lib().orc_affinity_nystrom_auto(m, _c(pcolB, np.int32), _c(irowB, np.int32), v, _c(sig, np.float64),
                                    _c(d_a, np.float64))
    return v


def auto_decomp_sparse(n, pcol, irow, dist, k_sigma, nev, perplexity=None, ncv=None, tol=0.0, maxiter=None):
    """auto_decomp_sparse oracle: per-landmark sigmas, affinity with
    exp(-d^2 / 2 s_c s_r), normalisation, ARPACK 'LA' eigenpairs.
    Returns (evals descending, evecs [nev, n], residuals, sigmas)."""
    from scipy.sparse.linalg import eigsh

    sig = auto_sigmas(n, pcol, irow, dist, k_sigma, perplexity)
    A, _ = affinity_auto(n, pcol, irow, dist, sig)
    op = sym_operator(n, pcol, irow, A)
    ncv = min(10 * nev + 1, n) if ncv is None else ncv
    maxiter = 100 * nev if maxiter is None else maxiter
    w, V = eigsh(op, k=nev, which="LA", ncv=ncv, tol=tol, maxiter=maxiter)
    order = np.argsort(w)[::-1]
    w = w[order]
    V = V[:, order].T.copy()
    res = np.array([np.linalg.norm(sp_dsymv(n, pcol, irow, A, V[x]) - w[x] * V[x]) / abs(w[x])
                    for x in range(nev)])
    return w, V, res, sig


def xtc_read(path_or_bytes, max_frames=None):
    """Decode an .xtc file: (xyz [frames, atoms, 3] float32 nm, steps, times)."""
    b = path_or_bytes if isinstance(path_or_bytes, (bytes, bytearray)) else open(path_or_bytes, "rb").read()
    buf = ctypes.create_string_buffer(bytes(b), len(b))
    na = np.zeros(1, np.int32)
    n = lib().orc_xtc_decode(buf, len(b), 1 << 30, na, None, None, None)
    if n < 0:
        raise ValueError("malformed xtc")
    if max_frames is not None:
        n = min(n, max_frames)
    xyz = np.zeros((n, int(na[0]), 3), np.float32)
    steps = np.zeros(n, np.int32)
    times = np.zeros(n, np.float32)
    vp = ctypes.c_void_p
    lib().orc_xtc_decode(buf, len(b), n, na, xyz.ctypes.data_as(vp), steps.ctypes.data_as(vp),
                         times.ctypes.data_as(vp))
    return xyz, steps, times


def dense_affinity(n, pcol, irow, dist, sigma):
    """Dense normalised affinity matrix (exact cross-check for small n)."""
    A, _ = affinity(n, pcol, irow, dist, sigma)
    M = np.zeros((n, n))
    for c in range(n):
        for p in range(pcol[c], pcol[c + 1]):
            r = irow[p]
            if r == c and p == pcol[c]:
                M[r, c] += A[p]
            else:
                M[r, c] += A[p]
                M[c, r] += A[p]
    return M


def nystrom_extend(evals, evecs, m, pcolB, irowB, B):
    """ext[x] = B^T (z_x / lambda_x) (decomp_sparse_nystrom.cpp:301-312)."""
    out = np.zeros((len(evals), m))
    for x in range(len(evals)):
        out[x] = sp_dgemv(m, pcolB, irowB, B, evecs[x] / evals[x])
    return out


# ---------------------------------------------------------------------------
# The reference's own functions, compiled from its checkout by ref_build.py
# (oracle/_ref/libmds_ref.so). Present only where the checkout is; the tests
# that pin the oracle on it skip elsewhere.
# ---------------------------------------------------------------------------
_ref_lib = None


def ref_lib():
    """The library built by ref_build.py, or None."""
    global _ref_lib
    if _ref_lib is None:
        import sys

        if _HERE not in sys.path:
            sys.path.insert(0, _HERE)
        import ref_build

        path = ref_build.build()
        if path is None or not os.path.exists(path):
            return None
        L = ctypes.CDLL(path)
        c_int, c_dbl = ctypes.c_int, ctypes.c_double
        _i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
        for nm in ("ref_euclidean_distance", "ref_correlation_distance"):
            getattr(L, nm).argtypes = [c_int, _f64p, _f64p]
            getattr(L, nm).restype = c_dbl
        L.ref_euclidean_distance_sparse.argtypes = [c_int, _i32p, _f64p, c_int, _i32p, _f64p]
        L.ref_euclidean_distance_sparse.restype = c_dbl
        for nm in ("ref_sp_dsymv", "ref_sp_dgemv"):
            getattr(L, nm).argtypes = [c_int, _i32p, _i32p, _f64p, _f64p, _f64p]
            getattr(L, nm).restype = None
        L.ref_affinity.argtypes = [c_int, _i32p, _i32p, _f64p, c_dbl, _f64p]
        L.ref_affinity.restype = None
        L.ref_entropic_sigmas.argtypes = [c_int, c_int, c_dbl, _f64p, _f64p]
        L.ref_entropic_sigmas.restype = None
        L.ref_knn_data.argtypes = [_f64p, c_int, _f64p, c_int, c_int, c_int, c_int, c_int, _f64p, _i32p]
        L.ref_knn_data.restype = None
        L.ref_knn_data_sparse.argtypes = [_i64p, _i32p, _f64p, c_int, _i64p, _i32p, _f64p, c_int, c_int,
                                          _f64p, _i32p]
        L.ref_knn_data_sparse.restype = None
        _ref_lib = L
    return _ref_lib


def ref_knn_data(ref, fit, k, correlation=False, sort=True):
    """knn_data's row loop around the reference's own distance functions and
    permutation::sort (entries [1..k] of the k+1 smallest)."""
    ref = _c(ref, np.float64)
    fit = ref if fit is None else _c(fit, np.float64)
    nref, dim = ref.shape
    nfit = fit.shape[0]
    kk = min(k, nref - 1)
    width = kk if sort else nref
    d = np.zeros(nfit * width, np.float64)
    i = np.zeros(nfit * width, np.int32)
    ref_lib().ref_knn_data(ref.reshape(-1), nref, fit.reshape(-1), nfit, dim, int(k), int(correlation),
                           int(sort), d, i)
    return d.reshape(nfit, width), i.reshape(nfit, width)


def ref_knn_data_sparse(ref, fit, k):
    """knn_data_sparse's row loop around the reference's
    euclidean_distance_sparse; ref / fit as for knn_data_sparse (CSR)."""
    ro, ri, rv = ref
    fo, fi, fv = ref if fit is None else fit
    nref, nfit = len(ro) - 1, len(fo) - 1
    kk = min(k, nref - 1)
    d = np.zeros(nfit * kk, np.float64)
    i = np.zeros(nfit * kk, np.int32)
    ref_lib().ref_knn_data_sparse(_c(ro, np.int64), _c(ri, np.int32), _c(rv, np.float64), nref,
                                  _c(fo, np.int64), _c(fi, np.int32), _c(fv, np.float64), nfit, int(k), d, i)
    return d.reshape(nfit, kk), i.reshape(nfit, kk)
