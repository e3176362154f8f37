"""Python mirror of the MDSCTK hot-path tools over the libmdsgpu C ABI.

Each method keeps the argument meaning of the reference tool it replaces
(knn_rms, knn_data, make_sysparse, make_gesparse, decomp_sparse,
decomp_sparse_nystrom) and returns the arrays the tool would write.
Host arrays are numpy; device-resident inputs may be passed as torch CUDA
tensors (their pointers go through the same C ABI with MDS_DEVICE_IO).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib as L


def _ptr(a):
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data_as(ctypes.c_void_p)
    return ctypes.c_void_p(int(a.data_ptr()))  # torch tensor


def _is_device(a) -> bool:
    return a is not None and not isinstance(a, np.ndarray) and getattr(a, "is_cuda", False)


class Context:
    """One libmdsgpu context (device + stream + HBM budget)."""

    def __init__(self, device: int = 0, hbm_budget: int = 0):
        self._lib = L.lib()
        h = ctypes.c_void_p()
        rc = self._lib.mds_create(int(device), int(hbm_budget), ctypes.byref(h))
        if rc != L.MDS_OK:
            raise L.MdsError(rc, f"mds_create(device={device}) failed")
        self.h = h
        self.device = device

    def close(self):
        if getattr(self, "h", None):
            self._lib.mds_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def xtc_read(self, path_or_bytes, device_out: bool = False):
        """Read a GROMACS .xtc trajectory (decoded on the GPU): returns
        (xyz [frames, atoms, 3] float32 nm, steps, times). With device_out the
        frames come back as a torch CUDA tensor, ready for knn_rms."""
        b = path_or_bytes if isinstance(path_or_bytes, (bytes, bytearray)) else open(path_or_bytes, "rb").read()
        buf = ctypes.create_string_buffer(bytes(b), len(b))
        nf, na = ctypes.c_int(0), ctypes.c_int(0)
        rc = self._lib.mds_xtc_index(buf, len(b), None, 0, ctypes.byref(nf), ctypes.byref(na))
        if rc != L.MDS_OK:
            raise L.MdsError(rc, "not an xtc trajectory (bad magic number or changing atom count)")
        off = np.zeros(nf.value + 1, np.int64)
        self._lib.mds_xtc_index(buf, len(b), _ptr(off), nf.value + 1, ctypes.byref(nf), ctypes.byref(na))
        steps = np.zeros(nf.value, np.int32)
        times = np.zeros(nf.value, np.float32)
        if device_out:
            import torch

            xyz = torch.empty((nf.value, na.value, 3), dtype=torch.float32, device=f"cuda:{self.device}")
            flags = L.MDS_DEVICE_IO
        else:
            xyz = np.zeros((nf.value, na.value, 3), np.float32)
            flags = 0
        L.check(self.h, self._lib.mds_xtc_decode(self.h, buf, len(b), _ptr(off), nf.value, na.value, flags,
                                                 _ptr(xyz), _ptr(steps), _ptr(times), None))
        return xyz, steps, times

    def stats(self) -> dict:
        s = L.KnnStats()
        L.check(self.h, self._lib.mds_get_knn_stats(self.h, ctypes.byref(s)))
        return s.as_dict()

    # ------------------------------------------------------------------ kNN
    def knn_rms(self, ref, fit=None, mass=None, k: int = 1, nofit: bool = False, sort: bool = True,
                precision: str = "fp32", out=None, skip: bool = True):
        """knn_rms: k nearest reference frames of every fit frame by minimum
        RMSD (Angstrom). ref/fit: [n, natoms, 3] float32 nm (uncentred).
        Returns (distances [n_fit, k] f64, indices [n_fit, k] i32), or the
        full [n_fit, n_ref] rows when sort=False. skip=False makes the screen
        compute every tile (same results; for like-for-like timing)."""
        dev = _is_device(ref)
        n_ref, natoms = int(ref.shape[0]), int(ref.shape[1])
        n_fit = n_ref if fit is None else int(fit.shape[0])
        flags = L.PRECISIONS[precision]
        if nofit:
            flags |= L.MDS_NOFIT
        if not sort:
            flags |= L.MDS_FULL
        if not skip:
            flags |= L.MDS_NO_SKIP
        if dev:
            import torch

            flags |= L.MDS_DEVICE_IO
            if mass is None:
                mass = torch.ones(natoms, dtype=torch.float32, device=ref.device)
            kk = n_ref if not sort else max(0, min(k, n_ref - 1))
            if out is None:
                out = (torch.empty((n_fit, kk), dtype=torch.float64, device=ref.device),
                       torch.empty((n_fit, kk), dtype=torch.int32, device=ref.device))
            d, i = out
        else:
            ref = np.ascontiguousarray(ref, dtype=np.float32)
            fit = None if fit is None else np.ascontiguousarray(fit, dtype=np.float32)
            mass = np.ones(natoms, np.float32) if mass is None else np.ascontiguousarray(mass, np.float32)
            kk = n_ref if not sort else max(0, min(k, n_ref - 1))
            if out is None:
                out = (np.empty((n_fit, kk), np.float64), np.empty((n_fit, kk), np.int32))
            d, i = out
        ku = ctypes.c_int(0)
        rc = self._lib.mds_knn_rms(self.h, _ptr(ref), n_ref, _ptr(fit), n_fit if fit is not None else 0,
                                   natoms, _ptr(mass), int(k), flags, _ptr(d), _ptr(i), ctypes.byref(ku))
        L.check(self.h, rc)
        return d, i

    def knn_rms_screen(self, ref, fit=None, mass=None, kprime: int = 32, nofit: bool = False,
                       precision: str = "fp32"):
        """Candidate screen diagnostic: per fit frame, the kprime smallest
        lower bounds of RMSD^2 (nm^2) and their reference indices, ascending.
        Returns (bounds [n_fit, kprime] f32, indices [n_fit, kprime] i32,
        counts [n_fit])."""
        ref = np.ascontiguousarray(ref, dtype=np.float32)
        fit = None if fit is None else np.ascontiguousarray(fit, dtype=np.float32)
        n_ref, natoms = ref.shape[0], ref.shape[1]
        n_fit = n_ref if fit is None else fit.shape[0]
        mass = np.ones(natoms, np.float32) if mass is None else np.ascontiguousarray(mass, np.float32)
        flags = L.PRECISIONS[precision] | (L.MDS_NOFIT if nofit else 0)
        keys = np.zeros((n_fit, kprime), np.uint64)
        counts = np.zeros(n_fit, np.int32)
        rc = self._lib.mds_knn_rms_screen(self.h, _ptr(ref), n_ref, _ptr(fit),
                                          n_fit if fit is not None else 0, natoms, _ptr(mass), int(kprime),
                                          flags, _ptr(keys), _ptr(counts))
        L.check(self.h, rc)
        bounds = (keys >> np.uint64(32)).astype(np.uint32).view(np.float32)
        idx = (keys & np.uint64(0xFFFFFFFF)).astype(np.uint32).view(np.int32)
        return bounds, idx, counts

    def knn_rms_superpose(self, ref, mass=None, nofit: bool = False):
        """Superposition diagnostic: (deviations [n, 3, Ap] f32, records [n, 16] f32)."""
        ref = np.ascontiguousarray(ref, dtype=np.float32)
        n, natoms = ref.shape[0], ref.shape[1]
        ap = (natoms + 63) // 64 * 64
        mass = np.ones(natoms, np.float32) if mass is None else np.ascontiguousarray(mass, np.float32)
        dev = np.zeros((n, 3, ap), np.float32)
        rec = np.zeros((n, 16), np.float32)
        rc = self._lib.mds_knn_rms_superpose(self.h, _ptr(ref), n, natoms, _ptr(mass),
                                             L.MDS_NOFIT if nofit else 0, _ptr(dev), _ptr(rec))
        L.check(self.h, rc)
        return dev, rec

    def knn_data(self, ref, fit=None, k: int = 1, correlation: bool = False, sort: bool = True,
                 precision: str = "fp32", out=None, skip: bool = True):
        """knn_data: k nearest reference vectors (Euclidean, or correlation
        distance). ref/fit: [n, dim] float64. Returns (distances, indices).
        skip=False: the tensor-core screen computes every tile in the input
        order (same results; MDS_NO_SKIP)."""
        dev = _is_device(ref)
        n_ref, dim = int(ref.shape[0]), int(ref.shape[1])
        n_fit = n_ref if fit is None else int(fit.shape[0])
        flags = L.PRECISIONS[precision]
        if not skip:
            flags |= L.MDS_NO_SKIP
        if correlation:
            flags |= L.MDS_CORRELATION
        if not sort:
            flags |= L.MDS_FULL
        kk = n_ref if not sort else max(0, min(k, n_ref - 1))
        if dev:
            import torch

            flags |= L.MDS_DEVICE_IO
            if out is None:
                out = (torch.empty((n_fit, kk), dtype=torch.float64, device=ref.device),
                       torch.empty((n_fit, kk), dtype=torch.int32, device=ref.device))
        else:
            ref = np.ascontiguousarray(ref, dtype=np.float64)
            fit = None if fit is None else np.ascontiguousarray(fit, dtype=np.float64)
            if out is None:
                out = (np.empty((n_fit, kk), np.float64), np.empty((n_fit, kk), np.int32))
        d, i = out
        ku = ctypes.c_int(0)
        rc = self._lib.mds_knn_data(self.h, _ptr(ref), n_ref, _ptr(fit), n_fit if fit is not None else 0,
                                    dim, int(k), flags, _ptr(d), _ptr(i), ctypes.byref(ku))
        L.check(self.h, rc)
        return d, i

    def knn_data_sparse(self, ref, fit=None, k: int = 1, sort: bool = True):
        """knn_data_sparse: k nearest sparse vectors (Euclidean). ref/fit:
        CSR triplets (off int64[n+1], idx int32, val float64), e.g. from
        sparse_vectors(); fit None = ref. Returns (distances, indices), or the
        full rows when sort=False."""
        ro, ri, rv = (np.ascontiguousarray(ref[0], np.int64), np.ascontiguousarray(ref[1], np.int32),
                      np.ascontiguousarray(ref[2], np.float64))
        n_ref = len(ro) - 1
        if fit is None:
            fo = fi = fv = None
            n_fit = n_ref
        else:
            fo, fi, fv = (np.ascontiguousarray(fit[0], np.int64), np.ascontiguousarray(fit[1], np.int32),
                          np.ascontiguousarray(fit[2], np.float64))
            n_fit = len(fo) - 1
        kk = n_ref if not sort else max(0, min(k, n_ref - 1))
        d = np.empty((n_fit, kk), np.float64)
        i = np.empty((n_fit, kk), np.int32)
        ku = ctypes.c_int(0)
        rc = self._lib.mds_knn_data_sparse(self.h, _ptr(ro), _ptr(ri), _ptr(rv), n_ref, _ptr(fo), _ptr(fi),
                                           _ptr(fv), n_fit, int(k), 0 if sort else L.MDS_FULL, _ptr(d), _ptr(i),
                                           ctypes.byref(ku))
        L.check(self.h, rc)
        return d, i

    def contact_profile(self, xyz, g1, g2, eps: float = 9.0):
        """contact_profile: xyz [nframes, natoms, 3] float32 nm; g1/g2 0-based
        atom indices. Returns (offsets int64[nframes+1], indices int32): frame
        f's contacts are indices[offsets[f]:offsets[f+1]] (grid index
        i * len(g2) + j, ascending), each of value 1.0."""
        xyz = np.ascontiguousarray(xyz, np.float32)
        g1 = np.ascontiguousarray(g1, np.int32)
        g2 = np.ascontiguousarray(g2, np.int32)
        nframes, natoms = int(xyz.shape[0]), int(xyz.shape[1])
        off = np.zeros(nframes + 1, np.int64)
        rc = self._lib.mds_contact_profile(self.h, _ptr(xyz), nframes, natoms, _ptr(g1), len(g1), _ptr(g2), len(g2),
                                           float(eps), _ptr(off), None, 0)
        L.check(self.h, rc)
        idx = np.empty(max(1, int(off[-1])), np.int32)
        rc = self._lib.mds_contact_profile(self.h, _ptr(xyz), nframes, natoms, _ptr(g1), len(g1), _ptr(g2), len(g2),
                                           float(eps), _ptr(off), _ptr(idx), int(len(idx)))
        L.check(self.h, rc)
        return off, idx[:int(off[-1])]

    # ------------------------------------------------------------ sparse
    def sysparse(self, dist, idx, k=None):
        """make_sysparse: returns (n, pcol, irow, val) of the strict lower
        triangle of distances (CSC)."""
        dist = np.ascontiguousarray(dist, np.float64)
        idx = np.ascontiguousarray(idx, np.int32)
        n, maxk = dist.shape
        k = maxk if k is None else int(k)
        cap = max(1, n * k)
        pcol = np.zeros(n + 1, np.int32)
        irow = np.zeros(cap, np.int32)
        val = np.zeros(cap, np.float64)
        nnz = ctypes.c_int64(0)
        L.check(self.h, self._lib.mds_sysparse(self.h, _ptr(dist), _ptr(idx), n, maxk, k, 0, _ptr(pcol),
                                               _ptr(irow), _ptr(val), cap, ctypes.byref(nnz)))
        return n, pcol, irow[:nnz.value].copy(), val[:nnz.value].copy()

    def gesparse(self, dist, idx, k=None, symmetric=False):
        """make_gesparse: returns (m, pcol, irow, val) (CSC, column = query)."""
        dist = np.ascontiguousarray(dist, np.float64)
        idx = np.ascontiguousarray(idx, np.int32)
        n, maxk = dist.shape
        k = maxk if k is None else int(k)
        cap = max(1, n * k * (2 if symmetric else 1))
        pcol = np.zeros(n + 1, np.int32)
        irow = np.zeros(cap, np.int32)
        val = np.zeros(cap, np.float64)
        nnz = ctypes.c_int64(0)
        L.check(self.h, self._lib.mds_gesparse(self.h, _ptr(dist), _ptr(idx), n, maxk, k, int(bool(symmetric)), 0,
                                               _ptr(pcol), _ptr(irow), _ptr(val), cap, ctypes.byref(nnz)))
        return n, pcol, irow[:nnz.value].copy(), val[:nnz.value].copy()

    def decomp_sparse(self, n, pcol, irow, dist, sigma, nev, ncv=0, tol=0.0, maxiter=0):
        """decomp_sparse: (evals descending [nev], evecs [nev, n], residuals [nev], nconv)."""
        pcol = np.ascontiguousarray(pcol, np.int32)
        irow = np.ascontiguousarray(irow, np.int32)
        dist = np.ascontiguousarray(dist, np.float64)
        ev = np.zeros(nev)
        V = np.zeros((nev, n))
        res = np.zeros(nev)
        nc = ctypes.c_int(0)
        L.check(self.h, self._lib.mds_decomp_sparse(self.h, int(n), _ptr(pcol), _ptr(irow), _ptr(dist), float(sigma),
                                                    int(nev), int(ncv), float(tol), int(maxiter), 0, _ptr(ev),
                                                    _ptr(V), _ptr(res), ctypes.byref(nc)))
        return ev, V, res, nc.value

    def decomp_sparse_nystrom(self, n, pcol, irow, dist, m, pcolB, irowB, distB, sigma, nev, ncv=0, tol=0.0,
                              maxiter=0):
        """decomp_sparse_nystrom: (evals, evecs [nev, n], ext [nev, m], residuals, nconv)."""
        a = [np.ascontiguousarray(v, t) for v, t in ((pcol, np.int32), (irow, np.int32), (dist, np.float64),
                                                      (pcolB, np.int32), (irowB, np.int32), (distB, np.float64))]
        ev = np.zeros(nev)
        V = np.zeros((nev, n))
        E = np.zeros((nev, m))
        res = np.zeros(nev)
        nc = ctypes.c_int(0)
        L.check(self.h, self._lib.mds_decomp_sparse_nystrom(
            self.h, int(n), _ptr(a[0]), _ptr(a[1]), _ptr(a[2]), int(m), _ptr(a[3]), _ptr(a[4]), _ptr(a[5]),
            float(sigma), int(nev), int(ncv), float(tol), int(maxiter), 0, _ptr(ev), _ptr(V), _ptr(E), _ptr(res),
            ctypes.byref(nc)))
        return ev, V, E, res, nc.value

    def auto_decomp_sparse(self, n, pcol, irow, dist, k_sigma, nev, perplexity=None, ncv=0, tol=0.0, maxiter=0):
        """auto_decomp_sparse: (evals, evecs [nev, n], residuals, nconv, sigmas [n])."""
        a = [np.ascontiguousarray(v, t) for v, t in ((pcol, np.int32), (irow, np.int32), (dist, np.float64))]
        ev = np.zeros(nev)
        V = np.zeros((nev, n))
        res = np.zeros(nev)
        sig = np.zeros(n)
        nc = ctypes.c_int(0)
        L.check(self.h, self._lib.mds_auto_decomp_sparse(
            self.h, int(n), _ptr(a[0]), _ptr(a[1]), _ptr(a[2]), int(k_sigma), float(perplexity or 0.0), int(nev),
            int(ncv), float(tol), int(maxiter), 0, _ptr(ev), _ptr(V), _ptr(res), ctypes.byref(nc), _ptr(sig)))
        return ev, V, res, nc.value, sig

    def auto_decomp_sparse_nystrom(self, n, pcol, irow, dist, m, pcolB, irowB, distB, k_sigma, nev, perplexity=None,
                                   ncv=0, tol=0.0, maxiter=0):
        """auto_decomp_sparse_nystrom: (evals, evecs [nev, n], ext [nev, m], residuals, nconv, sigmas [n])."""
        a = [np.ascontiguousarray(v, t) for v, t in ((pcol, np.int32), (irow, np.int32), (dist, np.float64),
                                                      (pcolB, np.int32), (irowB, np.int32), (distB, np.float64))]
        ev = np.zeros(nev)
        V = np.zeros((nev, n))
        E = np.zeros((nev, m))
        res = np.zeros(nev)
        sig = np.zeros(n)
        nc = ctypes.c_int(0)
        L.check(self.h, self._lib.mds_auto_decomp_sparse_nystrom(
            self.h, int(n), _ptr(a[0]), _ptr(a[1]), _ptr(a[2]), int(m), _ptr(a[3]), _ptr(a[4]), _ptr(a[5]),
            int(k_sigma), float(perplexity or 0.0), int(nev), int(ncv), float(tol), int(maxiter), 0, _ptr(ev),
            _ptr(V), _ptr(E),
            _ptr(res), ctypes.byref(nc), _ptr(sig)))
        return ev, V, E, res, nc.value, sig
