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

    def stats(self) -> dict:
        s = L.KnnStats()
        L.check(self.h, self._lib.mds_get_knn_stats(self.h, ctypes.byref(s)))
        return s.as_dict()

    # ------------------------------------------------------------------ kNN
    def knn_rms(self, ref, fit=None, mass=None, k: int = 1, nofit: bool = False, sort: bool = True,
                precision: str = "fp32", out=None):
        """knn_rms: k nearest reference frames of every fit frame by minimum
        RMSD (Angstrom). ref/fit: [n, natoms, 3] float32 nm (uncentred).
        Returns (distances [n_fit, k] f64, indices [n_fit, k] i32), or the
        full [n_fit, n_ref] rows when sort=False."""
        dev = _is_device(ref)
        n_ref, natoms = int(ref.shape[0]), int(ref.shape[1])
        n_fit = n_ref if fit is None else int(fit.shape[0])
        flags = L.PRECISIONS[precision]
        if nofit:
            flags |= L.MDS_NOFIT
        if not sort:
            flags |= L.MDS_FULL
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

    def knn_data(self, ref, fit=None, k: int = 1, correlation: bool = False, sort: bool = True,
                 precision: str = "fp32", out=None):
        """knn_data: k nearest reference vectors (Euclidean, or correlation
        distance). ref/fit: [n, dim] float64. Returns (distances, indices)."""
        dev = _is_device(ref)
        n_ref, dim = int(ref.shape[0]), int(ref.shape[1])
        n_fit = n_ref if fit is None else int(fit.shape[0])
        flags = L.PRECISIONS[precision]
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
