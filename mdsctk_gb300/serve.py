"""Python handle of the resident Nystrom server (mds_server_* in the C ABI).

    srv = Server(landmarks, masses, k=50, sigma=..., nev=10)
    t = srv.submit(frames)                      # returns immediately
    ext, d, i, info = srv.wait(t)               # ext [nev, m]; kNN [m, k]

Requests from any number of threads are batched continuously by the
library's scheduler thread; see include/mdsgpu.h for the semantics.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib as L


class Server:
    def __init__(self, landmarks, masses=None, k: int = 50, sigma: float = 1.0, nev: int = 10, ncv: int = 0,
                 tol: float = 0.0, maxiter: int = 0, precision: str = "bf16x3", nofit: bool = False,
                 max_batch_frames: int = 4096, slots: int = 0, hbm_budget: int = 0, use_graphs: bool = True,
                 device: int = 0):
        self._lib = L.lib()
        x = np.ascontiguousarray(landmarks, np.float32)
        self.n, self.natoms = x.shape[0], x.shape[1]
        m = np.ones(self.natoms, np.float32) if masses is None else np.ascontiguousarray(masses, np.float32)
        cfg = L.ServerConfig(device=device, k=k, sigma=sigma, nev=nev, ncv=ncv, tol=tol, maxiter=maxiter,
                             flags=L.PRECISIONS[precision] | (L.MDS_NOFIT if nofit else 0),
                             max_batch_frames=max_batch_frames, slots=slots, hbm_budget=hbm_budget,
                             use_graphs=int(bool(use_graphs)))
        h = ctypes.c_void_p()
        rc = self._lib.mds_server_create(ctypes.byref(cfg), x.ctypes.data_as(ctypes.c_void_p), self.n, self.natoms,
                                         m.ctypes.data_as(ctypes.c_void_p), ctypes.byref(h))
        if rc != L.MDS_OK:
            raise L.MdsError(rc, "mds_server_create failed")
        self.h = h
        self.k = min(k, self.n - 1)
        self.nev = nev
        self._sizes = {}  # ticket -> frames (dict operations are atomic under the GIL)

    def _check(self, rc):
        if rc != L.MDS_OK:
            msg = self._lib.mds_server_last_error(self.h)
            raise L.MdsError(rc, msg.decode() if msg else "")

    def model(self):
        ev = np.zeros(self.nev)
        V = np.zeros((self.nev, self.n))
        self._check(self._lib.mds_server_model(self.h, ev.ctypes.data_as(ctypes.c_void_p),
                                               V.ctypes.data_as(ctypes.c_void_p)))
        return ev, V

    def submit(self, frames) -> int:
        q = np.ascontiguousarray(frames, np.float32)
        t = ctypes.c_int64(0)
        self._check(self._lib.mds_server_submit(self.h, q.ctypes.data_as(ctypes.c_void_p), q.shape[0],
                                                ctypes.byref(t)))
        self._sizes[t.value] = q.shape[0]
        return t.value

    def wait(self, ticket: int, timeout_ms: int = 120000):
        m = self._sizes.pop(ticket)
        ext = np.zeros((self.nev, m))
        d = np.zeros((m, self.k))
        i = np.zeros((m, self.k), np.int32)
        info = L.RequestInfo()
        rc = self._lib.mds_server_wait(self.h, ticket, timeout_ms, ext.ctypes.data_as(ctypes.c_void_p),
                                       d.ctypes.data_as(ctypes.c_void_p), i.ctypes.data_as(ctypes.c_void_p),
                                       ctypes.byref(info))
        if rc != L.MDS_OK:
            self._sizes[ticket] = m
            self._check(rc)
        return ext, d, i, {"queue_ms": info.queue_ms, "total_ms": info.total_ms, "batch": info.batch,
                           "batch_frames": info.batch_frames}

    def hold(self, on: bool = True):
        """Admit no queued request into a batch while on (running batches
        finish, submissions keep queueing); hold(False) resumes."""
        self._check(self._lib.mds_server_hold(self.h, int(bool(on))))

    def stats(self) -> dict:
        s = L.ServerStats()
        self._check(self._lib.mds_server_get_stats(self.h, ctypes.byref(s)))
        return s.as_dict()

    def close(self):
        if getattr(self, "h", None):
            self._lib.mds_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
