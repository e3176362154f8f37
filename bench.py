"""Benchmark of the all-pairs kNN-RMSD hot path (knn_rms) on GB300.

Workload (one step): all-pairs kNN-RMSD of a synthetic trajectory of
N=20,000 frames x A=1,000 atoms (8 metastable basins, OU drift 0.08 nm,
quantised to 0.001 nm, uniform masses), k=100: 4e8 ordered pairs through the
candidate screen, fused top-k, exact recheck and output.

  value  pairs/s with the frames already resident in HBM (MDS_DEVICE_IO)
  e2e    pairs/s through the C ABI with pinned host buffers: the host->device
         copy of the frames and the device->host copy of the k-NN lists are
         inside the timed region
  roofline  the screen kernel: 18*A algorithmic flops (nine A-long
         contractions) per frame pair it computes -- the column tiles it does
         not skip (40 x 80 frame pairs each, counted by the kernel) plus the
         pivot pass -- over the screen stage's CUDA-event time, against the
         measured dense bf16 tensor peak. About 5% of the N^2 pairs are
         computed; pairs_equivalent / flops_equivalent give the N^2 figures
  roofline_recheck  the exact recheck stage: 30*A FP32 flops per candidate
         it computes (counted by the kernel) over its CUDA-event time, against
         the nominal FP32 rate; its operand bytes (12*A per candidate, served
         mostly from L2) as a rate beside it
  screen_guard  the recheck's audit of the screen's lower bound on every
         candidate it rechecks: the largest screen error per unit of
         |a_i|^2 + |a_j|^2 (which the guard coefficient must exceed) and the
         number of bounds found above their exact value (rows so found are
         finished by the wider FP32 screen or exactly)
  tc_vs_fp32  screen-stage times of the tensor-core screen and of the FP32
         CUDA-core screen on this workload, both with tile skipping switched
         off (every tile computed) and both skipping as they do by default
  parity  after the timed loops, 256 rows of the timed run's output (and of
         the FP32 path's) against the FP64 oracle (oracle/): largest distance
         error, index agreement, swaps inside tie bands of 1e-4 Angstrom
  cpu_baseline  the reference's per-pair procedure and OpenMP row loop
         restated in C++ (oracle/mds_oracle.cpp, orc_knn_rms_port) on a bounded
         sample of fit rows against all reference frames, all host cores

With --gpus N > 1 (one process per GPU under torchrun) every rank computes a
contiguous block of the fit rows against all reference frames (the kNN
stage's row sharding: no collective on the data path, strong scaling);
--replicas runs the whole workload on every rank instead.

`--impl reference` times that CPU restatement alone (the reference itself
needs GROMACS, Boost and Berkeley DB and cannot be built here).
Inputs (240 MB of frames) are larger than L2 (129 MB) in every step.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_FRAMES = 20_000
N_ATOMS = 1_000
K = 100
SEED = 2024
METRIC = "kNN-RMSD pairs/s"
UNIT = "pairs/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--precision", default=os.environ.get("MDS_BENCH_PRECISION", "bf16x3"))
    p.add_argument("--frames", type=int, default=N_FRAMES)
    p.add_argument("--atoms", type=int, default=N_ATOMS)
    p.add_argument("--k", type=int, default=K)
    p.add_argument("--cpu-rows", type=int, default=0, help="fit rows of the CPU sample (0 = auto)")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-parity", action="store_true", help="skip the oracle check of sampled rows")
    p.add_argument("--parity-rows", type=int, default=256)
    p.add_argument("--no-compare", action="store_true", help="skip the dense TC / FP32 screen comparison")
    p.add_argument("--replicas", action="store_true",
                   help="N > 1: every rank runs the whole workload (default: row shards)")
    p.add_argument("--serve", action="store_true",
                   help="Nystrom serving benchmark (50,000 landmarks x 304 atoms, k=50, nev=10)")
    p.add_argument("--serve-seconds", type=float, default=6.0, help="arrivals per rate, seconds")
    p.add_argument("--serve-rates", default="50,200,500,1000,2000", help="Poisson arrival rates, requests/s")
    p.add_argument("--serve-max-requests", type=int, default=3000)
    p.add_argument("--pipeline", choices=["small", "scale", "euclid", "sparse"],
                   help="per-stage wall time of a whole pipeline: small = 2,000 x 304 frames (parity vs the oracle), "
                        "scale = 100,000 x 304 (kNN k=64, sysparse, Lanczos nev=20 ncv=60 tol=1e-8), "
                        "euclid = knn_data 200,000 x 64, k=32 (Euclidean, then correlation), "
                        "sparse = contact_profile of 20,000 x 304 frames (atoms 0-151 vs 152-303, 12 A) "
                        "-> knn_data_sparse, k=32")
    p.add_argument("--pipeline-cpu", action="store_true", help="also time the CPU oracle's sysparse and eigsh")
    p.add_argument("--vectors", type=int, default=200_000, help="--pipeline euclid: vectors in the set")
    p.add_argument("--precision-report", action="store_true",
                   help="per-pair screen RMSD error vs FP64 and output agreement on sampled rows")
    return p.parse_args()


def run_serve(args):
    """Serving: landmarks stay resident; requests of 1-4096 frames (log-uniform
    sizes, 90% from the basin generator, 10% off-manifold) arrive as a Poisson
    stream; latency = submit -> results. Swept over the arrival rates of
    --serve-rates (each rate: up to --serve-seconds of arrivals, at most
    --serve-max-requests requests). The plain path serves one request at a
    time (one slot, no batching, no CUDA graphs): every request's service time
    is measured alone once, and each rate's arrivals are queued FIFO on them."""
    import numpy as np
    import threading

    from mdsctk_gb300 import Context, synth
    from mdsctk_gb300.serve import Server

    natoms, n_land, k, nev = 304, 50_000, 50, 10
    land = synth.trajectory(n_land, natoms, seed=SEED + 5, basins=16, dwell=500.0)
    m = np.ones(natoms, np.float32)
    with Context(0) as c:
        d, _ = c.knn_rms(land, None, m, k, precision=args.precision)
    sigma = float(np.median(d))
    rates = [float(r) for r in args.serve_rates.split(",")]
    nmax = max(8, min(args.serve_max_requests, int(max(rates) * args.serve_seconds)))
    rng = np.random.default_rng(SEED + 6)
    sizes = np.exp(rng.uniform(0, np.log(4096), nmax)).astype(int).clip(1, 4096)
    pool = synth.trajectory(8192, natoms, seed=SEED + 7, basins=16, dwell=500.0, off_manifold=0.1, off_sigma=0.3)
    starts = rng.integers(0, 8192 - 4096, nmax)
    unit_gaps = rng.exponential(1.0, nmax)  # scaled by 1/rate

    def nreq_of(rate):
        return max(8, min(nmax, int(rate * args.serve_seconds)))

    srv = Server(land, m, k=k, sigma=sigma, nev=nev, precision=args.precision, max_batch_frames=4096)
    # warm every size bucket of every slot (graph capture happens on first use)
    for bsz in (1, 2, 4, 8, 16, 32, 48, 64, 96, 128, 192, 256, 384, 512, 768, 1024, 1536, 2048, 3072, 4096):
        for t in [srv.submit(pool[:bsz]) for _ in range(srv.stats()["slots"])]:
            srv.wait(t)
    model = srv.stats()

    def run_batched(rate):
        nreq = nreq_of(rate)
        gaps = unit_gaps[:nreq] / rate
        st0 = srv.stats()
        lat, done = [None] * nreq, threading.Event()
        tickets = [None] * nreq
        bfr = [0] * nreq

        def waiter():
            for j in range(nreq):
                while tickets[j] is None:
                    time.sleep(1e-4)
                _, _, _, info = srv.wait(tickets[j])
                lat[j] = info["total_ms"]
                bfr[j] = info["batch_frames"]
            done.set()

        th = threading.Thread(target=waiter)
        th.start()
        t0 = time.perf_counter()
        tnext = t0
        for j in range(nreq):
            tnext += gaps[j]
            while time.perf_counter() < tnext:
                time.sleep(2e-5)
            tickets[j] = srv.submit(pool[starts[j]:starts[j] + sizes[j]])
        done.wait()
        wall = time.perf_counter() - t0
        th.join()
        st = srv.stats()
        lat = np.array(lat)
        return {"requests": nreq, "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                "mean_ms": float(lat.mean()), "queries_per_s": float(sizes[:nreq].sum() / wall),
                "requests_per_s": float(nreq / wall), "offered_queries_per_s": float(sizes[:nreq].sum() / gaps.sum()),
                "batches": st["batches"] - st0["batches"],
                "shared_batch_fraction": float(np.mean(np.array(bfr) > sizes[:nreq])),
                "rows_flagged": st["rows_flagged"] - st0["rows_flagged"]}

    # plain path: service time of every request alone, once
    plain = Server(land, m, k=k, sigma=sigma, nev=nev, precision=args.precision, max_batch_frames=4096,
                   slots=1, use_graphs=False)
    plain.wait(plain.submit(pool[:4096]))
    svc = np.zeros(nmax)
    for j in range(nmax):
        t0 = time.perf_counter()
        plain.wait(plain.submit(pool[starts[j]:starts[j] + sizes[j]]))
        svc[j] = time.perf_counter() - t0
    plain.close()

    def run_plain(rate):
        nreq = nreq_of(rate)
        arr = np.cumsum(unit_gaps[:nreq] / rate)
        fin, lat = 0.0, np.zeros(nreq)
        for j in range(nreq):
            fin = max(arr[j], fin) + svc[j]
            lat[j] = (fin - arr[j]) * 1e3
        return {"requests": nreq, "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                "mean_ms": float(lat.mean()), "queries_per_s": float(sizes[:nreq].sum() / max(fin, arr[-1])),
                "service_ms_mean": float(svc[:nreq].mean() * 1e3)}

    sweep = []
    for rate in rates:
        sweep.append({"rate_req_per_s": rate, "batched": run_batched(rate), "plain_per_request": run_plain(rate)})
    srv.close()
    out = {"metric": "Nystrom serving latency", "unit": "ms", "higher_is_better": False,
           "value": sweep[0]["batched"]["p99_ms"], "data": "synthetic", "dtype": args.precision,
           "config": {"workload": f"Nystrom serving: {n_land} landmarks x {natoms} atoms, k={k}, nev={nev}, "
                                  f"requests of 1-4096 frames (log-uniform), Poisson arrivals, 10% off-manifold",
                      "rates_req_per_s": rates, "sigma_A": sigma, "slots": model["slots"],
                      "model_knn_ms": model["model_knn_ms"], "model_decomp_ms": model["model_decomp_ms"]},
           "sweep": sweep}
    print(json.dumps(out))
    return 0


def run_precision_report(args):
    """Screen precision vs FP64 on two workloads: the benchmark trajectory
    (all pairs, sampled rows) and the serving case (off-trajectory queries
    against 50,000 landmarks, where neighbour distances are concentrated).
    Per candidate pair of the screen (the 256 smallest bounds of a row):
    coef = (screen value before the guard - exact RMSD^2) / (|a_i|^2 + |a_j|^2),
    the quantity the guard c * (|a_i|^2 + |a_j|^2) must cover (positive =
    over-estimate); the guard in use per precision; how many bounds exceed
    the exact value (must be 0); and knn_rms output agreement with the oracle."""
    import numpy as np

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from mdsctk_gb300 import Context, synth

    O.build()
    guards = {"fp32": 2.0 ** -16, "bf16x3": 2.0 ** -14, "fp16x3": 2.0 ** -14}  # MDS_GUARD_FP32 / _TC
    rep = {"metric": "kNN-RMSD screen error vs FP64"}
    x = workload(args.frames, args.atoms)
    land = synth.trajectory(50_000, 304, seed=SEED + 5, basins=16, dwell=500.0)
    qry = synth.trajectory(64, 304, seed=SEED + 7, basins=16, dwell=500.0, off_manifold=0.1, off_sigma=0.3)
    cases = {"trajectory": (x, x[np.linspace(0, x.shape[0] - 1, 64).astype(int)], args.k),
             "serving_queries": (land, qry, 50)}
    with Context(0) as c:
        for name, (ref, fit, k) in cases.items():
            m = np.ones(ref.shape[1], np.float32)
            _, rec = c.knn_rms_superpose(np.concatenate([ref, fit]), m)  # one template: ref[0]
            Ea_r, Ea_f = rec[:ref.shape[0], 15].astype(np.float64), rec[ref.shape[0]:, 15].astype(np.float64)
            exact = [dict() for _ in range(len(fit))]
            out = {"config": {"ref_frames": ref.shape[0], "atoms": ref.shape[1], "fit_rows": len(fit), "k": k}}
            for prec, guard in guards.items():
                lb, idx, cnt = c.knn_rms_screen(ref, fit, m, 256, precision=prec)
                coefs, viol = [], 0
                for r in range(len(fit)):
                    need = [j for j in idx[r] if j not in exact[r]]
                    if need:
                        ed, _ = O.knn_rms(ref[need], fit[r:r + 1], m, 0, sort=False)
                        for jj, j in enumerate(need):
                            exact[r][j] = (ed[0, jj] / 10.0) ** 2
                    ex2 = np.array([exact[r][j] for j in idx[r]])
                    E = Ea_f[r] + Ea_r[idx[r]]
                    viol += int(np.sum(lb[r] > ex2 * (1 + 1e-6) + 1e-12))
                    ok = lb[r] > 0  # unclamped values only
                    coefs.append(((lb[r] + guard * E) - ex2)[ok] / E[ok])
                cf = np.concatenate(coefs)
                d, i = c.knn_rms(ref, fit, m, k, precision=prec)
                st = c.stats()
                od, oi = O.knn_rms(ref, fit, m, k)
                out[prec] = {"guard_c": guard, "coef_max": float(cf.max()), "coef_p99_abs": float(np.percentile(
                    np.abs(cf), 99)), "coef_p50_abs": float(np.percentile(np.abs(cf), 50)), "pairs": int(cf.size),
                    "bounds_above_exact": viol, "mean_Ea_nm2": float(np.mean(Ea_f)),
                    "rows_flagged": st["rows_flagged"], "output_max_abs_err_A": float(np.max(np.abs(d - od))),
                    "index_agreement": float(np.mean(i == oi))}
            rep[name] = out
    print(json.dumps(rep))
    return 0


def run_pipeline(args):
    """Per-stage wall time (host arrays in and out, as the tools run) of one
    pipeline; each stage is timed once after one untimed run of the same
    stage. 'small' also checks every stage against the oracle."""
    import numpy as np

    from mdsctk_gb300 import Context, synth

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    O.build()
    out = {"metric": "pipeline stage wall time", "unit": "s", "pipeline": args.pipeline, "data": "synthetic"}
    st = {}

    def timed(name, fn, ctx=None):
        fn()
        t0 = time.perf_counter()
        r = fn()
        st[name] = time.perf_counter() - t0
        if ctx is not None:
            st[name + "_stats"] = ctx.stats()
        return r

    with Context(0) as c:
        if args.pipeline in ("small", "scale"):
            n, k, nev = (2000, 50, 10) if args.pipeline == "small" else (100_000, 64, 20)
            ncv, tol = (0, 0.0) if args.pipeline == "small" else (60, 1e-8)
            x = synth.trajectory(n, 304, seed=SEED + 11, basins=1 if args.pipeline == "small" else 16,
                                 drift_sigma=0.05, dwell=500.0)
            m = np.ones(304, np.float32)
            out["config"] = {"workload": f"knn_rms {n} x 304, k={k}; make_sysparse; decomp_sparse nev={nev} "
                                         f"ncv={ncv or 'min(10 nev + 1, n)'} tol={tol}", "precision": args.precision}
            d, i = timed("knn_rms", lambda: c.knn_rms(x, None, m, k, precision=args.precision), c)
            sigma = float(np.median(d))
            nn, pcol, irow, val = timed("make_sysparse", lambda: c.sysparse(d, i))
            w, V, res, nconv = timed("decomp_sparse",
                                     lambda: c.decomp_sparse(nn, pcol, irow, val, sigma, nev, ncv=ncv, tol=tol), c)
            st["nconv"] = nconv
            st["max_residual"] = float(np.max(res))
            st["pairs_per_s"] = n * n / st["knn_rms"]
            if args.pipeline == "small":
                od, oi = O.knn_rms(x, None, m, k)
                st["parity_knn_max_abs_err_A"] = float(np.max(np.abs(d - od)))
                st["parity_knn_index_agreement"] = float(np.mean(i == oi))
                on, op, oir, ov = O.sysparse(d, i)
                st["parity_sysparse_bit_exact"] = bool(np.array_equal(pcol, op) and np.array_equal(irow, oir)
                                                       and np.array_equal(val, ov))
                M = O.dense_affinity(nn, pcol, irow, val, sigma)
                ex = np.linalg.eigvalsh(M)[::-1][:nev]
                st["parity_evals_max_rel_err"] = float(np.max(np.abs(w - ex) / np.abs(ex)))
            if args.pipeline_cpu:
                t0 = time.perf_counter()
                O.sysparse(d, i)
                st["cpu_make_sysparse"] = time.perf_counter() - t0
                t0 = time.perf_counter()
                wo, Vo, reso = O.decomp_sparse(nn, pcol, irow, val, sigma, nev, ncv=ncv or None, tol=tol)
                st["cpu_decomp_sparse_eigsh"] = time.perf_counter() - t0
                # parity of the eigenpairs against ARPACK (scipy eigsh, same ncv/tol)
                st["parity_evals_max_rel_err_vs_eigsh"] = float(np.max(np.abs(w - wo) / np.abs(wo)))
                Qg = np.linalg.qr(np.asarray(V).T)[0]
                Qo = np.linalg.qr(np.asarray(Vo).T)[0]
                sv = np.linalg.svd(Qg.T @ Qo, compute_uv=False)
                st["parity_subspace_min_cos_vs_eigsh"] = float(np.min(sv))
                # Eigenvectors are determined only up to rotations inside a
                # cluster of near-equal eigenvalues: with residuals near tol,
                # a vector's error is about tol / gap. So (a) every GPU pair
                # is checked as an eigenpair of the same operator (the
                # oracle's sp_dsymv on the oracle's affinity), and (b) the
                # eigenvalues are grouped where neighbours lie within
                # 1e-4 (relative) of each other; each group separated by more
                # than that from the rest, the (nev+1)-th eigenvalue included
                # (from a GPU run for nev+1), is compared as a subspace with
                # eigsh's vectors of the same group.
                A_o, _ = O.affinity(nn, pcol, irow, val, sigma)
                Vg = np.asarray(V)
                st["parity_gpu_pair_max_residual"] = float(max(
                    np.linalg.norm(O.sp_dsymv(nn, pcol, irow, A_o, Vg[x]) - w[x] * Vg[x]) / abs(w[x])
                    for x in range(nev)))
                w1, _, _, _ = c.decomp_sparse(nn, pcol, irow, val, sigma, nev + 1, ncv=ncv, tol=tol)
                st["gap_nev_to_next"] = float(w1[nev - 1] - w1[nev])
                gtol = 1e-4
                groups, cur = [], [0]
                for x in range(1, nev):
                    if abs(w[x - 1] - w[x]) <= gtol * max(1.0, abs(w[x])):
                        cur.append(x)
                    else:
                        groups.append(cur)
                        cur = [x]
                groups.append(cur)
                Vo_ = np.asarray(Vo)
                res_g, open_g = [], 0
                for g in groups:
                    if abs(w[g[-1]] - w1[nev]) <= gtol * max(1.0, abs(w[g[-1]])):
                        open_g += len(g)  # the group continues past the nev-th eigenvalue
                        continue
                    Qg = np.linalg.qr(Vg[g].T)[0]
                    Qo = np.linalg.qr(Vo_[g].T)[0]
                    res_g.append(float(np.linalg.norm(Qg - Qo @ (Qo.T @ Qg), 2)))
                # eigenvalue 1 of the normalised affinity has one copy per
                # connected component of the neighbour graph: a Krylov solver
                # (ARPACK as much as this one) need not return them all
                from scipy.sparse import csc_matrix
                from scipy.sparse.csgraph import connected_components
                G = csc_matrix((np.ones(len(irow)), np.asarray(irow), np.asarray(pcol)), shape=(nn, nn))
                st["graph_components"] = int(connected_components(G, directed=False)[0])
                st["eigenvalue_1_copies_gpu"] = int(np.sum(np.abs(w - 1.0) < 1e-12))
                st["eigenvalue_1_copies_eigsh"] = int(np.sum(np.abs(np.asarray(wo) - 1.0) < 1e-12))
                st["parity_evec_groups"] = [len(g) for g in groups]
                st["parity_evec_group_max_residual_vs_eigsh"] = max(res_g) if res_g else None
                st["parity_evec_groups_checked"] = len(res_g)
                st["parity_evecs_in_groups_open_at_nev"] = open_g
                st["eigenvalues"] = [float(t) for t in w]
                gaps = [min(abs(wo[x] - wo[y]) for y in range(nev) if y != x) for x in range(nev)]
                errs = [float(np.max(np.abs(V[x] * np.sign(V[x] @ Vo[x]) - Vo[x])))
                        for x in range(nev) if gaps[x] > gtol]
                st["parity_evecs_max_abs_err_vs_eigsh_gapped"] = max(errs) if errs else None
                st["parity_evecs_gapped_count"] = len(errs)
                st["eigsh_max_residual"] = float(np.max(reso))
        elif args.pipeline == "sparse":
            n, na, k, eps = 20_000, 304, 32, 12.0
            x = synth.trajectory(n, na, seed=SEED + 17, basins=4, drift_sigma=0.05, dwell=500.0)
            g1 = np.arange(0, na // 2, dtype=np.int32)
            g2 = np.arange(na // 2, na, dtype=np.int32)
            out["config"] = {"workload": f"contact_profile {n} x {na} (groups {len(g1)} x {len(g2)}, eps {eps} A) "
                                         f"-> knn_data_sparse k={k}"}
            off, idx = timed("contact_profile", lambda: c.contact_profile(x, g1, g2, eps))
            st["contacts_per_frame"] = float(off[-1]) / n
            vecs = (off, idx, np.ones(len(idx), np.float64))
            d, i = timed("knn_data_sparse", lambda: c.knn_data_sparse(vecs, None, k), c)
            st["pairs_per_s"] = n * n / st["knn_data_sparse"]
            rows = np.linspace(0, n - 1, 64).astype(int)
            ooff, oidx = O.contact_profile(x[:200], g1, g2, eps)
            st["parity_contacts_frames_checked"] = 200
            st["parity_contacts_identical"] = bool(np.array_equal(ooff, off[:201] - off[0])
                                                   and np.array_equal(oidx, idx[:off[200]]))
            fit = (np.concatenate([[0], np.cumsum(off[rows + 1] - off[rows])]).astype(np.int64),
                   np.concatenate([idx[off[r]:off[r + 1]] for r in rows]).astype(np.int32),
                   np.ones(int(np.sum(off[rows + 1] - off[rows])), np.float64))
            t0 = time.perf_counter()
            od, oi = O.knn_data_sparse(vecs, fit, k)  # each sampled row finds itself at position 0, dropped
            st["cpu_oracle_knn_data_sparse_64_rows_s"] = time.perf_counter() - t0
            st["parity_rows_checked"] = len(rows)
            st["parity_bit_exact_distances"] = bool(np.array_equal(d[rows], od))
        else:
            n, dim, k = args.vectors, 64, 32
            x = synth.dihedral_vectors(n, dim, seed=SEED + 13).astype(np.float64)
            out["config"] = {"workload": f"knn_data {n} x {dim} (f64), k={k}", "precision": args.precision}
            d, i = timed("knn_data", lambda: c.knn_data(x, None, k, precision=args.precision), c)
            st["pairs_per_s"] = n * n / st["knn_data"]
            rows = np.linspace(0, n - 1, 256).astype(int)
            od, oi = O.knn_data(x, x[rows], k)
            st["parity_rows_checked"] = len(rows)
            st["parity_bit_exact_distances"] = bool(np.array_equal(d[rows], od))
            # the same set under the correlation metric (knn_data -c)
            d, i = timed("knn_data_correlation",
                         lambda: c.knn_data(x, None, k, correlation=True, precision=args.precision), c)
            st["correlation_pairs_per_s"] = n * n / st["knn_data_correlation"]
            od, oi = O.knn_data(x, x[rows], k, correlation=True)
            st["correlation_parity_bit_exact_distances"] = bool(np.array_equal(d[rows], od))
    out["stages"] = st
    print(json.dumps(out))
    return 0


# DRAM bytes (read + write) of one k_screen_tc screen launch (the second of
# the call; the first is the pivot pass, 0.27 + 0.03 GB) on the default workload
# (20,000 x 1,000 atoms, k = 100, bf16x3), from one ncu capture of
# dram__bytes_read.sum + dram__bytes_write.sum (a 1-pass metric pair) with
# the command `ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum
# --clock-control none -k regex:<the five kernels below> -s 24 -c 8 --csv python bench.py --steps 2 --warmup 3 --no-cpu` (regex
# "k_prep_sums|k_prep_out|k_screen_tc|k_recheck|k_tc_split"). Other
# workloads report null.
SCREEN_TRAFFIC_BYTES = 5.540e9 + 0.077e9


def screen_traffic(args):
    if (args.frames, args.atoms, args.k, args.precision) == (N_FRAMES, N_ATOMS, K, "bf16x3"):
        return SCREEN_TRAFFIC_BYTES
    return None


def workload(frames, atoms):
    from mdsctk_gb300 import synth

    return synth.trajectory(frames, atoms, seed=SEED, drift_sigma=0.08, basins=8, dwell=500.0)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def wait_first(self, timeout=10.0):
        """Block until nvidia-smi has produced its first sample, so that its
        start-up (NVML initialisation) falls before the timed region."""
        t0 = time.time()
        while self.proc is not None and not self.lines and time.time() - t0 < timeout:
            time.sleep(0.05)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        sm.sort()
        med = sm[len(sm) // 2] if sm else None
        return {"sm_mhz": med, "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def cpu_sample(x, rows, k, threads):
    """Time the restated reference loop on `rows` fit rows vs all frames."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import numpy as np
    import oracle as O

    O.build()
    m = np.ones(x.shape[1], np.float32)
    t0 = time.perf_counter()
    O.knn_rms_port(x, x[:rows], m, k, threads=threads)
    dt = time.perf_counter() - t0
    return rows * x.shape[0] / dt, dt


def bench_config(args, n, a, k, world, replicas):
    """The workload description both arms print (identical dicts)."""
    return {"workload": f"knn_rms all-pairs N={n} A={a} k={k}", "frames": n, "atoms": a, "k": k,
            "basins": 8, "drift_nm": 0.08,
            "l2": "inputs (240 MB of frames) larger than L2 every step",
            "parallelism": (f"replicas x{world}" if replicas else f"row shards x{world}")}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    x = workload(args.frames, args.atoms)
    threads = os.cpu_count() or 1
    rows = args.cpu_rows or 2 * threads
    vals = []
    for _ in range(args.warmup):
        cpu_sample(x, threads, args.k, threads)
    for _ in range(args.steps):
        v, dt = cpu_sample(x, rows, args.k, threads)
        vals.append(v)
    v = sorted(vals)[len(vals) // 2]
    sample = f"{rows} fit rows x {args.frames} reference frames x {args.atoms} atoms per step"
    out = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "fp32/fp64", "data": "synthetic",
           "config": bench_config(args, args.frames, args.atoms, args.k, args.gpus, args.replicas),
           "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                            "sample": sample},
           "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))
    return 0


TOL_A = 1e-4  # 1e-5 nm in the output's Angstrom units


def parity_rows(x, rows, k):
    """GPU rows against the FP64 oracle (outside every timed region). The
    oracle gives k+1 columns so that a swap at the k-th position can be
    recognised as a tie with the (k+1)-th."""
    import numpy as np

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    O.build()
    m = np.ones(x.shape[1], np.float32)
    t0 = time.perf_counter()
    od1, oi1 = O.knn_rms(x, x[rows], m, k + 1)
    dt = time.perf_counter() - t0
    return od1, oi1, dt


def parity_summary(d, i, od1, oi1, k):
    import numpy as np

    od, oi = od1[:, :k], oi1[:, :k]
    err = float(np.max(np.abs(d - od)))
    swaps, bad = 0, 0
    for r, c in np.argwhere(i != oi):
        v = od[r, c]
        near = np.abs(od1[r] - v) <= 2 * TOL_A
        if abs(d[r, c] - v) <= TOL_A and near.sum() >= 2:
            swaps += 1
        else:
            bad += 1
    return {"rows": int(d.shape[0]), "max_abs_err_A": err, "tolerance_A": TOL_A,
            "index_agreement": float(np.mean(i == oi)), "tie_swaps": swaps, "index_errors": bad,
            "ok": bool(err <= TOL_A and bad == 0)}


FP32_NOMINAL_TFLOPS = 152 * 128 * 2 * 2.07e9 / 1e12  # 152 SMs x 128 FP32 lanes x FMA x 2.07 GHz


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.serve:
        return run_serve(args)
    if args.precision_report:
        return run_precision_report(args)
    if args.pipeline:
        return run_pipeline(args)
    import numpy as np
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    from mdsctk_gb300 import Context
    from mdsctk_gb300.shard import row_range

    x = workload(args.frames, args.atoms)
    n, a, k = x.shape[0], x.shape[1], args.k
    # N > 1: each rank computes a contiguous block of fit rows against every
    # reference frame (the row sharding of the kNN stage, no collective on the
    # data path; total work fixed = strong scaling); --replicas runs the whole
    # workload on every rank instead (weak scaling)
    replicas = args.replicas or world == 1
    r0, r1 = (0, n) if replicas else row_range(n, rank, world)
    ctx = Context(local)
    dev = torch.device("cuda", local)
    xd = torch.from_numpy(x).to(dev)
    fitd = None if (r0, r1) == (0, n) else xd[r0:r1]
    md = torch.ones(a, dtype=torch.float32, device=dev)
    kk = min(k, n - 1)
    nrow = r1 - r0
    out = (torch.empty((nrow, kk), dtype=torch.float64, device=dev),
           torch.empty((nrow, kk), dtype=torch.int32, device=dev))
    # host side for e2e: pinned frames in, pinned k-NN lists out
    xh = torch.from_numpy(x).pin_memory()
    fith = None if fitd is None else xh[r0:r1]
    dh = torch.empty((nrow, kk), dtype=torch.float64).pin_memory()
    ih = torch.empty((nrow, kk), dtype=torch.int32).pin_memory()
    mh = np.ones(a, np.float32)

    def step_dev(precision=args.precision, skip=True):
        ctx.knn_rms(xd, fitd, md, k, precision=precision, out=out, skip=skip)

    def step_e2e():
        ctx.knn_rms(xh.numpy(), None if fith is None else fith.numpy(), mh, k, precision=args.precision,
                    out=(dh.numpy(), ih.numpy()))

    warm = max(args.warmup, 3)
    for _ in range(warm):
        step_dev()
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    sampler.wait_first()
    # identical steps back to back for ~2 s before the timed region, so the
    # clock record holds samples under this load (they count as warm-up)
    t_soak = time.perf_counter()
    soak = 0
    while time.perf_counter() - t_soak < 2.0:
        step_dev()
        soak += 1
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    stats = []
    for _ in range(args.steps):
        step_dev()
        stats.append(ctx.stats())
    ev1.record()
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / args.steps
    if world > 1:
        t = torch.tensor([ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        torch.distributed.barrier()
        ms = float(t.item())
    clocks = sampler.stop()
    clocks["window"] = "2 s of identical untimed steps immediately before the timed region, and the timed region"
    clocks["soak_steps"] = soak

    def med(key, st=None):
        v = sorted(s_[key] for s_ in (st or stats))
        return v[len(v) // 2]

    launches = sum(s_["launches"] for s_ in stats)
    flagged = max(s_["rows_flagged"] for s_ in stats)
    d_last, i_last = out[0].cpu().numpy(), out[1].cpu().numpy()
    # end to end through the C ABI with host buffers
    step_e2e()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step_e2e()
    e2e_ms = (time.perf_counter() - t0) * 1000.0 / args.steps
    if world > 1:
        t = torch.tensor([e2e_ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_ms = float(t.item())
    pairs_rank = float(nrow) * n
    pairs_all = pairs_rank * world if replicas else float(n) * n
    value = pairs_all / (ms / 1000.0)
    e2e = pairs_all / (e2e_ms / 1000.0)
    peaks, pk_kind = measured_peaks()
    scr = med("screen_ms")
    computed = float(med("screen_pairs")) or pairs_rank
    flops = 18.0 * a * computed
    achieved = flops / (scr / 1000.0) / 1e12
    peak = float(peaks.get("bf16_tflops", 1900.0))
    rc_ms = med("recheck_ms")
    rp = float(med("recheck_pairs"))
    Ap = (a + 63) // 64 * 64
    r_flops = 30.0 * a * rp  # per candidate and atom: d (3), D (3) and Q (9) FMAs
    r_bytes = 12.0 * a * rp + nrow * 12.0 * Ap
    res = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": warm, "ms_per_step": ms, "higher_is_better": True,
           "scaling": "weak" if replicas else "strong", "vs_baseline": None,
           "dtype": {"fp32": "fp32", "bf16x3": "bf16x3+fp32", "fp16x3": "fp16x3+fp32"}[args.precision],
           "data": "synthetic",
           "config": bench_config(args, n, a, k, world, replicas),
           "precision": args.precision,
           "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                        "frac": achieved / peak, "traffic": screen_traffic(args) if replicas else None,
                        "kernel": "screen", "kernel_ms": scr, "flops_per_launch": flops,
                        "pairs_computed": computed, "pairs_equivalent": pairs_rank,
                        "flops_equivalent": 18.0 * a * pairs_rank,
                        "peak_kind": f"{pk_kind} bf16 burst"},
           "roofline_recheck": {"bound": "fp32", "achieved": r_flops / (rc_ms / 1000.0) / 1e12,
                                "peak": FP32_NOMINAL_TFLOPS, "unit": "TFLOP/s",
                                "frac": r_flops / (rc_ms / 1000.0) / 1e12 / FP32_NOMINAL_TFLOPS,
                                "peak_kind": "nominal FP32 (152 SMs x 128 lanes x 2 x 2.07 GHz)",
                                "kernel": "recheck stage", "kernel_ms": rc_ms, "candidates": rp,
                                "candidates_per_row": rp / max(nrow, 1), "flops_per_launch": r_flops,
                                "bytes_per_launch": r_bytes, "l2_gbs": r_bytes / (rc_ms / 1000.0) / 1e9},
           "stages_ms": {"prep": med("prep_ms"), "screen": scr, "recheck": rc_ms, "call": med("total_ms")},
           "rows_flagged": flagged,
           "screen_guard": {"guard_coef": stats[-1]["guard_coef"],
                            "screen_err_max": max(s_["screen_err_max"] for s_ in stats),
                            "violations": max(s_["guard_violations"] for s_ in stats),
                            "rows_flagged_by_violation": max(s_["rows_audit_flagged"] for s_ in stats),
                            "pairs_audited_per_call": rp},
           "clocks": clocks,
           "gpu_launches": launches,
           "e2e": {"value": e2e, "unit": UNIT, "ms_per_step": e2e_ms,
                   "h2d_bytes_per_step": int(x.nbytes + a * 4),
                   "d2h_bytes_per_step": int(nrow * kk * 12)}}
    # Like-for-like screens on this workload: both dense (every tile), and
    # each as it runs by default (tensor-core with tile skipping, FP32 dense).
    cmp = {}
    if not args.no_compare:
        def screen_runs(precision, skip, reps):
            step_dev(precision, skip)
            sts = []
            for _ in range(reps):
                step_dev(precision, skip)
                sts.append(ctx.stats())
            return sts

        tcd = screen_runs(args.precision, False, 3)
        fpd = screen_runs("fp32", False, 1)
        fps = screen_runs("fp32", True, 3)
        d_fp32, i_fp32 = out[0].cpu().numpy(), out[1].cpu().numpy()
        cmp = {"tc_dense_screen_ms": med("screen_ms", tcd), "tc_dense_screen_pairs": med("screen_pairs", tcd),
               "fp32_dense_screen_ms": med("screen_ms", fpd), "fp32_dense_screen_pairs": med("screen_pairs", fpd),
               "tc_skip_screen_ms": scr, "tc_skip_screen_pairs": computed,
               "fp32_skip_screen_ms": med("screen_ms", fps), "fp32_skip_screen_pairs": med("screen_pairs", fps),
               "tc_vs_fp32_dense": med("screen_ms", fpd) / med("screen_ms", tcd),
               "tc_vs_fp32_skip": med("screen_ms", fps) / scr,
               "tc_call_ms": med("total_ms"), "fp32_call_ms": med("total_ms", fps),
               "tc_vs_fp32_call": med("total_ms", fps) / med("total_ms"),
               "note": "screen stage times by CUDA events (pivot pass included when skipping); dense = every "
                       "tile computed (MDS_NO_SKIP), skip = the default tile skipping of each screen; "
                       "*_pairs: frame pairs each screen computed"}
        res["tc_vs_fp32"] = cmp
    # parity of the timed run: sampled rows against the FP64 oracle
    if rank == 0 and not args.no_parity:
        rows = np.linspace(0, nrow - 1, min(args.parity_rows, nrow)).astype(int)
        od1, oi1, pdt = parity_rows(x, rows + r0, k)
        res["parity"] = parity_summary(d_last[rows], i_last[rows], od1, oi1, kk)
        res["parity"]["oracle"] = f"FP64 QCP restatement, {len(rows)} rows x {n} frames ({pdt:.1f} s)"
        if cmp:
            res["parity_fp32_path"] = parity_summary(d_fp32[rows], i_fp32[rows], od1, oi1, kk)
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        rows = args.cpu_rows or 16 * threads
        v, dt = cpu_sample(x, rows, k, threads)
        res["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                               "sample": f"{rows} fit rows x {n} reference frames ({dt:.1f} s)"}
    if rank == 0:
        print(json.dumps(res))
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
