"""Row-sharded kNN host logic on CPU: two gloo ranks each compute a block
of rows (the oracle stands in for the GPU call) and rank 0's gathered result
equals the single-process result, in row order, for knn_rms and knn_data."""
import os
import socket

import numpy as np
import pytest


def test_row_range_partitions():
    from mdsctk_gb300.shard import row_range

    for n in (0, 1, 7, 100, 101):
        for world in (1, 2, 3, 8):
            spans = [row_range(n, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
            sizes = [b - a for a, b in spans]
            assert max(sizes) - min(sizes) <= 1


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, outdir):
    import sys

    here = os.path.dirname(os.path.abspath(__file__))
    for p in (os.path.dirname(here), os.path.join(os.path.dirname(here), "oracle")):
        sys.path.insert(0, p)
    import torch.distributed as dist

    import oracle as O
    from mdsctk_gb300 import synth
    from mdsctk_gb300.shard import knn_sharded

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    x = synth.trajectory(90, 24, seed=3, basins=2, dwell=20)
    m = synth.uniform_masses(24)
    r1 = knn_sharded(lambda ref, fit, k: O.knn_rms(ref, fit, m, k), x, None, 7)
    v = synth.dihedral_vectors(75, 6, seed=4).astype(np.float64)
    q = synth.dihedral_vectors(33, 6, seed=5).astype(np.float64)
    r2 = knn_sharded(lambda ref, fit, k: O.knn_data(ref, fit, k), v, q, 5)
    if rank == 0:
        np.savez(os.path.join(outdir, "sharded.npz"), d1=r1[0], i1=r1[1], d2=r2[0], i2=r2[1])
    else:
        assert r1 is None and r2 is None
    dist.barrier()
    dist.destroy_process_group()


def test_knn_sharded_gloo_two_ranks(tmp_path, oracle):
    import torch.multiprocessing as mp

    from mdsctk_gb300 import synth

    mp.spawn(_rank_main, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    got = np.load(tmp_path / "sharded.npz")
    x = synth.trajectory(90, 24, seed=3, basins=2, dwell=20)
    m = synth.uniform_masses(24)
    d1, i1 = oracle.knn_rms(x, None, m, 7)
    assert np.array_equal(got["d1"], d1) and np.array_equal(got["i1"], i1)
    v = synth.dihedral_vectors(75, 6, seed=4).astype(np.float64)
    q = synth.dihedral_vectors(33, 6, seed=5).astype(np.float64)
    d2, i2 = oracle.knn_data(v, q, 5)
    assert np.array_equal(got["d2"], d2) and np.array_equal(got["i2"], i2)
