"""The drop-in tools end to end on the GPU, file for file against the
oracle: knn_data -> make_sysparse -> decomp_sparse on the reference's rings
example, knn_rms on a synthetic trajectory with a PDB topology, and the
Nystrom pipeline (make_gesparse + decomp_sparse_nystrom)."""
import os
import subprocess

import numpy as np
import pytest

from mdsctk_gb300 import synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")


def _run(build, tmp, name, *args):
    r = subprocess.run([os.path.join(build.BINDIR, name), *args], cwd=tmp, capture_output=True, text=True)
    assert r.returncode == 0, (name, r.stdout, r.stderr)
    return r.stdout


def _read_csc(path):
    b = open(path, "rb").read()
    n = np.frombuffer(b[:4], np.int32)[0]
    pcol = np.frombuffer(b[4:4 + 4 * (n + 1)], np.int32)
    nnz = pcol[-1]
    o = 4 + 4 * (n + 1)
    irow = np.frombuffer(b[o:o + 4 * nnz], np.int32)
    val = np.frombuffer(b[o + 4 * nnz:o + 12 * nnz], np.float64)
    return n, pcol, irow, val


@pytest.mark.gpu
def test_cluster_data_pipeline(ctx, oracle, tmp_path):
    from mdsctk_gb300 import build

    build.build()
    x = np.fromfile(os.path.join(GOLD, "rings.pts"), np.float64).reshape(-1, 2)
    x.tofile(tmp_path / "reference.pts")
    k = 20
    _run(build, tmp_path, "knn_data", "-k", str(k), "-v", "2", "-r", "reference.pts")
    d = np.fromfile(tmp_path / "distances.dat", np.float64).reshape(-1, k)
    i = np.fromfile(tmp_path / "indices.dat", np.int32).reshape(-1, k)
    od, oi = oracle.knn_data(x, None, k)
    assert np.array_equal(d, od)
    _run(build, tmp_path, "make_sysparse", "-k", str(k), "-n", "10")
    n, pcol, irow, val = _read_csc(tmp_path / "distances.ssm")
    on, op, oir, ov = oracle.sysparse(od, oi, 10)
    assert n == on and np.array_equal(pcol, op) and np.array_equal(irow, oir) and np.array_equal(val, ov)
    out = _run(build, tmp_path, "decomp_sparse", "-q", "0.5", "-n", "4", "--binary-out")
    assert "Number of converged eigenvalues/vectors found: 4" in out
    w = np.fromfile(tmp_path / "eigenvalues.dat", np.float64)
    V = np.fromfile(tmp_path / "eigenvectors.dat", np.float64).reshape(4, n)
    wo, Vo, _ = oracle.decomp_sparse(on, op, oir, ov, 0.5, 4)
    assert np.allclose(w, wo, rtol=1e-6, atol=1e-9)
    # text mode writes the same values with six significant digits
    _run(build, tmp_path, "decomp_sparse", "-q", "0.5", "-n", "4")
    wt = np.loadtxt(tmp_path / "eigenvalues.dat")
    assert np.allclose(wt, wo, rtol=1e-5)
    lines = open(tmp_path / "eigenvectors.dat").read().splitlines()
    assert len(lines) == 4 and lines[0].endswith(" ")


@pytest.mark.gpu
def test_knn_rms_tool_with_pdb(ctx, oracle, tmp_path):
    from mdsctk_gb300 import build

    build.build()
    natoms = 30
    x = synth.trajectory(120, natoms, seed=4)
    names = ["N", "CA", "C"] * (natoms // 3)
    with open(tmp_path / "topology.pdb", "w") as f:
        for a, nm in enumerate(names):
            f.write("ATOM  %5d %-4s ALA A%4d    %8.3f%8.3f%8.3f  1.00  0.00\n" % (a + 1, nm, a // 3 + 1, 0, 0, 0))
    x.tofile(tmp_path / "traj.crd")
    _run(build, tmp_path, "knn_rms", "-k", "8", "-p", "topology.pdb", "-r", "traj.crd")
    d = np.fromfile(tmp_path / "distances.dat", np.float64).reshape(-1, 8)
    m = np.array([14.0067 if nm == "N" else 12.011 for nm in names], np.float32)
    od, oi = oracle.knn_rms(x, None, m, 8)
    assert np.max(np.abs(d - od)) < 1e-4


@pytest.mark.gpu
def test_nystrom_tools(ctx, oracle, tmp_path):
    from mdsctk_gb300 import build

    build.build()
    rng = np.random.default_rng(3)
    land = np.concatenate([rng.normal(size=(150, 2)), rng.normal(size=(150, 2)) + 5])
    qry = np.concatenate([rng.normal(size=(40, 2)), rng.normal(size=(40, 2)) + 5])
    land.tofile(tmp_path / "land.pts")
    qry.tofile(tmp_path / "query.pts")
    _run(build, tmp_path, "knn_data", "-k", "10", "-v", "2", "-r", "land.pts")
    _run(build, tmp_path, "make_sysparse", "-k", "10")
    _run(build, tmp_path, "knn_data", "-k", "10", "-v", "2", "-r", "land.pts", "-f", "query.pts",
         "-d", "qd.dat", "-i", "qi.dat")
    _run(build, tmp_path, "make_gesparse", "-k", "10", "-d", "qd.dat", "-i", "qi.dat")
    m, pb, ib, vb = _read_csc(tmp_path / "distances.gsm")
    dq, iq = oracle.knn_data(land, qry, 10)
    om, opb, oib, ovb = oracle.gesparse(dq, iq)
    assert m == om and np.array_equal(pb, opb) and np.array_equal(ib, oib) and np.array_equal(vb, ovb)
    _run(build, tmp_path, "decomp_sparse_nystrom", "-q", "1.0", "-n", "3", "--binary-out")
    V = np.fromfile(tmp_path / "eigenvectors.dat", np.float64).reshape(3, 300 + 80)
    assert np.all(np.isfinite(V))


@pytest.mark.gpu
def test_auto_decomp_tools(ctx, oracle, tmp_path):
    from mdsctk_gb300 import build

    build.build()
    x = np.fromfile(os.path.join(GOLD, "rings.pts"), np.float64).reshape(-1, 2)
    x.tofile(tmp_path / "reference.pts")
    _run(build, tmp_path, "knn_data", "-k", "20", "-v", "2", "-r", "reference.pts")
    _run(build, tmp_path, "make_sysparse", "-k", "20", "-n", "12")
    n, pcol, irow, val = _read_csc(tmp_path / "distances.ssm")
    out = _run(build, tmp_path, "auto_decomp_sparse", "-k", "10", "-K", "6", "-n", "4", "--binary-out")
    assert "Average sigma:" in out and "Maximum residual:" in out
    w = np.fromfile(tmp_path / "eigenvalues.dat", np.float64)
    wo, _, _, osig = oracle.auto_decomp_sparse(n, pcol, irow, val, 10, 4, perplexity=6.0)
    assert np.allclose(w, wo, rtol=1e-6, atol=1e-9)
    avg = float(out.split("Average sigma:")[1].split()[0])
    assert abs(avg - osig.mean()) <= 1e-5 * osig.mean()
    r = subprocess.run([os.path.join(build.BINDIR, "auto_decomp_sparse"), "-k", "3", "-K", "6", "-n", "4"],
                       cwd=tmp_path, capture_output=True, text=True)
    assert "WARNING: --k-perplexity (6) is higher than --k-sigma (3)" in r.stdout
