"""GPU .xtc decoding (mds_xtc_decode) against the oracle's decoder, bit for
bit: the reference's example trajectory, synthetic frames that reach the
format's other paths, a malformed frame, and knn_rms on .xtc input through
the drop-in tool (atom-count mismatch exits with status 4)."""
import os
import subprocess

import numpy as np
import pytest

import xtc_synth as X

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.gpu
def test_xtc_trp_cage_bit_exact(ctx, oracle):
    b = open(os.path.join(GOLD, "trp-cage.xtc"), "rb").read()
    xyz, steps, times = ctx.xtc_read(b)
    oxyz, osteps, otimes = oracle.xtc_read(b)
    assert xyz.shape == (1000, 60, 3)
    assert np.array_equal(xyz, oxyz) and np.array_equal(steps, osteps) and np.array_equal(times, otimes)
    dxyz, _, _ = ctx.xtc_read(b, device_out=True)
    assert np.array_equal(dxyz.cpu().numpy(), oxyz)


@pytest.mark.gpu
def test_xtc_synthetic_paths(ctx, oracle):
    groups = [(2, 0, True), (2, 0, False), (3, 1, True), (1, -1, True), (5, 0, True), (5, 0, False),
              (0, -1, True), (4, 0, True)]
    groups += [(0, 0, True)] * (60 - sum(g[0] + 1 for g in groups))
    frames = [X.encode_frame(X.walk(60, s), prec=1000.0, step=s, groups=groups) for s in range(3)]
    q = X.walk(60, 9, step=3)
    q[7] += 30_000_000
    frames.append(X.encode_frame(q, prec=1e6, step=3))
    b = b"".join(frames)
    xyz, steps, _ = ctx.xtc_read(b)
    oxyz, osteps, _ = oracle.xtc_read(b)
    assert np.array_equal(xyz, oxyz) and steps.tolist() == [0, 1, 2, 3]
    small = X.encode_frame(X.walk(5, 4))
    xyz, _, _ = ctx.xtc_read(small * 3)
    assert np.array_equal(xyz, oracle.xtc_read(small * 3)[0])


@pytest.mark.gpu
def test_xtc_malformed_frame_is_an_error(ctx):
    from mdsctk_gb300 import MdsError

    f = bytearray(X.encode_frame(X.walk(60, 5), prec=1000.0))
    f[84:88] = (80).to_bytes(4, "big")  # small index outside the table
    with pytest.raises(MdsError):
        ctx.xtc_read(bytes(f))
    # a truncated last frame is dropped, as a reader stops there
    g = X.encode_frame(X.walk(60, 6), prec=1000.0)
    xyz, _, _ = ctx.xtc_read(g + g[:-8])
    assert xyz.shape[0] == 1


@pytest.mark.gpu
def test_knn_rms_tool_on_xtc(ctx, oracle, tmp_path):
    from mdsctk_gb300 import build

    build.build()
    tool = os.path.join(build.BINDIR, "knn_rms")
    for f in ("trp-cage.xtc", "trp-cage.pdb"):
        (tmp_path / f).write_bytes(open(os.path.join(GOLD, f), "rb").read())
    r = subprocess.run([tool, "-k", "10", "-p", "trp-cage.pdb", "-r", "trp-cage.xtc"], cwd=tmp_path,
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    d = np.fromfile(tmp_path / "distances.dat", np.float64).reshape(-1, 10)
    i = np.fromfile(tmp_path / "indices.dat", np.int32).reshape(-1, 10)
    x, _, _ = oracle.xtc_read(os.path.join(GOLD, "trp-cage.xtc"))
    m = np.array([14.0067 if j % 3 == 0 else 12.011 for j in range(60)], np.float32)
    od, oi = oracle.knn_rms(x, None, m, 10)
    assert d.shape == (1000, 10)
    assert np.max(np.abs(d - od)) < 1e-4
    assert np.mean(i == oi) > 0.999
    # topology with a different atom count: exit status 4
    pdb = open(os.path.join(GOLD, "trp-cage.pdb")).read().splitlines()
    atoms = [ln for ln in pdb if ln.startswith("ATOM")][:-3]
    (tmp_path / "short.pdb").write_text("\n".join(atoms) + "\n")
    r = subprocess.run([tool, "-k", "10", "-p", "short.pdb", "-r", "trp-cage.xtc"], cwd=tmp_path,
                       capture_output=True, text=True)
    assert r.returncode == 4 and "does not match the number of atoms" in r.stdout
