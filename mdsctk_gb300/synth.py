"""Seeded synthetic workloads with the shapes of the benchmark configurations.

No public trajectory set is used: every input is generated here from a seed.

* ``trajectory``: a self-avoiding random-walk chain (0.15 nm bonds) as the
  base structure; optional metastable basins (a seeded Markov chain with a
  mean dwell time picks the basin, each basin displaces the chain smoothly);
  per-atom Ornstein-Uhlenbeck conformational drift; a uniform random rigid
  rotation and a translation in [0, 5] nm per frame; coordinates quantised to
  0.001 nm (the XTC precision) and stored as float32 [n, natoms, 3] in nm.
* ``dihedral_vectors``: sin/cos of D/2 dihedral angles drawn from a seeded
  von Mises mixture, stored as float32 (exact in float64 for the .pts file).
"""
from __future__ import annotations

import numpy as np


def _saw_chain(natoms: int, rng: np.random.Generator, step: float = 0.15,
               min_dist: float = 0.12) -> np.ndarray:
    """Self-avoiding random walk: reject steps that come within min_dist."""
    pos = np.zeros((natoms, 3))
    for i in range(1, natoms):
        for _ in range(200):
            v = rng.normal(size=3)
            v *= step / np.linalg.norm(v)
            p = pos[i - 1] + v
            if i < 3 or np.min(np.sum((pos[: i - 1] - p) ** 2, axis=1)) >= min_dist ** 2:
                break
        pos[i] = p
    return pos - pos.mean(axis=0)


def _random_rotations(n: int, rng: np.random.Generator) -> np.ndarray:
    """Uniform random rotation matrices from normalised Gaussian quaternions."""
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    R = np.empty((n, 3, 3))
    R[:, 0, 0] = 1 - 2 * (y * y + z * z)
    R[:, 0, 1] = 2 * (x * y - z * w)
    R[:, 0, 2] = 2 * (x * z + y * w)
    R[:, 1, 0] = 2 * (x * y + z * w)
    R[:, 1, 1] = 1 - 2 * (x * x + z * z)
    R[:, 1, 2] = 2 * (y * z - x * w)
    R[:, 2, 0] = 2 * (x * z - y * w)
    R[:, 2, 1] = 2 * (y * z + x * w)
    R[:, 2, 2] = 1 - 2 * (x * x + y * y)
    return R


def trajectory(n: int, natoms: int, seed: int = 0, drift_sigma: float = 0.05,
               tau: float = 200.0, basins: int = 1, dwell: float = 500.0,
               basin_sigma: float = 0.25, off_manifold: float = 0.0,
               off_sigma: float = 0.3, base=None, rotate: bool = True,
               quantise: bool = True) -> np.ndarray:
    """Synthetic trajectory [n, natoms, 3] float32 in nm (see module doc)."""
    rng = np.random.default_rng(seed)
    base_rng = np.random.default_rng(10_000 + natoms) if base is None else None
    chain = _saw_chain(natoms, base_rng) if base is None else np.asarray(base, np.float64)
    # Basin offsets: smooth displacement fields along the chain.
    brng = np.random.default_rng(20_000 + natoms)
    offs = np.zeros((max(basins, 1), natoms, 3))
    if basins > 1:
        t = np.linspace(0, 1, natoms)[:, None]
        for b in range(basins):
            coef = brng.normal(size=(6, 3)) * basin_sigma
            field = np.zeros((natoms, 3))
            for h in range(6):
                field += np.sin((h + 1) * np.pi * t + brng.uniform(0, 2 * np.pi)) * coef[h]
            offs[b] = field
    # Basin sequence: leave the current basin with probability 1/dwell.
    state = np.zeros(n, np.int64)
    if basins > 1:
        s = int(rng.integers(basins))
        switch = rng.random(n) < 1.0 / dwell
        nxt = rng.integers(basins, size=n)
        for f in range(n):
            if switch[f]:
                s = int(nxt[f])
            state[f] = s
    # Per-atom Ornstein-Uhlenbeck drift, stationary variance drift_sigma^2.
    a = np.exp(-1.0 / tau)
    b = drift_sigma * np.sqrt(1.0 - a * a)
    x = np.zeros((n, natoms, 3))
    cur = rng.normal(size=(natoms, 3)) * drift_sigma
    noise = rng.normal(size=(n, natoms, 3))
    for f in range(n):
        cur = a * cur + b * noise[f]
        x[f] = cur
    x += chain[None] + offs[state]
    if off_manifold > 0:
        sel = rng.random(n) < off_manifold
        x[sel] += rng.normal(size=(int(sel.sum()), natoms, 3)) * off_sigma
    if rotate:
        R = _random_rotations(n, rng)
        x = np.einsum("fij,faj->fai", R, x)
        x += rng.uniform(0, 5, size=(n, 1, 3))
    if quantise:
        x = np.round(x * 1000.0) / 1000.0
    return x.astype(np.float32)


def dihedral_vectors(n: int, dim: int = 64, components: int = 12, seed: int = 0) -> np.ndarray:
    """sin/cos of dim/2 dihedrals from a seeded von Mises mixture, float32 [n, dim]."""
    rng = np.random.default_rng(seed)
    nang = dim // 2
    mus = rng.uniform(-np.pi, np.pi, size=(components, nang))
    kappas = rng.uniform(2.0, 20.0, size=(components, nang))
    weights = rng.dirichlet(np.ones(components))
    comp = rng.choice(components, size=n, p=weights)
    ang = rng.vonmises(mus[comp], kappas[comp])
    out = np.empty((n, dim), np.float32)
    out[:, 0::2] = np.sin(ang)
    out[:, 1::2] = np.cos(ang)
    return out


def uniform_masses(natoms: int) -> np.ndarray:
    return np.ones(natoms, np.float32)
