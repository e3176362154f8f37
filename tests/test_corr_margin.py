"""The correlation metric's tile bounds (knn_data, locality order) rest on
one inequality: for the reference's squared distance (1 - r)/2 of two
vectors (correlation_distance, mdsctk.cpp:337-360, single-pass sums) and
the FP32 standardised vectors z the screen works on,

    | (1 - r)/2 - |z_x - z_y|^2 / 4 |  <=  m,
    m = 0.5 max | |z|^2 - 1 |  +  1e-7 Dp  +  1e-6    (corr_margin)

where |z|^2 is the FP32 norm the split kernel sees and Dp the padded
dimension. The lower side lets a tile be skipped (dlo^2 / 4 - m above the
threshold), the upper side makes a threshold seed (a quarter of the
Euclidean seed plus m). Checked here on the CPU on every pair of sets
built to stress it: a large common offset (the single-pass standard
deviation loses digits, so the norms stray from 1), mixed scales, and a
plain Gaussian set."""
import numpy as np
import pytest


def _standardise(x):
    """k_vec_prep's correlation operand: sequential FP64 sums, the
    single-pass standard deviation, z = (x - mean) / (sd sqrt(dim - 1)) in
    FP64 rounded to FP32, and its FP32 squared norm."""
    n, dim = x.shape
    s = np.zeros(n)
    q = np.zeros(n)
    for i in range(dim):
        s = s + x[:, i]
        q = q + x[:, i] * x[:, i]
    d = float(dim)
    sd = np.sqrt((d * q - s * s) / (d * (d - 1.0)))
    mu = s / d
    inv = np.where(sd > 0, 1.0 / (sd * np.sqrt(d - 1.0)), 0.0)
    z = ((x - mu[:, None]) * inv[:, None]).astype(np.float32)
    nrm = np.zeros(n, np.float32)
    for i in range(dim):
        nrm = (nrm + z[:, i] * z[:, i]).astype(np.float32)
    return z, nrm, mu, sd


def _ref_d2(x, mu, sd):
    """(1 - r)/2 clamped at 0, as correlation_distance forms it before the
    square root: sequential sum of (a - ma)(b - mb) for every pair."""
    n, dim = x.shape
    c = x - mu[:, None]
    acc = np.zeros((n, n))
    for i in range(dim):
        acc = acc + c[:, i][:, None] * c[:, i][None, :]
    v = (1.0 - acc / ((dim - 1.0) * sd[:, None] * sd[None, :])) / 2.0
    return np.maximum(v, 0.0)


@pytest.mark.parametrize("case", ["offset", "scales", "gauss"])
def test_correlation_margin_brackets_reference(case):
    rng = np.random.default_rng({"offset": 1, "scales": 2, "gauss": 3}[case])
    n, dim = 300, 24
    if case == "offset":
        x = 1e4 + 0.01 * rng.normal(size=(n, dim))
    elif case == "scales":
        x = rng.normal(size=(n, dim)) * 10.0 ** rng.uniform(-3, 3, size=(n, 1)) + rng.normal(size=(n, 1)) * 50
    else:
        x = rng.normal(size=(n, dim))
    z, nrm, mu, sd = _standardise(x)
    dp = (dim + 31) // 32 * 32
    m = 0.5 * float(np.max(np.abs(nrm.astype(np.float64) - 1.0))) + 1e-7 * dp + 1e-6
    zd = z.astype(np.float64)
    e2 = np.sum((zd[:, None, :] - zd[None, :, :]) ** 2, axis=2) / 4.0
    d2 = _ref_d2(x, mu, sd)
    assert np.all(d2 >= e2 - m), float(np.max(e2 - m - d2))
    assert np.all(d2 <= e2 + m), float(np.max(d2 - e2 - m))
    if case == "offset":
        # the case the margin's first term exists for: norms well off 1
        assert np.max(np.abs(nrm - 1.0)) > 1e-6
