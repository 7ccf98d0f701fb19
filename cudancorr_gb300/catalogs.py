"""Seeded synthetic catalogues (float32 positions, N x 4 float64 arrays).

The reference reads DESI/mock files that are not available and draws its
randoms with a time seed (source/utils.cu:41-52 of cudaNcorr); these
generators stand in for them with fixed seeds and the shapes, sizes and
distributions of the benchmark workloads. Positions are drawn in float64,
rounded to float32 (the catalogues are float32 xyz) and returned as float64
(x, y, z, w) rows, the layout of std::vector<double4>.
"""
from __future__ import annotations

import math

import numpy as np


def _pack(xyz: np.ndarray, w=None) -> np.ndarray:
    n = xyz.shape[0]
    out = np.empty((n, 4), dtype=np.float64)
    out[:, :3] = xyz.astype(np.float32).astype(np.float64)
    out[:, 3] = 1.0 if w is None else np.asarray(w, dtype=np.float32).astype(np.float64)
    return out


def _wrap(x: np.ndarray, box: float) -> np.ndarray:
    """Periodic wrap into [0, box) that stays inside after float32 rounding."""
    y = np.mod(x, box).astype(np.float32)
    y[y >= np.float32(box)] = 0.0
    y[y < 0] = 0.0
    return y.astype(np.float64)


def uniform_box(n: int, box: float, seed: int) -> np.ndarray:
    """n points uniform in [0, box)^3, unit weights."""
    rng = np.random.default_rng(seed)
    return _pack(_wrap(rng.random((n, 3)) * box, box))


def neyman_scott(n_parents: int, mean_children: float, sigma: float, box: float, seed: int) -> np.ndarray:
    """Neyman-Scott process: uniform parent centres, Poisson(mean) children
    each displaced by N(0, sigma^2) per axis, periodically wrapped. Only the
    children are returned."""
    rng = np.random.default_rng(seed)
    parents = rng.random((n_parents, 3)) * box
    k = rng.poisson(mean_children, n_parents)
    centres = np.repeat(parents, k, axis=0)
    pts = centres + rng.normal(0.0, sigma, centres.shape)
    return _pack(_wrap(pts, box))


def survey_wedge(n: int, seed: int, weighted: bool, ra_max_deg: float = 90.0, dec_max_deg: float = 60.0,
                 r_mean: float = 1000.0, r_sigma: float = 150.0, r_lo: float = 600.0,
                 r_hi: float = 1400.0, w_sigma: float = 0.3) -> np.ndarray:
    """Sky wedge: RA uniform in [0, ra_max), Dec uniform on the sphere in
    [0, dec_max), comoving distance Gaussian truncated to [r_lo, r_hi];
    xyz = r (cos d cos a, cos d sin a, sin d) (the formula of
    source/survey.cu:48-50). Weights lognormal(0, w_sigma) or 1."""
    rng = np.random.default_rng(seed)
    ra = rng.random(n) * math.radians(ra_max_deg)
    dec = np.arcsin(rng.random(n) * math.sin(math.radians(dec_max_deg)))
    r = np.empty(n)
    filled = 0
    while filled < n:
        draw = rng.normal(r_mean, r_sigma, 2 * (n - filled) + 16)
        draw = draw[(draw >= r_lo) & (draw <= r_hi)][: n - filled]
        r[filled:filled + draw.size] = draw
        filled += draw.size
    xyz = np.stack([r * np.cos(dec) * np.cos(ra), r * np.cos(dec) * np.sin(ra), r * np.sin(dec)], axis=1)
    w = rng.lognormal(0.0, w_sigma, n) if weighted else None
    return _pack(xyz, w)


def soneira_peebles(n_top: int, levels: int, eta: int, lam: float, radius: float, box: float,
                    seed: int) -> np.ndarray:
    """Soneira-Peebles hierarchy: n_top clumps uniform in the box; each clump
    of radius R places eta sub-centres uniformly in its sphere, with radius
    R/lam, for `levels` levels; the last level's centres are the points
    (n_top * eta**levels points), periodically wrapped."""
    rng = np.random.default_rng(seed)
    centres = rng.random((n_top, 3)) * box
    r = radius
    for _ in range(levels):
        m = centres.shape[0]
        # uniform in a ball of radius r
        d = rng.normal(size=(m * eta, 3))
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        d *= (r * rng.random(m * eta) ** (1.0 / 3.0))[:, None]
        centres = np.repeat(centres, eta, axis=0) + d
        r /= lam
    return _pack(_wrap(centres, box))


def linear_edges(r_max: float, n_bins: int) -> np.ndarray:
    """n_bins linear bins on [0, r_max): edges i * r_max / n_bins."""
    return np.array([i * (r_max / n_bins) for i in range(n_bins + 1)], dtype=np.float64)


# Workload definitions of the benchmark configurations.
def config_box_uniform(seed: int = 1):
    """20,000 uniform points, L=1000, 10 linear bins on [0, 50)."""
    return uniform_box(20000, 1000.0, seed), 1000.0, linear_edges(50.0, 10)


def config_box_clustered(seed: int = 2, n_parents: int = 200000):
    """Neyman-Scott, 200,000 parents x Poisson(10), sigma 2, L=2000,
    20 linear bins on [0, 100)."""
    return neyman_scott(n_parents, 10.0, 2.0, 2000.0, seed), 2000.0, linear_edges(100.0, 20)


def config_soneira_peebles(seed: int = 5, n_top: int = 3906):
    """Soneira-Peebles, 5 levels, eta=4, lambda=1.9, top radius 200,
    3906 top clumps (~4M points), L=1500, 16 linear bins on [0, 80)."""
    return soneira_peebles(n_top, 5, 4, 1.9, 200.0, 1500.0, seed), 1500.0, linear_edges(80.0, 16)


def batch_mock_sizes(seed: int = 4, n_mocks: int = 64, n_min: int = 50_000, n_max: int = 1_000_000):
    """Target sizes of the batched mocks: log-uniform in [n_min, n_max]."""
    rng = np.random.default_rng(seed)
    return np.exp(rng.uniform(np.log(n_min), np.log(n_max), n_mocks))


def batch_mock(i: int, size: float, seed: int = 4) -> np.ndarray:
    """Mock i of the batch: N/8 parents x Poisson(8), sigma 1.5, L=1000."""
    return neyman_scott(max(1, int(round(size / 8.0))), 8.0, 1.5, 1000.0, seed * 1000 + i)


def config_batch_mocks(seed: int = 4, n_mocks: int = 64, n_min: int = 50_000, n_max: int = 1_000_000):
    """64 Neyman-Scott mocks in L=1000 with sizes log-uniform in
    [50,000, 1,000,000]: N/8 parents, Poisson(8) children, sigma 1.5;
    r_max=60 (17 cells, the last 40 wide), 12 linear bins."""
    sizes = batch_mock_sizes(seed, n_mocks, n_min, n_max)
    mocks = [batch_mock(i, s, seed) for i, s in enumerate(sizes)]
    return mocks, 1000.0, linear_edges(60.0, 12)


def config_survey(seed: int = 7):
    """Survey wedge: data 500,000 points with lognormal(0, 0.3) weights and
    randoms 2,500,000 points with unit weights, RA 0-90 deg, Dec 0-60 deg,
    r ~ N(1000, 150) in [600, 1400], jointly shifted by prep_cat_survey
    (source/survey.cu:106-128); 15 log bins in [5, 120).
    Returns (data, randoms, box, ori, edges)."""
    from . import api
    d = survey_wedge(500_000, seed, True)
    r = survey_wedge(2_500_000, seed + 1, False)
    box, ori = api.prep_cat_survey(d, r)
    return d, r, box, ori, api.logspace(5.0, 120.0, 16)


def training_soneira_peebles(index: int):
    """Training catalogue `index` of the scheduler's work model: the 4M-point
    Soneira-Peebles process at the same clump density in L=600 (250 top
    clumps, 256,000 points), r_max=80, 16 linear bins."""
    return soneira_peebles(250, 5, 4, 1.9, 200.0, 600.0, 100 + index), 600.0, linear_edges(80.0, 16)
