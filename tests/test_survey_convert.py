"""survey::convert_coordinates (source/survey.cu:17-57 of cudaNcorr) on CPU.

The reference integrates 1/E(z) with GSL's qags to 1e-7 relative; GSL is not
in this image, so the engine's own quadrature is checked here against
independent FP64 integrals: composite Simpson with 1e5 panels in numpy, and
the closed forms of the Einstein-de Sitter (OmegaM = 1) and pure-Lambda
(OmegaLambda = 1) cosmologies. The RA/Dec -> xyz formula of
source/survey.cu:48-50 is checked on fixed points.
"""
import math
import threading

import numpy as np
import pytest

from cudancorr_gb300 import api

C_OVER_100 = 299792.458 / 100.0


def simpson_distance(z: float, om: float, ol: float, panels: int = 100_000) -> float:
    x = np.linspace(0.0, z, 2 * panels + 1)
    f = 1.0 / np.sqrt(om * (1.0 + x) ** 3 + ol)
    h = z / (2 * panels)
    return C_OVER_100 * h / 3.0 * (f[0] + f[-1] + 4.0 * f[1:-1:2].sum() + 2.0 * f[2:-1:2].sum())


def distances(z, om, ol):
    """Comoving distances of redshifts z through the C ABI (RA = Dec = 0, so
    x is the distance itself)."""
    z = np.asarray(z, dtype=np.float64)
    cat = np.zeros((z.size, 4))
    cat[:, 2] = z
    cat[:, 3] = 1.0
    return api.convert_coordinates(cat, 67.7, om, ol)[:, 0]


@pytest.mark.parametrize("om,ol", [(0.3, 0.7), (0.315, 0.685), (0.25, 0.75), (0.5, 0.5), (1.0, 0.0)])
def test_distance_matches_simpson(om, ol):
    zs = np.array([1e-4, 0.01, 0.1, 0.35, 0.5, 0.8, 1.0, 1.5, 2.0, 2.5, 3.0])
    got = distances(zs, om, ol)
    for z, d in zip(zs, got):
        ref = simpson_distance(float(z), om, ol)
        assert abs(d - ref) <= 1e-9 * ref, (z, d, ref)


def test_distance_closed_forms():
    zs = np.array([0.05, 0.5, 1.0, 3.0, 10.0, 1000.0])
    eds = distances(zs, 1.0, 0.0)
    assert np.allclose(eds, C_OVER_100 * 2.0 * (1.0 - 1.0 / np.sqrt(1.0 + zs)), rtol=1e-12, atol=0)
    lam = distances(zs, 0.0, 1.0)
    assert np.allclose(lam, C_OVER_100 * zs, rtol=1e-12, atol=0)


def test_distance_edge_values():
    d = distances([0.0, -0.2, -1.0, np.nan, np.inf], 0.3, 0.7)
    assert d[0] == 0.0
    # qags from 0 to a negative z gives the negative integral (Simpson with a
    # negative step is the same signed integral)
    assert d[1] < 0
    assert abs(d[1] - simpson_distance(-0.2, 0.3, 0.7)) <= 1e-9 * abs(d[1])
    assert np.isnan(d[2]) and np.isnan(d[3]) and np.isnan(d[4])


def test_ra_dec_formula():
    """x = d cos(dec) cos(ra), y = d cos(dec) sin(ra), z = d sin(dec), weight
    carried (source/survey.cu:43-53)."""
    ra = np.array([0.0, 90.0, 180.0, 45.0, 300.0, 12.5])
    dec = np.array([0.0, 0.0, 30.0, 60.0, -45.0, 89.0])
    z = np.array([0.5, 0.5, 1.0, 0.2, 2.0, 0.7])
    w = np.array([1.0, 2.0, 0.5, 3.25, 1.0, 0.75])
    cat = np.stack([ra, dec, z, w], axis=1)
    out = api.convert_coordinates(cat, 67.7, 0.3, 0.7)
    d = np.array([simpson_distance(float(zz), 0.3, 0.7) for zz in z])
    a, b = np.radians(ra), np.radians(dec)
    want = np.stack([d * np.cos(b) * np.cos(a), d * np.cos(b) * np.sin(a), d * np.sin(b)], axis=1)
    assert np.allclose(out[:, :3], want, rtol=1e-9, atol=1e-9 * d.max())
    assert np.array_equal(out[:, 3], w)
    # on the axes the formula is exact up to the distance itself
    assert out[1, 1] == pytest.approx(d[1], rel=1e-9) and abs(out[1, 0]) < 1e-9 * d[1]
    assert math.hypot(*out[3, :3]) == pytest.approx(d[3], rel=1e-12)


def test_concurrent_conversions_agree():
    """Threads converting at once share the quadrature rule, built once on
    first use; every thread gets the single-threaded result."""
    rng = np.random.default_rng(3)
    cat = np.stack([rng.uniform(0, 360, 2000), rng.uniform(-90, 90, 2000), rng.uniform(0, 3, 2000),
                    np.ones(2000)], axis=1)
    want = api.convert_coordinates(cat, 67.7, 0.31, 0.69)
    results = [None] * 8

    def work(i):
        results[i] = api.convert_coordinates(cat, 67.7, 0.31, 0.69)

    threads = [threading.Thread(target=work, args=(i,)) for i in range(8)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    for r in results:
        assert np.array_equal(r, want)
