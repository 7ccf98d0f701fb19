"""Hand-built known-answer inputs and seeded parity cases shared by the tests.

Expected values of the known-answer cases are derived by hand from the
reference's arithmetic (source/device.cu:154-201, :259-315, :381-431 and
source/cudaNcorr.cu:37-58, :118-157 of cudaNcorr): every anchor counts each
ordered (p2, p3) pair, so a triangle seen from all three vertices counts 6.
"""
import numpy as np

from cudancorr_gb300 import catalogs as C

EDGES_20 = np.array([0.0, 5.0, 10.0, 15.0, 20.0])  # nb = 4, r_max = 20


def flat(i, j, k, nb=4):
    """triCountsAll_ index of sorted bins i <= j <= k (source/device.cu:198)."""
    return k + j * nb + i * nb * nb


def pts(*rows):
    a = np.array([list(r) + ([1.0] if len(r) == 3 else []) for r in rows], dtype=np.float64)
    return a


def kat_345():
    """A 5-8-sqrt(89) triangle in a divisible box (L=100, cell 20, nc=5).
    AB^2 = 25 sits exactly on edge 5^2 and belongs to bin 1 (r^2 >= edge^2)."""
    p = pts((50, 50, 50), (53, 54, 50), (50, 50, 58))
    expect = {flat(1, 1, 1): 6.0}
    return dict(box=100.0, edges=EDGES_20, p=p, expect=expect, survey=False)


def kat_rmax_excluded():
    """Adds D at distance exactly r_max = 20 from A: r^2 < r_max^2 is strict,
    so D joins no triangle (BD is in range, but AD and CD are not)."""
    p = pts((50, 50, 50), (53, 54, 50), (50, 50, 58), (70, 50, 50))
    return dict(box=100.0, edges=EDGES_20, p=p, expect={flat(1, 1, 1): 6.0}, survey=False)


def kat_coincident():
    """A duplicate of A: the zero side fails r^2 > r_min^2 = 0, but the
    duplicate forms its own copy of the triangle with B and C."""
    p = pts((50, 50, 50), (53, 54, 50), (50, 50, 58), (50, 50, 50))
    return dict(box=100.0, edges=EDGES_20, p=p, expect={flat(1, 1, 1): 12.0}, survey=False)


def kat_collinear():
    """Collinear 5, 5, 10: sqrtf(25)+sqrtf(25) <= sqrtf(100) rejects it."""
    p = pts((10, 10, 10), (15, 10, 10), (20, 10, 10))
    return dict(box=100.0, edges=EDGES_20, p=p, expect={}, survey=False)


def kat_wrap():
    """3-4-5 triangle across the periodic x face: P and Q are 3 apart through
    the wrap. Bins (0, 0, 1); (0,0,1) is absent from the compacted output
    because mid[1] = 7.5 > mid[0] + mid[0] = 5."""
    p = pts((1, 50, 50), (98, 50, 50), (1, 54, 50))
    return dict(box=100.0, edges=EDGES_20, p=p, expect={flat(0, 0, 1): 6.0}, survey=False)


def kat_wrap_survey():
    """The same three points in survey mode: no wrap, so P-Q is never a pair;
    only P-R (4) is, and no triangle closes."""
    p = pts((1, 50, 50), (98, 50, 50), (1, 54, 50))
    return dict(box=100.0, edges=EDGES_20, p=p, expect={}, survey=True)


def kat_nondivisible():
    """L = 90 with cell 20: five cells, the last 10 wide. P (cell 0) and Q
    (cell 3) are 17 apart through the wrap but two cells apart, so neither
    sees the other; R (cell 4) sees both and counts the triangle in its two
    orders only: 2, not 6 (the reference's cell predicate)."""
    p = pts((2, 45, 45), (75, 45, 45), (85, 48, 45))
    return dict(box=90.0, edges=EDGES_20, p=p, expect={flat(1, 2, 3): 2.0}, survey=False)


KATS = [kat_345, kat_rmax_excluded, kat_coincident, kat_collinear, kat_wrap, kat_wrap_survey,
        kat_nondivisible]


def expected_hist(case):
    nb = len(case["edges"]) - 1
    h = np.zeros(nb ** 3)
    for k, v in case["expect"].items():
        h[k] = v
    return h


# ------------------------------------------------------------------ seeded parity cases
def small_box_uniform(seed=11, n=3000, box=300.0):
    return C.uniform_box(n, box, seed), box, C.linear_edges(30.0, 6)


def small_box_clustered(seed=12):
    """Neyman-Scott in a divisible box: L=400, r_max=100 (nc=4), 20 bins."""
    return C.neyman_scott(800, 10.0, 2.0, 400.0, seed), 400.0, C.linear_edges(100.0, 20)


def small_box_nondivisible(seed=13):
    """Neyman-Scott mock, L=1000, r_max=60 (17 cells, the last 40 wide)."""
    return C.neyman_scott(1500, 8.0, 1.5, 1000.0, seed), 1000.0, C.linear_edges(60.0, 12)


def small_box_tiny_grid(seed=14):
    """L=150 with r_max=100: two cells per axis, so every cell is visited
    twice with different images (the single-wrap rule at nc=2)."""
    return C.uniform_box(600, 150.0, seed), 150.0, C.linear_edges(100.0, 10)


def small_box_one_cell(seed=15):
    """L=80 with r_max=100: one cell, all 27 images of every point."""
    return C.uniform_box(60, 80.0, seed), 80.0, C.linear_edges(100.0, 5)


def small_survey(seed=16, nd=4000, nr=9000, weighted=False):
    """Survey wedge scaled down: D and R jointly shifted by prep_cat_survey,
    15 log bins in [5, 120)."""
    from oracle import oracle as O
    d = C.survey_wedge(nd, seed, weighted, ra_max_deg=20.0, dec_max_deg=15.0)
    r = C.survey_wedge(nr, seed + 1000, False, ra_max_deg=20.0, dec_max_deg=15.0)
    box, ori = O.prep_cat_survey(d, r)
    edges = O.logspace(5.0, 120.0, 16)
    return d, r, box, ori, edges


def fma_probe(seed=17, n_clusters=48):
    """Isolated triangles whose short side lands within a few ulps of a bin
    edge, chosen so that the contraction patterns of sqrSep disagree on its
    bin. Cluster i targets edge 2i+2, so its outcome is readable from the
    histogram alone: sorted bins (2i+1 or 2i+2, last, last).

    Double-precision coordinates (not float32), 4x4x3 clusters 60 apart in a
    240 box with r_max 20 (cells of 20, 12 per axis)."""
    from oracle import oracle as O
    rng = np.random.default_rng(seed)
    n_inner = 2 * n_clusters + 1
    edges = [0.0] + list(np.linspace(2.0, 12.0, n_inner)) + [20.0]
    edges = np.array(edges)
    rows = []
    centres = [(30.0 + 60.0 * i, 30.0 + 60.0 * j, 30.0 + 60.0 * k)
               for i in range(4) for j in range(4) for k in range(3)][:n_clusters]
    for ci, c in enumerate(centres):
        e = edges[2 * ci + 2]  # inner edge with two neighbours of its own
        target = e * e
        for _ in range(200000):
            a = np.array([c[0] + rng.random(), c[1] + rng.random(), c[2] + rng.random(), 1.0])
            u = rng.normal(size=3)
            u /= np.linalg.norm(u)
            b = a.copy()
            b[:3] = a[:3] + e * u
            cls = {O.sqr_sep(a, b, k) >= target for k in range(6)}
            if len(cls) > 1:
                break
        else:
            raise RuntimeError("no distinguishing pair found")
        # third vertex ~16 from both, off the AB line
        v = np.cross(u, rng.normal(size=3))
        v /= np.linalg.norm(v)
        m = (a[:3] + b[:3]) / 2.0
        cpt = np.append(m + np.sqrt(16.0 ** 2 - (e / 2.0) ** 2) * v, 1.0)
        rows += [a, b, cpt]
    return dict(box=240.0, edges=edges, p=np.array(rows), survey=False)


# ------------------------------------------------------------------ rppi (rp, pi) bin type
RPPI_EDGES = np.array([0.0, 5.0, 10.0, 15.0, 20.0])  # nb = 4, rpMax = 20
RPPI_NPI = 10  # unit pi bins 0..10, piMax = 10; box cells (20, 20, 10)


def rppi_flat(ip2, ip1, i3, i2, i1, nb=4, npi=RPPI_NPI):
    """getTriangleIndexRppi's flat index (source/device.cu:251)."""
    return ip2 + ip1 * npi + i3 * npi * npi + i2 * nb * npi * npi + i1 * nb * nb * npi * npi


def rppi_kat_tie():
    """Sides AB (rp^2 25, pi^2 4), AC (64, 1), BC (25, 1). AB and BC tie on
    rp^2, so the pi bins of the two shortest sides follow the reference's
    swap order: anchors A (both orders) and B (A then C) give pi bins (2, 1),
    the other three orderings (1, 2)."""
    p = pts((50, 50, 50), (53, 54, 52), (50, 58, 51))
    expect = {rppi_flat(1, 2, 1, 1, 1): 3.0, rppi_flat(2, 1, 1, 1, 1): 3.0}
    return dict(box=100.0, edges=RPPI_EDGES, npi=RPPI_NPI, p=p, expect=expect, overflow=0.0, survey=False)


def rppi_kat_pi_cut():
    """AB has pi^2 = 100 = piMax^2 exactly: pi^2 < piMax^2 is strict, so no
    ordering of ABC counts, although AC and BC are in range."""
    p = pts((50, 50, 45), (53, 54, 55), (50, 58, 50))
    return dict(box=100.0, edges=RPPI_EDGES, npi=RPPI_NPI, p=p, expect={}, overflow=0.0, survey=False)


def rppi_kat_pi_overflow():
    """AB has pi^2 = (10 - 2^-30)^2 < 100, whose FP32 square root rounds to
    10 = nPi. All sides fall in the last rp bin and AB sorts second, so every
    ordering's index is nb^3 * nPi^2: one past the histogram, where the
    reference writes out of bounds. All six go to the overflow counter."""
    t = np.deg2rad(70.0)
    p = pts((50.0, 50.0, 40.0), (66.0, 50.0, 50.0 - 2.0 ** -30),
            (50.0 + 15.5 * np.cos(t), 50.0 + 15.5 * np.sin(t), 49.5))
    return dict(box=100.0, edges=RPPI_EDGES, npi=RPPI_NPI, p=p, expect={}, overflow=6.0, survey=False)


RPPI_KATS = [rppi_kat_tie, rppi_kat_pi_cut, rppi_kat_pi_overflow]


def rppi_expected_hist(case):
    nb = len(case["edges"]) - 1
    h = np.zeros(nb ** 3 * case["npi"] ** 2)
    for k, v in case["expect"].items():
        h[k] = v
    return h


def rppi_small_box(seed=21, n=2500, box=200.0):
    """Uniform box, L = 200, rp edges 0..25 in 5 bins, 15 pi bins
    (cells 25 x 25 x 15: 8 x 8 x 14)."""
    return C.uniform_box(n, box, seed), box, C.linear_edges(25.0, 5), 15


def rppi_small_box_clustered(seed=22):
    """Neyman-Scott, L = 300, rp 12 log bins in [1, 30), 20 pi bins; the last
    z cell is 20 wide of 20 (divisible) and x cells 30 (divisible)."""
    from oracle import oracle as O
    return C.neyman_scott(300, 8.0, 2.0, 300.0, seed), 300.0, O.logspace(1.0, 30.0, 13), 20


def rppi_small_box_nondivisible(seed=23):
    """L = 100, rpMax = 30 (4 cells, the last 10 wide), 12 pi bins (9 cells,
    the last 4 wide)."""
    return C.uniform_box(1200, 100.0, seed), 100.0, C.linear_edges(30.0, 6), 12


def rppi_small_box_tiny_grid(seed=28):
    """L = 50, rpMax = 25 (two cells in x and y, so every x-y cell is visited
    as two images), 15 pi bins (4 cells, the last 5 wide)."""
    return C.uniform_box(300, 50.0, seed), 50.0, C.linear_edges(25.0, 5), 15


def rppi_small_box_one_cell(seed=29):
    """L = 20 below rpMax = 25 and piMax = 22: one cell per axis, so the 27
    slots are 27 images of every point."""
    return C.uniform_box(40, 20.0, seed), 20.0, C.linear_edges(25.0, 5), 22


def rppi_small_survey(seed=24, nd=1500, nr=3000, weighted=False):
    """Survey wedge scaled down, jointly shifted; rp 8 log bins in [2, 30),
    20 pi bins (cells of sqrtf(30^2 + 20^2))."""
    from oracle import oracle as O
    d = C.survey_wedge(nd, seed, weighted, ra_max_deg=12.0, dec_max_deg=10.0)
    r = C.survey_wedge(nr, seed + 1000, False, ra_max_deg=12.0, dec_max_deg=10.0)
    box, ori = O.prep_cat_survey(d, r)
    return d, r, box, ori, O.logspace(2.0, 30.0, 9), 20


def _probe_edges(n_clusters):
    """Inner edges 1..4 (two per cluster plus one), rpMax 6: small enough a
    histogram with 5 pi bins (nb^3 * 25 entries) for the oracle."""
    n_inner = 2 * n_clusters + 1
    return np.array([0.0] + list(np.linspace(1.0, 4.0, n_inner)) + [6.0])


def rppi_box_probe(seed=25, n_clusters=12):
    """Isolated box triangles whose side AB has rp^2 within a few ulps of a
    bin edge, chosen so that the three contraction candidates of sqrRpBox
    disagree on its bin (as fma_probe does for sqrSep). 5 pi bins; clusters
    60 apart in a 240 box (cells 6 x 6 x 5)."""
    from oracle import oracle as O
    rng = np.random.default_rng(seed)
    edges = _probe_edges(n_clusters)
    rows = []
    centres = [(30.0 + 60.0 * i, 30.0 + 60.0 * j, 30.0 + 60.0 * k)
               for i in range(4) for j in range(4) for k in range(3)][:n_clusters]
    for ci, c in enumerate(centres):
        e = edges[2 * ci + 2]
        target = e * e
        for _ in range(200000):
            a = np.array([c[0] + rng.random(), c[1] + rng.random(), c[2] + rng.random(), 1.0])
            phi = rng.random() * 2 * np.pi
            u = np.array([np.cos(phi), np.sin(phi), 0.0])
            b = a.copy()
            b[:3] = a[:3] + e * u
            b[2] = a[2] + rng.uniform(0.2, 0.9)
            if len({O.sqr_rp(a, b, k) >= target for k in range(3)}) > 1:
                break
        else:
            raise RuntimeError("no distinguishing pair found")
        v = np.array([-u[1], u[0], 0.0])
        m = (a[:3] + b[:3]) / 2.0
        cpt = np.append(m + np.sqrt(4.5 ** 2 - (e / 2.0) ** 2) * v + np.array([0.0, 0.0, 0.3]), 1.0)
        rows += [a, b, cpt]
    return dict(box=240.0, edges=edges, npi=5, p=np.array(rows), survey=False, ori=(0.0, 0.0, 0.0))


def rppi_survey_probe(seed=27, n_clusters=12):
    """Isolated survey triangles whose side AB has rp^2 = s^2 - pi^2 within a
    few ulps of a bin edge with pi^2 of the same size, chosen so that the six
    contraction candidates of dotProduct_d3 disagree on its bin. B is placed
    at A + e*u + p*n with u perpendicular to the line of sight n, so
    rp^2 ~ e^2 and pi^2 ~ p^2; n is re-derived from the final positions.
    5 pi bins, clusters 60 apart in a 240 box, ori.x = -700."""
    from oracle import oracle as O
    rng = np.random.default_rng(seed)
    edges = _probe_edges(n_clusters)
    ori = np.array([-700.0, -800.0, -900.0])
    rows = []
    centres = [(30.0 + 60.0 * i, 30.0 + 60.0 * j, 30.0 + 60.0 * k)
               for i in range(4) for j in range(4) for k in range(3)][:n_clusters]
    off = np.array([ori[0], 0.0, 0.0])
    for ci, c in enumerate(centres):
        e = edges[2 * ci + 2]
        target = e * e
        found = False
        for _ in range(20000):
            a = np.array([c[0] + rng.random(), c[1] + rng.random(), c[2] + rng.random(), 1.0])
            cpt = a.copy()
            cpt[:3] = a[:3] + rng.normal(size=3) * 1.5
            p = e * rng.uniform(0.8, 1.2)
            b = a.copy()
            u = None
            for _ in range(12):  # the line of sight moves with B: iterate to a fixed point
                los = (a[:3] - off) + (b[:3] - off) + (cpt[:3] - off)
                n = los / np.linalg.norm(los)
                if u is None:
                    u = np.cross(n, rng.normal(size=3))
                u = u - np.dot(u, n) * n
                u /= np.linalg.norm(u)
                b[:3] = a[:3] + e * u + p * n
            sides = [O.survey_rppi_sides(a, b, cpt, ori, dot_pattern=k) for k in range(6)]
            if len({s[0] >= target for s in sides}) > 1:
                s = sides[O.DOT_PATTERN]
                if all(0.0 < s[i] < 36.0 for i in range(3)) and all(s[3 + i] < 25.0 for i in range(3)):
                    found = True
                    break
        if not found:
            raise RuntimeError("no distinguishing triangle found")
        rows += [a, b, cpt]
    return dict(box=np.array([240.0, 240.0, 240.0]), edges=edges, npi=5, p=np.array(rows), survey=True,
                ori=tuple(ori))
