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
