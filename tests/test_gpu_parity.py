"""GPU parity: the engine, called through the C ABI, against the CPU oracle.

Unweighted counts must be bit-identical; weighted bins within 1e-6 relative
of the oracle's compensated FP64 sums (the precision stated for weighted
survey bins).
"""
import numpy as np
import pytest

from cudancorr_gb300 import api
from cudancorr_gb300 import catalogs as C
from tests import cases

pytestmark = pytest.mark.gpu

WEIGHTED_RTOL = 1e-6


def run_engine(box, edges, p1, p2=None, p3=None, survey=False, ori=(0.0, 0.0, 0.0)):
    p2 = p1 if p2 is None else p2
    p3 = p2 if p3 is None else p3
    b = np.broadcast_to(np.asarray(box, dtype=np.float64), (3,))
    with api.ncorr(b, api.threeD, edges, survey, ori) as corr:
        corr.calculateD1D2D3(p1, p2, p3)
        return corr.getTriCountsAll(), corr.getTriCountsOut(), corr.stats()


@pytest.mark.parametrize("make", cases.KATS, ids=lambda f: f.__name__)
def test_known_answers(engine_lib, make):
    c = make()
    h, _, _ = run_engine(c["box"], c["edges"], c["p"], survey=c["survey"])
    assert np.array_equal(h, cases.expected_hist(c))


@pytest.mark.parametrize("make", [cases.small_box_uniform, cases.small_box_clustered,
                                  cases.small_box_nondivisible, cases.small_box_tiny_grid,
                                  cases.small_box_one_cell], ids=lambda f: f.__name__)
def test_box_parity(engine_lib, oracle, make):
    p, box, edges = make()
    h, out, st = run_engine(box, edges, p)
    ref = oracle.count_threeD(box, edges, p)
    assert np.array_equal(h, ref)
    ref_out, _ = oracle.compact(edges, ref)
    assert np.array_equal(out, ref_out)
    assert st["triangles"] == ref.sum()


def test_box_uniform_20k(engine_lib, oracle):
    """20,000 uniform points, L=1000, 10 bins on [0, 50): full parity."""
    p, box, edges = C.config_box_uniform()
    h, out, st = run_engine(box, edges, p)
    ref = oracle.count_threeD(box, edges, p)
    assert np.array_equal(h, ref)
    assert ref.sum() > 1e6 - 1e5


@pytest.mark.parametrize("make", [cases.small_box_clustered, cases.small_box_uniform,
                                  cases.small_box_nondivisible], ids=lambda f: f.__name__)
def test_symmetry_modes_agree(engine_lib, oracle, make):
    """The three loop forms give the same histogram bit for bit: all (j, l)
    (p3 a distinct copy), pairs j<l x2 (p1 a distinct copy), and -- where the
    geometry allows it -- i<j<l x6 (one catalogue for all three)."""
    p, box, edges = make()
    h6, _, st6 = run_engine(box, edges, p, p, p)
    h2, _, st2 = run_engine(box, edges, p.copy(), p, p)
    h1, _, st1 = run_engine(box, edges, p, p, p.copy())
    assert st2["symmetric"] == 2 and st1["symmetric"] == 1
    divisible = make is not cases.small_box_nondivisible
    assert st6["symmetric"] == (6 if divisible else 2)
    assert np.array_equal(h6, h2) and np.array_equal(h2, h1)
    assert np.array_equal(h6, oracle.count_threeD(box, edges, p))


def test_cross_catalogue_box(engine_lib, oracle):
    rng_a = C.uniform_box(2500, 300.0, 21)
    rng_b = C.neyman_scott(300, 6.0, 2.0, 300.0, 22)
    edges = C.linear_edges(40.0, 8)
    for args in [(rng_a, rng_b, rng_b), (rng_a, rng_a, rng_b), (rng_b, rng_a, rng_b)]:
        h, _, _ = run_engine(300.0, edges, *args)
        ref = oracle.count_threeD(300.0, edges, *args)
        assert np.array_equal(h, ref)


@pytest.mark.parametrize("combo", ["DDD", "DDR", "DRR", "RRR"])
def test_survey_unweighted(engine_lib, oracle, combo):
    d, r, box, ori, edges = cases.small_survey()
    cat = {"D": d, "R": r}
    args = [cat[c] for c in combo]
    h, _, _ = run_engine(box, edges, *args, survey=True, ori=ori)
    ref = oracle.count_threeD(box, edges, *args, survey=True)
    assert np.array_equal(h, ref)


@pytest.mark.parametrize("combo", ["DDD", "DDR", "DRR"])
def test_survey_weighted(engine_lib, oracle, combo):
    d, r, box, ori, edges = cases.small_survey(weighted=True)
    cat = {"D": d, "R": r}
    args = [cat[c] for c in combo]
    h, _, st = run_engine(box, edges, *args, survey=True, ori=ori)
    assert st["weighted"] == 1
    ref = oracle.count_threeD(box, edges, *args, survey=True)
    nz = ref != 0
    assert np.array_equal(h != 0, nz)
    rel = np.abs(h[nz] - ref[nz]) / np.abs(ref[nz])
    assert rel.max() < WEIGHTED_RTOL


def test_weighted_box_with_negative_weights(engine_lib, oracle):
    p, box, edges = cases.small_box_uniform(n=2000)
    rng = np.random.default_rng(9)
    p = p.copy()
    p[:, 3] = rng.normal(0.5, 1.0, len(p)).astype(np.float32)
    h, _, _ = run_engine(box, edges, p)
    ref = oracle.count_threeD(box, edges, p)
    # per-bin error relative to the bin's sum of |w1 w2 w3| scale
    scale = oracle.count_threeD(box, edges, np.abs(p))
    nz = scale != 0
    assert np.max(np.abs(h[nz] - ref[nz]) / scale[nz]) < WEIGHTED_RTOL


def test_many_bins_global_histogram(engine_lib, oracle):
    """Bin counts whose histogram does not fit in shared memory (63 bins
    unweighted, 40 weighted) take the global-histogram path."""
    p, box, edges = cases.small_box_uniform(n=2500)
    e63 = C.linear_edges(30.0, 63)
    h, _, _ = run_engine(box, e63, p)
    assert np.array_equal(h, oracle.count_threeD(box, e63, p))
    d, r, sbox, ori, _ = cases.small_survey(nd=1500, nr=3000, weighted=True)
    e40 = oracle.logspace(5.0, 120.0, 41)
    h, _, _ = run_engine(sbox, e40, d, d, r, survey=True, ori=ori)
    ref = oracle.count_threeD(sbox, e40, d, d, r, survey=True)
    nz = ref != 0
    assert np.array_equal(h != 0, nz)
    assert np.max(np.abs(h[nz] - ref[nz]) / np.abs(ref[nz])) < WEIGHTED_RTOL


def test_empty_and_single(engine_lib):
    edges = C.linear_edges(20.0, 4)
    one = cases.pts((5, 5, 5))
    empty = np.zeros((0, 4))
    h, out, _ = run_engine(100.0, edges, one)
    assert not h.any() and not out.any()
    h, _, _ = run_engine(100.0, edges, empty, one, one)
    assert not h.any()
    h, _, _ = run_engine(100.0, edges, one, empty, empty)
    assert not h.any()


def test_points_outside_grid_raise(engine_lib):
    edges = C.linear_edges(20.0, 4)
    for bad in [cases.pts((150, 5, 5)), cases.pts((-25, 5, 5)), cases.pts((np.nan, 5, 5))]:
        p = np.vstack([cases.pts((5, 5, 5)), bad])
        with pytest.raises(api.NcorrError) as e:
            run_engine(100.0, edges, p)
        assert e.value.code == api.NCORR_ERR_OUT_OF_GRID


def test_box_face_point_is_clamped(engine_lib, oracle):
    """x == L maps to cell nc (clamped to nc-1) as in the reference."""
    edges = C.linear_edges(20.0, 4)
    p = cases.pts((100, 50, 50), (97, 50, 50), (99, 54, 50), (3, 52, 50))
    h, _, _ = run_engine(100.0, edges, p)
    ref = oracle.count_threeD(100.0, edges, p)
    assert np.array_equal(h, ref) and ref.sum() > 0


def test_exact_queue_overflow_settles_in_place(engine_lib, oracle, monkeypatch):
    """With no room in the deferred exact queue every uncertain candidate is
    settled inside the triangle kernel; results are unchanged."""
    c = cases.fma_probe()
    monkeypatch.setenv("NCORR_EXACT_QUEUE_CAP", "0")
    h0, _, st0 = run_engine(c["box"], c["edges"], c["p"])
    monkeypatch.setenv("NCORR_EXACT_QUEUE_CAP", "3")
    h3, _, _ = run_engine(c["box"], c["edges"], c["p"])
    monkeypatch.delenv("NCORR_EXACT_QUEUE_CAP")
    h, _, _ = run_engine(c["box"], c["edges"], c["p"])
    ref = oracle.count_threeD(c["box"], c["edges"], c["p"])
    assert np.array_equal(h0, ref) and np.array_equal(h3, ref) and np.array_equal(h, ref)
    assert st0["n_exact_tris"] + st0["n_exact_pairs"] > 0


def test_repeatable(engine_lib):
    p, box, edges = cases.small_box_clustered()
    h1, _, _ = run_engine(box, edges, p)
    h2, _, _ = run_engine(box, edges, p)
    assert np.array_equal(h1, h2)


def test_device_entry_matches_host_entry(engine_lib):
    torch = pytest.importorskip("torch")
    p, box, edges = cases.small_box_nondivisible()
    b = np.full(3, box)
    with api.ncorr(b, api.threeD, edges, False, (0, 0, 0)) as corr:
        corr.calculateD1D2D3(p, p, p)
        h_host = corr.getTriCountsAll()
        t = torch.from_numpy(p).cuda()
        corr.calculateD1D2D3(t, t, t)
        h_dev = corr.getTriCountsAll()
    assert np.array_equal(h_host, h_dev)


def test_clustered_full_size_properties(engine_lib):
    """2,000,000-point Neyman-Scott box (L=2000, r_max=100, 20 bins) at full
    size: anchor linearity over a partition, the symmetric and asymmetric
    loops agree, and every count is a multiple of 6 (divisible box)."""
    p, box, edges = C.config_box_clustered()
    b = np.full(3, box)
    with api.ncorr(b, api.threeD, edges, False, (0, 0, 0)) as corr:
        corr.calculateD1D2D3(p, p, p)
        h = corr.getTriCountsAll()
        n = len(p) // 3
        a = np.ascontiguousarray(p[:n])
        rest = np.ascontiguousarray(p[n:])
        corr.calculateD1D2D3(a, p, p)
        ha = corr.getTriCountsAll()
        corr.calculateD1D2D3(rest, p, p)
        hb = corr.getTriCountsAll()
        corr.calculateD1D2D3(a, p, p.copy())
        ha_asym = corr.getTriCountsAll()
    assert np.array_equal(h, ha + hb)
    assert np.array_equal(ha, ha_asym)
    assert np.all(np.mod(h, 6) == 0)
    assert h.sum() > 5e11
