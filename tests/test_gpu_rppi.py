"""GPU parity of the rppi bin type: the engine, called through the C ABI,
against the CPU oracle and against the reference's own rppi kernels.

Unweighted counts (and the count of triangles indexed past the histogram)
must be bit-identical; weighted sums, which the engine and the reference
both add with FP64 atomics in an arbitrary order, within 1e-12 relative of
the oracle's compensated sums.
"""
import numpy as np
import pytest

from cudancorr_gb300 import api
from tests import cases

pytestmark = pytest.mark.gpu

WEIGHTED_RTOL = 1e-12


def run_rppi(box, edges, npi, p1, p2=None, p3=None, survey=False, ori=(0.0, 0.0, 0.0)):
    p2 = p1 if p2 is None else p2
    p3 = p2 if p3 is None else p3
    b = np.broadcast_to(np.asarray(box, dtype=np.float64), (3,))
    with api.ncorr(b, api.rppi, edges, int(npi), survey, ori) as corr:
        corr.calculateD1D2D3(p1, p2, p3)
        return (corr.getTriCountsAll(), corr.stats(), corr.getTriCountsOut(), corr.getTriBinsOut(),
                corr.getPiBinsOut())


def assert_weighted_close(h, ref):
    nz = ref != 0
    assert np.array_equal(h != 0, nz)
    assert np.max(np.abs(h[nz] - ref[nz]) / np.abs(ref[nz])) < WEIGHTED_RTOL


@pytest.mark.parametrize("make", cases.RPPI_KATS, ids=lambda f: f.__name__)
def test_rppi_known_answers(engine_lib, make):
    c = make()
    h, st, _, _, _ = run_rppi(c["box"], c["edges"], c["npi"], c["p"])
    assert np.array_equal(h, cases.rppi_expected_hist(c))
    assert st["overflow"] == c["overflow"]


@pytest.mark.parametrize("make", [cases.rppi_small_box, cases.rppi_small_box_clustered,
                                  cases.rppi_small_box_nondivisible, cases.rppi_small_box_tiny_grid,
                                  cases.rppi_small_box_one_cell], ids=lambda f: f.__name__)
def test_rppi_box_parity(engine_lib, oracle, make):
    p, box, edges, npi = make()
    h, st, out, bins, pis = run_rppi(box, edges, npi, p)
    ref, ov = oracle.count_rppi(box, edges, npi, p)
    assert np.array_equal(h, ref)
    assert st["overflow"] == ov
    assert st["triangles"] == ref.sum()
    c_out, b_out, p_out = oracle.compact_rppi(edges, npi, ref)
    assert np.array_equal(out, c_out) and np.array_equal(bins, b_out) and np.array_equal(pis, p_out)


def test_rppi_box_distinct_catalogues(engine_lib, oracle):
    """p2 != p3 (all ordered pairs) and p1 != p2 == p3 (pairs j < l, twice)."""
    p, box, edges, npi = cases.rppi_small_box(n=3000)
    a, b = p[:1500].copy(), p[1500:].copy()
    for args in [(a, b, b), (a, a, b), (b, a, b)]:
        h, _, _, _, _ = run_rppi(box, edges, npi, *args)
        ref, _ = oracle.count_rppi(box, edges, npi, *args)
        assert np.array_equal(h, ref)


def test_rppi_empty_partner_catalogues(engine_lib, oracle):
    """Anchors with empty p2 and p3: every list is empty and nothing counts."""
    p, box, edges, npi = cases.rppi_small_box(n=500)
    empty = np.zeros((0, 4))
    h, st, _, _, _ = run_rppi(box, edges, npi, p, empty, empty)
    ref, _ = oracle.count_rppi(box, edges, npi, p, empty, empty)
    assert not ref.any() and np.array_equal(h, ref)
    assert st["overflow"] == 0 and st["n_pairs"] == 0


@pytest.mark.parametrize("combo", ["DDD", "DDR", "DRR", "RRR"])
def test_rppi_survey_parity(engine_lib, oracle, combo):
    d, r, box, ori, edges, npi = cases.rppi_small_survey()
    cat = {"D": d, "R": r}
    args = [cat[ch] for ch in combo]
    h, st, _, _, _ = run_rppi(box, edges, npi, *args, survey=True, ori=ori)
    ref, ov = oracle.count_rppi(box, edges, npi, *args, survey=True, ori=ori)
    assert np.array_equal(h, ref)
    assert st["overflow"] == ov
    assert ref.sum() > 0


def test_rppi_weighted(engine_lib, oracle):
    d, r, box, ori, edges, npi = cases.rppi_small_survey(weighted=True)
    h, _, _, _, _ = run_rppi(box, edges, npi, d, d, r, survey=True, ori=ori)
    ref, _ = oracle.count_rppi(box, edges, npi, d, d, r, survey=True, ori=ori)
    assert_weighted_close(h, ref)
    p, box, edges, npi = cases.rppi_small_box_clustered()
    q = p.copy()
    q[:, 3] = np.random.default_rng(3).lognormal(0.0, 0.3, len(q))
    h, _, _, _, _ = run_rppi(box, edges, npi, q)
    ref, _ = oracle.count_rppi(box, edges, npi, q)
    assert_weighted_close(h, ref)


def test_rppi_device_entry_matches_host(engine_lib):
    torch = pytest.importorskip("torch")
    p, box, edges, npi = cases.rppi_small_box_clustered()
    h_host, _, _, _, _ = run_rppi(box, edges, npi, p)
    t = torch.from_numpy(p).cuda()
    with api.ncorr(np.full(3, box), api.rppi, edges, npi, False, (0, 0, 0)) as corr:
        corr.calculateD1D2D3(t, t, t)
        assert np.array_equal(corr.getTriCountsAll(), h_host)


def test_rppi_out_of_grid_is_rejected(engine_lib):
    p = np.array([[10.0, 10.0, 10.0, 1.0], [250.0, 10.0, 10.0, 1.0]])
    with pytest.raises(api.NcorrError) as e:
        run_rppi(200.0, [0.0, 10.0, 20.0], 10, p)
    assert e.value.code == api.NCORR_ERR_OUT_OF_GRID


# ------------------------------------------------------------ against the reference's own kernels
@pytest.fixture(scope="module")
def ref(oracle):
    if not oracle.REF_CUBIN.exists():
        pytest.skip("reference cubin not built (needs the reference sources)")
    oracle.runner()
    return oracle


@pytest.mark.parametrize("make,key,n,default", [(cases.rppi_box_probe, "rp_pattern", 3, "RP_PATTERN"),
                                                (cases.rppi_survey_probe, "dot_pattern", 6, "DOT_PATTERN")],
                         ids=["box_rp", "survey_dot"])
def test_rppi_contraction_patterns(ref, make, key, n, default):
    """Exactly one contraction candidate reproduces the reference kernel on
    its probe, and it is the one the oracle and the engine use."""
    c = make()
    h_ref, ov_ref, _, _ = ref.reference_count_rppi(c["box"], c["edges"], c["npi"], c["p"], survey=c["survey"],
                                                   ori=c["ori"])
    matches = [k for k in range(n)
               if np.array_equal(ref.count_rppi(c["box"], c["edges"], c["npi"], c["p"], survey=c["survey"],
                                                ori=c["ori"], **{key: k})[0], h_ref)]
    assert matches == [getattr(ref, default)]
    h, _, _, _, _ = run_rppi(c["box"], c["edges"], c["npi"], c["p"], survey=c["survey"], ori=c["ori"])
    assert np.array_equal(h, h_ref)


@pytest.mark.parametrize("make", cases.RPPI_KATS, ids=lambda f: f.__name__)
def test_rppi_reference_known_answers(ref, make):
    """The reference kernel itself gives the hand-derived answers, including
    the triangles it writes past the end of its histogram."""
    c = make()
    h, ov, _, _ = ref.reference_count_rppi(c["box"], c["edges"], c["npi"], c["p"])
    assert np.array_equal(h, cases.rppi_expected_hist(c))
    assert ov == c["overflow"]


@pytest.mark.parametrize("make", [cases.rppi_small_box, cases.rppi_small_box_clustered,
                                  cases.rppi_small_box_nondivisible, cases.rppi_small_box_tiny_grid,
                                  cases.rppi_small_box_one_cell], ids=lambda f: f.__name__)
def test_rppi_reference_box(ref, make):
    p, box, edges, npi = make()
    h_ref, ov_ref, _, _ = ref.reference_count_rppi(box, edges, npi, p)
    h, st, _, _, _ = run_rppi(box, edges, npi, p)
    assert np.array_equal(h, h_ref) and st["overflow"] == ov_ref


@pytest.mark.parametrize("combo", ["DDD", "DDR", "DRR", "RRR"])
def test_rppi_reference_survey(ref, combo):
    d, r, box, ori, edges, npi = cases.rppi_small_survey()
    cat = {"D": d, "R": r}
    args = [cat[ch] for ch in combo]
    h_ref, ov_ref, _, _ = ref.reference_count_rppi(box, edges, npi, *args, survey=True, ori=ori)
    h, st, _, _, _ = run_rppi(box, edges, npi, *args, survey=True, ori=ori)
    assert np.array_equal(h, h_ref) and st["overflow"] == ov_ref


def test_rppi_reference_weighted(ref):
    d, r, box, ori, edges, npi = cases.rppi_small_survey(weighted=True)
    h_ref, _, _, _ = ref.reference_count_rppi(box, edges, npi, d, d, r, survey=True, ori=ori)
    h, _, _, _, _ = run_rppi(box, edges, npi, d, d, r, survey=True, ori=ori)
    assert_weighted_close(h, h_ref)
