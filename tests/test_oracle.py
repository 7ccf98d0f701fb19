"""CPU checks of the oracle: known answers, internal consistency, fixtures.

The oracle is the checker of every GPU parity test, so it is pinned here:
against hand-derived answers, against its own literal loop nest (the
reference's loop structure), and against outputs of the reference's kernel
recorded in tests/golden/ (generated on a GB300 by tests/golden/make_golden.py).
"""
import json
import pathlib

import numpy as np
import pytest

from tests import cases

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden"


@pytest.mark.parametrize("make", cases.KATS, ids=lambda f: f.__name__)
def test_known_answers(oracle, make):
    c = make()
    h = oracle.count_threeD(c["box"], c["edges"], c["p"], survey=c["survey"])
    assert np.array_equal(h, cases.expected_hist(c))
    h_lit = oracle.count_threeD(c["box"], c["edges"], c["p"], survey=c["survey"], literal=True)
    assert np.array_equal(h_lit, h)


@pytest.mark.parametrize("make", [cases.small_box_uniform, cases.small_box_clustered,
                                  cases.small_box_nondivisible, cases.small_box_tiny_grid,
                                  cases.small_box_one_cell], ids=lambda f: f.__name__)
def test_list_form_equals_literal_loops(oracle, make):
    p, box, edges = make()
    p = p[:1500]
    h_lit = oracle.count_threeD(box, edges, p, literal=True)
    h = oracle.count_threeD(box, edges, p)
    assert np.array_equal(h, h_lit)
    assert h.sum() > 0


def test_ddr_list_form_equals_literal(oracle):
    d, r, box, ori, edges = cases.small_survey(nd=600, nr=1500)
    for args in [(d, d, r), (d, r, r), (r, d, r)]:
        h_lit = oracle.count_threeD(box, edges, *args, survey=True, literal=True)
        h = oracle.count_threeD(box, edges, *args, survey=True)
        assert np.array_equal(h, h_lit)


def test_unweighted_counts_are_integers_and_symmetric(oracle):
    p, box, edges = cases.small_box_clustered()
    h = oracle.count_threeD(box, edges, p[:2000])
    assert np.all(h == np.round(h))
    nb = len(edges) - 1
    idx = np.nonzero(h)[0]
    i, j, k = idx // (nb * nb), (idx // nb) % nb, idx % nb
    assert np.all((i <= j) & (j <= k))  # only sorted bin triples are filled


def test_divisible_box_counts_multiple_of_six(oracle):
    """In a divisible box with nc >= 4 every triangle is seen from all three
    vertices in both orders."""
    p, box, edges = cases.small_box_uniform()
    h = oracle.count_threeD(box, edges, p)
    assert np.all(np.mod(h, 6) == 0)


def test_anchor_linearity(oracle):
    """Counts are additive over a partition of the anchor catalogue."""
    p, box, edges = cases.small_box_nondivisible()
    p = p[:2500]
    h = oracle.count_threeD(box, edges, p, p, p)
    a, b = p[:1000], p[1000:]
    ha = oracle.count_threeD(box, edges, a, p, p)
    hb = oracle.count_threeD(box, edges, b, p, p)
    assert np.array_equal(h, ha + hb)


def test_compaction_matches_reference_rule(oracle):
    edges = np.array([0.0, 5.0, 10.0, 15.0, 20.0])
    nb = 4
    h = np.arange(nb ** 3, dtype=np.float64)
    c, b = oracle.compact(edges, h)
    mids = (edges[1:] + edges[:-1]) / 2.0
    exp_c, exp_b = [], []
    for i in range(nb):
        for j in range(i, nb):
            for k in range(j, nb):
                if mids[k] <= mids[i] + mids[j]:
                    exp_c.append(h[k + j * nb + i * nb * nb])
                    exp_b.append((mids[i], mids[j], mids[k]))
    assert np.array_equal(c, exp_c)
    assert np.array_equal(b, np.array(exp_b))


def test_logspace_and_survey_prep(oracle):
    e = oracle.logspace(5.0, 120.0, 16)
    assert e[0] == pytest.approx(5.0) and e[-1] == pytest.approx(120.0)
    assert np.all(np.diff(e) > 0)
    rng = np.random.default_rng(3)
    c1 = rng.random((50, 4)) * 100 - 20
    c2 = rng.random((70, 4)) * 100 - 40
    m = np.minimum(c1[:, :3].min(0), c2[:, :3].min(0))
    mx = np.maximum(c1[:, :3].max(0), c2[:, :3].max(0))
    a1, a2 = c1.copy(), c2.copy()
    box, ori = oracle.prep_cat_survey(a1, a2)
    assert np.array_equal(box, mx - m + 1.0)
    assert np.array_equal(ori, -m)
    assert np.array_equal(a1[:, :3], c1[:, :3] - m)
    assert np.array_equal(a1[:, 3], c1[:, 3])


def test_fma_patterns_differ_on_adversarial_pairs(oracle):
    """The contraction patterns of sqrSep are distinguishable: on generic
    double inputs they disagree in the last bits."""
    rng = np.random.default_rng(5)
    diffs = 0
    for _ in range(200):
        a = np.append(rng.random(3) * 10, 1.0)
        b = np.append(rng.random(3) * 10, 1.0)
        vals = {oracle.sqr_sep(a, b, k) for k in range(6)}
        diffs += len(vals) > 1
    assert diffs > 20


def _golden_files():
    return sorted(p for p in GOLDEN.glob("*.json") if not p.name.startswith("rppi_"))


@pytest.mark.parametrize("path", _golden_files(), ids=lambda p: p.stem)
def test_oracle_matches_reference_golden(oracle, path):
    """Outputs of the reference's own kernel, recorded on a GB300."""
    g = json.loads(path.read_text())
    arrays = np.load(path.with_suffix(".npz"))
    cats = {k: arrays[k] for k in arrays.files if k.startswith("cat")}
    roles = [cats[name] for name in g["roles"]]
    h = oracle.count_threeD(g["box"], np.array(g["edges"]), *roles, survey=g["survey"])
    ref = arrays["hist"]
    if g["weighted"]:
        scale = np.maximum(np.abs(ref), 1e-300)
        assert np.max(np.abs(h - ref) / scale) < 1e-12
    else:
        assert np.array_equal(h, ref)
