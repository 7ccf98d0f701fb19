"""The reference's own kernel on the GB300, against the oracle and the engine.

The reference's device code (source/device.cu of cudaNcorr) is compiled
unmodified into oracle/_ref/reference_device.cubin and launched by
oracle/ref_runner.cu with the reference's host flow. These tests pin the CPU
oracle to the reference (including the FMA contraction nvcc applied to its
sqrSep) and check the engine against the reference directly.
"""
import numpy as np
import pytest

from cudancorr_gb300 import catalogs as C
from tests import cases
from tests.test_gpu_parity import run_engine

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ref(oracle):
    if not oracle.REF_CUBIN.exists():
        pytest.skip("reference cubin not built (needs the reference sources)")
    oracle.runner()
    return oracle


def test_fma_pattern(ref):
    """Exactly one contraction pattern reproduces the reference kernel on
    inputs built to separate them, and it is the one the oracle and the
    engine's exact path use."""
    c = cases.fma_probe()
    h_ref, _, _ = ref.reference_count(c["box"], c["edges"], c["p"])
    matches = [k for k in range(6)
               if np.array_equal(ref.count_threeD(c["box"], c["edges"], c["p"], fma_pattern=k), h_ref)]
    assert matches == [ref.FMA_PATTERN]
    h, _, st = run_engine(c["box"], c["edges"], c["p"])
    assert np.array_equal(h, h_ref)
    assert st["n_exact_pairs"] > 0


@pytest.mark.parametrize("make", cases.KATS, ids=lambda f: f.__name__)
def test_reference_known_answers(ref, make):
    c = make()
    h, _, _ = ref.reference_count(c["box"], c["edges"], c["p"], survey=c["survey"])
    assert np.array_equal(h, cases.expected_hist(c))


@pytest.mark.parametrize("make", [cases.small_box_uniform, cases.small_box_clustered,
                                  cases.small_box_nondivisible, cases.small_box_tiny_grid,
                                  cases.small_box_one_cell], ids=lambda f: f.__name__)
def test_reference_box(ref, make):
    p, box, edges = make()
    h_ref, _, _ = ref.reference_count(box, edges, p)
    assert np.array_equal(ref.count_threeD(box, edges, p), h_ref)
    h, _, _ = run_engine(box, edges, p)
    assert np.array_equal(h, h_ref)


@pytest.mark.parametrize("combo", ["DDD", "DDR", "DRR", "RRR"])
def test_reference_survey(ref, combo):
    d, r, box, ori, edges = cases.small_survey(nd=2000, nr=4000)
    cat = {"D": d, "R": r}
    args = [cat[ch] for ch in combo]
    h_ref, _, _ = ref.reference_count(box, edges, *args, survey=True, ori=ori)
    assert np.array_equal(ref.count_threeD(box, edges, *args, survey=True), h_ref)
    h, _, _ = run_engine(box, edges, *args, survey=True, ori=ori)
    assert np.array_equal(h, h_ref)


def test_reference_survey_weighted(ref):
    d, r, box, ori, edges = cases.small_survey(nd=2000, nr=4000, weighted=True)
    h_ref, _, _ = ref.reference_count(box, edges, d, d, r, survey=True, ori=ori)
    h_o = ref.count_threeD(box, edges, d, d, r, survey=True)
    nz = h_o != 0
    assert np.array_equal(h_ref != 0, nz)
    assert np.max(np.abs(h_ref[nz] - h_o[nz]) / np.abs(h_o[nz])) < 1e-12
    h, _, _ = run_engine(box, edges, d, d, r, survey=True, ori=ori)
    assert np.max(np.abs(h[nz] - h_o[nz]) / np.abs(h_o[nz])) < 1e-6


def test_reference_full_size_anchor_subset(ref):
    """2,000,000-point clustered box at full size, 1,024 random anchors: the
    reference kernel and the engine agree bit for bit."""
    p, box, edges = C.config_box_clustered()
    rng = np.random.default_rng(99)
    sub = np.ascontiguousarray(p[rng.choice(len(p), 1024, replace=False)])
    h_ref, kms, _ = ref.reference_count(box, edges, sub, p, p)
    h, _, _ = run_engine(box, edges, sub, p, p)
    assert h_ref.sum() > 0
    assert np.array_equal(h, h_ref)
