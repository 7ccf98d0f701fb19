"""CPU checks of the oracle's rppi restatement (the reference's second bin
type): hand-derived answers, its literal loop nests against the list form,
the contraction probes, the output tables, and outputs of the reference's
own rppi kernels recorded in tests/golden/rppi_*.
"""
import json
import pathlib

import numpy as np
import pytest

from tests import cases

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden"
RPPI_GOLDEN = sorted(GOLDEN.glob("rppi_*.json"))


@pytest.mark.parametrize("make", cases.RPPI_KATS, ids=lambda f: f.__name__)
def test_rppi_known_answers(oracle, make):
    c = make()
    for literal in (False, True):
        h, ov = oracle.count_rppi(c["box"], c["edges"], c["npi"], c["p"], literal=literal)
        assert np.array_equal(h, cases.rppi_expected_hist(c))
        assert ov == c["overflow"]


def test_rppi_index_follows_the_reference_swap_order(oracle):
    """Equal rp^2 on the first two sides: no swap, so pi bins keep the input
    order (source/device.cu:215-229)."""
    e = cases.RPPI_EDGES
    a = oracle.rppi_index(25.0, 25.0, 64.0, 4.0, 1.0, 1.0, e, 10)
    b = oracle.rppi_index(25.0, 25.0, 64.0, 1.0, 4.0, 1.0, e, 10)
    assert a == cases.rppi_flat(1, 2, 1, 1, 1) and b == cases.rppi_flat(2, 1, 1, 1, 1)
    # collinear: sqrtf(25) + sqrtf(25) <= sqrtf(100) rejects
    assert oracle.rppi_index(25.0, 25.0, 100.0, 0.0, 0.0, 0.0, e, 10) == -1


def test_rppi_grid_is_the_constructors(oracle):
    """Box cells (rpMax, rpMax, piMax); survey cubes of sqrtf(rpMax^2 + piMax^2)
    evaluated in FP32 (source/cudaNcorr.cu:182-193)."""
    cell, nc = oracle.rppi_grid(200.0, [0.0, 10.0, 25.0], 15)
    assert np.array_equal(cell, [25.0, 25.0, 15.0]) and np.array_equal(nc, [8, 8, 14])
    cell, nc = oracle.rppi_grid(200.0, [0.0, 10.0, 25.0], 15, survey=True)
    rmax = float(np.sqrt(np.float32(25.0 ** 2 + 15.0 ** 2)))
    assert np.all(cell == rmax) and np.all(nc == int(np.ceil(200.0 / rmax)))


@pytest.mark.parametrize("make", [cases.rppi_small_box, cases.rppi_small_box_clustered,
                                  cases.rppi_small_box_nondivisible], ids=lambda f: f.__name__)
def test_rppi_list_form_equals_literal(oracle, make):
    p, box, edges, npi = make()
    p = p[:1200]
    h, ov = oracle.count_rppi(box, edges, npi, p)
    hl, ovl = oracle.count_rppi(box, edges, npi, p, literal=True)
    assert np.array_equal(h, hl) and ov == ovl
    assert h.sum() > 0


@pytest.mark.parametrize("combo", ["DDD", "DDR", "DRR", "RRR", "RDR"])
def test_rppi_survey_list_form_equals_literal(oracle, combo):
    d, r, box, ori, edges, npi = cases.rppi_small_survey(nd=500, nr=1000)
    cat = {"D": d, "R": r}
    args = [cat[ch] for ch in combo]
    h, ov = oracle.count_rppi(box, edges, npi, *args, survey=True, ori=ori)
    hl, ovl = oracle.count_rppi(box, edges, npi, *args, survey=True, ori=ori, literal=True)
    assert np.array_equal(h, hl) and ov == ovl
    assert h.sum() > 0


def test_rppi_survey_uses_only_ori_x(oracle):
    """The reference uploads sizeof(double) of ori (source/cudaNcorr.cu:254),
    so ori.y and ori.z never reach the line of sight."""
    d, r, box, ori, edges, npi = cases.rppi_small_survey(nd=400, nr=10)
    h1, _ = oracle.count_rppi(box, edges, npi, d, survey=True, ori=ori)
    h2, _ = oracle.count_rppi(box, edges, npi, d, survey=True, ori=(ori[0], 1e4, -1e4))
    h3, _ = oracle.count_rppi(box, edges, npi, d, survey=True, ori=(ori[0] + 500.0, ori[1], ori[2]))
    assert np.array_equal(h1, h2)
    assert not np.array_equal(h1, h3)


def test_rppi_weighted_equals_unweighted_with_unit_weights(oracle):
    p, box, edges, npi = cases.rppi_small_box()
    p = p[:1000].copy()
    h, _ = oracle.count_rppi(box, edges, npi, p)
    q = p.copy()
    q[:, 3] = 2.0
    hw, _ = oracle.count_rppi(box, edges, npi, q)
    assert np.array_equal(hw, 8.0 * h)


@pytest.mark.parametrize("make,key,n", [(cases.rppi_box_probe, "rp_pattern", 3),
                                        (cases.rppi_survey_probe, "dot_pattern", 6)],
                         ids=["box_rp", "survey_dot"])
def test_rppi_probes_separate_every_contraction(oracle, make, key, n):
    """Each candidate contraction gives a different histogram on its probe,
    so running the reference kernel on the probe identifies the one nvcc
    chose."""
    c = make()
    res = [oracle.count_rppi(c["box"], c["edges"], c["npi"], c["p"], survey=c["survey"], ori=c["ori"],
                             **{key: k})[0] for k in range(n)]
    for i in range(n):
        for j in range(i + 1, n):
            assert not np.array_equal(res[i], res[j]), (i, j)


def test_rppi_compaction_layout(oracle):
    """prepTriCountsOutRppi (source/cudaNcorr.cu:88-105): entry order and
    tables, checked against a histogram that stores its own index."""
    edges = oracle.logspace(1.0, 30.0, 7)
    npi = 3
    nb = len(edges) - 1
    hist = np.arange(nb ** 3 * npi * npi, dtype=np.float64)
    counts, bins, pis = oracle.compact_rppi(edges, npi, hist)
    mids = (edges[1:] + edges[:-1]) / 2.0
    k = 0
    for i in range(nb):
        for j in range(i, nb):
            for kk in range(j, nb):
                if mids[kk] <= mids[i] + mids[j]:
                    for l in range(npi):
                        for m in range(npi):
                            assert counts[k] == m + l * npi + kk * npi * npi + j * npi * npi * nb + i * npi * npi * nb * nb
                            assert np.array_equal(bins[k], [mids[i], mids[j], mids[kk]])
                            assert np.array_equal(pis[k], [l, m])
                            k += 1
    assert k == len(counts)


@pytest.mark.skipif(not RPPI_GOLDEN, reason="no rppi fixtures recorded")
@pytest.mark.parametrize("meta_path", RPPI_GOLDEN, ids=lambda p: p.stem)
def test_rppi_golden_reference_outputs(oracle, meta_path):
    """The oracle reproduces the reference's rppi kernels on recorded inputs:
    exactly for counts (the weight written past the histogram included),
    within 1e-12 relative for weighted sums (the reference adds them with
    FP64 atomics in an arbitrary order)."""
    meta = json.loads(meta_path.read_text())
    data = np.load(meta_path.with_suffix(".npz"))
    cats = {k: data[k] for k in data.files if k.startswith("cat")}
    args = [cats[r] for r in meta["roles"]]
    if meta["roles"][1] == meta["roles"][2]:
        args[2] = args[1]
    if meta["roles"][0] == meta["roles"][1]:
        args[1] = args[0]
        args[2] = args[0] if meta["roles"][2] == meta["roles"][0] else args[2]
    h, ov = oracle.count_rppi(np.array(meta["box"]), np.array(meta["edges"]), meta["num_pi_bins"], *args,
                              survey=meta["survey"], ori=meta["ori"])
    ref = data["hist"]
    if meta["weighted"]:
        nz = ref != 0
        assert np.array_equal(nz, h != 0)
        assert np.max(np.abs(h[nz] - ref[nz]) / np.abs(ref[nz])) < 1e-12
    else:
        assert np.array_equal(h, ref)
        assert ov == meta["overflow"]


def test_rppi_gather_prefilter_never_drops_a_kept_point(tmp_path):
    """The FP32 prefilter of the rppi neighbour gather (rppi_gather_cut in
    cudancorr_gb300/csrc/rppi_fast.cuh), with the kernel's FP32 operations
    repeated on the host, against the reference's FP64 cut: neighbours on the
    cut surfaces to a few 2^-20 relative, at coordinates up to the grid's far
    face and through periodic images, in two boxes and a survey extent. Also
    the survey line-of-sight cut of list entries (rppi_los_cut): no entry it
    drops passes the reference's anchor-side test with any of its partners;
    and the survey pair classifier (rppi_survey_index): with pairs on the pi3,
    rp3 and pi1 limits of their own line of sight, rp1 or rp3 on a bin edge,
    pi1 on an integer and rp1 = rp2, every pair it rejects is not counted by
    the reference and every pair it indexes is counted at that index."""
    import shutil
    import subprocess
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    src = GOLDEN.parent / "cpp" / "rppi_gather_check.cu"
    exe = tmp_path / "rppi_gather_check"
    r = subprocess.run([nvcc, "-std=c++17", "-O2", "-Xcompiler", "-ffp-contract=off", "-o", str(exe), str(src)],
                       capture_output=True, text=True)
    if r.returncode != 0:
        pytest.skip(f"nvcc could not build the host check: {r.stderr[:200]}")
    for seed in (1, 2):
        out = subprocess.run([str(exe), "100000", str(seed)], capture_output=True, text=True)
        assert out.returncode == 0, out.stdout + out.stderr
        n = dict(zip(out.stdout.split()[0::2], map(int, out.stdout.split()[1::2])))
        assert n["violations"] == 0 and n["near"] > n["checked"] // 100 and n["kept"] > n["checked"] // 10
        assert n["los_violations"] == 0 and n["los_cut"] > n["los_checked"] // 10 and n["los_partners"] > 0
        assert n["pair_violations"] == 0 and n["pair_near"] > n["pair_checked"] // 10 and n["pair_idx"] > 0


def test_rppi_fp32_classifier_agrees_with_the_exact_computation(tmp_path):
    """The box-mode FP32 classifier (cudancorr_gb300/csrc/rppi_fast.cuh),
    compiled for the host, against an FP64 restatement of the reference on
    random and adversarial triangles (third side on a bin edge or equal to an
    anchor side, pi3 next to k^2, nearly collinear): whenever it answers, the
    answer is the reference's."""
    import shutil
    import subprocess
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    src = GOLDEN.parent / "cpp" / "rppi_fast_check.cu"
    exe = tmp_path / "rppi_fast_check"
    r = subprocess.run([nvcc, "-std=c++17", "-O2", "-Xcompiler", "-ffp-contract=off", "-o", str(exe), str(src)],
                       capture_output=True, text=True)
    if r.returncode != 0:
        pytest.skip(f"nvcc could not build the host check: {r.stderr[:200]}")
    for seed in (1, 2):
        out = subprocess.run([str(exe), "200000", str(seed)], capture_output=True, text=True)
        assert out.returncode == 0, out.stdout + out.stderr
        n = dict(zip(out.stdout.split()[0::2], map(int, out.stdout.split()[1::2])))
        assert n["mismatches"] == 0 and n["certain"] > n["checked"] // 4 and n["counted"] > 0
