"""Parity at the full sizes of the benchmark workloads, on anchor subsets.

Each workload is generated at its full size (every point is a neighbour
candidate); the anchors (p1) are a subset, so the oracle and the reference
kernel finish in seconds:
  * the 4M-point Soneira-Peebles box (L=1500, r_max=80, 16 bins: 19 cells per
    axis, the last one 60 wide, so the one-step wrap of
    source/device.cu:89-122 misses some face pairs and the engine must miss
    the same ones);
  * the survey wedge, 500k data (lognormal weights) and 2.5M randoms, jointly
    shifted, 15 log bins in [5, 120): DDD, DDR, DRR and RRR unweighted, and
    weighted DDD/DDR/DRR against the FP64 oracle;
  * the batched mocks' largest catalogue (about 1M points, L=1000, r_max=60,
    17 cells, the last 40 wide), inside a batch with three other mocks;
  * the rppi bin type on the 2M-point clustered box and on the survey wedge
    (rp 12 log bins in [1, 30), 30 unit pi bins): box, and survey DDD, DDR,
    DRR against the oracle, survey DDD against the reference's rppi kernel.
Against the CPU oracle the anchors are drawn at random. The reference kernel
(source/device.cu:259-315, :381-431, compiled unmodified) runs one thread per
anchor in FP64, so its time per anchor grows with (in-range neighbours) x
(points in the 27 cells); its anchors are the ones with the smallest such
cost, half of them chosen among anchors in the first or last cell layer of
the grid (the cells the periodic wrap involves), which bounds its run time.
"""
import time

import numpy as np
import pytest

from cudancorr_gb300 import api
from cudancorr_gb300 import catalogs as C
from oracle import oracle as O
from tests.test_gpu_parity import run_engine

pytestmark = pytest.mark.gpu

WEIGHTED_RTOL = 1e-6


@pytest.fixture(scope="module")
def ref(oracle):
    if not oracle.REF_CUBIN.exists():
        pytest.skip("reference cubin not built (needs the reference sources)")
    oracle.runner()
    return oracle


def cheap_anchors(p1, p2, p3, box, rmax, survey, n, seed):
    """n anchors of p1 with the smallest estimated reference-kernel cost
    (oracle.reference_anchor_cost); half of them from the first and last
    cell layers, half from the rest."""
    cost, face = O.reference_anchor_cost(p1, p2, p3, box, rmax, survey)
    rng = np.random.default_rng(seed)
    jitter = rng.random(len(p1)) * 1e-3  # random among equal costs
    pick = []
    for mask in (face, ~face):
        idx = np.flatnonzero(mask)
        pick.extend(idx[np.argsort(cost[idx] + jitter[idx])][: n // 2].tolist())
    pick = np.sort(np.array(pick))
    return np.ascontiguousarray(p1[pick]), float(cost[pick].max()), int(face[pick].sum())


def random_anchors(p, n, seed):
    rng = np.random.default_rng(seed)
    return np.ascontiguousarray(p[np.sort(rng.choice(len(p), n, replace=False))])


# --------------------------------------------------------------------------- 4M Soneira-Peebles box
@pytest.fixture(scope="module")
def sp4m():
    return C.config_soneira_peebles()


def test_soneira_peebles_4M_reference_anchors(ref, engine_lib, sp4m):
    """The reference kernel and the engine, bit for bit, on 128 anchors of the
    full 4M-point catalogue, 64 of them in the wrapped face layers."""
    p, box, edges = sp4m
    sub, cmax, nface = cheap_anchors(p, p, p, box, edges[-1], False, 128, 51)
    t0 = time.perf_counter()
    h_ref, kms, _ = ref.reference_count(box, edges, sub, p, p)
    print(f"\nSP4M reference: {len(sub)} anchors ({nface} on faces, cost <= {cmax:.3g}), "
          f"kernel {kms / 1e3:.1f} s, call {time.perf_counter() - t0:.1f} s")
    h, _, _ = run_engine(box, edges, sub, p, p)
    assert h_ref.sum() > 0
    assert np.array_equal(h, h_ref)


def test_soneira_peebles_4M_oracle_anchors(oracle, engine_lib, sp4m):
    """The oracle and the engine, bit for bit, on 256 random anchors of the
    full 4M-point catalogue; and the engine's schedules agree on them."""
    p, box, edges = sp4m
    sub = random_anchors(p, 256, 52)
    t0 = time.perf_counter()
    h_o = oracle.count_threeD(box, edges, sub, p, p)
    print(f"\nSP4M oracle: 256 anchors, {time.perf_counter() - t0:.1f} s")
    b = np.full(3, box)
    for mode in (api.SCHED_DYNAMIC, api.SCHED_STATIC):
        with api.ncorr(b, api.threeD, edges, False, (0.0, 0.0, 0.0)) as corr:
            corr.set_schedule(mode)
            corr.calculateD1D2D3(sub, p, p)
            assert np.array_equal(corr.getTriCountsAll(), h_o)
    assert h_o.sum() > 0


# --------------------------------------------------------------------------- survey wedge, 500k + 2.5M
@pytest.fixture(scope="module")
def survey_full():
    d, r, box, ori, edges = C.config_survey(7)
    d1, r1 = d.copy(), r.copy()
    d1[:, 3] = 1.0
    r1[:, 3] = 1.0
    return dict(D=d, R=r, D1=d1, R1=r1, box=box, ori=ori, edges=edges)


def _survey_args(s, combo, unit):
    cat = {"D": s["D1"] if unit else s["D"], "R": s["R1"] if unit else s["R"]}
    c2, c3 = cat[combo[1]], cat[combo[2]]
    return cat[combo[0]], c2, (c2 if combo[2] == combo[1] else c3)


@pytest.mark.parametrize("combo,n_anc", [("DDD", 256), ("DDR", 64), ("DRR", 24), ("RRR", 24)])
def test_survey_full_unweighted_oracle(oracle, engine_lib, survey_full, combo, n_anc):
    """Unit weights, random anchors of the full catalogues: bit for bit."""
    s = survey_full
    c1, c2, c3 = _survey_args(s, combo, True)
    sub = random_anchors(c1, n_anc, 60 + len(combo) * n_anc)
    t0 = time.perf_counter()
    h_o = oracle.count_threeD(s["box"], s["edges"], sub, c2, c3, survey=True)
    print(f"\nsurvey {combo} oracle: {n_anc} anchors, {time.perf_counter() - t0:.1f} s")
    h, _, _ = run_engine(s["box"], s["edges"], sub, c2, c3, survey=True, ori=s["ori"])
    assert h_o.sum() > 0
    assert np.array_equal(h, h_o)


@pytest.mark.parametrize("combo", ["DDD", "DDR"])
def test_survey_full_reference_anchors(ref, engine_lib, survey_full, combo):
    """Unit weights, the reference kernel on 64 anchors of the full
    catalogues (half in the clipped boundary layers): bit for bit."""
    s = survey_full
    c1, c2, c3 = _survey_args(s, combo, True)
    sub, cmax, nface = cheap_anchors(c1, c2, c3, s["box"], s["edges"][-1], True, 64, 70)
    t0 = time.perf_counter()
    h_ref, kms, _ = ref.reference_count(s["box"], s["edges"], sub, c2, c3, survey=True, ori=s["ori"])
    print(f"\nsurvey {combo} reference: {len(sub)} anchors ({nface} on faces, cost <= {cmax:.3g}), "
          f"kernel {kms / 1e3:.1f} s, call {time.perf_counter() - t0:.1f} s")
    h, _, _ = run_engine(s["box"], s["edges"], sub, c2, c3, survey=True, ori=s["ori"])
    assert h_ref.sum() > 0
    assert np.array_equal(h, h_ref)


@pytest.mark.parametrize("combo,n_anc", [("DDD", 64), ("DDR", 16), ("DRR", 8)])
def test_survey_full_weighted(oracle, engine_lib, survey_full, combo, n_anc):
    """Lognormal data weights: every bin within 1e-6 relative of the FP64
    oracle (the reference's (w1 w2) w3 in double, summed in FP64), and the
    same bins non-zero."""
    s = survey_full
    c1, c2, c3 = _survey_args(s, combo, False)
    sub = random_anchors(c1, n_anc, 80 + n_anc)
    h_o = oracle.count_threeD(s["box"], s["edges"], sub, c2, c3, survey=True)
    h, _, _ = run_engine(s["box"], s["edges"], sub, c2, c3, survey=True, ori=s["ori"])
    nz = h_o != 0
    assert nz.sum() > 100
    assert np.array_equal(h != 0, nz)
    rel = np.abs(h[nz] - h_o[nz]) / np.abs(h_o[nz])
    print(f"\nsurvey {combo} weighted: {n_anc} anchors, {int(nz.sum())} bins, max rel err {rel.max():.3g}")
    assert rel.max() < WEIGHTED_RTOL


# --------------------------------------------------------------------------- batched mocks, largest mock
@pytest.fixture(scope="module")
def mocks4():
    sizes = C.batch_mock_sizes()
    order = np.argsort(sizes)
    pick = [int(order[-1]), int(order[-2]), int(order[len(order) // 2]), int(order[0])]
    return [C.batch_mock(i, sizes[i]) for i in pick], 1000.0, C.linear_edges(60.0, 12)


def test_batch_with_largest_mock(engine_lib, mocks4):
    """The largest mock (about 1M points) and three others in one autotuned
    batch (one persistent launch in a CUDA graph), replayed twice: per-mock
    counts identical to separate calculateD1D2D3 calls."""
    torch = pytest.importorskip("torch")
    mocks, box, edges = mocks4
    assert len(mocks[0]) > 900_000
    b3 = np.full(3, box)
    plain = []
    with api.ncorr(b3, api.threeD, edges, False, (0.0, 0.0, 0.0)) as corr:
        for m in mocks:
            corr.calculateD1D2D3(m, m, m)
            plain.append(corr.getTriCountsAll())
        tm = [torch.from_numpy(m).cuda() for m in mocks]
        batch = api.Batch(corr, [(t, t, t) for t in tm], autotune=True)
        for _ in range(2):
            batch.run()
            for i in range(len(mocks)):
                assert np.array_equal(batch.counts_all(i), plain[i]), i
        batch.close()
    assert all(h.sum() > 0 for h in plain)


def test_largest_mock_reference_and_oracle_anchors(ref, engine_lib, mocks4):
    """The largest mock: the reference kernel on 128 anchors (64 in the
    wrapped face layers, where the last cell is 40 wide) and the oracle on
    256 random anchors, each bit for bit against the engine."""
    mocks, box, edges = mocks4
    p = mocks[0]
    sub, cmax, nface = cheap_anchors(p, p, p, box, edges[-1], False, 128, 90)
    t0 = time.perf_counter()
    h_ref, kms, _ = ref.reference_count(box, edges, sub, p, p)
    print(f"\nlargest mock reference: {len(sub)} anchors ({nface} on faces, cost <= {cmax:.3g}), "
          f"kernel {kms / 1e3:.1f} s, call {time.perf_counter() - t0:.1f} s")
    h, _, _ = run_engine(box, edges, sub, p, p)
    assert h_ref.sum() > 0
    assert np.array_equal(h, h_ref)
    sub2 = random_anchors(p, 256, 91)
    h_o = ref.count_threeD(box, edges, sub2, p, p)
    h2, _, _ = run_engine(box, edges, sub2, p, p)
    assert np.array_equal(h2, h_o)


# --------------------------------------------------------------------------- rppi at the benchmark sizes
def _rppi_run(box, edges, npi, p1, p2, p3, survey=False, ori=(0.0, 0.0, 0.0)):
    from tests.test_gpu_rppi import run_rppi
    h, st, _, _, _ = run_rppi(box, edges, npi, p1, p2, p3, survey=survey, ori=ori)
    return h, st


def test_rppi_box_clustered_2M_oracle_anchors(oracle, engine_lib):
    """rppi on the 2M-point clustered box of the rppi benchmark (rp 12 log
    bins in [1, 30), 30 unit pi bins), 4,096 random anchors against the
    oracle: bit for bit, with the triangles past the histogram."""
    p, box, _ = C.config_box_clustered(seed=2)
    edges = api.logspace(1.0, 30.0, 13)
    sub = random_anchors(p, 4096, 71)
    t0 = time.perf_counter()
    h_o, ov_o = oracle.count_rppi(box, edges, 30, sub, p, p)
    print(f"\nrppi box 2M oracle: {len(sub)} anchors, {time.perf_counter() - t0:.1f} s")
    h, st = _rppi_run(box, edges, 30, sub, p, p)
    assert h_o.sum() > 0
    assert np.array_equal(h, h_o) and st["overflow"] == ov_o


@pytest.mark.parametrize("combo,n_anc", [("DDD", 2048), ("DDR", 512), ("DRR", 192)])
def test_rppi_survey_full_oracle_anchors(oracle, engine_lib, survey_full, combo, n_anc):
    """Survey-mode rppi (rp 12 log bins in [1, 30), 30 unit pi bins) on the
    full wedge catalogues with unit weights, random anchors against the
    oracle: bit for bit."""
    s = survey_full
    c1, c2, c3 = _survey_args(s, combo, True)
    sub = random_anchors(c1, n_anc, 80 + n_anc)
    edges = api.logspace(1.0, 30.0, 13)
    t0 = time.perf_counter()
    h_o, ov_o = oracle.count_rppi(s["box"], edges, 30, sub, c2, c3, survey=True, ori=s["ori"])
    print(f"\nrppi survey {combo} oracle: {n_anc} anchors, {time.perf_counter() - t0:.1f} s")
    h, st = _rppi_run(s["box"], edges, 30, sub, c2, c3, survey=True, ori=s["ori"])
    assert h_o.sum() > 0
    assert np.array_equal(h, h_o) and st["overflow"] == ov_o


def test_rppi_survey_full_reference_anchors(ref, engine_lib, survey_full):
    """Survey-mode rppi DDD on the full data catalogue, the reference's own
    rppi kernel on 64 random anchors: bit for bit."""
    s = survey_full
    c1, c2, c3 = _survey_args(s, "DDD", True)
    sub = random_anchors(c1, 64, 97)
    edges = api.logspace(1.0, 30.0, 13)
    t0 = time.perf_counter()
    h_ref, ov_ref, _, _ = ref.reference_count_rppi(s["box"], edges, 30, sub, c2, c3, survey=True, ori=s["ori"])
    print(f"\nrppi survey DDD reference: {len(sub)} anchors, {time.perf_counter() - t0:.1f} s")
    h, st = _rppi_run(s["box"], edges, 30, sub, c2, c3, survey=True, ori=s["ori"])
    assert h_ref.sum() > 0
    assert np.array_equal(h, h_ref) and st["overflow"] == ov_ref
