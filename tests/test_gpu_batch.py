"""Batches: one persistent launch in a CUDA graph, per-item counts identical to
separate calculateD1D2D3 runs."""
import numpy as np
import pytest

from cudancorr_gb300 import api
from cudancorr_gb300 import catalogs as C
from tests import cases

pytestmark = pytest.mark.gpu


def mocks(n_mocks, seed, box=500.0):
    """Neyman-Scott mocks of uneven size (parents N/8, Poisson(8), sigma 1.5)."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(4000), np.log(40000), n_mocks)).astype(int)
    return [C.neyman_scott(max(1, s // 8), 8.0, 1.5, box, seed * 100 + i) for i, s in enumerate(sizes)]


def plain(box, edges, p1, p2, p3, survey=False, ori=(0, 0, 0)):
    with api.ncorr(np.broadcast_to(np.asarray(box, dtype=np.float64), (3,)), api.threeD, edges, survey,
                   ori) as corr:
        corr.calculateD1D2D3(p1, p2, p3)
        return corr.getTriCountsAll()


@pytest.mark.parametrize("autotune", [True, False])
def test_batch_of_mocks_matches_plain_runs(engine_lib, autotune):
    box, edges = 500.0, C.linear_edges(60.0, 12)  # 9 cells, the last 20 wide
    ms = mocks(6, 1, box)
    refs = [plain(box, edges, m, m, m) for m in ms]
    with api.ncorr(np.full(3, box), api.threeD, edges, False, (0, 0, 0)) as corr:
        b = api.Batch(corr, [(m, m, m) for m in ms], autotune=autotune)
        for _ in range(2):
            b.run()
            for i, m in enumerate(ms):
                assert np.array_equal(b.counts_all(i), refs[i]), i
        st = b.stats()
        assert st["n_items"] == 6 and st["n_catalogues"] == 6 and st["graph_nodes"] > 10
        assert st["triangles"] == int(sum(r.sum() for r in refs))
        assert st["n_work"] == sum(len(m) for m in ms)
        b.close()


def test_batch_device_inputs_and_schedules(engine_lib):
    torch = pytest.importorskip("torch")
    box, edges = 500.0, C.linear_edges(60.0, 12)
    ms = mocks(5, 2, box)
    refs = [plain(box, edges, m, m, m) for m in ms]
    ts = [torch.from_numpy(m).cuda() for m in ms]
    model = api.WorkModel(seed=4)
    for mode, mdl in [(api.SCHED_DYNAMIC, None), (api.SCHED_STATIC, None), (api.SCHED_LEARNED, model)]:
        with api.ncorr(np.full(3, box), api.threeD, edges, False, (0, 0, 0)) as corr:
            corr.set_schedule(mode, mdl)
            b = api.Batch(corr, [(t, t, t) for t in ts], autotune=False)
            b.run()
            for i in range(len(ms)):
                assert np.array_equal(b.counts_all(i), refs[i]), (mode, i)
            assert 0.0 < b.stats()["ms_count"] <= b.stats()["ms_run"]
            b.close()
            # The library leaves no CUDA error pending for the next launch.
            torch.ones(4, device="cuda").fill_(2.0)
            torch.cuda.synchronize()


def test_batch_divisible_box_six_fold(engine_lib, oracle):
    p1, box, edges = cases.small_box_clustered(seed=12)
    p2, _, _ = cases.small_box_clustered(seed=13)
    with api.ncorr(np.full(3, box), api.threeD, edges, False, (0, 0, 0)) as corr:
        b = api.Batch(corr, [(p1, p1, p1), (p2, p2, p2)], autotune=True)
        b.run()
        assert np.array_equal(b.counts_all(0), oracle.count_threeD(box, edges, p1))
        assert np.array_equal(b.counts_all(1), oracle.count_threeD(box, edges, p2))
        b.close()


def test_batch_survey_weighted_shared_catalogues(engine_lib, oracle):
    """Data plus randoms: DDR and RDR share the gridded D and R."""
    d, r, box, ori, edges = cases.small_survey(nd=2000, nr=4000, weighted=True)
    with api.ncorr(box, api.threeD, edges, True, ori) as corr:
        b = api.Batch(corr, [(d, d, r), (r, d, r)], autotune=True)
        b.run()
        assert b.stats()["n_catalogues"] == 2 and b.stats()["weighted"] == 1
        for i, (p1, p2, p3) in enumerate([(d, d, r), (r, d, r)]):
            ref = oracle.count_threeD(box, edges, p1, p2, p3, survey=True)
            h = b.counts_all(i)
            nz = ref != 0
            assert np.array_equal(h != 0, nz)
            assert np.max(np.abs(h[nz] - ref[nz]) / np.abs(ref[nz])) < 1e-6
        b.close()


def test_batch_rejects_mixed_pair_loops(engine_lib):
    d, r, box, ori, edges = cases.small_survey(nd=500, nr=1000)
    with api.ncorr(box, api.threeD, edges, True, ori) as corr:
        with pytest.raises(api.NcorrError) as e:
            api.Batch(corr, [(d, d, d), (d, d, r)])
        assert e.value.code == api.NCORR_ERR_INVALID_ARGUMENT


def test_batch_replay_sees_new_contents_and_stale_weights(engine_lib):
    box, edges = 500.0, C.linear_edges(60.0, 12)
    ms = mocks(3, 3, box)
    with api.ncorr(np.full(3, box), api.threeD, edges, False, (0, 0, 0)) as corr:
        b = api.Batch(corr, [(m, m, m) for m in ms], autotune=False)
        b.run()
        # Same sizes, new positions: the replay recomputes cell lists and queue.
        new = C.neyman_scott(len(ms[1]) // 8, 8.0, 1.5, box, 999)[: len(ms[1])]
        if len(new) == len(ms[1]):
            ms[1][:] = new
            b.run()
            assert np.array_equal(b.counts_all(1), plain(box, edges, ms[1], ms[1], ms[1]))
        # Weights appear after an unweighted plan: refused, not miscounted.
        ms[0][:, 3] = 2.0
        with pytest.raises(api.NcorrError) as e:
            b.run()
        assert e.value.code == api.NCORR_ERR_CAPACITY
        b.close()
