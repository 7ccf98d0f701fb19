"""Work-queue scheduling on the GPU: the work model's kernels against the CPU
oracle, and counts that do not depend on the schedule or the tuning."""
import numpy as np
import pytest

from cudancorr_gb300 import api
from cudancorr_gb300 import catalogs as C
from oracle import mlp_oracle as M
from tests import cases

pytestmark = pytest.mark.gpu


def small_sp(seed):
    """Soneira-Peebles box, 100 top clumps (102,400 points) in L=600, r_max=80
    (8 cells, non-divisible), 16 bins: clustered enough to spread cell work."""
    return C.soneira_peebles(100, 5, 4, 1.9, 200.0, 600.0, seed), 600.0, C.linear_edges(80.0, 16)


def counts(box, edges, p, mode=api.SCHED_DYNAMIC, model=None, tuning=(32, 1), record=False):
    with api.ncorr(np.full(3, box), api.threeD, edges, False, (0, 0, 0)) as corr:
        corr.set_schedule(mode, model)
        corr.set_tuning(*tuning)
        corr.set_record_work(record)
        corr.calculateD1D2D3(p, p, p)
        out = corr.getTriCountsAll(), corr.stats()
        if record:
            out = out + corr.cell_work()
        return out


def training_rows(seeds):
    xs, ys = [], []
    for s in seeds:
        p, box, edges = small_sp(s)
        _, _, feats, work = counts(box, edges, p, record=True)
        keep = feats[:, 0] > 0  # cells holding anchors
        xs.append(feats[keep])
        ys.append(np.log1p(work[keep]).astype(np.float32))
    return np.concatenate(xs), np.concatenate(ys)


def test_gradient_matches_cpu_oracle(engine_lib):
    rng = np.random.default_rng(11)
    model = api.WorkModel(seed=7)
    p = model.get_params().astype(np.float64)
    x = rng.uniform(0.0, 7.0, (300, 28)).astype(np.float32)  # 300: a partial last tile
    t = rng.uniform(5.0, 20.0, 300).astype(np.float32)
    g, sse = model.gradient(x, t)
    sse_o, g_o = M.loss_and_grad(p, x.astype(np.float64), t.astype(np.float64))
    assert abs(sse - sse_o) <= 1e-5 * sse_o
    assert np.max(np.abs(g - g_o)) <= 2e-4 * np.max(np.abs(g_o))
    # Per block of parameters as well (W1, b1, W2, b2, w3, b3).
    for lo, hi in [(M.OFF_W1, M.OFF_B1), (M.OFF_B1, M.OFF_W2), (M.OFF_W2, M.OFF_B2),
                   (M.OFF_B2, M.OFF_W3), (M.OFF_W3, M.OFF_B3), (M.OFF_B3, M.N_PARAMS)]:
        scale = max(np.max(np.abs(g_o[lo:hi])), 1e-12)
        assert np.max(np.abs(g[lo:hi] - g_o[lo:hi])) <= 1e-3 * scale


def test_predict_matches_cpu_oracle(engine_lib):
    rng = np.random.default_rng(12)
    model = api.WorkModel(seed=8)
    x = rng.uniform(0.0, 7.0, (1000, 28)).astype(np.float32)
    y = model.predict(x)
    y_o = M.forward(model.get_params().astype(np.float64), x.astype(np.float64))
    assert np.allclose(y, y_o, rtol=1e-5, atol=1e-5)


def test_set_params_round_trip_and_sgd_direction(engine_lib):
    """One Adam step from the oracle's point of view lowers the loss."""
    rng = np.random.default_rng(13)
    model = api.WorkModel(seed=9)
    x = rng.uniform(0.0, 7.0, (512, 28)).astype(np.float32)
    t = (x[:, 0] * 2.0 + x[:, 1:].mean(axis=1)).astype(np.float32)
    p0 = model.get_params()
    model.set_params(p0)
    assert np.array_equal(model.get_params(), p0)
    before, _ = M.loss_and_grad(p0.astype(np.float64), x, t)
    model.train(x, t, epochs=5, batch=256, lr=1e-2, seed=1)
    after, _ = M.loss_and_grad(model.get_params().astype(np.float64), x, t)
    assert after < 0.5 * before


def test_recorded_work_adds_up(engine_lib):
    p, box, edges = small_sp(21)
    h, st, feats, work = counts(box, edges, p, record=True)
    assert feats.shape == (8 ** 3, 28)
    assert work.sum() == st["n_pairs"]
    cell = np.minimum((p[:, :3] / edges[-1]).astype(int), 7)
    occ = np.bincount((cell[:, 0] * 8 + cell[:, 1]) * 8 + cell[:, 2], minlength=512)
    assert np.allclose(feats[:, 0], np.log1p(occ).astype(np.float32))
    assert np.all(work[occ == 0] == 0)


@pytest.mark.parametrize("tuning", [(32, 1), (16, 2), (8, 4), (32, 4)])
def test_tuning_does_not_change_counts(engine_lib, oracle, tuning):
    p, box, edges = cases.small_box_nondivisible()
    h, _ = counts(box, edges, p, tuning=tuning)
    assert np.array_equal(h, oracle.count_threeD(box, edges, p))
    p, box, edges = cases.small_box_clustered()  # six-fold loop, 20 bins
    h, _ = counts(box, edges, p, tuning=tuning)
    assert np.array_equal(h, oracle.count_threeD(box, edges, p))


def test_schedules_give_identical_counts(engine_lib):
    x, y = training_rows([31, 32])
    model = api.WorkModel(seed=1)
    model.train(x, y, epochs=20, batch=256, lr=3e-3, seed=2)
    p, box, edges = small_sp(33)
    h_dyn, st_dyn = counts(box, edges, p)
    h_sta, st_sta = counts(box, edges, p, mode=api.SCHED_STATIC)
    h_lrn, st_lrn = counts(box, edges, p, mode=api.SCHED_LEARNED, model=model)
    assert np.array_equal(h_dyn, h_sta) and np.array_equal(h_dyn, h_lrn)
    assert st_dyn["n_pairs"] == st_sta["n_pairs"] == st_lrn["n_pairs"]
    assert st_lrn["n_anchors"] == len(p)


def test_learned_schedule_time_against_static_and_dynamic(engine_lib):
    """What the trained network gains in time. A model trained on the cell
    work of six 256k-point Soneira-Peebles boxes (L=600, r_max=80) orders a
    seventh, held-out one. Counts are identical under all three schedules.
    The learned order leaves less of the launch idle at its end than the
    static schedule (one contiguous range per CTA) and is faster than it.
    Against the dynamic counter, whose tail is already about one anchor long,
    any order can gain at most that idle share, so the learned one is only
    required to match it (within 5%). Best of three calls each."""
    torch = pytest.importorskip("torch")
    xs, ys = [], []
    for i in range(6):
        q, qbox, qedges = C.training_soneira_peebles(i)
        _, _, feats, work = counts(qbox, qedges, q, record=True)
        keep = feats[:, 0] > 0
        xs.append(feats[keep])
        ys.append(np.log1p(work[keep]).astype(np.float32))
    model = api.WorkModel(seed=1)
    model.train(np.concatenate(xs), np.concatenate(ys), epochs=200, batch=256, lr=3e-3, seed=2)
    p, box, edges = C.training_soneira_peebles(20)
    t = torch.from_numpy(p).cuda()
    res = {}
    with api.ncorr(np.full(3, box), api.threeD, edges, False, (0, 0, 0)) as corr:
        for name, mode in (("static", api.SCHED_STATIC), ("dynamic", api.SCHED_DYNAMIC),
                           ("learned", api.SCHED_LEARNED)):
            corr.set_schedule(mode, model if mode == api.SCHED_LEARNED else None)
            best = None
            for _ in range(3):
                corr.calculateD1D2D3(t, t, t)
                st = corr.stats()
                if best is None or st["ms_count"] < best["ms_count"]:
                    best = st
            res[name] = (best["ms_count"], best["tail_idle"], corr.getTriCountsAll())
    model.close()
    print("\n" + ", ".join(f"{k} {v[0]:.1f} ms (tail idle {100 * v[1]:.2f}%)" for k, v in res.items()))
    assert np.array_equal(res["learned"][2], res["static"][2])
    assert np.array_equal(res["learned"][2], res["dynamic"][2])
    assert res["learned"][1] < res["static"][1]
    assert res["learned"][0] < res["static"][0]
    assert res["learned"][0] <= 1.05 * res["dynamic"][0]


def test_learned_schedule_with_weights_and_survey(engine_lib, oracle):
    """The learned queue in survey mode with weights (p2 != p3)."""
    d, r, box, ori, edges = cases.small_survey(nd=2000, nr=4000, weighted=True)
    model = api.WorkModel(seed=3)
    with api.ncorr(box, api.threeD, edges, True, ori) as corr:
        corr.calculateD1D2D3(d, d, r)
        h0 = corr.getTriCountsAll()
        corr.set_schedule(api.SCHED_LEARNED, model)  # untrained: any order is correct
        corr.calculateD1D2D3(d, d, r)
        h1 = corr.getTriCountsAll()
    ref = oracle.count_threeD(box, edges, d, d, r, survey=True)
    nz = ref != 0
    for h in (h0, h1):
        assert np.array_equal(h != 0, nz)
        assert np.max(np.abs(h[nz] - ref[nz]) / np.abs(ref[nz])) < 1e-6


def test_model_learns_cell_work(engine_lib):
    """Trained on three catalogues of the process, the model predicts the
    held-out catalogue's per-cell log-work far better than its mean."""
    x, y = training_rows([41, 42, 43])
    xt, yt = training_rows([44])
    model = api.WorkModel(seed=5)
    model.train(x, y, epochs=200, batch=256, lr=3e-3, seed=6)
    pred = model.predict(xt)
    mse = np.mean((pred - yt) ** 2)
    var = np.var(yt)
    # The float64 oracle trained the same way reaches about 0.31 of the variance.
    assert mse < 0.5 * var, (mse, var)


def test_bf16_forward_matches_cpu_oracle(engine_lib):
    """The BF16 forward pass (weights, inputs and hidden activations rounded
    to bfloat16, FP32 accumulation) against the oracle's restatement of the
    same roundings with float64 sums. Tolerance: the two sum the same
    products in different precision, so a sum that falls next to a bfloat16
    rounding boundary can round one bfloat16 step differently; 99% of the
    outputs agree to 1e-4 of the output scale, all to 2e-2. Against the FP32
    model the BF16 outputs stay within 0.1 of the scale."""
    rng = np.random.default_rng(21)
    model = api.WorkModel(seed=8)
    p = model.get_params().astype(np.float64)
    x = rng.uniform(0.0, 7.0, (1000, 28)).astype(np.float32)
    y32 = model.predict(x)
    model.set_precision(api.MLP_BF16)
    y16 = model.predict(x)
    y_o = M.forward(p, x, bf16_forward=True)
    scale = max(1.0, float(np.max(np.abs(y_o))))
    err = np.abs(y16 - y_o)
    assert np.quantile(err, 0.99) <= 1e-4 * scale
    assert err.max() <= 2e-2 * scale
    assert np.max(np.abs(y16 - y32)) <= 0.1 * scale
    assert np.max(np.abs(y16 - y32)) > 0  # the roundings do happen
    # Training gradient with the BF16 forward pass.
    t = rng.uniform(5.0, 20.0, 300).astype(np.float32)
    g, sse = model.gradient(x[:300], t)
    sse_o, g_o = M.loss_and_grad(p, x[:300].astype(np.float64), t.astype(np.float64), bf16_forward=True)
    assert abs(sse - sse_o) <= 1e-3 * sse_o
    assert np.max(np.abs(g - g_o)) <= 1e-2 * np.max(np.abs(g_o))
    assert np.mean(np.abs(g - g_o)) <= 1e-3 * np.max(np.abs(g_o))
    model.close()


def test_bf16_model_orders_like_fp32_and_keeps_counts():
    """A work model trained with the BF16 forward pass predicts cell work like
    the FP32 one on a held-out catalogue, and the learned queue it builds
    gives counts identical to the dynamic schedule (the order never changes
    the counts)."""
    x, y = training_rows([61, 62, 63])
    m32 = api.WorkModel(seed=3)
    m32.train(x, y, epochs=60, batch=256, lr=3e-3, seed=4)
    m16 = api.WorkModel(seed=3)
    m16.set_precision(api.MLP_BF16)
    m16.train(x, y, epochs=60, batch=256, lr=3e-3, seed=4)
    p, box, edges = small_sp(64)
    h_dyn, _, feats, work = counts(box, edges, p, record=True)
    keep = feats[:, 0] > 0
    yt = np.log1p(work[keep])
    p32 = m32.predict(feats[keep]).astype(np.float64)
    p16 = m16.predict(feats[keep]).astype(np.float64)
    r2_32 = 1.0 - np.mean((p32 - yt) ** 2) / np.var(yt)
    r2_16 = 1.0 - np.mean((p16 - yt) ** 2) / np.var(yt)
    assert r2_16 > 0.3 and r2_16 > r2_32 - 0.1
    h16, _ = counts(box, edges, p, mode=api.SCHED_LEARNED, model=m16)
    assert np.array_equal(h16, h_dyn)
    m32.close()
    m16.close()
