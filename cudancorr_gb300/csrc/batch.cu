// Batches (include/ncorr_gb300.h, ncorr_batch_*): many catalogue triples --
// mocks, or data plus randoms -- counted by ONE persistent launch of the
// triangle kernel, with the copies, cell lists, work queue, exact pass and
// fold around it captured once into a CUDA graph and replayed per run.
//
// Planning grids every distinct catalogue once, reads back what the launch
// shape depends on (weights, neighbourhood bounds, the six-fold conditions),
// optionally times tuning candidates on a sample of the queue, and captures
// the graph. A replay recomputes the cell lists and the queue from the
// arrays' current contents; whatever the plan fixed is re-checked on the
// device (weights, list capacity) and reported as an error if the contents
// no longer fit the plan.
#include "host.cuh"

using namespace ncorr_gb300;
using namespace ncorr_host;

// Set in the kernel-flag word when the catalogues no longer fit the plan.
constexpr int kFlagPlanStale = 64;

namespace ncorr_gb300 {

// Re-checks, inside the graph, the plan's assumptions on the weights.
__global__ void k_plan_check(const int* __restrict__ cat_flags, int n_cats, const unsigned* __restrict__ wmax_bits,
                             int weighted, unsigned wmax_planned, int* __restrict__ kflags) {
  bool stale = false;
  for (int c = threadIdx.x; c < n_cats; c += blockDim.x)
    if (!weighted && (cat_flags[c] & kFlagWeighted)) stale = true;
  if (threadIdx.x == 0 && weighted && *wmax_bits > wmax_planned) stale = true;
  if (stale) atomicOr(kflags, kFlagPlanStale);
}

// Every stride-th position of a queue (the autotuner's sample).
__global__ void k_sample_queue(const int* __restrict__ q_item, const int* __restrict__ q_anchor, int stride,
                               int n_out, int* __restrict__ s_item, int* __restrict__ s_anchor) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_out) return;
  s_item[i] = q_item[static_cast<size_t>(i) * stride];
  s_anchor[i] = q_anchor[static_cast<size_t>(i) * stride];
}

}  // namespace ncorr_gb300

struct ncorr_batch {
  ncorr_handle* h = nullptr;
  int n_items = 0, n_cats = 0;
  bool on_device = false;
  std::vector<const double*> cat_src;
  std::vector<int64_t> cat_n, cat_off;
  std::vector<char> registered;  // host arrays this batch page-locked
  std::vector<int> role[3];      // item -> catalogue
  Geom g;
  // Concatenated cell lists of all catalogues.
  DevBuf in, cid, pd, pq, pc, count, start, cursor, flags, wmax, bound;
  // Items, histograms, results and the launch's own buffers.
  DevBuf items, hist, out, total, item_off, q_item, q_anchor, s_item, s_anchor, work, stats, xq, xq_count;
  DevBuf slab_e, slab_w, slab_q, slab_x, args, args_probe, table, feats;
  OrderBufs order;
  unsigned xq_cap = 0;
  // Page-locked host mirrors the graph writes.
  double* h_out = nullptr;
  int* h_flags = nullptr;
  unsigned long long* h_stats = nullptr;
  unsigned long long* h_total = nullptr;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  // The plan.
  KArgs a;
  bool sym = false, weighted = false, hg = false, learned = false;
  unsigned wmax_planned = 0;
  int grid = 0, nsm = 0;
  size_t smem = 0;
  float wscale = 1.0f;
  int64_t n_work = 0;
  ncorr_batch_stats st;
};

namespace {

size_t hist_words(const ncorr_batch* b) {
  const size_t nbin = static_cast<size_t>(b->h->nb) * b->h->nb * b->h->nb;
  return b->weighted ? 2 * nbin : nbin;
}

// Copies (host inputs), cell lists and neighbourhood bounds of all
// catalogues, on b->stream; eager in planning, captured in the graph.
int enqueue_grid(ncorr_batch* b) {
  cudaStream_t s = b->stream;
  const long ncell = b->h->ncell;
  CU(cudaMemsetAsync(b->flags.p, 0, (b->n_cats + 8) * sizeof(int), s));
  CU(cudaMemsetAsync(b->wmax.p, 0, sizeof(unsigned), s));
  CU(cudaMemsetAsync(b->bound.p, 0, b->n_cats * sizeof(int), s));
  CU(cudaMemsetAsync(b->count.p, 0, static_cast<size_t>(b->n_cats) * ncell * sizeof(int), s));
  for (int c = 0; c < b->n_cats; ++c) {
    const int64_t off = b->cat_off[c];
    const int n = static_cast<int>(b->cat_n[c]);
    const double4_16a* src = b->on_device ? reinterpret_cast<const double4_16a*>(b->cat_src[c])
                                          : b->in.as<double4_16a>() + off;
    if (!b->on_device && n > 0)
      CU(cudaMemcpyAsync(b->in.as<double4_16a>() + off, b->cat_src[c], n * sizeof(double4_16a),
                         cudaMemcpyHostToDevice, s));
    int* cnt = b->count.as<int>() + static_cast<size_t>(c) * ncell;
    int* cur = b->cursor.as<int>() + static_cast<size_t>(c) * ncell;
    int* stt = b->start.as<int>() + static_cast<size_t>(c) * (ncell + 1);
    launch_assign(src, n, b->g, b->cid.as<int>() + off, cnt, b->flags.as<int>() + c, b->wmax.as<unsigned>(), s);
    launch_scan(cnt, static_cast<int>(ncell), stt, cur, s);
    launch_scatter(src, n, b->g, b->cid.as<int>() + off, cur, b->pd.as<double4_16a>() + off,
                   b->pq.as<float4>() + off, b->pc.as<int>() + off, s);
    launch_nbr_bound(cnt, b->g, b->bound.as<int>() + c, s);
  }
  CU(cudaGetLastError());
  return NCORR_OK;
}

Catalog cat_view(const ncorr_batch* b, int c) {
  Catalog v;
  const int64_t off = b->cat_off[c];
  const long ncell = b->h->ncell;
  v.pd = b->pd.as<double4_16a>() + off;
  v.pq = b->pq.as<float4>() + off;
  v.pc = b->pc.as<int>() + off;
  v.start = b->start.as<int>() + static_cast<size_t>(c) * (ncell + 1);
  v.count = b->count.as<int>() + static_cast<size_t>(c) * ncell;
  v.n = static_cast<int>(b->cat_n[c]);
  return v;
}

// Work queue for b->a: identity (cell order, items in order) or learned.
int enqueue_queue(ncorr_batch* b) {
  cudaStream_t s = b->stream;
  const int n_work = static_cast<int>(b->n_work);
  if (b->learned) {
    OrderScratch os;
    CU(b->order.ensure(b->n_items, b->h->ncell, &os));
    const int m = b->n_items * static_cast<int>(b->h->ncell);
    launch_cell_features(b->items.as<BatchItem>(), b->n_items, b->g, b->feats.as<float>(), s);
    launch_mlp_predict(b->h->sched_model->params.as<float>(), b->feats.as<float>(), m, os.pred, s,
                       b->h->sched_model->bf16);
    launch_learned_queue(b->items.as<BatchItem>(), b->n_items, static_cast<int>(b->h->ncell), os,
                         b->q_item.as<int>(), b->q_anchor.as<int>(), s);
  } else {
    launch_identity_queue(b->item_off.as<int>(), b->n_items, b->q_item.as<int>(), b->q_anchor.as<int>(), n_work, s);
  }
  CU(cudaGetLastError());
  return NCORR_OK;
}

// Everything after the cell lists: plan check, zeroing, queue, count, exact
// pass, fold and the read-back into page-locked memory.
int enqueue_count(ncorr_batch* b, bool set_attr) {
  cudaStream_t s = b->stream;
  const size_t nbin = static_cast<size_t>(b->h->nb) * b->h->nb * b->h->nb;
  k_plan_check<<<1, 256, 0, s>>>(b->flags.as<int>(), b->n_cats, b->wmax.as<unsigned>(), b->weighted ? 1 : 0,
                                 b->wmax_planned, b->flags.as<int>() + b->n_cats);
  CU(cudaMemsetAsync(b->hist.p, 0, b->n_items * hist_words(b) * sizeof(unsigned long long), s));
  CU(cudaMemsetAsync(b->total.p, 0, b->n_items * sizeof(unsigned long long), s));
  CU(cudaMemsetAsync(b->work.p, 0, sizeof(int), s));
  CU(cudaMemsetAsync(b->xq_count.p, 0, sizeof(unsigned), s));
  CU(cudaMemsetAsync(b->stats.p, 0, 8 * sizeof(unsigned long long), s));
  if (int rc = enqueue_queue(b)) return rc;
  // External records: inside a capture they become event-record nodes that
  // the replay timestamps (a plain record only orders the capture).
  CU(cudaEventRecordWithFlags(b->ev[1], s, cudaEventRecordExternal));
  if (b->n_work > 0) {
    CU(launch_triangles(b->a, b->h->survey != 0, b->sym, b->weighted, b->hg, b->grid, b->smem, s, set_attr));
    CU(cudaEventRecordWithFlags(b->ev[2], s, cudaEventRecordExternal));
    launch_exact(b->a, b->h->survey != 0, b->weighted, b->nsm * 4, s);
  } else {
    CU(cudaEventRecordWithFlags(b->ev[2], s, cudaEventRecordExternal));
  }
  launch_fold(b->items.as<BatchItem>(), b->n_items, b->h->nb, b->weighted, b->sym, 1.0 / b->wscale, s);
  CU(cudaGetLastError());
  CU(cudaMemcpyAsync(b->h_out, b->out.p, b->n_items * nbin * sizeof(double), cudaMemcpyDeviceToHost, s));
  CU(cudaMemcpyAsync(b->h_flags, b->flags.p, (b->n_cats + 8) * sizeof(int), cudaMemcpyDeviceToHost, s));
  CU(cudaMemcpyAsync(b->h_stats, b->stats.p, 8 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
  CU(cudaMemcpyAsync(b->h_total, b->total.p, b->n_items * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
  return NCORR_OK;
}

// Launch shape for a tuning choice (histogram copies) and the largest
// 27-cell occupancy of any catalogue. Returns false when the kernel cannot
// run with exactly that many copies.
bool shape(ncorr_batch* b, int copies, int kmax, TriShape* out) {
  if (!tri_shape(b->h->nb, b->h->survey != 0, b->sym, b->weighted, b->hg, copies, b->nsm, b->n_work, kmax, kmax,
                 out))
    return false;
  return out->copies == copies;
}

int plan(ncorr_batch* b, int autotune) {
  ncorr_handle* h = b->h;
  cudaStream_t s = b->stream;
  const long ncell = h->ncell;
  const int nb = h->nb;
  const size_t nbin = static_cast<size_t>(nb) * nb * nb;
  int64_t total_pts = 0;
  for (int c = 0; c < b->n_cats; ++c) total_pts += b->cat_n[c];
  const size_t tp = static_cast<size_t>(std::max<int64_t>(total_pts, 1));
  if (!b->on_device) CU(b->in.ensure(tp * sizeof(double4_16a)));
  CU(b->cid.ensure(tp * sizeof(int)));
  CU(b->pd.ensure(tp * sizeof(double4_16a)));
  CU(b->pq.ensure(tp * sizeof(float4)));
  CU(b->pc.ensure(tp * sizeof(int)));
  CU(b->count.ensure(static_cast<size_t>(b->n_cats) * ncell * sizeof(int)));
  CU(b->cursor.ensure(static_cast<size_t>(b->n_cats) * ncell * sizeof(int)));
  CU(b->start.ensure(static_cast<size_t>(b->n_cats) * (ncell + 1) * sizeof(int)));
  CU(b->flags.ensure((b->n_cats + 8) * sizeof(int)));
  CU(b->wmax.ensure(sizeof(unsigned)));
  CU(b->bound.ensure(b->n_cats * sizeof(int)));
  b->g = h->g;

  // Eager pass over the cell lists: what the launch shape depends on.
  if (int rc = enqueue_grid(b)) return rc;
  std::vector<int> flags(b->n_cats), bound(b->n_cats);
  unsigned wmax_bits = 0;
  CU(cudaMemcpyAsync(flags.data(), b->flags.p, b->n_cats * sizeof(int), cudaMemcpyDeviceToHost, s));
  CU(cudaMemcpyAsync(bound.data(), b->bound.p, b->n_cats * sizeof(int), cudaMemcpyDeviceToHost, s));
  CU(cudaMemcpyAsync(&wmax_bits, b->wmax.p, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  CU(cudaStreamSynchronize(s));
  b->weighted = false;
  for (int c = 0; c < b->n_cats; ++c) {
    if (flags[c] & kFlagNonFinite) return fail(NCORR_ERR_OUT_OF_GRID, "non-finite coordinate or weight");
    if (flags[c] & kFlagOutOfGrid) return fail(NCORR_ERR_OUT_OF_GRID, "a point lies outside the cell grid of the box");
    if (flags[c] & kFlagWeighted) b->weighted = true;
  }
  for (int i = 0; i < b->n_items; ++i)
    if (h->survey && (flags[b->role[0][i]] & kFlagSurveyFace))
      return fail(NCORR_ERR_OUT_OF_GRID, "survey anchor on the upper face of the cell grid");
  b->wmax_planned = wmax_bits;
  b->wscale = 1.0f;
  if (b->weighted) {
    float wm = 0.0f;
    std::memcpy(&wm, &wmax_bits, sizeof(float));
    const double p3 = static_cast<double>(wm) * wm * wm;
    int e = 0;
    if (p3 > 0) e = static_cast<int>(std::floor(std::log2(std::ldexp(1.0, 30) / p3)));
    b->wscale = static_cast<float>(std::ldexp(1.0, std::max(-120, std::min(120, e))));
  }
  bool divisible = true;
  for (int d = 0; d < 3; ++d)
    if (h->g.nc[d] < 4 || __builtin_fma(-static_cast<double>(h->g.nc[d]), h->g.cell, h->box[d]) != 0.0)
      divisible = false;
  const int elem = b->weighted ? 8 : 4;
  b->hg = hist_global(nb, elem);
  const int code_scale = b->hg ? 1 : elem;
  {
    std::vector<unsigned char> tab;
    build_table(b->g, code_scale, tab);
    CU(b->table.ensure(tab.size()));
    CU(cudaMemcpy(b->table.p, tab.data(), tab.size(), cudaMemcpyHostToDevice));
  }

  // Items and their buffers.
  CU(b->hist.ensure(b->n_items * hist_words(b) * sizeof(unsigned long long)));
  CU(b->out.ensure(b->n_items * nbin * sizeof(double)));
  CU(b->total.ensure(b->n_items * sizeof(unsigned long long)));
  std::vector<BatchItem> items(b->n_items);
  std::vector<int> item_off(b->n_items + 1, 0);
  for (int i = 0; i < b->n_items; ++i) {
    BatchItem& it = items[i];
    std::memset(&it, 0, sizeof(it));
    it.c1 = cat_view(b, b->role[0][i]);
    it.c2 = cat_view(b, b->role[1][i]);
    it.c3 = cat_view(b, b->role[2][i]);
    unsigned long long* hw = b->hist.as<unsigned long long>() + i * hist_words(b);
    it.hist.counts = b->weighted ? nullptr : hw;
    it.hist.wsum = b->weighted ? hw : nullptr;
    it.out = b->out.as<double>() + i * nbin;
    it.total = b->total.as<unsigned long long>() + i;
    it.flags1 = b->flags.as<int>() + b->role[0][i];
    const bool one_cat = b->role[0][i] == b->role[1][i] && b->role[1][i] == b->role[2][i];
    it.sym6_ok = (one_cat && (h->survey || divisible)) ? 1 : 0;
    it.cell_base = static_cast<int>(i * ncell);
    item_off[i + 1] = item_off[i] + static_cast<int>(b->cat_n[b->role[0][i]]);
  }
  b->n_work = item_off[b->n_items];
  CU(b->items.ensure(b->n_items * sizeof(BatchItem)));
  CU(cudaMemcpy(b->items.p, items.data(), b->n_items * sizeof(BatchItem), cudaMemcpyHostToDevice));
  CU(b->item_off.ensure((b->n_items + 1) * sizeof(int)));
  CU(cudaMemcpy(b->item_off.p, item_off.data(), (b->n_items + 1) * sizeof(int), cudaMemcpyHostToDevice));
  const size_t nw = static_cast<size_t>(std::max<int64_t>(b->n_work, 1));
  CU(b->q_item.ensure(nw * sizeof(int)));
  CU(b->q_anchor.ensure(nw * sizeof(int)));
  CU(b->work.ensure(sizeof(int)));
  CU(b->stats.ensure(8 * sizeof(unsigned long long)));
  b->xq_cap = h->xq_cap;
  CU(b->xq.ensure(static_cast<size_t>(std::max(b->xq_cap, 1u)) * sizeof(ExactEntry)));
  CU(b->xq_count.ensure(sizeof(unsigned)));
  CU(b->args.ensure(sizeof(KArgs)));
  CU(b->args_probe.ensure(sizeof(KArgs)));
  b->learned = h->sched_mode == NCORR_SCHED_LEARNED;
  if (b->learned) {
    // Allocated now: nothing may be allocated while the graph is captured.
    CU(b->feats.ensure(static_cast<size_t>(b->n_items) * ncell * kMlpIn * sizeof(float)));
    OrderScratch os;
    CU(b->order.ensure(b->n_items, ncell, &os));
  }
  CU(cudaDeviceGetAttribute(&b->nsm, cudaDevAttrMultiProcessorCount, h->device));
  if (cudaHostAlloc(&b->h_out, b->n_items * nbin * sizeof(double), cudaHostAllocDefault) != cudaSuccess ||
      cudaHostAlloc(&b->h_flags, (b->n_cats + 8) * sizeof(int), cudaHostAllocDefault) != cudaSuccess ||
      cudaHostAlloc(&b->h_stats, 8 * sizeof(unsigned long long), cudaHostAllocDefault) != cudaSuccess ||
      cudaHostAlloc(&b->h_total, b->n_items * sizeof(unsigned long long), cudaHostAllocDefault) != cudaSuccess)
    return fail(NCORR_ERR_CUDA, "cudaHostAlloc failed");

  // Tuning candidates (histogram copies; the flag-group height is the
  // handle's) and the slabs the largest list needs under any of them.
  struct Cand {
    int sub_j, copies;
    TriShape shp;
  };
  std::vector<Cand> cands;
  const int kmax = *std::max_element(bound.begin(), bound.end());
  for (int cp : {1, 2, 4}) {
    if (!autotune && cp != h->hist_copies) continue;
    Cand c{h->sub_j, cp, TriShape()};
    if (!shape(b, cp, kmax, &c.shp)) continue;
    cands.push_back(c);
  }
  if (cands.empty()) {
    Cand c{h->sub_j, 1, TriShape()};
    if (!shape(b, 1, kmax, &c.shp)) return fail(NCORR_ERR_CUDA, "triangle kernel does not fit on the device, or a 27-cell neighbourhood holds "
                                  "more than 2^24 points");
    cands.push_back(c);
  }
  size_t slab_n = 0;
  int grid_max = 0;
  for (const Cand& c : cands) {
    slab_n = std::max(slab_n, tri_slab_entries(c.shp));
    grid_max = std::max(grid_max, c.shp.grid);
  }
  CU(b->slab_e.ensure(slab_n * sizeof(ListEnt)));
  if (b->weighted) CU(b->slab_w.ensure(slab_n * sizeof(float)));
  CU(b->slab_q.ensure(static_cast<size_t>(grid_max) * kWarps * kQueueCap * sizeof(unsigned long long)));
  CU(b->slab_x.ensure(static_cast<size_t>(grid_max) * kWarps * 32 * sizeof(ExactEntry)));

  KArgs& a = b->a;
  std::memset(&a, 0, sizeof(a));
  a.g = b->g;
  a.items = b->items.as<BatchItem>();
  a.n_items = b->n_items;
  a.q_item = b->q_item.as<int>();
  a.q_anchor = b->q_anchor.as<int>();
  a.n_work = static_cast<int>(b->n_work);
  a.sched_static = h->sched_mode == NCORR_SCHED_STATIC ? 1 : 0;
  a.cell_work = nullptr;
  a.table = b->table.as<unsigned char>();
  a.work = b->work.as<int>();
  a.flags = b->flags.as<int>() + b->n_cats;
  a.slab_e = b->slab_e.as<ListEnt>();
  a.slab_w = b->weighted ? b->slab_w.as<float>() : nullptr;
  a.slab_q = b->slab_q.as<unsigned long long>();
  a.slab_x = b->slab_x.as<ExactEntry>();
  a.code_scale = code_scale;
  a.wscale = b->wscale;
  a.stats = b->stats.as<unsigned long long>();
  a.xq = b->xq.as<ExactEntry>();
  a.xq_count = b->xq_count.as<unsigned>();
  a.xq_cap = b->xq_cap;
  a.self = b->args.as<KArgs>();
  auto apply = [&](const Cand& c) -> int {
    a.sub_j = c.sub_j;
    a.hist_copies = c.copies;
    a.kcap2 = c.shp.kcap2;
    a.kcap3 = c.shp.kcap3;
    b->grid = c.shp.grid;
    b->smem = c.shp.smem;
    CU(cudaMemcpy(b->args.p, &a, sizeof(KArgs), cudaMemcpyHostToDevice));
    return NCORR_OK;
  };

  // Autotune: each candidate counts every stride-th queue position (twice;
  // the faster time counts). Counts are identical for all candidates.
  auto t0 = std::chrono::steady_clock::now();
  if (int rc = apply(cands[0])) return rc;
  if (cands.size() > 1 && b->n_work > 0) {
    if (int rc = enqueue_queue(b)) return rc;
    const int64_t n_probe = std::min<int64_t>(b->n_work, std::max<int64_t>(4096, b->n_work / 32));
    const int stride = static_cast<int>(b->n_work / n_probe);
    const int n_s = static_cast<int>(b->n_work / stride);
    CU(b->s_item.ensure(n_s * sizeof(int)));
    CU(b->s_anchor.ensure(n_s * sizeof(int)));
    k_sample_queue<<<(n_s + 255) / 256, 256, 0, s>>>(b->q_item.as<int>(), b->q_anchor.as<int>(), stride, n_s,
                                                     b->s_item.as<int>(), b->s_anchor.as<int>());
    double best = 1e300;
    size_t best_i = 0;
    for (size_t i = 0; i < cands.size(); ++i) {
      if (int rc = apply(cands[i])) return rc;
      KArgs probe = a;
      probe.q_item = b->s_item.as<int>();
      probe.q_anchor = b->s_anchor.as<int>();
      probe.n_work = n_s;
      probe.stats = nullptr;
      probe.xq = nullptr;  // settle in place: nothing outlives the probe
      probe.cell_work = nullptr;
      probe.self = b->args_probe.as<KArgs>();
      CU(cudaMemcpy(b->args_probe.p, &probe, sizeof(KArgs), cudaMemcpyHostToDevice));
      double t_best = 1e300;
      for (int rep = 0; rep < 2; ++rep) {
        CU(cudaMemsetAsync(b->hist.p, 0, b->n_items * hist_words(b) * sizeof(unsigned long long), s));
        CU(cudaMemsetAsync(b->work.p, 0, sizeof(int), s));
        CU(cudaEventRecord(b->ev[1], s));
        CU(launch_triangles(probe, h->survey != 0, b->sym, b->weighted, b->hg, std::min(b->grid, n_s), b->smem, s,
                            true));
        CU(cudaEventRecord(b->ev[2], s));
        CU(cudaEventSynchronize(b->ev[2]));
        float ms = 0.0f;
        CU(cudaEventElapsedTime(&ms, b->ev[1], b->ev[2]));
        t_best = std::min(t_best, static_cast<double>(ms));
      }
      if (t_best < best) {
        best = t_best;
        best_i = i;
      }
    }
    if (int rc = apply(cands[best_i])) return rc;
  }
  // The launch that the graph records sets no attribute: the occupancy query
  // sets the kernel's shared-memory limit to the chosen size.
  if (triangles_occupancy(h->survey != 0, b->sym, b->weighted, b->hg, b->smem) <= 0)
    return fail(NCORR_ERR_CUDA, "triangle kernel does not fit on the device, or a 27-cell neighbourhood holds "
                                  "more than 2^24 points");
  CU(cudaStreamSynchronize(s));
  b->st.ms_autotune = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();

  // Capture the whole count.
  CU(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  int rc = enqueue_grid(b);
  if (!rc) rc = enqueue_count(b, false);
  cudaGraph_t graph = nullptr;
  const cudaError_t ec = cudaStreamEndCapture(s, &graph);
  if (rc) {
    if (graph) cudaGraphDestroy(graph);
    return rc;
  }
  if (ec != cudaSuccess) return fail(NCORR_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ec));
  b->graph = graph;
  CU(cudaGraphInstantiate(&b->exec, graph, 0));
  size_t n_nodes = 0;
  cudaGraphGetNodes(graph, nullptr, &n_nodes);
  b->st.graph_nodes = static_cast<int>(n_nodes);
  b->st.sub_j = a.sub_j;
  b->st.hist_copies = a.hist_copies;
  b->st.grid_ctas = b->grid;
  b->st.weighted = b->weighted ? 1 : 0;
  b->st.n_work = static_cast<uint64_t>(b->n_work);
  return NCORR_OK;
}

}  // namespace

extern "C" {

void ncorr_batch_destroy(ncorr_batch* b) {
  if (!b) return;
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  for (DevBuf* d : {&b->in, &b->cid, &b->pd, &b->pq, &b->pc, &b->count, &b->start, &b->cursor, &b->flags, &b->wmax,
                    &b->bound, &b->items, &b->hist, &b->out, &b->total, &b->item_off, &b->q_item, &b->q_anchor,
                    &b->s_item, &b->s_anchor, &b->work, &b->stats, &b->xq, &b->xq_count, &b->slab_e,
                    &b->slab_w, &b->slab_q, &b->slab_x, &b->args, &b->args_probe, &b->table, &b->feats})
    d->release();
  b->order.release();
  for (double* p : {b->h_out})
    if (p) cudaFreeHost(p);
  if (b->h_flags) cudaFreeHost(b->h_flags);
  if (b->h_stats) cudaFreeHost(b->h_stats);
  if (b->h_total) cudaFreeHost(b->h_total);
  for (size_t c = 0; c < b->registered.size(); ++c)
    if (b->registered[c]) cudaHostUnregister(const_cast<double*>(b->cat_src[c]));
  for (auto& e : b->ev)
    if (e) cudaEventDestroy(e);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

int ncorr_batch_create(ncorr_handle* h, int n_items, const double* const* p1, const int64_t* n1,
                       const double* const* p2, const int64_t* n2, const double* const* p3, const int64_t* n3,
                       int on_device, int autotune, ncorr_batch** out) {
  auto t0 = std::chrono::steady_clock::now();
  if (!out) return fail(NCORR_ERR_INVALID_ARGUMENT, "null output pointer");
  *out = nullptr;
  if (!h) return fail(NCORR_ERR_INVALID_ARGUMENT, "null handle");
  if (h->bin_type != NCORR_BIN_THREED)
    return fail(NCORR_ERR_NOT_IMPLEMENTED, "batches are implemented for the threeD bin type");
  if (n_items < 1 || n_items > (1 << 20) || !p1 || !n1 || !p2 || !n2 || !p3 || !n3)
    return fail(NCORR_ERR_INVALID_ARGUMENT, "bad batch arrays");
  cudaGetLastError();
  ncorr_batch* b = new ncorr_batch();
  std::memset(&b->st, 0, sizeof(b->st));
  b->h = h;
  b->n_items = n_items;
  b->on_device = on_device != 0;
  auto bail = [&](int rc) {
    ncorr_batch_destroy(b);
    return rc;
  };
  const double* const* ps[3] = {p1, p2, p3};
  const int64_t* ns[3] = {n1, n2, n3};
  int64_t total = 0;
  for (int i = 0; i < n_items; ++i) {
    for (int r = 0; r < 3; ++r) {
      const double* p = ps[r][i];
      const int64_t n = ns[r][i];
      if (int rc = validate_catalog_ptr(p, n)) return bail(rc);
      if (b->on_device && p && (reinterpret_cast<uintptr_t>(p) & 15u))
        return bail(fail(NCORR_ERR_INVALID_ARGUMENT, "device catalogues must be 16-byte aligned"));
      int c = -1;
      for (int q = 0; q < b->n_cats; ++q)
        if (b->cat_src[q] == p && b->cat_n[q] == n) c = q;
      if (c < 0) {
        c = b->n_cats++;
        b->cat_src.push_back(p);
        b->cat_n.push_back(n);
        b->cat_off.push_back(total);
        total += n;
      }
      b->role[r].push_back(c);
    }
    if (n1[i] > 0 && total > (int64_t(1) << 30))
      return bail(fail(NCORR_ERR_INVALID_ARGUMENT, "batch larger than 2^30 points"));
  }
  // All items visit pairs the same way (one kernel variant per launch).
  b->sym = b->role[1][0] == b->role[2][0];
  for (int i = 1; i < n_items; ++i)
    if ((b->role[1][i] == b->role[2][i]) != b->sym)
      return bail(fail(NCORR_ERR_INVALID_ARGUMENT, "items must all have p2 == p3, or all p2 != p3"));
  int64_t n_work = 0;
  for (int i = 0; i < n_items; ++i) n_work += n1[i];
  if (n_work >= (int64_t(1) << 31)) return bail(fail(NCORR_ERR_INVALID_ARGUMENT, "more than 2^31 anchors"));
  if (h->sched_mode == NCORR_SCHED_LEARNED && (static_cast<int64_t>(n_items) * h->ncell >= (int64_t(1) << 31)))
    return bail(fail(NCORR_ERR_INVALID_ARGUMENT, "too many (item, cell) pairs for the learned queue"));
  cudaSetDevice(h->device);
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess)
    return bail(fail(NCORR_ERR_CUDA, "cudaStreamCreate failed"));
  for (auto& e : b->ev)
    if (cudaEventCreate(&e) != cudaSuccess) return bail(fail(NCORR_ERR_CUDA, "cudaEventCreate failed"));
  // Host arrays are page-locked in place so the graph copies them directly.
  b->registered.assign(b->n_cats, 0);
  if (!b->on_device)
    for (int c = 0; c < b->n_cats; ++c) {
      if (b->cat_n[c] == 0) continue;
      const cudaError_t e = cudaHostRegister(const_cast<double*>(b->cat_src[c]),
                                             b->cat_n[c] * sizeof(double4_16a), cudaHostRegisterDefault);
      if (e == cudaSuccess) {
        b->registered[c] = 1;
      } else if (e == cudaErrorHostMemoryAlreadyRegistered) {
        cudaGetLastError();
      } else {
        cudaGetLastError();
        return bail(fail(NCORR_ERR_CUDA, std::string("cudaHostRegister: ") + cudaGetErrorString(e)));
      }
    }
  if (int rc = plan(b, autotune)) return bail(rc);
  b->st.n_items = n_items;
  b->st.n_catalogues = b->n_cats;
  b->st.ms_plan = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  *out = b;
  return NCORR_OK;
}

int ncorr_batch_run(ncorr_batch* b, void* stream) {
  if (!b) return fail(NCORR_ERR_INVALID_ARGUMENT, "null batch");
  cudaGetLastError();
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : b->stream;
  CU(cudaEventRecord(b->ev[0], s));
  CU(cudaGraphLaunch(b->exec, s));
  CU(cudaEventRecord(b->ev[3], s));
  CU(cudaStreamSynchronize(s));
  for (int c = 0; c < b->n_cats; ++c) {
    const int f = b->h_flags[c];
    if (f & kFlagNonFinite) return fail(NCORR_ERR_OUT_OF_GRID, "non-finite coordinate or weight");
    if (f & kFlagOutOfGrid) return fail(NCORR_ERR_OUT_OF_GRID, "a point lies outside the cell grid of the box");
  }
  const int kf = b->h_flags[b->n_cats];
  if (kf & kFlagSchedStall) return fail(NCORR_ERR_CUDA, "triangle kernel: histogram binding wait timed out");
  if (kf & (kFlagListOverflow | kFlagPlanStale))
    return fail(NCORR_ERR_CAPACITY, "the catalogues no longer fit the batch plan (weights or neighbourhood "
                                    "density grew): create the batch again");
  float ms = 0.0f, msc = -1.0f;
  CU(cudaEventElapsedTime(&ms, b->ev[0], b->ev[3]));
  if (cudaEventElapsedTime(&msc, b->ev[1], b->ev[2]) != cudaSuccess) {
    cudaGetLastError();  // no kernel time on this driver: report -1, leave no error behind
    msc = -1.0f;
  }
  b->st.ms_run = ms;
  b->st.ms_count = msc;
  b->st.n_pairs = b->h_stats[3];
  b->st.n_pair_evals = b->h_stats[4];
  uint64_t tri = 0;
  for (int i = 0; i < b->n_items; ++i) tri += b->h_total[i];
  b->st.triangles = b->weighted ? 0 : tri;
  return NCORR_OK;
}

int ncorr_batch_get_counts_all(const ncorr_batch* b, int item, double* out, int64_t cap) {
  if (!b) return fail(NCORR_ERR_INVALID_ARGUMENT, "null batch");
  const int64_t nbin = static_cast<int64_t>(b->h->nb) * b->h->nb * b->h->nb;
  if (item < 0 || item >= b->n_items) return fail(NCORR_ERR_INVALID_ARGUMENT, "item out of range");
  if (!out || cap < nbin) return fail(NCORR_ERR_INVALID_ARGUMENT, "output too small");
  std::memcpy(out, b->h_out + item * nbin, nbin * sizeof(double));
  return NCORR_OK;
}

int ncorr_batch_get_stats(const ncorr_batch* b, ncorr_batch_stats* out) {
  if (!b || !out) return fail(NCORR_ERR_INVALID_ARGUMENT, "null argument");
  *out = b->st;
  return NCORR_OK;
}

}  // extern "C"
