// C ABI of the engine (include/ncorr_gb300.h): handle life cycle, host
// orchestration of one calculateD1D2D3, result compaction.
#include <mutex>
#include <new>
#include <stdexcept>

#include "host.cuh"

using namespace ncorr_gb300;
using namespace ncorr_host;

namespace ncorr_host {
thread_local std::string t_err;
}  // namespace ncorr_host

namespace {

void compact(ncorr_handle* h) {
  const int nb = h->nb;
  h->counts_out.clear();
  for (int i = 0; i < nb; ++i)
    for (int j = i; j < nb; ++j)
      for (int k = j; k < nb; ++k)
        if (h->mids[k] <= h->mids[i] + h->mids[j])
          h->counts_out.push_back(h->counts_all[k + j * nb + i * nb * nb]);
}

int run(ncorr_handle* h, const double4_16a* d1, int n1, const double4_16a* d2, int n2, const double4_16a* d3,
        int n3, cudaStream_t st, const void* key1, const void* key2, const void* key3) {
  auto t0 = std::chrono::steady_clock::now();
  cudaGetLastError();  // clear any error left by an earlier failed call
  // Distinct catalogues: identical inputs are gridded once.
  int role[3];
  role[0] = 0;
  role[1] = (key2 == key1 && n2 == n1) ? 0 : 1;
  if (key3 == key2 && n3 == n2)
    role[2] = role[1];
  else if (key3 == key1 && n3 == n1)
    role[2] = 0;
  else
    role[2] = 2;
  const bool sym = role[1] == role[2];
  const double4_16a* src[3] = {d1, d2, d3};
  const int ns[3] = {n1, n2, n3};

  CU(h->d_flags.ensure(8 * sizeof(int)));
  CU(h->d_wmax.ensure(sizeof(unsigned)));
  CU(h->d_work.ensure(sizeof(int)));
  CU(h->d_bound.ensure(2 * sizeof(int)));
  CU(h->d_stats.ensure(8 * sizeof(unsigned long long)));
  CU(h->d_total.ensure(sizeof(unsigned long long)));
  CU(cudaMemsetAsync(h->d_flags.p, 0, 8 * sizeof(int), st));
  CU(cudaMemsetAsync(h->d_wmax.p, 0, sizeof(unsigned), st));
  CU(cudaMemsetAsync(h->d_bound.p, 0, 2 * sizeof(int), st));
  CU(cudaMemsetAsync(h->d_stats.p, 0, 8 * sizeof(unsigned long long), st));
  CU(cudaMemsetAsync(h->d_total.p, 0, sizeof(unsigned long long), st));

  CU(cudaEventRecord(h->ev[0], st));
  bool done[3] = {false, false, false};
  for (int r = 0; r < 3; ++r) {
    int ci = role[r];
    if (done[ci]) continue;
    done[ci] = true;
    int rc = grid_catalog(h, ci, src[r], ns[r], st);
    if (rc) return rc;
  }
  launch_nbr_bound(h->cat[role[1]].count.as<int>(), h->g, h->d_bound.as<int>(), st);
  if (!sym) launch_nbr_bound(h->cat[role[2]].count.as<int>(), h->g, h->d_bound.as<int>() + 1, st);
  CU(cudaGetLastError());
  CU(cudaEventRecord(h->ev[1], st));

  int flags[8];
  unsigned wmax_bits = 0;
  int bound[2] = {0, 0};
  CU(cudaMemcpyAsync(flags, h->d_flags.p, sizeof(flags), cudaMemcpyDeviceToHost, st));
  CU(cudaMemcpyAsync(&wmax_bits, h->d_wmax.p, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
  CU(cudaMemcpyAsync(bound, h->d_bound.p, sizeof(bound), cudaMemcpyDeviceToHost, st));
  CU(cudaStreamSynchronize(st));
  bool weighted = false;
  for (int r = 0; r < 3; ++r) {
    const int f = flags[role[r]];
    if (f & kFlagNonFinite) return fail(NCORR_ERR_OUT_OF_GRID, "non-finite coordinate or weight");
    if (f & kFlagOutOfGrid)
      return fail(NCORR_ERR_OUT_OF_GRID,
                  "a point lies outside the cell grid of the box (the reference would index out of bounds)");
    if (f & kFlagWeighted) weighted = true;
  }
  if (h->survey && (flags[role[0]] & kFlagSurveyFace))
    return fail(NCORR_ERR_OUT_OF_GRID,
                "survey anchor on the upper face of the cell grid (unclamped cell index == nc)");

  // Fixed-point scale for weighted sums: |w1*w2*w3| * scale <= 2^30.
  float wscale = 1.0f;
  if (weighted) {
    float wmax = 0.0f;
    std::memcpy(&wmax, &wmax_bits, sizeof(float));
    double p3 = static_cast<double>(wmax) * wmax * wmax;
    int e = 0;
    if (p3 > 0) e = static_cast<int>(std::floor(std::log2(std::ldexp(1.0, 30) / p3)));
    e = std::max(-120, std::min(120, e));
    wscale = static_cast<float>(std::ldexp(1.0, e));
  }

  // Count each triangle once for all six orderings when the three catalogues
  // are one and the geometry makes every triangle's vertices see each other
  // through bit-identical differences: survey mode, or a box divided exactly
  // into >= 4 cells per axis; plus every point exactly inside its cell and,
  // in a box, exact +-box images (kFlagNoSym6).
  bool sym6 = sym && role[0] == role[1] && !(flags[role[0]] & kFlagNoSym6);
  if (sym6 && !h->survey)
    for (int d = 0; d < 3; ++d)
      if (h->g.nc[d] < 4 || __builtin_fma(-static_cast<double>(h->g.nc[d]), h->g.cell, h->box[d]) != 0.0)
        sym6 = false;

  // CTA histogram in shared memory when it fits; a bin's byte stride is
  // encoded in the table codes (u8).
  const int nbin = h->nb * h->nb * h->nb;
  const int elem = weighted ? 8 : 4;
  const bool hg = hist_global(h->nb, elem);
  const int code_scale = hg ? 1 : elem;
  if (h->table_scale != code_scale) {
    build_table(h->g, code_scale, h->table);
    CU(h->d_table.ensure(h->table.size()));
    CU(cudaMemcpyAsync(h->d_table.p, h->table.data(), h->table.size(), cudaMemcpyHostToDevice, st));
    h->table_scale = code_scale;
  }

  // Launch shape (histogram copies that fit, shared memory, grid) and the
  // per-warp slabs: neighbour lists sized by the largest 27-cell occupancy,
  // careful queues, exact buffers.
  int nsm = 0;
  CU(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, h->device));
  TriShape shp;
  if (!tri_shape(h->nb, h->survey != 0, sym, weighted, hg, h->hist_copies, nsm, n1, bound[0], bound[1], &shp))
    return fail(NCORR_ERR_CUDA, "triangle kernel does not fit on the device, or a 27-cell neighbourhood holds "
                                "more than 2^24 points");
  const size_t slab_n = tri_slab_entries(shp);
  CU(h->slab_e.ensure(slab_n * sizeof(ListEnt)));
  if (weighted) CU(h->slab_w.ensure(slab_n * sizeof(float)));
  CU(h->slab_q.ensure(static_cast<size_t>(shp.grid) * kWarps * kQueueCap * sizeof(unsigned long long)));
  CU(h->slab_x.ensure(static_cast<size_t>(shp.grid) * kWarps * 32 * sizeof(ExactEntry)));
  CU(h->cta_time.ensure(static_cast<size_t>(shp.grid) * 2 * sizeof(unsigned long long)));

  const size_t hist_words = weighted ? 2 * static_cast<size_t>(nbin) : static_cast<size_t>(nbin);
  CU(h->d_hist.ensure(hist_words * sizeof(unsigned long long)));
  CU(cudaMemsetAsync(h->d_hist.p, 0, hist_words * sizeof(unsigned long long), st));
  CU(cudaMemsetAsync(h->d_work.p, 0, sizeof(int), st));
  CU(h->d_out.ensure(nbin * sizeof(double)));

  // The call is a batch of one item.
  BatchItem it;
  std::memset(&it, 0, sizeof(it));
  it.c1 = view(h->cat[role[0]]);
  it.c2 = view(h->cat[role[1]]);
  it.c3 = view(h->cat[role[2]]);
  it.hist.counts = weighted ? nullptr : h->d_hist.as<unsigned long long>();
  it.hist.wsum = weighted ? h->d_hist.as<unsigned long long>() : nullptr;
  it.out = h->d_out.as<double>();
  it.total = h->d_total.as<unsigned long long>();
  it.flags1 = h->d_flags.as<int>() + role[0];
  it.sym6_ok = sym6 ? 1 : 0;
  it.cell_base = 0;
  CU(h->d_items.ensure(sizeof(BatchItem)));
  CU(cudaMemcpyAsync(h->d_items.p, &it, sizeof(it), cudaMemcpyHostToDevice, st));

  KArgs a;
  std::memset(&a, 0, sizeof(a));
  a.g = h->g;
  a.items = h->d_items.as<BatchItem>();
  a.n_items = 1;
  a.n_work = n1;
  a.q_item = nullptr;
  a.q_anchor = nullptr;
  a.sched_static = h->sched_mode == NCORR_SCHED_STATIC ? 1 : 0;
  a.sub_j = h->sub_j;
  a.hist_copies = shp.copies;
  a.cell_work = nullptr;
  const bool need_feats = h->record_work || h->sched_mode == NCORR_SCHED_LEARNED;
  if (need_feats) {
    CU(h->d_feats.ensure(static_cast<size_t>(h->ncell) * kMlpIn * sizeof(float)));
    launch_cell_features(a.items, 1, h->g, h->d_feats.as<float>(), st);
  }
  if (h->sched_mode == NCORR_SCHED_LEARNED && n1 > 0) {
    // Cells heaviest first, as the work model predicts them.
    OrderScratch os;
    CU(h->order.ensure(1, h->ncell, &os));
    CU(h->q_item.ensure(static_cast<size_t>(n1) * sizeof(int)));
    CU(h->q_anchor.ensure(static_cast<size_t>(n1) * sizeof(int)));
    launch_mlp_predict(h->sched_model->params.as<float>(), h->d_feats.as<float>(), static_cast<int>(h->ncell),
                       os.pred, st, h->sched_model->bf16);
    launch_learned_queue(a.items, 1, static_cast<int>(h->ncell), os, h->q_item.as<int>(), h->q_anchor.as<int>(),
                         st);
    a.q_item = h->q_item.as<int>();
    a.q_anchor = h->q_anchor.as<int>();
  }
  if (h->record_work) {
    CU(h->d_cell_work.ensure(static_cast<size_t>(h->ncell) * sizeof(unsigned long long)));
    CU(cudaMemsetAsync(h->d_cell_work.p, 0, static_cast<size_t>(h->ncell) * sizeof(unsigned long long), st));
    a.cell_work = h->d_cell_work.as<unsigned long long>();
  }
  a.table = h->d_table.as<unsigned char>();
  a.work = h->d_work.as<int>();
  a.flags = h->d_flags.as<int>() + 4;
  a.slab_e = h->slab_e.as<ListEnt>();
  a.slab_w = weighted ? h->slab_w.as<float>() : nullptr;
  a.slab_q = h->slab_q.as<unsigned long long>();
  a.slab_x = h->slab_x.as<ExactEntry>();
  a.kcap2 = shp.kcap2;
  a.kcap3 = shp.kcap3;
  a.cta_time = h->cta_time.as<unsigned long long>();
  a.code_scale = code_scale;
  a.wscale = wscale;
  a.stats = h->d_stats.as<unsigned long long>();
  // Deferred exact candidates: about one in 10^4 candidates at the clustered
  // 2M-point workload; beyond the capacity they are settled in place.
  CU(h->xq.ensure(static_cast<size_t>(std::max(h->xq_cap, 1u)) * sizeof(ExactEntry)));
  CU(h->xq_count.ensure(sizeof(unsigned)));
  CU(cudaMemsetAsync(h->xq_count.p, 0, sizeof(unsigned), st));
  a.xq = h->xq.as<ExactEntry>();
  a.xq_count = h->xq_count.as<unsigned>();
  a.xq_cap = h->xq_cap;

  CU(h->d_args.ensure(sizeof(KArgs)));
  a.self = h->d_args.as<KArgs>();
  CU(cudaMemcpyAsync(h->d_args.p, &a, sizeof(KArgs), cudaMemcpyHostToDevice, st));
  CU(cudaEventRecord(h->ev[2], st));
  if (n1 > 0) CU(launch_triangles(a, h->survey != 0, sym, weighted, hg, shp.grid, shp.smem, st));
  if (n1 > 0) launch_exact(a, h->survey != 0, weighted, nsm * 4, st);
  CU(cudaEventRecord(h->ev[3], st));
  launch_fold(a.items, 1, h->nb, weighted, sym, 1.0 / wscale, st);
  CU(cudaGetLastError());
  h->counts_all.assign(nbin, 0.0);
  if (h->record_work) {
    h->rec_feats.resize(static_cast<size_t>(h->ncell) * kMlpIn);
    std::vector<unsigned long long> w(h->ncell);
    CU(cudaMemcpyAsync(h->rec_feats.data(), h->d_feats.p, h->rec_feats.size() * sizeof(float),
                       cudaMemcpyDeviceToHost, st));
    CU(cudaMemcpyAsync(w.data(), h->d_cell_work.p, w.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                       st));
    CU(cudaStreamSynchronize(st));
    h->rec_work.assign(w.begin(), w.end());
  }
  unsigned long long st_host[8];
  unsigned long long total = 0;
  int kflags = 0;
  std::vector<unsigned long long> cta_t(static_cast<size_t>(shp.grid) * 2, 0ull);
  if (n1 > 0)
    CU(cudaMemcpyAsync(cta_t.data(), h->cta_time.p, cta_t.size() * sizeof(unsigned long long),
                       cudaMemcpyDeviceToHost, st));
  CU(cudaMemcpyAsync(h->counts_all.data(), h->d_out.p, nbin * sizeof(double), cudaMemcpyDeviceToHost, st));
  CU(cudaMemcpyAsync(st_host, h->d_stats.p, sizeof(st_host), cudaMemcpyDeviceToHost, st));
  CU(cudaMemcpyAsync(&total, h->d_total.p, sizeof(total), cudaMemcpyDeviceToHost, st));
  CU(cudaMemcpyAsync(&kflags, h->d_flags.as<int>() + 4, sizeof(int), cudaMemcpyDeviceToHost, st));
  cudaEvent_t ev_end;
  CU(cudaEventCreate(&ev_end));
  CU(cudaEventRecord(ev_end, st));
  CU(cudaStreamSynchronize(st));
  if (kflags & kFlagListOverflow) return fail(NCORR_ERR_CAPACITY, "neighbour list overflow");
  if (kflags & kFlagSchedStall) return fail(NCORR_ERR_CUDA, "triangle kernel: histogram binding wait timed out");
  float ms0 = 0, ms1 = 0, ms2 = 0;
  cudaEventElapsedTime(&ms0, h->ev[0], h->ev[1]);
  cudaEventElapsedTime(&ms1, h->ev[2], h->ev[3]);
  cudaEventElapsedTime(&ms2, h->ev[3], ev_end);
  cudaEventDestroy(ev_end);
  compact(h);
  auto t1 = std::chrono::steady_clock::now();
  ncorr_stats& s = h->stats;
  s.ms_grid = ms0;
  s.ms_count = ms1;
  s.ms_fold = ms2;
  s.ms_total = std::chrono::duration<double, std::milli>(t1 - t0).count();
  s.n_exact_tris = st_host[0];
  s.n_exact_pairs = st_host[1];
  s.n_anchors = st_host[2];
  s.n_pairs = st_host[3];
  s.n_pair_evals = st_host[4];
  s.n_flagged_rows = st_host[5];
  s.n_queued = st_host[6];
  s.triangles = weighted ? 0 : total;
  s.weighted = weighted ? 1 : 0;
  s.symmetric = sym6 ? 6 : (sym ? 2 : 1);
  s.grid_ctas = shp.grid;
  s.list_capacity = shp.kcap2;
  s.tail_idle = n1 > 0 ? tail_idle_fraction(cta_t, shp.grid) : 0.0;
  return NCORR_OK;
}

}  // namespace

extern "C" {

const char* ncorr_last_error(void) { return t_err.c_str(); }

int ncorr_create(const double box[3], int bin_type, const double* edges, int n_edges, int is_survey,
                 const double ori[3], ncorr_handle** out) {
  if (!out) return fail(NCORR_ERR_INVALID_ARGUMENT, "null handle pointer");
  *out = nullptr;
  if (bin_type != NCORR_BIN_THREED)
    return fail(NCORR_ERR_INVALID_ARGUMENT, "Invalid constructor call for bin_type.");
  if (!box || !edges) return fail(NCORR_ERR_INVALID_ARGUMENT, "null box or edges");
  if (n_edges < 2 || n_edges > kMaxEdges)
    return fail(NCORR_ERR_INVALID_ARGUMENT, "need 2..128 bin edges");
  for (int i = 0; i < n_edges; ++i)
    if (!std::isfinite(edges[i])) return fail(NCORR_ERR_INVALID_ARGUMENT, "non-finite bin edge");
  if (edges[0] < 0.0) return fail(NCORR_ERR_INVALID_ARGUMENT, "negative first bin edge");
  for (int i = 1; i < n_edges; ++i)
    if (!(edges[i] > edges[i - 1]) || !(edges[i] * edges[i] > edges[i - 1] * edges[i - 1]))
      return fail(NCORR_ERR_INVALID_ARGUMENT, "bin edges must be strictly increasing");
  for (int d = 0; d < 3; ++d)
    if (!(box[d] > 0.0) || !std::isfinite(box[d]))
      return fail(NCORR_ERR_INVALID_ARGUMENT, "box sides must be positive");
  int dev_count = 0;
  if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count <= 0)
    return fail(NCORR_ERR_NO_DEVICE, "no CUDA device");

  ncorr_handle* h = new ncorr_handle();
  h->survey = is_survey ? 1 : 0;
  for (int d = 0; d < 3; ++d) {
    h->box[d] = box[d];
    h->ori[d] = ori ? ori[d] : 0.0;
  }
  h->edges.assign(edges, edges + n_edges);
  h->nb = n_edges - 1;
  for (int i = 1; i < n_edges; ++i) h->mids.push_back((edges[i] + edges[i - 1]) / 2.0);
  Geom& g = h->g;
  std::memset(&g, 0, sizeof(g));
  g.nb = h->nb;
  g.survey = h->survey;
  g.fma_pattern = kDefaultFmaPattern;
  const double rmax = edges[n_edges - 1], rmin = edges[0];
  g.cell = rmax;
  g.sqr_rmax = rmax * rmax;
  g.sqr_rmin = rmin * rmin;
  long ncell = 1;
  for (int d = 0; d < 3; ++d) {
    g.box[d] = box[d];
    double n = std::ceil(box[d] / rmax);
    if (n > 4096.0) {
      delete h;
      return fail(NCORR_ERR_INVALID_ARGUMENT, "cell grid too large (box/r_max > 4096)");
    }
    g.nc[d] = static_cast<int>(n);
    ncell *= g.nc[d];
  }
  if (ncell > (1L << 26)) {
    delete h;
    return fail(NCORR_ERR_INVALID_ARGUMENT, "cell grid too large (more than 2^26 cells)");
  }
  h->ncell = ncell;
  for (int i = 0; i < n_edges; ++i) {
    g.sqr_bins[i] = edges[i] * edges[i];
    g.e2lo[i] = f32_down(g.sqr_bins[i]);
    g.e2hi[i] = f32_up(g.sqr_bins[i]);
  }
  set_error_model(g);
  // Bin mids and the compacted (r1,r2,r3) table (source/cudaNcorr.cu:145-154).
  for (int i = 0; i < h->nb; ++i)
    for (int j = i; j < h->nb; ++j)
      for (int k = j; k < h->nb; ++k)
        if (h->mids[k] <= h->mids[i] + h->mids[j]) {
          h->tri_bins_out.push_back(h->mids[i]);
          h->tri_bins_out.push_back(h->mids[j]);
          h->tri_bins_out.push_back(h->mids[k]);
          h->counts_out.push_back(0.0);
        }
  h->counts_all.assign(static_cast<size_t>(h->nb) * h->nb * h->nb, 0.0);
  std::memset(&h->stats, 0, sizeof(h->stats));
  // Capacity of the deferred exact queue; NCORR_EXACT_QUEUE_CAP overrides it
  // (0 settles every uncertain candidate in place).
  h->xq_cap = kExactQueueCap;
  if (const char* env = std::getenv("NCORR_EXACT_QUEUE_CAP")) h->xq_cap = static_cast<unsigned>(std::strtoul(env, nullptr, 10));
  cudaGetDevice(&h->device);
  cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
  for (int i = 0; i < 4 && e == cudaSuccess; ++i) e = cudaEventCreate(&h->ev[i]);
  if (e != cudaSuccess) {
    ncorr_destroy(h);
    return fail(NCORR_ERR_CUDA, std::string("stream/event creation: ") + cudaGetErrorString(e));
  }
  *out = h;
  return NCORR_OK;
}

int ncorr_create_rppi(const double box[3], int bin_type, const double* edges, int n_edges,
                      int num_minor_bins, int is_survey, const double ori[3], ncorr_handle** out) {
  if (!out) return fail(NCORR_ERR_INVALID_ARGUMENT, "null handle pointer");
  *out = nullptr;
  if (bin_type != NCORR_BIN_RPPI)
    return fail(NCORR_ERR_INVALID_ARGUMENT, "Invalid constructor call for bin_type.");
  if (!box || !edges) return fail(NCORR_ERR_INVALID_ARGUMENT, "null box or edges");
  if (n_edges < 2 || n_edges > kMaxEdges)
    return fail(NCORR_ERR_INVALID_ARGUMENT, "need 2..128 bin edges");
  for (int i = 0; i < n_edges; ++i)
    if (!std::isfinite(edges[i])) return fail(NCORR_ERR_INVALID_ARGUMENT, "non-finite bin edge");
  if (edges[0] < 0.0) return fail(NCORR_ERR_INVALID_ARGUMENT, "negative first bin edge");
  for (int i = 1; i < n_edges; ++i)
    if (!(edges[i] > edges[i - 1]) || !(edges[i] * edges[i] > edges[i - 1] * edges[i - 1]))
      return fail(NCORR_ERR_INVALID_ARGUMENT, "bin edges must be strictly increasing");
  // The reference builds piBins_ = 0, 1, ..., numMinorBins and throws when
  // their count disagrees (source/cudaNcorr.cu:174-180); with fewer than one
  // pi bin its z cell would be 0 wide.
  if (num_minor_bins < 1 || num_minor_bins > 4096)
    return fail(NCORR_ERR_INVALID_ARGUMENT, "numMinorBins must be 1..4096");
  for (int d = 0; d < 3; ++d)
    if (!(box[d] > 0.0) || !std::isfinite(box[d]))
      return fail(NCORR_ERR_INVALID_ARGUMENT, "box sides must be positive");
  int dev_count = 0;
  if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count <= 0)
    return fail(NCORR_ERR_NO_DEVICE, "no CUDA device");
  ncorr_handle* h = new ncorr_handle();
  h->bin_type = NCORR_BIN_RPPI;
  h->survey = is_survey ? 1 : 0;
  for (int d = 0; d < 3; ++d) {
    h->box[d] = box[d];
    h->ori[d] = ori ? ori[d] : 0.0;
  }
  h->edges.assign(edges, edges + n_edges);
  h->nb = n_edges - 1;
  for (int i = 1; i < n_edges; ++i) h->mids.push_back((edges[i] + edges[i - 1]) / 2.0);
  std::memset(&h->g, 0, sizeof(h->g));
  std::memset(&h->stats, 0, sizeof(h->stats));
  int rc;
  try {
    rc = rppi_init(h, box, edges, n_edges, num_minor_bins, is_survey, ori);
  } catch (const std::bad_alloc&) {
    rc = fail(NCORR_ERR_CAPACITY, "host memory exhausted (output tables of nb^3 * numMinorBins^2 entries)");
  }
  if (rc) {
    delete h;
    return rc;
  }
  cudaGetDevice(&h->device);
  cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
  for (int i = 0; i < 4 && e == cudaSuccess; ++i) e = cudaEventCreate(&h->ev[i]);
  if (e != cudaSuccess) {
    ncorr_destroy(h);
    return fail(NCORR_ERR_CUDA, std::string("stream/event creation: ") + cudaGetErrorString(e));
  }
  *out = h;
  return NCORR_OK;
}

void ncorr_destroy(ncorr_handle* h) {
  if (!h) return;
  for (auto& c : h->cat) {
    c.in.release();
    c.cid.release();
    c.count.release();
    c.start.release();
    c.cursor.release();
    c.pd.release();
    c.pq.release();
    c.pc.release();
  }
  for (DevBuf* b : {&h->d_table, &h->d_flags, &h->d_wmax, &h->d_work, &h->d_bound, &h->d_hist,
                    &h->d_out, &h->d_stats, &h->d_total, &h->slab_e,
                    &h->slab_w, &h->slab_q, &h->slab_x, &h->cta_time, &h->xq, &h->xq_count, &h->d_args, &h->d_items, &h->d_cell_work,
                    &h->d_feats, &h->q_item, &h->q_anchor, &h->rp_pos, &h->rp_ab, &h->rp_rel, &h->rp_meta, &h->rp_pw, &h->rp_tab})
    b->release();
  h->order.release();
  for (auto& e : h->ev)
    if (e) cudaEventDestroy(e);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
}

static int calculate_host(ncorr_handle* h, const double* p1, int64_t n1, const double* p2, int64_t n2,
                          const double* p3, int64_t n3) {
  if (!h) return fail(NCORR_ERR_INVALID_ARGUMENT, "null handle");
  int rc;
  if ((rc = validate_catalog_ptr(p1, n1)) || (rc = validate_catalog_ptr(p2, n2)) ||
      (rc = validate_catalog_ptr(p3, n3)))
    return rc;
  cudaStream_t st = h->stream;
  const double* src[3] = {p1, p2, p3};
  const int64_t ns[3] = {n1, n2, n3};
  const double4_16a* dev[3] = {nullptr, nullptr, nullptr};
  // Host -> device, each distinct array once.
  for (int r = 0; r < 3; ++r) {
    int same = -1;
    for (int q = 0; q < r; ++q)
      if (src[q] == src[r] && ns[q] == ns[r]) same = q;
    if (same >= 0) {
      dev[r] = dev[same];
      continue;
    }
    DevBuf& b = h->cat[r].in;
    CU(b.ensure(std::max<int64_t>(ns[r], 1) * sizeof(double4_16a)));
    if (ns[r] > 0)
      CU(cudaMemcpyAsync(b.p, src[r], ns[r] * sizeof(double4_16a), cudaMemcpyHostToDevice, st));
    dev[r] = b.as<double4_16a>();
  }
  if (h->bin_type == NCORR_BIN_RPPI)
    return rppi_run(h, dev[0], static_cast<int>(n1), dev[1], static_cast<int>(n2), dev[2], static_cast<int>(n3), st,
                    p1, p2, p3);
  return run(h, dev[0], static_cast<int>(n1), dev[1], static_cast<int>(n2), dev[2],
             static_cast<int>(n3), st, p1, p2, p3);
}

static int calculate_device(ncorr_handle* h, const double* d_p1, int64_t n1, const double* d_p2, int64_t n2,
                            const double* d_p3, int64_t n3, void* stream) {
  if (!h) return fail(NCORR_ERR_INVALID_ARGUMENT, "null handle");
  int rc;
  if ((rc = validate_catalog_ptr(d_p1, n1)) || (rc = validate_catalog_ptr(d_p2, n2)) ||
      (rc = validate_catalog_ptr(d_p3, n3)))
    return rc;
  for (const double* p : {d_p1, d_p2, d_p3})
    if (p && (reinterpret_cast<uintptr_t>(p) & 15u))
      return fail(NCORR_ERR_INVALID_ARGUMENT, "device catalogues must be 16-byte aligned");
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : h->stream;
  if (h->bin_type == NCORR_BIN_RPPI)
    return rppi_run(h, reinterpret_cast<const double4_16a*>(d_p1), static_cast<int>(n1),
                    reinterpret_cast<const double4_16a*>(d_p2), static_cast<int>(n2),
                    reinterpret_cast<const double4_16a*>(d_p3), static_cast<int>(n3), st, d_p1, d_p2, d_p3);
  return run(h, reinterpret_cast<const double4_16a*>(d_p1), static_cast<int>(n1),
             reinterpret_cast<const double4_16a*>(d_p2), static_cast<int>(n2),
             reinterpret_cast<const double4_16a*>(d_p3), static_cast<int>(n3), st, d_p1, d_p2, d_p3);
}

// Host allocations (result tables, read-back buffers) may throw; nothing
// throws across the C ABI.
int ncorr_calculate_d1d2d3(ncorr_handle* h, const double* p1, int64_t n1, const double* p2,
                           int64_t n2, const double* p3, int64_t n3) {
  try {
    return calculate_host(h, p1, n1, p2, n2, p3, n3);
  } catch (const std::bad_alloc&) {
    return fail(NCORR_ERR_CAPACITY, "host memory exhausted");
  } catch (const std::exception& e) {
    return fail(NCORR_ERR_INVALID_ARGUMENT, e.what());
  }
}

int ncorr_calculate_d1d2d3_device(ncorr_handle* h, const double* d_p1, int64_t n1,
                                  const double* d_p2, int64_t n2, const double* d_p3, int64_t n3,
                                  void* stream) {
  try {
    return calculate_device(h, d_p1, n1, d_p2, n2, d_p3, n3, stream);
  } catch (const std::bad_alloc&) {
    return fail(NCORR_ERR_CAPACITY, "host memory exhausted");
  } catch (const std::exception& e) {
    return fail(NCORR_ERR_INVALID_ARGUMENT, e.what());
  }
}

int64_t ncorr_num_out(const ncorr_handle* h) {
  return h ? static_cast<int64_t>(h->counts_out.size()) : 0;
}

int ncorr_num_bins(const ncorr_handle* h) { return h ? h->nb : 0; }

int ncorr_num_pi_bins(const ncorr_handle* h) { return (h && h->bin_type == NCORR_BIN_RPPI) ? h->rg.npi : 0; }

int ncorr_get_tri_bins_out(const ncorr_handle* h, double* out, int64_t cap) {
  if (!h || !out) return fail(NCORR_ERR_INVALID_ARGUMENT, "null argument");
  if (cap < static_cast<int64_t>(h->tri_bins_out.size()))
    return fail(NCORR_ERR_INVALID_ARGUMENT, "output capacity too small");
  std::memcpy(out, h->tri_bins_out.data(), h->tri_bins_out.size() * sizeof(double));
  return NCORR_OK;
}

int ncorr_get_pi_bins_out(const ncorr_handle* h, double* out, int64_t cap, int64_t* n) {
  if (!h) return fail(NCORR_ERR_INVALID_ARGUMENT, "null handle");
  const int64_t m = static_cast<int64_t>(h->pi_bins_out.size() / 2);
  if (n) *n = m;
  if (m == 0) return NCORR_OK;
  if (!out || cap < 2 * m) return fail(NCORR_ERR_INVALID_ARGUMENT, "output capacity too small");
  std::memcpy(out, h->pi_bins_out.data(), h->pi_bins_out.size() * sizeof(double));
  return NCORR_OK;
}

int ncorr_get_tri_counts_out(const ncorr_handle* h, double* out, int64_t cap) {
  if (!h || !out) return fail(NCORR_ERR_INVALID_ARGUMENT, "null argument");
  if (cap < static_cast<int64_t>(h->counts_out.size()))
    return fail(NCORR_ERR_INVALID_ARGUMENT, "output capacity too small");
  std::memcpy(out, h->counts_out.data(), h->counts_out.size() * sizeof(double));
  return NCORR_OK;
}

int ncorr_get_tri_counts_all(const ncorr_handle* h, double* out, int64_t cap) {
  if (!h || !out) return fail(NCORR_ERR_INVALID_ARGUMENT, "null argument");
  if (cap < static_cast<int64_t>(h->counts_all.size()))
    return fail(NCORR_ERR_INVALID_ARGUMENT, "output capacity too small");
  std::memcpy(out, h->counts_all.data(), h->counts_all.size() * sizeof(double));
  return NCORR_OK;
}

int ncorr_set_schedule(ncorr_handle* h, int mode, const ncorr_sched* model) {
  if (!h) return fail(NCORR_ERR_INVALID_ARGUMENT, "null handle");
  if (mode != NCORR_SCHED_DYNAMIC && mode != NCORR_SCHED_STATIC && mode != NCORR_SCHED_LEARNED)
    return fail(NCORR_ERR_INVALID_ARGUMENT, "unknown schedule");
  if (h->bin_type != NCORR_BIN_THREED && mode != NCORR_SCHED_DYNAMIC)
    return fail(NCORR_ERR_NOT_IMPLEMENTED, "the rppi kernel takes anchors from a dynamic counter only");
  if (mode == NCORR_SCHED_LEARNED && !model)
    return fail(NCORR_ERR_INVALID_ARGUMENT, "the learned schedule needs a model");
  if (model && model->device != h->device)
    return fail(NCORR_ERR_INVALID_ARGUMENT, "scheduler model belongs to another device");
  h->sched_mode = mode;
  h->sched_model = mode == NCORR_SCHED_LEARNED ? model : nullptr;
  return NCORR_OK;
}

int ncorr_set_tuning(ncorr_handle* h, int sub_j, int hist_copies) {
  if (!h) return fail(NCORR_ERR_INVALID_ARGUMENT, "null handle");
  if (sub_j != 8 && sub_j != 16 && sub_j != 32) return fail(NCORR_ERR_INVALID_ARGUMENT, "sub_j must be 8, 16 or 32");
  if (hist_copies != 1 && hist_copies != 2 && hist_copies != 4)
    return fail(NCORR_ERR_INVALID_ARGUMENT, "hist_copies must be 1, 2 or 4");
  h->sub_j = sub_j;
  h->hist_copies = hist_copies;
  return NCORR_OK;
}

int ncorr_set_record_work(ncorr_handle* h, int on) {
  if (!h) return fail(NCORR_ERR_INVALID_ARGUMENT, "null handle");
  if (h->bin_type != NCORR_BIN_THREED && on)
    return fail(NCORR_ERR_NOT_IMPLEMENTED, "work recording is implemented for the threeD bin type");
  h->record_work = on != 0;
  return NCORR_OK;
}

int64_t ncorr_num_cells(const ncorr_handle* h) { return h ? static_cast<int64_t>(h->ncell) : 0; }

int ncorr_get_cell_work(const ncorr_handle* h, float* feats, double* work, int64_t cap_cells) {
  if (!h) return fail(NCORR_ERR_INVALID_ARGUMENT, "null handle");
  if (h->rec_work.size() != static_cast<size_t>(h->ncell))
    return fail(NCORR_ERR_INVALID_ARGUMENT, "no recorded call (ncorr_set_record_work)");
  if (cap_cells < h->ncell) return fail(NCORR_ERR_INVALID_ARGUMENT, "output too small");
  if (feats) std::memcpy(feats, h->rec_feats.data(), h->rec_feats.size() * sizeof(float));
  if (work) std::memcpy(work, h->rec_work.data(), h->rec_work.size() * sizeof(double));
  return NCORR_OK;
}

int ncorr_get_stats(const ncorr_handle* h, ncorr_stats* out) {
  if (!h || !out) return fail(NCORR_ERR_INVALID_ARGUMENT, "null argument");
  *out = h->stats;
  return NCORR_OK;
}

static void minmax(const double* c, int64_t n, double mn[3], double mx[3]) {
  for (int64_t i = 0; i < n; ++i)
    for (int d = 0; d < 3; ++d) {
      const double v = c[4 * i + d];
      if (v < mn[d]) mn[d] = v;
      if (v > mx[d]) mx[d] = v;
    }
}

int survey_prep_cat2(double* c1, int64_t n1, double* c2, int64_t n2, double box[3], double ori[3]) {
  if (!box || !ori || (n1 > 0 && !c1) || (n2 > 0 && !c2) || n1 < 0 || n2 < 0)
    return fail(NCORR_ERR_INVALID_ARGUMENT, "null or negative argument");
  double mn[3], mx[3];
  for (int d = 0; d < 3; ++d) {
    mn[d] = std::numeric_limits<double>::max();
    mx[d] = std::numeric_limits<double>::lowest();
  }
  minmax(c1, n1, mn, mx);
  if (c2) minmax(c2, n2, mn, mx);
  for (int d = 0; d < 3; ++d) {
    box[d] = mx[d] - mn[d] + 1.0;
    ori[d] = -mn[d];
  }
  for (int64_t i = 0; i < n1; ++i)
    for (int d = 0; d < 3; ++d) c1[4 * i + d] -= mn[d];
  if (c2)
    for (int64_t i = 0; i < n2; ++i)
      for (int d = 0; d < 3; ++d) c2[4 * i + d] -= mn[d];
  return NCORR_OK;
}

int survey_prep_cat(double* cat, int64_t n, double box[3], double ori[3]) {
  return survey_prep_cat2(cat, n, nullptr, 0, box, ori);
}

// Gauss-Legendre nodes and weights on [-1, 1] by Newton iteration on P_n.
static void gauss_legendre(int n, std::vector<double>& x, std::vector<double>& w) {
  x.assign(n, 0.0);
  w.assign(n, 0.0);
  const double pi = 3.14159265358979323846;
  for (int i = 0; i < (n + 1) / 2; ++i) {
    double z = std::cos(pi * (i + 0.75) / (n + 0.5)), dp = 0.0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = 0.0;
      for (int k = 1; k <= n; ++k) {
        const double p2 = p1;
        p1 = p0;
        p0 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p2) / k;
      }
      dp = n * (z * p0 - p1) / (z * z - 1.0);
      const double dz = p0 / dp;
      z -= dz;
      if (std::fabs(dz) < 1e-16) break;
    }
    x[i] = -z;
    x[n - 1 - i] = z;
    w[i] = w[n - 1 - i] = 2.0 / ((1.0 - z * z) * dp * dp);
  }
}

// The 48-point Gauss-Legendre rule, built once on first use (a function-local
// static: its initialisation is thread-safe, so concurrent conversions share
// it without a race).
struct GaussLegendre48 {
  std::vector<double> x, w;
  GaussLegendre48() { gauss_legendre(48, x, w); }
};
static const GaussLegendre48& gl48() {
  static const GaussLegendre48 rule;
  return rule;
}

// Comoving distance in Mpc/h: (c/100) * integral_0^z dz' / E(z'),
// E(z) = sqrt(OmegaM (1+z)^3 + OmegaLambda) (source/survey.cu:17-37, where
// GSL's qags integrates to 1e-7 relative). The integral is taken in
// u = ln(1 + z'), dz' = (1 + z') du, whose integrand (1+z)/E(z) is smooth for
// every z > -1; 48-point Gauss-Legendre panels of width <= 0.25 in u keep
// the error near 1e-15 relative, with at most a few dozen panels for any
// finite z. A negative z gives the negative integral, as qags from 0 to z
// does; z <= -1 or a non-finite z gives NaN.
static double comoving_distance(double z, double om, double ol) {
  constexpr double c_over_100 = 299792.458 / 100.0;  // source/survey.cu:12, :36
  if (z == 0.0) return 0.0;
  if (!(z > -1.0) || !std::isfinite(z)) return std::numeric_limits<double>::quiet_NaN();
  const GaussLegendre48& gl = gl48();
  const double umax = std::log1p(z);
  const int panels = std::max(1, static_cast<int>(std::ceil(std::fabs(umax) / 0.25)));
  const double hw = umax / panels / 2.0;
  double s = 0.0;
  for (int p = 0; p < panels; ++p) {
    const double mid = (2 * p + 1) * hw;
    for (size_t k = 0; k < gl.x.size(); ++k) {
      const double a = std::exp(mid + hw * gl.x[k]);  // 1 + z'
      s += gl.w[k] * a / std::sqrt(om * a * a * a + ol);
    }
  }
  return c_over_100 * s * hw;
}

int survey_convert_coordinates(const double cosmo[3], const double* in, int64_t n, double* out) {
  if (!cosmo || n < 0 || (n > 0 && (!in || !out)))
    return fail(NCORR_ERR_INVALID_ARGUMENT, "null or negative argument");
  try {
    const double om = cosmo[1], ol = cosmo[2];
    const double deg = 3.14159265358979323846 / 180.0;
    for (int64_t i = 0; i < n; ++i) {
      const double ra = in[4 * i] * deg, dec = in[4 * i + 1] * deg, z = in[4 * i + 2], w = in[4 * i + 3];
      const double d = comoving_distance(z, om, ol);
      // source/survey.cu:48-50
      out[4 * i] = d * std::cos(dec) * std::cos(ra);
      out[4 * i + 1] = d * std::cos(dec) * std::sin(ra);
      out[4 * i + 2] = d * std::sin(dec);
      out[4 * i + 3] = w;
    }
  } catch (const std::bad_alloc&) {
    return fail(NCORR_ERR_CAPACITY, "host memory exhausted");
  } catch (const std::exception& e) {
    return fail(NCORR_ERR_INVALID_ARGUMENT, e.what());
  }
  return NCORR_OK;
}

int ncorr_logspace(double start, double end, int n, double* out) {
  if (!out || n < 2) return fail(NCORR_ERR_INVALID_ARGUMENT, "need n >= 2 and an output array");
  const double a = std::log10(start), b = std::log10(end);
  const double step = (b - a) / (n - 1);
  for (int i = 0; i < n; ++i) out[i] = std::pow(10, a + i * step);
  return NCORR_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Entry point that allocates nothing.
//
// Some callers may not allocate device memory at all: code that hands the GPU
// a fixed memory budget up front (a pre-sized pool, an embedding runtime), or
// code on a path where a cudaMalloc/cudaFree would synchronise the device and
// stall work queued by others. For them, ncorr_count_noalloc runs the same
// kernels as calculateD1D2D3 with every working buffer carved out of one
// file-scope device array. Its size is fixed at build time and every GPU
// that loads the library holds it until the process exits.
namespace {

constexpr long long kNoAllocPoints = 65536;  // points per catalogue (p1, p2, p3)
constexpr long long kNoAllocCells = 32768;   // cells of the grid
constexpr int kNoAllocMaxBins = 31;          // bins per side
constexpr unsigned kNoAllocExactCap = 65536; // deferred exact candidates
constexpr int kNoAllocMaxDevices = 64;

// Bytes of one catalogue's cell list: cid, count, start, cursor, pd, pq, pc.
constexpr size_t kNoAllocCatBytes =
    ((kNoAllocPoints * (4 + 32 + 16 + 4) + kNoAllocCells * 12 + 4 + 255) / 256) * 256;
constexpr size_t kNoAllocHistBytes = 2ull * kNoAllocMaxBins * kNoAllocMaxBins * kNoAllocMaxBins * 8;
constexpr size_t kNoAllocBytes = 16ull << 20;  // 16 MiB

}  // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

namespace {

std::mutex g_noalloc_mutex;
void* g_noalloc_ptr[kNoAllocMaxDevices] = {};

// Device address of the scratch array on the current device (the host-side
// name of a __device__ array is not a device address). It is looked up on
// every call made outside a stream capture, so that a device reset, after
// which the module is loaded again, cannot leave a stale address behind; a
// call inside a capture uses the address found by an earlier call on that
// device, or looks it up if there is none.
int noalloc_scratch(int dev, cudaStream_t st, unsigned char** out) {
  if (dev < 0 || dev >= kNoAllocMaxDevices) return fail(NCORR_ERR_INVALID_ARGUMENT, "device index out of range");
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cap) != cudaSuccess) {
    cudaGetLastError();
    cap = cudaStreamCaptureStatusNone;
  }
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_ptr[dev] || cap == cudaStreamCaptureStatusNone) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return fail(NCORR_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
    g_noalloc_ptr[dev] = p;
  }
  *out = static_cast<unsigned char*>(g_noalloc_ptr[dev]);
  return NCORR_OK;
}

}  // namespace

static int count_noalloc_impl(const double box[3], const double* edges, int n_edges, int is_survey,
                              const double* d_p1, int64_t n1, const double* d_p2, int64_t n2, const double* d_p3,
                              int64_t n3, double* d_counts_all, void* stream) {
  static_assert(3 * kNoAllocCatBytes + kNoAllocHistBytes + kTableSize + kNoAllocExactCap * sizeof(ExactEntry) +
                        sizeof(KArgs) + sizeof(BatchItem) + 64 * 1024 <= kNoAllocBytes,
                "scratch layout exceeds the scratch array");
  if (!box || !edges || !d_counts_all) return fail(NCORR_ERR_INVALID_ARGUMENT, "null box, edges or output");
  if (n_edges < 2 || n_edges - 1 > kNoAllocMaxBins)
    return fail(NCORR_ERR_INVALID_ARGUMENT, "ncorr_count_noalloc: 1..31 bins per side");
  for (int i = 0; i < n_edges; ++i)
    if (!std::isfinite(edges[i])) return fail(NCORR_ERR_INVALID_ARGUMENT, "non-finite bin edge");
  if (edges[0] < 0.0) return fail(NCORR_ERR_INVALID_ARGUMENT, "negative first bin edge");
  for (int i = 1; i < n_edges; ++i)
    if (!(edges[i] > edges[i - 1]) || !(edges[i] * edges[i] > edges[i - 1] * edges[i - 1]))
      return fail(NCORR_ERR_INVALID_ARGUMENT, "bin edges must be strictly increasing");
  for (int d = 0; d < 3; ++d)
    if (!(box[d] > 0.0) || !std::isfinite(box[d])) return fail(NCORR_ERR_INVALID_ARGUMENT, "box sides must be positive");
  const int64_t ns[3] = {n1, n2, n3};
  const double* src[3] = {d_p1, d_p2, d_p3};
  for (int r = 0; r < 3; ++r) {
    if (ns[r] < 0 || ns[r] > kNoAllocPoints)
      return fail(NCORR_ERR_CAPACITY, "ncorr_count_noalloc: at most 65536 points per catalogue");
    if (ns[r] > 0 && (!src[r] || (reinterpret_cast<uintptr_t>(src[r]) & 15u)))
      return fail(NCORR_ERR_INVALID_ARGUMENT, "device catalogues must be non-null and 16-byte aligned");
  }
  // Geometry, as ncorr_create builds it, on the stack.
  Geom g;
  std::memset(&g, 0, sizeof(g));
  g.nb = n_edges - 1;
  g.survey = is_survey ? 1 : 0;
  g.fma_pattern = kDefaultFmaPattern;
  const double rmax = edges[n_edges - 1], rmin = edges[0];
  g.cell = rmax;
  g.sqr_rmax = rmax * rmax;
  g.sqr_rmin = rmin * rmin;
  long long ncell = 1;
  for (int d = 0; d < 3; ++d) {
    g.box[d] = box[d];
    const double n = std::ceil(box[d] / rmax);
    if (n > 4096.0) return fail(NCORR_ERR_CAPACITY, "ncorr_count_noalloc: cell grid too large");
    g.nc[d] = static_cast<int>(n);
    ncell *= g.nc[d];
  }
  if (ncell > kNoAllocCells) return fail(NCORR_ERR_CAPACITY, "ncorr_count_noalloc: at most 32768 cells");
  for (int i = 0; i < n_edges; ++i) {
    g.sqr_bins[i] = edges[i] * edges[i];
    g.e2lo[i] = f32_down(g.sqr_bins[i]);
    g.e2hi[i] = f32_up(g.sqr_bins[i]);
  }
  set_error_model(g);

  int dev = 0;
  CU(cudaGetDevice(&dev));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  unsigned char* base = nullptr;
  if (int rc = noalloc_scratch(dev, st, &base)) return rc;
  cudaGetLastError();

  // Distinct catalogues (same pointer and size: gridded once).
  int role[3];
  role[0] = 0;
  role[1] = (d_p2 == d_p1 && n2 == n1) ? 0 : 1;
  role[2] = (d_p3 == d_p2 && n3 == n2) ? role[1] : ((d_p3 == d_p1 && n3 == n1) ? 0 : 2);
  const bool sym = role[1] == role[2];

  // Carve the scratch: the distinct catalogues' cell lists (by their sizes),
  // histogram, table, exact queue, small counters, kernel arguments; the
  // rest holds the triangle kernel's per-warp slabs.
  size_t off = 0;
  auto take = [&](size_t bytes) {
    unsigned char* p = base + off;
    off += (bytes + 255) & ~size_t(255);
    return p;
  };
  struct CatScratch {
    int *cid, *count, *start, *cursor, *pc;
    double4_16a* pd;
    float4* pq;
  } cat[3];
  {
    bool carved[3] = {false, false, false};
    for (int r = 0; r < 3; ++r) {
      const int ci = role[r];
      if (carved[ci]) continue;
      carved[ci] = true;
      CatScratch& c = cat[ci];
      const size_t n = static_cast<size_t>(std::max<int64_t>(ns[r], 1));
      c.pd = reinterpret_cast<double4_16a*>(take(n * 32));
      c.pq = reinterpret_cast<float4*>(take(n * 16));
      c.cid = reinterpret_cast<int*>(take(n * 4));
      c.pc = reinterpret_cast<int*>(take(n * 4));
      c.count = reinterpret_cast<int*>(take(ncell * 4));
      c.start = reinterpret_cast<int*>(take((ncell + 1) * 4));
      c.cursor = reinterpret_cast<int*>(take(ncell * 4));
    }
  }
  unsigned long long* hist = reinterpret_cast<unsigned long long*>(take(kNoAllocHistBytes));
  unsigned char* table = take(kTableSize);
  ExactEntry* xq = reinterpret_cast<ExactEntry*>(take(kNoAllocExactCap * sizeof(ExactEntry)));
  KArgs* d_args = reinterpret_cast<KArgs*>(take(sizeof(KArgs)));
  BatchItem* d_item = reinterpret_cast<BatchItem*>(take(sizeof(BatchItem)));
  int* flags = reinterpret_cast<int*>(take(8 * sizeof(int)));
  unsigned* wmax = reinterpret_cast<unsigned*>(take(sizeof(unsigned)));
  int* work = reinterpret_cast<int*>(take(sizeof(int)));
  int* bound = reinterpret_cast<int*>(take(2 * sizeof(int)));
  unsigned long long* stats = reinterpret_cast<unsigned long long*>(take(8 * sizeof(unsigned long long)));
  unsigned long long* total = reinterpret_cast<unsigned long long*>(take(sizeof(unsigned long long)));
  unsigned* xq_count = reinterpret_cast<unsigned*>(take(sizeof(unsigned)));
  if (off > kNoAllocBytes) return fail(NCORR_ERR_CAPACITY, "scratch layout exceeds the scratch array");
  const size_t slab_bytes = kNoAllocBytes - off;

  // Everything read before being written starts at zero on every call: the
  // array keeps the previous call's contents.
  CU(cudaMemsetAsync(flags, 0, 8 * sizeof(int), st));
  CU(cudaMemsetAsync(wmax, 0, sizeof(unsigned), st));
  CU(cudaMemsetAsync(bound, 0, 2 * sizeof(int), st));
  CU(cudaMemsetAsync(stats, 0, 8 * sizeof(unsigned long long), st));
  CU(cudaMemsetAsync(total, 0, sizeof(unsigned long long), st));
  CU(cudaMemsetAsync(work, 0, sizeof(int), st));
  CU(cudaMemsetAsync(xq_count, 0, sizeof(unsigned), st));

  bool done[3] = {false, false, false};
  for (int r = 0; r < 3; ++r) {
    const int ci = role[r];
    if (done[ci]) continue;
    done[ci] = true;
    CatScratch& c = cat[ci];
    const int n = static_cast<int>(ns[r]);
    CU(cudaMemsetAsync(c.count, 0, ncell * sizeof(int), st));
    launch_assign(reinterpret_cast<const double4_16a*>(src[r]), n, g, c.cid, c.count, flags + ci, wmax, st);
    launch_scan(c.count, static_cast<int>(ncell), c.start, c.cursor, st);
    launch_scatter(reinterpret_cast<const double4_16a*>(src[r]), n, g, c.cid, c.cursor, c.pd, c.pq, c.pc, st);
  }
  launch_nbr_bound(cat[role[1]].count, g, bound, st);
  if (!sym) launch_nbr_bound(cat[role[2]].count, g, bound + 1, st);
  CU(cudaGetLastError());
  int hflags[8];
  unsigned hwmax = 0;
  int hbound[2] = {0, 0};
  CU(cudaMemcpyAsync(hflags, flags, sizeof(hflags), cudaMemcpyDeviceToHost, st));
  CU(cudaMemcpyAsync(&hwmax, wmax, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
  CU(cudaMemcpyAsync(hbound, bound, sizeof(hbound), cudaMemcpyDeviceToHost, st));
  CU(cudaStreamSynchronize(st));
  bool weighted = false;
  for (int r = 0; r < 3; ++r) {
    const int f = hflags[role[r]];
    if (f & (kFlagNonFinite | kFlagOutOfGrid))
      return fail(NCORR_ERR_OUT_OF_GRID, "a point lies outside the cell grid or is non-finite");
    if (f & kFlagWeighted) weighted = true;
  }
  if (g.survey && (hflags[role[0]] & kFlagSurveyFace))
    return fail(NCORR_ERR_OUT_OF_GRID, "survey anchor on the upper face of the cell grid");
  bool sym6 = sym && role[0] == role[1] && !(hflags[role[0]] & kFlagNoSym6);
  if (sym6 && !g.survey)
    for (int d = 0; d < 3; ++d)
      if (g.nc[d] < 4 || __builtin_fma(-static_cast<double>(g.nc[d]), g.cell, g.box[d]) != 0.0) sym6 = false;
  float wscale = 1.0f;
  if (weighted) {
    float wm = 0.0f;
    std::memcpy(&wm, &hwmax, sizeof(float));
    const double p3 = static_cast<double>(wm) * wm * wm;
    int e = 0;
    if (p3 > 0) e = static_cast<int>(std::floor(std::log2(std::ldexp(1.0, 30) / p3)));
    wscale = static_cast<float>(std::ldexp(1.0, std::max(-120, std::min(120, e))));
  }
  const int nbin = g.nb * g.nb * g.nb;
  const int elem = weighted ? 8 : 4;
  const bool hg = hist_global(g.nb, elem);
  const int code_scale = hg ? 1 : elem;
  // Launch shape; the grid shrinks until the per-warp slabs (lists sized by
  // the largest 27-cell occupancy, careful queues, exact buffers) fit the
  // part of the scratch left after the fixed buffers.
  int nsm = 0;
  CU(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  TriShape shp;
  if (!tri_shape(g.nb, g.survey != 0, sym, weighted, hg, 1, nsm, n1, hbound[0], hbound[1], &shp))
    return fail(NCORR_ERR_CUDA, "triangle kernel does not fit on the device, or a 27-cell neighbourhood holds "
                                "more than 2^24 points");
  const size_t per_warp_entries = static_cast<size_t>(shp.kcap2) + shp.kcap3;
  const size_t per_cta = kWarps * (per_warp_entries * (sizeof(ListEnt) + sizeof(float)) +
                                   kQueueCap * sizeof(unsigned long long) + 32 * sizeof(ExactEntry));
  // Four 256-byte roundings of the slab arrays, at most.
  const size_t usable = slab_bytes > 4 * 256 ? slab_bytes - 4 * 256 : 0;
  const int fit = static_cast<int>(std::min<size_t>(usable / per_cta, static_cast<size_t>(shp.grid)));
  if (fit < 1)
    return fail(NCORR_ERR_CAPACITY, "ncorr_count_noalloc: neighbourhoods too dense for its fixed scratch");
  shp.grid = fit;
  const size_t slab_n = tri_slab_entries(shp);
  ListEnt* slab_e = reinterpret_cast<ListEnt*>(take(slab_n * sizeof(ListEnt)));
  float* slab_w = reinterpret_cast<float*>(take(slab_n * sizeof(float)));
  unsigned long long* slab_q = reinterpret_cast<unsigned long long*>(
      take(static_cast<size_t>(shp.grid) * kWarps * kQueueCap * sizeof(unsigned long long)));
  ExactEntry* slab_x =
      reinterpret_cast<ExactEntry*>(take(static_cast<size_t>(shp.grid) * kWarps * 32 * sizeof(ExactEntry)));
  if (off > kNoAllocBytes)
    return fail(NCORR_ERR_CAPACITY, "ncorr_count_noalloc: neighbourhoods too dense for its fixed scratch");

  // Bin table, built on the host stack and copied in (a pageable source:
  // the copy has completed when cudaMemcpyAsync returns).
  unsigned char tab_host[kTableSize];
  build_table(g, code_scale, tab_host);
  CU(cudaMemcpyAsync(table, tab_host, kTableSize, cudaMemcpyHostToDevice, st));
  CU(cudaMemsetAsync(hist, 0, (weighted ? 2 : 1) * static_cast<size_t>(nbin) * sizeof(unsigned long long), st));

  auto catview = [&](int ci, int64_t n) {
    Catalog v;
    v.pd = cat[ci].pd;
    v.pq = cat[ci].pq;
    v.pc = cat[ci].pc;
    v.start = cat[ci].start;
    v.count = cat[ci].count;
    v.n = static_cast<int>(n);
    return v;
  };
  BatchItem it;
  std::memset(&it, 0, sizeof(it));
  it.c1 = catview(role[0], n1);
  it.c2 = catview(role[1], n2);
  it.c3 = catview(role[2], n3);
  it.hist.counts = weighted ? nullptr : hist;
  it.hist.wsum = weighted ? hist : nullptr;
  it.out = d_counts_all;
  it.total = total;
  it.flags1 = flags + role[0];
  it.sym6_ok = sym6 ? 1 : 0;
  CU(cudaMemcpyAsync(d_item, &it, sizeof(it), cudaMemcpyHostToDevice, st));
  KArgs a;
  std::memset(&a, 0, sizeof(a));
  a.g = g;
  a.items = d_item;
  a.n_items = 1;
  a.n_work = static_cast<int>(n1);
  a.sub_j = kSubJDefault;
  a.hist_copies = shp.copies;
  a.table = table;
  a.work = work;
  a.flags = flags + 4;
  a.slab_e = slab_e;
  a.slab_w = weighted ? slab_w : nullptr;
  a.slab_q = slab_q;
  a.slab_x = slab_x;
  a.kcap2 = shp.kcap2;
  a.kcap3 = shp.kcap3;
  a.code_scale = code_scale;
  a.wscale = wscale;
  a.stats = stats;
  a.xq = xq;
  a.xq_count = xq_count;
  a.xq_cap = kNoAllocExactCap;
  a.self = d_args;
  CU(cudaMemcpyAsync(d_args, &a, sizeof(KArgs), cudaMemcpyHostToDevice, st));
  if (n1 > 0) {
    CU(launch_triangles(a, g.survey != 0, sym, weighted, hg, shp.grid, shp.smem, st));
    launch_exact(a, g.survey != 0, weighted, nsm * 4, st);
  }
  launch_fold(d_item, 1, g.nb, weighted, sym, 1.0 / wscale, st);
  CU(cudaGetLastError());
  int kflags = 0;
  CU(cudaMemcpyAsync(&kflags, flags + 4, sizeof(int), cudaMemcpyDeviceToHost, st));
  CU(cudaStreamSynchronize(st));
  if (kflags & kFlagListOverflow) return fail(NCORR_ERR_CAPACITY, "neighbour list overflow");
  if (kflags & kFlagSchedStall) return fail(NCORR_ERR_CUDA, "triangle kernel: histogram binding wait timed out");
  return NCORR_OK;
}

// Nothing throws across the C ABI: the mutex and the error strings may.
extern "C" int ncorr_count_noalloc(const double box[3], const double* edges, int n_edges, int is_survey,
                                   const double* d_p1, int64_t n1, const double* d_p2, int64_t n2,
                                   const double* d_p3, int64_t n3, double* d_counts_all, void* stream) {
  try {
    return count_noalloc_impl(box, edges, n_edges, is_survey, d_p1, n1, d_p2, n2, d_p3, n3, d_counts_all, stream);
  } catch (const std::bad_alloc&) {
    return fail(NCORR_ERR_CAPACITY, "host memory exhausted");
  } catch (const std::exception& e) {
    return fail(NCORR_ERR_INVALID_ARGUMENT, e.what());
  }
}
