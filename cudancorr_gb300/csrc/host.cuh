// Host-side pieces shared by the C ABI translation units: error reporting,
// device buffers, the handle, the FP32 error model and the bin table.
#pragma once
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

#include "../../include/ncorr_gb300.h"
#include "engine.cuh"
#include "rppi.cuh"
#include "sched.cuh"
#include "triangles.cuh"

namespace ncorr_gb300 {
void launch_assign(const double4_16a* in, int n, const Geom& g, int* cid, int* count, int* flags,
                   unsigned* wmax_bits, cudaStream_t st);
void launch_scan(const int* count, int ncell, int* start, int* cursor, cudaStream_t st);
void launch_scatter(const double4_16a* in, int n, const Geom& g, const int* cid, int* cursor,
                    double4_16a* pd, float4* pq, int* pc, cudaStream_t st);
void launch_nbr_bound(const int* count, const Geom& g, int* out, cudaStream_t st);
cudaError_t launch_triangles(const KArgs& a, bool survey, bool sym, bool weighted, bool hg, int grid,
                             size_t smem, cudaStream_t st, bool set_attr = true);
int triangles_occupancy(bool survey, bool sym, bool weighted, bool hg, size_t smem);
void launch_exact(const KArgs& a, bool survey, bool weighted, int grid, cudaStream_t st);
void launch_fold(const BatchItem* items, int n_items, int nb, bool weighted, bool sym, double inv_scale,
                 cudaStream_t st);
}  // namespace ncorr_gb300

namespace ncorr_host {

using namespace ncorr_gb300;

// Message of the last failed call on this thread (ncorr_last_error).
extern thread_local std::string t_err;

inline int fail(int code, const std::string& msg) {
  t_err = msg;
  return code;
}

// Contraction pattern of the reference's sqrSep as compiled by nvcc for the
// GB300, established by running the reference kernel on inputs built to
// separate the candidates: fma(dz, dz, fma(dx, dx, dy*dy)).
constexpr int kDefaultFmaPattern = 2;
// Contractions of the rppi helpers under nvcc, established the same way:
// sqrRpBox as fma(dx, dx, dy*dy) and dotProduct_d3 as
// fma(a.z, b.z, fma(a.x, b.x, a.y*b.y)).
constexpr int kDefaultRpPattern = 2;
constexpr int kDefaultDotPattern = 2;

// The largest histogram (all copies) the triangle kernel keeps in shared
// memory; what the kernel leaves of the SM's 256 KB serves as L1 for the
// neighbour lists.
constexpr long kHistSmemMax = 96 * 1024;

// Whether the triangle kernel keeps its histogram in global memory: the CTA
// histogram (nb^2 (nb + 2) bins of elem bytes, sinks included) must fit
// kHistSmemMax and its table codes, the careful sink's included, one byte.
// Largest neighbour list (points of one 27-cell neighbourhood) per anchor.
constexpr int kListMax = 1 << 24;

inline bool hist_global(int nb, int elem) {
  return static_cast<long>(hist_words(nb)) * elem > kHistSmemMax || (nb + 1) * elem > 0xFF;
}
constexpr unsigned kExactQueueCap = 1u << 24;  // 16M entries, 256 MiB

struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
  cudaError_t ensure(size_t bytes) {
    if (bytes <= cap && p) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    size_t b = std::max<size_t>(bytes, 256);
    cudaError_t e = cudaMalloc(&p, b);
    if (e == cudaSuccess) cap = b;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
  template <class T>
  T* as() const {
    return static_cast<T*>(p);
  }
};

struct CatDev {
  DevBuf in, cid, count, start, cursor, pd, pq, pc;
  int n = 0;
};

// Device scratch of the learned queue order (OrderScratch), grown on demand.
struct OrderBufs {
  DevBuf pred, item_total, item_rank, ekey, kcount, kstart, kcursor, sorted, acount, aoff, acursor;
  cudaError_t ensure(int n_items, long ncell, OrderScratch* out) {
    const size_t m = static_cast<size_t>(n_items) * ncell;
    const size_t nk = static_cast<size_t>(n_items) * kSchedBuckets + 1;
    cudaError_t e;
    if ((e = pred.ensure(m * sizeof(float))) || (e = item_total.ensure(n_items * sizeof(double))) ||
        (e = item_rank.ensure(n_items * sizeof(int))) || (e = ekey.ensure(m * sizeof(int))) ||
        (e = kcount.ensure(nk * sizeof(int))) || (e = kstart.ensure(nk * sizeof(int))) ||
        (e = kcursor.ensure(nk * sizeof(int))) || (e = sorted.ensure(m * sizeof(int))) ||
        (e = acount.ensure((m + 1) * sizeof(int))) || (e = aoff.ensure((m + 1) * sizeof(int))) ||
        (e = acursor.ensure((m + 1) * sizeof(int))))
      return e;
    out->pred = pred.as<float>();
    out->item_total = item_total.as<double>();
    out->item_rank = item_rank.as<int>();
    out->ekey = ekey.as<int>();
    out->kcount = kcount.as<int>();
    out->kstart = kstart.as<int>();
    out->kcursor = kcursor.as<int>();
    out->sorted = sorted.as<int>();
    out->acount = acount.as<int>();
    out->aoff = aoff.as<int>();
    out->acursor = acursor.as<int>();
    return cudaSuccess;
  }
  void release() {
    for (DevBuf* b : {&pred, &item_total, &item_rank, &ekey, &kcount, &kstart, &kcursor, &sorted, &acount, &aoff,
                      &acursor})
      b->release();
  }
};

}  // namespace ncorr_host

struct ncorr_handle {
  int bin_type = NCORR_BIN_THREED;
  int survey = 0;
  double box[3] = {0, 0, 0};
  double ori[3] = {0, 0, 0};
  std::vector<double> edges, mids;
  int nb = 0;
  long ncell = 0;
  ncorr_gb300::Geom g;
  std::vector<unsigned char> table;
  int table_scale = 0;  // code scale the uploaded table was built with
  std::vector<double> counts_all, counts_out, tri_bins_out;
  ncorr_stats stats;
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  ncorr_host::CatDev cat[3];
  ncorr_host::DevBuf d_table, d_flags, d_wmax, d_work, d_bound, d_hist, d_out, d_stats, d_total;
  ncorr_host::DevBuf slab_e, slab_w, slab_q, slab_x, cta_time;
  ncorr_host::DevBuf xq, xq_count;  // deferred exact candidates
  ncorr_host::DevBuf d_args;        // global copy of the triangle kernel's arguments
  unsigned xq_cap = 0;
  bool table_uploaded = false;
  // Work queue (ncorr_set_schedule, ncorr_set_tuning, ncorr_set_record_work).
  int sched_mode = NCORR_SCHED_DYNAMIC;
  const ncorr_sched* sched_model = nullptr;
  int sub_j = ncorr_gb300::kSubJDefault;
  int hist_copies = 1;
  bool record_work = false;
  ncorr_host::DevBuf d_items, d_cell_work, d_feats, q_item, q_anchor;
  ncorr_host::OrderBufs order;
  std::vector<float> rec_feats;   // features of the last recorded call, ncell x 28
  std::vector<double> rec_work;   // its candidate pairs per cell of catalogue 1
  // rppi bin type: geometry, piBinsOut_ table (2 per entry), per-warp lists,
  // weight of the last call's triangles indexed past triCountsAll_.
  ncorr_gb300::RppiGeom rg;
  std::vector<double> pi_bins_out;
  ncorr_host::DevBuf rp_pos, rp_ab, rp_rel, rp_meta, rp_pw, rp_tab;
  std::vector<unsigned char> rp_tab_host;  // the box classifier's rp3 table
  double rppi_overflow = 0.0;
};

// The scheduler's work-prediction MLP: parameters, Adam state and training
// scratch on one device.
struct ncorr_sched {
  int device = 0;
  cudaStream_t stream = nullptr;
  int step = 0;  // Adam steps taken
  bool bf16 = false;  // BF16 forward pass in prediction and training
  ncorr_host::DevBuf params, m, v, grad, loss, partial, partial_loss, feats, target, idx, pred;
};

namespace ncorr_host {

inline float f32_down(double x) {
  float f = static_cast<float>(x);
  if (static_cast<double>(f) > x) f = std::nextafter(f, -std::numeric_limits<float>::infinity());
  return f;
}
inline float f32_up(double x) {
  float f = static_cast<float>(x);
  if (static_cast<double>(f) < x) f = std::nextafter(f, std::numeric_limits<float>::infinity());
  return f;
}

// FP32 error model (u = 2^-24).
//  * List entries hold d = fl32(D), D the exact anchor-relative offset
//    (computed in FP64), |D| < r_max, and rho = sqrt_rn(a) of the pair
//    estimate a = fl32(|d|^2), which satisfies |a - A| <= 5.1u A.
//  * The pair loop forms the third side as v = p + s with p = -2 d_j.d_l
//    (one product, two FMAs: error <= 6u r_max^2) and
//    s = fma(rho_l, rho_l, fl(rho_j^2)) (within 13u r_max^2 of
//    |d_j|^2 + |d_l|^2). |d_j - d_l|^2 itself is within 7u V + 2u r_max^2 of
//    the reference's V (componentwise error u(|D_j| + |D_l|), Cauchy-Schwarz,
//    AM-GM on the cross term). So |v - V| <= 8.1u V + 21u r_max^2. The
//    exact-difference form used by the careful path and the pair stage is
//    tighter. ka = 12u, kb = 32u r_max^2 bound all of them with margin, also
//    covering the rounding of the band arithmetic itself. A slightly negative
//    v (a side near zero) still maps to table entry 0, since
//    kb * tab_scale < 0.25.
//  * The prefilter estimate from cell-local coordinates (error <= 5u*cell +
//    u|D| per component) satisfies |v - V| <= 14u V + 9u r_max^2; only used
//    to skip candidates that are certainly out of range (pa, pb).
//  * Triangle test. Let A, B, C be the reference's r^2 of the sides
//    anchor-j, anchor-l, j-l, all below r_max^2 for a candidate that can
//    count, and Q = 2 sqrt(AB) - |C - A - B|. The sorted quantity
//    (p + q)^2 - r^2 of the reference's test (p <= q <= r the square roots)
//    is >= Q whichever side is longest, and the FP32 test sqrtf(x1) +
//    sqrtf(x2) > sqrtf(x3) errs by at most 6.5u r_max in p + q - r; so
//    Q > 19.8u r_max^2 proves the triangle is kept. The list stores
//    rho = sqrt_rn(a) with a within 5.1u A, so rho^2 is within 7.2u A and
//    2 rho_j rho_l within 7.2u of 2 sqrt(AB). The pair loop tests
//    |p| < w with p = -2 d_j.d_l as above (C - A - B = -2 D_j.D_l exactly
//    for the exact sides; |p - (C - A - B)| <= 10u r_max^2) and
//    w = fma(2 rho_j, rho_l, -M) (error <= 16.5u r_max^2): then
//    Q > M - 26.5u r_max^2. The careful path tests t = v - (a + b) with v
//    from exact differences (error <= 30.7u r_max^2): Q > M - 47.2u r_max^2.
//    M = 128u r_max^2 leaves a factor of two or more for both.
// Margins are generous on purpose: a wider band only sends more candidates
// to the exact FP64 path.
inline void set_error_model(Geom& g) {
  const double u = std::ldexp(1.0, -24);
  const double r2 = g.sqr_rmax;
  g.ka = static_cast<float>(12.0 * u);
  g.kb = static_cast<float>(32.0 * u * r2);
  g.hm = -f32_up(128.0 * u * r2);
  // Prefilter thresholds: candidates with v >= pre_hi or v <= pre_lo are
  // certainly outside (r_min^2, r_max^2).
  const double eb = 20.0 * u, ec = 12.0 * u * r2;
  g.pre_hi = f32_up((r2 + ec) / (1.0 - eb) * (1.0 + 4.0 * u));
  g.pre_lo = f32_down((g.sqr_rmin - ec) / (1.0 + eb) * (1.0 - 4.0 * u) - 4.0 * u * ec);
}

// Bin table: entry i covers every v with rint(v * scale) == i. Its code is the
// bin that contains the whole error band of every such v (times code_scale,
// the byte stride of a bin in the CTA histogram), "reject" when the band lies
// outside (rmin^2, rmax^2), or "careful" otherwise (table_code_reject /
// table_code_careful: sink bins of the CTA histogram, or plain markers for
// the global one). `tab` holds kTableSize entries.
inline void build_table(Geom& g, int code_scale, unsigned char* tab) {
  const int n = kTableSize;
  const double vmax = g.sqr_rmax * 1.05;
  const float scale = static_cast<float>((n - 2) / vmax);
  g.tab_scale = scale;
  g.tab_n = n;
  const double ka = g.ka, kb = g.kb;
  const auto rej = static_cast<unsigned char>(table_code_reject(g.nb, code_scale));
  const auto car = static_cast<unsigned char>(table_code_careful(g.nb, code_scale));
  for (int i = 0; i < n; ++i) {
    double lo = (i - 0.5) / static_cast<double>(scale);
    double hi = (i + 0.5) / static_cast<double>(scale);
    if (lo < 0) lo = 0;
    if (i == n - 1) hi = std::numeric_limits<double>::infinity();
    // Inflate slightly for the rounding of the band arithmetic itself.
    const double blo = lo - (ka * lo + kb) * 1.01;
    const double bhi = hi + (ka * hi + kb) * 1.01;
    unsigned char code = car;
    if (bhi <= g.sqr_rmin || blo >= g.sqr_rmax) {
      code = rej;
    } else if (blo > g.sqr_rmin && bhi < g.sqr_rmax) {
      for (int b = 0; b < g.nb; ++b) {
        if (g.sqr_bins[b] <= blo && bhi < g.sqr_bins[b + 1]) {
          code = static_cast<unsigned char>(b * code_scale);
          break;
        }
      }
    }
    tab[i] = code;
  }
}

inline void build_table(Geom& g, int code_scale, std::vector<unsigned char>& tab) {
  tab.assign(kTableSize, 0);
  build_table(g, code_scale, tab.data());
}

// Launch shape of the triangle kernel: histogram copies that fit (at most
// `copies`), dynamic shared memory, persistent grid (one CTA of kWarps warps
// per SM and resident slot, fewer for small queues), and the per-warp list
// capacities (kcap2 for p2, kcap3 for p3 or 0 when p2 == p3), from the
// largest 27-cell occupancies bound2/bound3.
struct TriShape {
  int copies = 1;
  size_t smem = 0;
  int grid = 0;
  int kcap2 = 0, kcap3 = 0;
};

inline bool tri_shape(int nb, bool survey, bool sym, bool weighted, bool hg, int copies, int nsm, int64_t n_work,
                      int bound2, int bound3, TriShape* out) {
  const long nbp = hist_words(nb);
  const int elem = weighted ? 8 : 4;
  if (hg) copies = 1;
  copies = std::max(1, copies);
  while (copies > 1 && static_cast<long>(copies) * nbp * elem > kHistSmemMax) copies >>= 1;
  const SmemLayout L = make_layout(nb, weighted, hg, copies);
  const int occ = triangles_occupancy(survey, sym, weighted, hg, static_cast<size_t>(L.total));
  if (occ <= 0) return false;
  out->copies = copies;
  out->smem = static_cast<size_t>(L.total);
  const int64_t ctas_needed = std::max<int64_t>(1, (n_work + kWarps - 1) / kWarps);
  out->grid = static_cast<int>(std::min<int64_t>(static_cast<int64_t>(nsm) * occ, ctas_needed));
  // kListPad entries more than the largest list: the padding rows after it.
  out->kcap2 = ((std::max(bound2, 1) + kListPad + 31) / 32) * 32;
  out->kcap3 = sym ? 0 : ((std::max(bound3, 1) + kListPad + 31) / 32) * 32;
  // The careful queue names list rows in 24 bits.
  return out->kcap2 <= kListMax && out->kcap3 <= kListMax;
}

// Share of the launch's CTA-time spent idle at its end: CTA b ran from
// t[2b] to t[2b+1] (ns); the launch lasted from the first start to the last
// end.
inline double tail_idle_fraction(const std::vector<unsigned long long>& t, int grid) {
  if (grid <= 0) return 0.0;
  unsigned long long t0 = ~0ull, t1 = 0;
  for (int b = 0; b < grid; ++b) {
    t0 = std::min(t0, t[2 * b]);
    t1 = std::max(t1, t[2 * b + 1]);
  }
  if (t1 <= t0) return 0.0;
  double idle = 0.0;
  for (int b = 0; b < grid; ++b) idle += static_cast<double>(t1 - t[2 * b + 1]);
  return idle / (static_cast<double>(grid) * static_cast<double>(t1 - t0));
}

// Entries of the per-warp list slabs of a launch.
inline size_t tri_slab_entries(const TriShape& s) {
  return static_cast<size_t>(s.grid) * kWarps * (static_cast<size_t>(s.kcap2) + s.kcap3);
}

#define CU(call)                                                              \
  do {                                                                        \
    cudaError_t e_ = (call);                                                  \
    if (e_ != cudaSuccess)                                                    \
      return fail(NCORR_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

inline int validate_catalog_ptr(const double* p, int64_t n) {
  if (n < 0) return fail(NCORR_ERR_INVALID_ARGUMENT, "negative catalogue size");
  if (n > 0 && !p) return fail(NCORR_ERR_INVALID_ARGUMENT, "null catalogue");
  if (n > (int64_t(1) << 30)) return fail(NCORR_ERR_INVALID_ARGUMENT, "catalogue larger than 2^30 points");
  return NCORR_OK;
}

// Builds the cell list of one catalogue already in device memory.
inline int grid_catalog(ncorr_handle* h, int ci, const double4_16a* d_in, int n, cudaStream_t st) {
  CatDev& c = h->cat[ci];
  c.n = n;
  const size_t nn = static_cast<size_t>(std::max(n, 1));
  CU(c.cid.ensure(nn * sizeof(int)));
  CU(c.count.ensure(h->ncell * sizeof(int)));
  CU(c.start.ensure((h->ncell + 1) * sizeof(int)));
  CU(c.cursor.ensure(h->ncell * sizeof(int)));
  CU(c.pd.ensure(nn * sizeof(double4_16a)));
  CU(c.pq.ensure(nn * sizeof(float4)));
  CU(c.pc.ensure(nn * sizeof(int)));
  CU(cudaMemsetAsync(c.count.p, 0, h->ncell * sizeof(int), st));
  launch_assign(d_in, n, h->g, c.cid.as<int>(), c.count.as<int>(), h->d_flags.as<int>() + ci,
                h->d_wmax.as<unsigned>(), st);
  launch_scan(c.count.as<int>(), static_cast<int>(h->ncell), c.start.as<int>(), c.cursor.as<int>(), st);
  launch_scatter(d_in, n, h->g, c.cid.as<int>(), c.cursor.as<int>(), c.pd.as<double4_16a>(),
                 c.pq.as<float4>(), c.pc.as<int>(), st);
  CU(cudaGetLastError());
  return NCORR_OK;
}

// The rppi bin type (rppi.cu).
int rppi_init(ncorr_handle* h, const double box[3], const double* edges, int n_edges, int num_minor_bins,
              int is_survey, const double ori[3]);
int rppi_run(ncorr_handle* h, const double4_16a* d1, int n1, const double4_16a* d2, int n2, const double4_16a* d3,
             int n3, cudaStream_t st, const void* key1, const void* key2, const void* key3);

inline Catalog view(const CatDev& c) {
  Catalog v;
  v.pd = c.pd.as<double4_16a>();
  v.pq = c.pq.as<float4>();
  v.pc = c.pc.as<int>();
  v.start = c.start.as<int>();
  v.count = c.count.as<int>();
  v.n = c.n;
  return v;
}

}  // namespace ncorr_host
