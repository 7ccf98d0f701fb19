// CPU oracle for the three-point (r1,r2,r3) triangle count of cudaNcorr.
//
// TEST INFRASTRUCTURE ONLY. This file restates, in plain C++ with OpenMP, the
// arithmetic of the reference's threeD counting path so that tests and the
// benchmark's CPU baseline can check the CUDA engine against it. Nothing in
// the product links or calls it.
//
// Parity status: pinned. The reference ships no tests or golden files, so the
// restatement is pinned against outputs of the reference's own kernel
// (source/device.cu, compiled unmodified and run through oracle/ref_runner.cu)
// on seeded inputs, recorded under tests/golden/.
//
// Build: -O2 -fopenmp -ffp-contract=off (no implicit FMA: every fused
// multiply-add below is spelled out with std::fma, to restate exactly the
// contraction the CUDA compiler applied to the reference's sqrSep).
//
// Reference lines restated here (paths inside the cudaNcorr project):
//   source/cudaNcorr.cu:26-35    getBinsMid
//   source/cudaNcorr.cu:37-48    getShifts (27 offsets, i,j,k nested -1..1)
//   source/cudaNcorr.cu:50-58    getCellIndex (host gridding, clamp == nc)
//   source/cudaNcorr.cu:72-86    prepTriCountsOutThreeD (compaction)
//   source/cudaNcorr.cu:118-157  threeD constructor (edges^2, cell = r_max, nc = ceil)
//   source/device.cu:30-36       sqrSep
//   source/device.cu:75-87       initCellIndexBox / initCellIndexSurvey
//   source/device.cu:89-153      shiftCellIndexBox / shiftCellIndexSurvey
//   source/device.cu:154-201     getTriangleIndexThreeD
//   source/device.cu:259-315     countTrianglesThreeDBox
//   source/device.cu:381-431     countTrianglesThreeDSurvey
//   source/survey.cu:60-128      find_min_max_elements / shift_catalog / prep_cat_survey
//   source/utils.cu:16-27        logspace
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>
#include <omp.h>

namespace {

// Contraction patterns for `dx*dx + dy*dy + dz*dz` (source/device.cu:35).
// The expression parses as ((dx*dx + dy*dy) + dz*dz); these are all the ways a
// compiler may fuse its two additions with the products beside them.
enum SqrSepPattern {
  kNoFma = 0,        // (dx*dx + dy*dy) + dz*dz, every operation rounded
  kFmaInnerDy = 1,   // fma(dz,dz, fma(dy,dy, dx*dx))
  kFmaInnerDx = 2,   // fma(dz,dz, fma(dx,dx, dy*dy)): what nvcc emits for the
                     // reference (pinned by the fma_probe fixture)
  kFmaOuterOnly = 3, // fma(dz,dz, dx*dx + dy*dy)
  kFmaInnerDyOnly = 4, // fma(dy,dy, dx*dx) + dz*dz
  kFmaInnerDxOnly = 5, // fma(dx,dx, dy*dy) + dz*dz
};

template <int P>
inline double sqr_sum(double dx, double dy, double dz) {
  if constexpr (P == kNoFma) {
    double a = dx * dx;
    double b = dy * dy;
    double c = dz * dz;
    return (a + b) + c;
  } else if constexpr (P == kFmaInnerDy) {
    return std::fma(dz, dz, std::fma(dy, dy, dx * dx));
  } else if constexpr (P == kFmaInnerDx) {
    return std::fma(dz, dz, std::fma(dx, dx, dy * dy));
  } else if constexpr (P == kFmaOuterOnly) {
    double a = dx * dx;
    double b = dy * dy;
    return std::fma(dz, dz, a + b);
  } else if constexpr (P == kFmaInnerDyOnly) {
    double c = dz * dz;
    return std::fma(dy, dy, dx * dx) + c;
  } else {
    double c = dz * dz;
    return std::fma(dx, dx, dy * dy) + c;
  }
}

struct Pt {
  double x, y, z, w;
};

// source/device.cu:30-36: dx = p1 - p2 per axis, then the sum of squares.
template <int P>
inline double sqr_sep(const Pt& a, const Pt& b) {
  double dx = a.x - b.x;
  double dy = a.y - b.y;
  double dz = a.z - b.z;
  return sqr_sum<P>(dx, dy, dz);
}

struct Geometry {
  int nb = 0;
  std::vector<double> sqr_bins;  // bins[i]^2 (source/cudaNcorr.cu:124-127)
  double sqr_rmin = 0, sqr_rmax = 0;
  double cell[3] = {0, 0, 0};
  double box[3] = {0, 0, 0};
  int nc[3] = {0, 0, 0};
  bool survey = false;
  int shifts[27][3];
};

int make_geometry(const double* box, const double* edges, int n_edges, int is_survey, Geometry* g) {
  if (n_edges < 2) return -1;
  for (int i = 0; i < n_edges; ++i)
    if (!std::isfinite(edges[i])) return -1;
  if (edges[0] < 0.0) return -1;
  for (int i = 1; i < n_edges; ++i)
    if (!(edges[i] > edges[i - 1])) return -1;
  for (int d = 0; d < 3; ++d)
    if (!(box[d] > 0.0) || !std::isfinite(box[d])) return -1;
  g->nb = n_edges - 1;
  g->sqr_bins.resize(n_edges);
  for (int i = 0; i < n_edges; ++i) g->sqr_bins[i] = edges[i] * edges[i];
  double rmax = edges[n_edges - 1], rmin = edges[0];
  g->sqr_rmax = rmax * rmax;  // source/cudaNcorr.cu:131-134
  g->sqr_rmin = rmin * rmin;
  for (int d = 0; d < 3; ++d) {
    g->cell[d] = rmax;  // cell size = r_max (source/cudaNcorr.cu:137)
    g->box[d] = box[d];
    double n = std::ceil(box[d] / rmax);  // source/cudaNcorr.cu:138-140
    if (n > 4096.0) return -2;
    g->nc[d] = static_cast<int>(n);
  }
  g->survey = is_survey != 0;
  // source/cudaNcorr.cu:37-48: i, j, k nested over -1..1.
  int s = 0;
  for (int i = -1; i <= 1; ++i)
    for (int j = -1; j <= 1; ++j)
      for (int k = -1; k <= 1; ++k) {
        g->shifts[s][0] = i;
        g->shifts[s][1] = j;
        g->shifts[s][2] = k;
        ++s;
      }
  return 0;
}

// int(x / cell) as the reference computes it (C++ truncation toward zero),
// guarded so that the conversion itself is defined.
inline bool axis_index(double x, double cell, long* out) {
  if (!std::isfinite(x)) return false;
  double q = x / cell;
  if (!(q > -2147483000.0 && q < 2147483000.0)) return false;
  *out = static_cast<long>(static_cast<int>(q));
  return true;
}

// Host gridding cell of a point (source/cudaNcorr.cu:50-58): truncation, then
// `== nc` clamps to nc-1. Returns -1 where the reference would index outside
// its cell array (undefined behaviour there); such inputs are rejected.
inline long host_cell(const Geometry& g, const Pt& p, int ijk[3]) {
  const double c[3] = {p.x, p.y, p.z};
  for (int d = 0; d < 3; ++d) {
    long i;
    if (!axis_index(c[d], g.cell[d], &i)) return -1;
    if (i == g.nc[d]) --i;
    if (i < 0 || i >= g.nc[d]) return -1;
    ijk[d] = static_cast<int>(i);
  }
  return ijk[2] + static_cast<long>(g.nc[2]) * (ijk[1] + static_cast<long>(g.nc[1]) * ijk[0]);
}

// Anchor cell on the device (source/device.cu:75-87): box clamps like the
// host; survey does not clamp. An unclamped survey index of nc is rejected.
inline bool anchor_cell(const Geometry& g, const Pt& p, int ijk[3]) {
  const double c[3] = {p.x, p.y, p.z};
  for (int d = 0; d < 3; ++d) {
    long i;
    if (!axis_index(c[d], g.cell[d], &i)) return false;
    if (!g.survey && i == g.nc[d]) --i;
    if (i < 0 || i >= g.nc[d]) return false;
    ijk[d] = static_cast<int>(i);
  }
  return true;
}

// source/device.cu:89-122 (box): one-step wrap, image shift of +-box.
// source/device.cu:123-153 (survey): out-of-grid neighbours are skipped.
inline long neighbour_cell(const Geometry& g, const int home[3], int s, double shift[3]) {
  int c[3];
  for (int d = 0; d < 3; ++d) {
    c[d] = home[d] + g.shifts[s][d];
    shift[d] = 0.0;
  }
  if (g.survey) {
    for (int d = 0; d < 3; ++d)
      if (c[d] == g.nc[d] || c[d] == -1) return -1;
  } else {
    for (int d = 0; d < 3; ++d) {
      if (c[d] == g.nc[d]) {
        c[d] = 0;
        shift[d] = g.box[d];
      }
    }
    for (int d = 0; d < 3; ++d) {
      if (c[d] == -1) {
        c[d] = g.nc[d] - 1;
        shift[d] = -g.box[d];
      }
    }
  }
  return c[2] + static_cast<long>(g.nc[2]) * (c[1] + static_cast<long>(g.nc[1]) * c[0]);
}

// source/device.cu:154-201. Returns the flat bin or -1 when the FP32 triangle
// test rejects. With strictly increasing non-negative edges and r^2 in
// (rmin^2, rmax^2) exactly one bin matches, so the reference's "last match
// wins" scan and its uninitialised indices reduce to this search.
inline int triangle_index(double r1, double r2, double r3, const std::vector<double>& sb, int nb) {
  double t;
  if (r1 > r2) { t = r1; r1 = r2; r2 = t; }
  if (r1 > r3) { t = r1; r1 = r3; r3 = t; }
  if (r2 > r3) { t = r2; r2 = r3; r3 = t; }
  float s1 = std::sqrt(static_cast<float>(r1));
  float s2 = std::sqrt(static_cast<float>(r2));
  float s3 = std::sqrt(static_cast<float>(r3));
  float sum = s1 + s2;
  if (sum <= s3) return -1;
  int idx[3] = {-1, -1, -1};
  const double r[3] = {r1, r2, r3};
  for (int i = 0; i < nb; ++i)
    for (int m = 0; m < 3; ++m)
      if (r[m] >= sb[i] && r[m] < sb[i + 1]) idx[m] = i;
  if (idx[0] < 0 || idx[1] < 0 || idx[2] < 0) return -1;
  return idx[2] + idx[1] * nb + idx[0] * nb * nb;
}

// Compensated (Neumaier) accumulator: the oracle's per-bin sums are far more
// accurate than a plain FP64 sum, so it serves as the FP64 reference for
// weighted bins.
struct Acc {
  double s = 0.0, c = 0.0;
  inline void add(double v) {
    double t = s + v;
    if (std::fabs(s) >= std::fabs(v))
      c += (s - t) + v;
    else
      c += (v - t) + s;
    s = t;
  }
  inline double value() const { return s + c; }
};

struct Grid {
  std::vector<long> start;  // per cell
  std::vector<long> count;
  std::vector<Pt> pts;      // grouped by cell, input order within a cell
};

int build_grid(const Geometry& g, const Pt* p, long n, Grid* grid) {
  long ncell = static_cast<long>(g.nc[0]) * g.nc[1] * g.nc[2];
  std::vector<long> cid(n);
  grid->count.assign(ncell, 0);
  grid->start.assign(ncell + 1, 0);
  int ijk[3];
  for (long i = 0; i < n; ++i) {
    long c = host_cell(g, p[i], ijk);
    if (c < 0) return -3;
    cid[i] = c;
    grid->count[c]++;
  }
  for (long c = 0; c < ncell; ++c) grid->start[c + 1] = grid->start[c] + grid->count[c];
  grid->pts.resize(n);
  std::vector<long> cur(grid->start.begin(), grid->start.end() - 1);
  for (long i = 0; i < n; ++i) grid->pts[cur[cid[i]]++] = p[i];
  return 0;
}

// Literal restatement of the reference's loop nest (source/device.cu:259-315
// and :381-431): for every anchor, walk 27 cells for p2, and for every p2 in
// range walk the 27 cells again for p3.
template <int P>
void count_literal(const Geometry& g, const Pt* p1, long n1, const Grid& g2, const Grid& g3,
                   int nthreads, std::vector<Acc>* out) {
  const int nb = g.nb;
  const long nbin = static_cast<long>(nb) * nb * nb;
  std::vector<std::vector<Acc>> part(nthreads, std::vector<Acc>(nbin));
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 16)
  for (long a = 0; a < n1; ++a) {
    std::vector<Acc>& h = part[omp_get_thread_num()];
    const Pt q1 = p1[a];
    int home[3];
    anchor_cell(g, q1, home);
    for (int s2 = 0; s2 < 27; ++s2) {
      double sh2[3];
      long c2 = neighbour_cell(g, home, s2, sh2);
      if (c2 < 0) continue;
      for (long j = g2.start[c2]; j < g2.start[c2] + g2.count[c2]; ++j) {
        Pt q2 = g2.pts[j];
        q2.x += sh2[0];
        q2.y += sh2[1];
        q2.z += sh2[2];
        double r1 = sqr_sep<P>(q1, q2);
        if (!(r1 < g.sqr_rmax && r1 > g.sqr_rmin)) continue;
        for (int s3 = 0; s3 < 27; ++s3) {
          double sh3[3];
          long c3 = neighbour_cell(g, home, s3, sh3);
          if (c3 < 0) continue;
          for (long l = g3.start[c3]; l < g3.start[c3] + g3.count[c3]; ++l) {
            Pt q3 = g3.pts[l];
            q3.x += sh3[0];
            q3.y += sh3[1];
            q3.z += sh3[2];
            double r2 = sqr_sep<P>(q1, q3);
            double r3 = sqr_sep<P>(q2, q3);
            if (r2 < g.sqr_rmax && r3 < g.sqr_rmax && r2 > g.sqr_rmin && r3 > g.sqr_rmin) {
              int t = triangle_index(r1, r2, r3, g.sqr_bins, nb);
              if (t != -1) h[t].add(q1.w * q2.w * q3.w);
            }
          }
        }
      }
    }
  }
  out->assign(nbin, Acc());
  for (int t = 0; t < nthreads; ++t)
    for (long b = 0; b < nbin; ++b) {
      (*out)[b].add(part[t][b].s);
      (*out)[b].add(part[t][b].c);
    }
}

struct Nbr {
  Pt p;       // shifted image of the neighbour
  double r;   // exact r^2 to the anchor
};

template <int P>
inline void gather(const Geometry& g, const Pt& q1, const int home[3], const Grid& gr,
                   std::vector<Nbr>* lst) {
  lst->clear();
  for (int s = 0; s < 27; ++s) {
    double sh[3];
    long c = neighbour_cell(g, home, s, sh);
    if (c < 0) continue;
    for (long j = gr.start[c]; j < gr.start[c] + gr.count[c]; ++j) {
      Pt q = gr.pts[j];
      q.x += sh[0];
      q.y += sh[1];
      q.z += sh[2];
      double r = sqr_sep<P>(q1, q);
      if (r < g.sqr_rmax && r > g.sqr_rmin) lst->push_back({q, r});
    }
  }
}

// Same arithmetic as count_literal, with each anchor's in-range neighbours
// gathered once: the p3 walk of the reference recomputes sqrSep(p1, p3) for
// every p2, which yields the same list every time. Used as the timed CPU
// cell-list counter and for larger parity cases.
template <int P>
void count_lists(const Geometry& g, const Pt* p1, long n1, const Grid& g2, const Grid& g3,
                 bool same23, int nthreads, std::vector<Acc>* out) {
  const int nb = g.nb;
  const long nbin = static_cast<long>(nb) * nb * nb;
  std::vector<std::vector<Acc>> part(nthreads, std::vector<Acc>(nbin));
#pragma omp parallel num_threads(nthreads)
  {
    std::vector<Nbr> l2, l3;
    std::vector<Acc>& h = part[omp_get_thread_num()];
#pragma omp for schedule(dynamic, 4)
    for (long a = 0; a < n1; ++a) {
      const Pt q1 = p1[a];
      int home[3];
      anchor_cell(g, q1, home);
      gather<P>(g, q1, home, g2, &l2);
      const std::vector<Nbr>* pl3 = &l2;
      if (!same23) {
        gather<P>(g, q1, home, g3, &l3);
        pl3 = &l3;
      }
      const std::vector<Nbr>& L3 = *pl3;
      for (size_t j = 0; j < l2.size(); ++j) {
        const Nbr& b = l2[j];
        const double w12 = q1.w * b.p.w;
        for (size_t l = 0; l < L3.size(); ++l) {
          const Nbr& c = L3[l];
          double r3 = sqr_sep<P>(b.p, c.p);
          if (r3 < g.sqr_rmax && r3 > g.sqr_rmin) {
            int t = triangle_index(b.r, c.r, r3, g.sqr_bins, nb);
            if (t != -1) h[t].add(w12 * c.p.w);
          }
        }
      }
    }
  }
  out->assign(nbin, Acc());
  for (int t = 0; t < nthreads; ++t)
    for (long b = 0; b < nbin; ++b) {
      (*out)[b].add(part[t][b].s);
      (*out)[b].add(part[t][b].c);
    }
}

template <int P>
int run(const Geometry& g, const Pt* p1, long n1, const Pt* p2, long n2, const Pt* p3, long n3,
        int nthreads, int variant, double* hist) {
  int ijk[3];
  for (long i = 0; i < n1; ++i) {
    if (host_cell(g, p1[i], ijk) < 0) return -3;
    if (!anchor_cell(g, p1[i], ijk)) return -3;
  }
  Grid g2, g3;
  int rc = build_grid(g, p2, n2, &g2);
  if (rc) return rc;
  bool same23 = (p2 == p3 && n2 == n3);
  if (!same23) {
    rc = build_grid(g, p3, n3, &g3);
    if (rc) return rc;
  }
  const Grid& G3 = same23 ? g2 : g3;
  std::vector<Acc> acc;
  if (variant == 0)
    count_literal<P>(g, p1, n1, g2, G3, nthreads, &acc);
  else
    count_lists<P>(g, p1, n1, g2, G3, same23, nthreads, &acc);
  for (size_t b = 0; b < acc.size(); ++b) hist[b] = acc[b].value();
  return 0;
}

}  // namespace

extern "C" {

// Full (r1,r2,r3) histogram of the reference's calculateD1D2D3 for the threeD
// bin type (source/cudaNcorr.cu:220-430 with source/device.cu:259-315 or
// :381-431), laid out as the reference's triCountsAll_: index
// idx3 + idx2*nb + idx1*nb*nb with idx1 <= idx2 <= idx3.
// Points are N x 4 doubles (x, y, z, w), the layout of std::vector<double4>.
// Returns 0, -1 (bad edges/box), -2 (grid too large), -3 (a point outside
// the cell grid: the reference indexes out of bounds there), -4 (bad args).
int oracle_count_threeD(const double* box, const double* edges, int n_edges, int is_survey,
                        const double* p1, long n1, const double* p2, long n2, const double* p3,
                        long n3, int fma_pattern, int nthreads, int variant, double* hist_out) {
  Geometry g;
  int rc = make_geometry(box, edges, n_edges, is_survey, &g);
  if (rc) return rc;
  if (n1 < 0 || n2 < 0 || n3 < 0 || !hist_out) return -4;
  if (nthreads <= 0) nthreads = omp_get_max_threads();
  const Pt* a = reinterpret_cast<const Pt*>(p1);
  const Pt* b = reinterpret_cast<const Pt*>(p2);
  const Pt* c = reinterpret_cast<const Pt*>(p3);
  switch (fma_pattern) {
    case 0: return run<0>(g, a, n1, b, n2, c, n3, nthreads, variant, hist_out);
    case 1: return run<1>(g, a, n1, b, n2, c, n3, nthreads, variant, hist_out);
    case 2: return run<2>(g, a, n1, b, n2, c, n3, nthreads, variant, hist_out);
    case 3: return run<3>(g, a, n1, b, n2, c, n3, nthreads, variant, hist_out);
    case 4: return run<4>(g, a, n1, b, n2, c, n3, nthreads, variant, hist_out);
    case 5: return run<5>(g, a, n1, b, n2, c, n3, nthreads, variant, hist_out);
    default: return -4;
  }
}

// sqrSep of two points under a given contraction pattern (source/device.cu:30-36).
double oracle_sqr_sep(const double* a, const double* b, int fma_pattern) {
  const Pt& p = *reinterpret_cast<const Pt*>(a);
  const Pt& q = *reinterpret_cast<const Pt*>(b);
  switch (fma_pattern) {
    case 0: return sqr_sep<0>(p, q);
    case 1: return sqr_sep<1>(p, q);
    case 2: return sqr_sep<2>(p, q);
    case 3: return sqr_sep<3>(p, q);
    case 4: return sqr_sep<4>(p, q);
    default: return sqr_sep<5>(p, q);
  }
}

// getTriangleIndexThreeD (source/device.cu:154-201) on three r^2 values.
int oracle_triangle_index(double r1, double r2, double r3, const double* edges, int n_edges) {
  std::vector<double> sb(n_edges);
  for (int i = 0; i < n_edges; ++i) sb[i] = edges[i] * edges[i];
  return triangle_index(r1, r2, r3, sb, n_edges - 1);
}

// Number of entries of the compacted output (source/cudaNcorr.cu:145-154).
long oracle_n_out_threeD(const double* edges, int n_edges) {
  int nb = n_edges - 1;
  std::vector<double> mid(nb);
  for (int i = 1; i < n_edges; ++i) mid[i - 1] = (edges[i] + edges[i - 1]) / 2.0;
  long n = 0;
  for (int i = 0; i < nb; ++i)
    for (int j = i; j < nb; ++j)
      for (int k = j; k < nb; ++k)
        if (mid[k] <= mid[i] + mid[j]) ++n;
  return n;
}

// prepTriCountsOutThreeD (source/cudaNcorr.cu:72-86) and the triBinsOut_
// table built beside it in the constructor (source/cudaNcorr.cu:145-154).
// bins_out receives n_out x 3 bin mids; either output may be null.
long oracle_compact_threeD(const double* edges, int n_edges, const double* hist_all,
                           double* counts_out, double* bins_out) {
  int nb = n_edges - 1;
  std::vector<double> mid(nb);
  for (int i = 1; i < n_edges; ++i) mid[i - 1] = (edges[i] + edges[i - 1]) / 2.0;
  long n = 0;
  for (int i = 0; i < nb; ++i)
    for (int j = i; j < nb; ++j)
      for (int k = j; k < nb; ++k)
        if (mid[k] <= mid[i] + mid[j]) {
          if (counts_out) counts_out[n] = hist_all[k + j * nb + i * nb * nb];
          if (bins_out) {
            bins_out[3 * n] = mid[i];
            bins_out[3 * n + 1] = mid[j];
            bins_out[3 * n + 2] = mid[k];
          }
          ++n;
        }
  return n;
}

// logspace (source/utils.cu:16-27).
void oracle_logspace(double start, double end, int n_edge, double* out) {
  double a = std::log10(start);
  double b = std::log10(end);
  double step = (b - a) / (n_edge - 1);
  for (int i = 0; i < n_edge; ++i) out[i] = std::pow(10, a + i * step);
}

static void min_max(const double* c, long n, double mn[3], double mx[3]) {
  for (int d = 0; d < 3; ++d) {
    mn[d] = std::numeric_limits<double>::max();
    mx[d] = std::numeric_limits<double>::lowest();
  }
  for (long i = 0; i < n; ++i)
    for (int d = 0; d < 3; ++d) {
      double v = c[4 * i + d];
      if (v < mn[d]) mn[d] = v;
      if (v > mx[d]) mx[d] = v;
    }
}

// prep_cat_survey for one catalogue (source/survey.cu:94-104) and for two
// (source/survey.cu:106-128): joint bounding box, box = max - min + 1.0,
// ori = -min, catalogues shifted in place by -min.
void oracle_prep_cat_survey(double* c1, long n1, double* c2, long n2, double* box, double* ori) {
  double mn[3], mx[3];
  min_max(c1, n1, mn, mx);
  if (c2) {
    double mn2[3], mx2[3];
    min_max(c2, n2, mn2, mx2);
    for (int d = 0; d < 3; ++d) {
      mn[d] = std::min(mn[d], mn2[d]);
      mx[d] = std::max(mx[d], mx2[d]);
    }
  }
  for (int d = 0; d < 3; ++d) {
    box[d] = mx[d] - mn[d] + 1.0;
    ori[d] = -mn[d];
  }
  for (long i = 0; i < n1; ++i)
    for (int d = 0; d < 3; ++d) c1[4 * i + d] -= mn[d];
  if (c2)
    for (long i = 0; i < n2; ++i)
      for (int d = 0; d < 3; ++d) c2[4 * i + d] -= mn[d];
}

}  // extern "C"
