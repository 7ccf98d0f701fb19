// CPU oracle for the three-point (r1,r2,r3) triangle count of cudaNcorr.
//
// TEST INFRASTRUCTURE ONLY. This file restates, in plain C++ with OpenMP, the
// arithmetic of the reference's threeD counting path so that tests and the
// benchmark's CPU baseline can check the CUDA engine against it. Nothing in
// the product links or calls it.
//
// Parity status: pinned. The reference ships no tests or golden files, so the
// restatement is pinned against outputs of the reference's own kernels
// (source/device.cu, compiled unmodified and run through oracle/ref_runner.cu)
// on seeded inputs, recorded under tests/golden/ (threeD and rppi, box and
// survey).
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
// and of its rppi bin type:
//   source/cudaNcorr.cu:88-105   prepTriCountsOutRppi
//   source/cudaNcorr.cu:159-216  rppi constructor (pi bins, cells, rMax = sqrtf)
//   source/device.cu:23-25       dotProduct_d3 (six contraction candidates)
//   source/device.cu:38-68       sqrRpBox / sqrPiBox / getLOS / getSqrSdotL /
//                                getSqrRpSqrPi
//   source/device.cu:203-255     getTriangleIndexRppi
//   source/device.cu:317-379     countTrianglesRppiBox
//   source/device.cu:434-505     countTrianglesRppiSurvey
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
  // The reference scans every bin for each side (the last match wins); with
  // strictly increasing edges at most one bin matches, which a binary search
  // finds directly.
  const double r[3] = {r1, r2, r3};
  int idx[3];
  for (int m = 0; m < 3; ++m) {
    if (!(r[m] >= sb[0] && r[m] < sb[nb])) return -1;
    int lo = 0, hi = nb - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (r[m] >= sb[mid]) lo = mid; else hi = mid - 1;
    }
    idx[m] = lo;
  }
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
  // Row j of one anchor's pair loop. With p2 == p3 the ordered pairs (j, l)
  // and (l, j) have bit-identical sides ((a-b)^2 == (b-a)^2, and the triangle
  // index sorts the three), so each unordered pair is evaluated once and adds
  // both orderings' weight products; l == j has r3 = 0, which the strict
  // r_min test rejects.
  auto row = [&](const Pt& q1, const std::vector<Nbr>& l2, const std::vector<Nbr>& L3, size_t j,
                 std::vector<Acc>& h) {
    const Nbr& b = l2[j];
    const double w12 = q1.w * b.p.w;
    const size_t lend = same23 ? j : L3.size();
    for (size_t l = 0; l < lend; ++l) {
      const Nbr& c = L3[l];
      double r3 = sqr_sep<P>(b.p, c.p);
      if (r3 < g.sqr_rmax && r3 > g.sqr_rmin) {
        int t = triangle_index(b.r, c.r, r3, g.sqr_bins, nb);
        if (t != -1) {
          h[t].add(w12 * c.p.w);
          if (same23) h[t].add((q1.w * c.p.w) * b.p.w);
        }
      }
    }
  };
  if (n1 >= 8L * nthreads) {
    // Many anchors: threads take whole anchors.
#pragma omp parallel num_threads(nthreads)
    {
      std::vector<Nbr> l2, l3;
      std::vector<Acc>& h = part[omp_get_thread_num()];
#pragma omp for schedule(dynamic, 1)
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
        for (size_t j = 0; j < l2.size(); ++j) row(q1, l2, *pl3, j, h);
      }
    }
  } else {
    // Few anchors: the rows of each anchor's pair loop are shared out.
    std::vector<Nbr> l2, l3;
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
      const long nrow = static_cast<long>(l2.size());
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 8)
      for (long j = 0; j < nrow; ++j) row(q1, l2, *pl3, static_cast<size_t>(j), part[omp_get_thread_num()]);
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


// ======================================================================= rppi
// The (rp, pi) bin type: ncorr's second constructor (source/cudaNcorr.cu:159-216)
// with the kernels countTrianglesRppiBox (source/device.cu:317-379) and
// countTrianglesRppiSurvey (source/device.cu:434-505).

// sqrRpBox (source/device.cu:38-43): dx*dx + dy*dy under one of the three
// ways a compiler may contract it.
enum RpPattern {
  kRpNoFma = 0,   // dx*dx + dy*dy, every operation rounded
  kRpFmaDy = 1,   // fma(dy, dy, dx*dx)
  kRpFmaDx = 2,   // fma(dx, dx, dy*dy)
};

inline double rp_sum(int pat, double dx, double dy) {
  if (pat == kRpNoFma) {
    double a = dx * dx;
    double b = dy * dy;
    return a + b;
  }
  if (pat == kRpFmaDy) return std::fma(dy, dy, dx * dx);
  return std::fma(dx, dx, dy * dy);
}

// dotProduct_d3 (source/device.cu:23-25): a.x*b.x + a.y*b.y + a.z*b.z with
// the same six contraction candidates as sqrSep (SqrSepPattern numbering).
inline double dot3(int pat, const double a[3], const double b[3]) {
  switch (pat) {
    case kNoFma: {
      double x = a[0] * b[0];
      double y = a[1] * b[1];
      double z = a[2] * b[2];
      return (x + y) + z;
    }
    case kFmaInnerDy: return std::fma(a[2], b[2], std::fma(a[1], b[1], a[0] * b[0]));
    case kFmaInnerDx: return std::fma(a[2], b[2], std::fma(a[0], b[0], a[1] * b[1]));
    case kFmaOuterOnly: {
      double x = a[0] * b[0];
      double y = a[1] * b[1];
      return std::fma(a[2], b[2], x + y);
    }
    case kFmaInnerDyOnly: {
      double z = a[2] * b[2];
      return std::fma(a[1], b[1], a[0] * b[0]) + z;
    }
    default: {
      double z = a[2] * b[2];
      return std::fma(a[0], b[0], a[1] * b[1]) + z;
    }
  }
}

struct RppiGeometry {
  Geometry g;            // bins, shifts, nc, box, survey flag (cell unused)
  int npi = 0;           // numPiBins_
  double cellv[3] = {0, 0, 0};
  double sqr_rpmax = 0, sqr_rpmin = 0, sqr_pimax = 0;
  double sqr_rmax = 0;   // rpMax^2 + piMax^2 (source/cudaNcorr.cu:182)
  double sqr_rmin = 0;   // never set by the reference (see make_rppi_geometry)
  double ori[3] = {0, 0, 0};  // d_ori as the kernels see it: (ori.x, 0, 0)
  int rp_pat = kRpFmaDx;
  int dot_pat = kFmaInnerDx;
};

// The rppi constructor (source/cudaNcorr.cu:159-216). Pi bins are unit wide,
// 0..numMinorBins; the box grid uses cells (rpMax, rpMax, piMax), the survey
// grid cubes of rMax = sqrtf(rpMax^2 + piMax^2) evaluated in FP32
// (source/cudaNcorr.cu:183, float sqrtf of the double). sqrRMin_ is left
// uninitialised there yet uploaded to d_sqrRMin and used by the survey kernel
// (source/cudaNcorr.cu:229, source/device.cu:459, :466); any value in
// [0, rpMin^2] gives the same counts, because every side that counts has
// sqrS >= sqrRp > rpMin^2, so it is defined as 0 here. The reference uploads
// only d_ori.x (sizeof(double) at source/cudaNcorr.cu:254), so the kernels see
// (ori.x, 0, 0).
int make_rppi_geometry(const double* box, const double* edges, int n_edges, int npi, int is_survey,
                       const double* ori, RppiGeometry* r) {
  Geometry& g = r->g;
  if (n_edges < 2 || npi < 1 || npi > 4096) return -1;
  for (int i = 0; i < n_edges; ++i)
    if (!std::isfinite(edges[i])) return -1;
  if (edges[0] < 0.0) return -1;
  for (int i = 1; i < n_edges; ++i)
    if (!(edges[i] > edges[i - 1])) return -1;
  for (int d = 0; d < 3; ++d)
    if (!(box[d] > 0.0) || !std::isfinite(box[d])) return -1;
  g.nb = n_edges - 1;
  g.sqr_bins.resize(n_edges);
  for (int i = 0; i < n_edges; ++i) g.sqr_bins[i] = edges[i] * edges[i];
  const double rpmax = edges[n_edges - 1], rpmin = edges[0];
  r->npi = npi;
  const double pimax = static_cast<double>(npi);
  r->sqr_rpmax = rpmax * rpmax;
  r->sqr_rpmin = rpmin * rpmin;
  r->sqr_pimax = pimax * pimax;
  r->sqr_rmax = rpmax * rpmax + pimax * pimax;
  r->sqr_rmin = 0.0;
  const double rmax = static_cast<double>(std::sqrt(static_cast<float>(r->sqr_rmax)));
  g.survey = is_survey != 0;
  if (g.survey) {
    r->cellv[0] = r->cellv[1] = r->cellv[2] = rmax;
  } else {
    r->cellv[0] = r->cellv[1] = rpmax;
    r->cellv[2] = pimax;
  }
  for (int d = 0; d < 3; ++d) {
    g.box[d] = box[d];
    g.cell[d] = r->cellv[d];
    double n = std::ceil(box[d] / r->cellv[d]);
    if (n > 4096.0) return -2;
    g.nc[d] = static_cast<int>(n);
  }
  r->ori[0] = (g.survey && ori) ? ori[0] : 0.0;
  r->ori[1] = 0.0;
  r->ori[2] = 0.0;
  int s = 0;
  for (int i = -1; i <= 1; ++i)
    for (int j = -1; j <= 1; ++j)
      for (int k = -1; k <= 1; ++k) {
        g.shifts[s][0] = i;
        g.shifts[s][1] = j;
        g.shifts[s][2] = k;
        ++s;
      }
  return 0;
}

// getTriangleIndexRppi (source/device.cu:203-255): sort the three sides by
// rp^2 carrying their pi^2 along, FP32 sqrtf triangle test, rp bin of each
// side, unit pi bins floor(sqrtf(pi^2)) of the two shortest sides, flat index
// idxPi2 + idxPi1*nPi + idx3*nPi^2 + idx2*nb*nPi^2 + idx1*nb^2*nPi^2. The
// returned index is the reference's even where it lands outside the nb^3*nPi^2
// histogram (a pi^2 just below piMax^2 whose FP32 square root rounds up to
// piMax gives pi bin nPi).
inline long rppi_index(double r1, double r2, double r3, double q1, double q2, double q3,
                       const std::vector<double>& sb, int nb, int npi) {
  double t;
  if (r1 > r2) {
    t = r1; r1 = r2; r2 = t;
    t = q1; q1 = q2; q2 = t;
  }
  if (r1 > r3) {
    t = r1; r1 = r3; r3 = t;
    t = q1; q1 = q3; q3 = t;
  }
  if (r2 > r3) {
    t = r2; r2 = r3; r3 = t;
    t = q2; q2 = q3; q3 = t;
  }
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
  if (idx[0] < 0 || idx[1] < 0 || idx[2] < 0) return -1;  // unreachable for in-range sides
  const long p1 = static_cast<long>(std::floor(std::sqrt(static_cast<float>(q1))));
  const long p2 = static_cast<long>(std::floor(std::sqrt(static_cast<float>(q2))));
  const long P = npi, B = nb;
  return p2 + p1 * P + idx[2] * P * P + idx[1] * B * P * P + idx[0] * B * B * P * P;
}

// Histogram of an rppi count plus the weight that the reference writes past
// its end (index >= nb^3 * nPi^2).
struct RppiHist {
  std::vector<Acc> bins;
  Acc overflow;
};

inline void rppi_add(RppiHist& h, long idx, double w) {
  if (idx < 0) return;
  if (idx < static_cast<long>(h.bins.size()))
    h.bins[idx].add(w);
  else
    h.overflow.add(w);
}

inline void shifted(const Pt& p, const double sh[3], Pt* q) {
  *q = p;
  q->x += sh[0];
  q->y += sh[1];
  q->z += sh[2];
}

// countTrianglesRppiSurvey's per-triangle body (source/device.cu:460-500)
// after its sqrS range tests: line of sight from getLOS (:45-56), squared
// projections from getSqrSdotL (:58-63), pi^2 = (s.L)^2 / L^2 and
// rp^2 = s^2 - pi^2 (getSqrRpSqrPi, :65-68), the three projection cuts, then
// the rp and pi range tests. Returns the flat index or -1.
inline long survey_rppi_body(const RppiGeometry& R, const Pt& p1, const Pt& p2, const Pt& p3, double s1,
                             double s2, double s3) {
  const double* o = R.ori;
  const double a[3] = {p1.x - o[0], p1.y - o[1], p1.z - o[2]};
  const double b[3] = {p2.x - o[0], p2.y - o[1], p2.z - o[2]};
  const double c[3] = {p3.x - o[0], p3.y - o[1], p3.z - o[2]};
  const double los[3] = {a[0] + b[0] + c[0], a[1] + b[1] + c[1], a[2] + b[2] + c[2]};
  const double sqrL = dot3(R.dot_pat, los, los);
  const double pm = R.sqr_pimax * sqrL;
  const double d12[3] = {p1.x - p2.x, p1.y - p2.y, p1.z - p2.z};
  double t = dot3(R.dot_pat, los, d12);
  const double q1 = t * t;
  if (pm < q1) return -1;
  const double d13[3] = {p1.x - p3.x, p1.y - p3.y, p1.z - p3.z};
  t = dot3(R.dot_pat, los, d13);
  const double q2 = t * t;
  if (pm < q2) return -1;
  const double d23[3] = {p2.x - p3.x, p2.y - p3.y, p2.z - p3.z};
  t = dot3(R.dot_pat, los, d23);
  const double q3 = t * t;
  if (pm < q3) return -1;
  const double pi1 = q1 / sqrL, pi2 = q2 / sqrL, pi3 = q3 / sqrL;
  const double rp1 = s1 - pi1, rp2 = s2 - pi2, rp3 = s3 - pi3;
  if (rp1 < R.sqr_rpmax && rp2 < R.sqr_rpmax && rp3 < R.sqr_rpmax && rp1 > R.sqr_rpmin &&
      rp2 > R.sqr_rpmin && rp3 > R.sqr_rpmin && pi1 < R.sqr_pimax && pi2 < R.sqr_pimax)
    return rppi_index(rp1, rp2, rp3, pi1, pi2, pi3, R.g.sqr_bins, R.g.nb, R.npi);
  return -1;
}

// Literal restatement of both rppi loop nests (source/device.cu:317-379 and
// :434-505): for every anchor, 27 cells for p2 and, for each p2 that passes,
// 27 cells again for p3.
template <int P>
void count_rppi_literal(const RppiGeometry& R, const Pt* p1, long n1, const Grid& g2, const Grid& g3,
                        int nthreads, RppiHist* out) {
  const Geometry& g = R.g;
  const long nbin = static_cast<long>(g.nb) * g.nb * g.nb * R.npi * R.npi;
  std::vector<RppiHist> part(nthreads);
  for (auto& h : part) h.bins.assign(nbin, Acc());
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 16)
  for (long a = 0; a < n1; ++a) {
    RppiHist& h = part[omp_get_thread_num()];
    const Pt q1 = p1[a];
    int home[3];
    anchor_cell(g, q1, home);
    for (int s2 = 0; s2 < 27; ++s2) {
      double sh2[3];
      long c2 = neighbour_cell(g, home, s2, sh2);
      if (c2 < 0) continue;
      for (long j = g2.start[c2]; j < g2.start[c2] + g2.count[c2]; ++j) {
        Pt q2;
        if (g.survey) {
          q2 = g2.pts[j];
        } else {
          shifted(g2.pts[j], sh2, &q2);
        }
        double pi1 = 0, rp1 = 0, s1 = 0;
        if (g.survey) {
          s1 = sqr_sep<P>(q1, q2);
          if (!(s1 < R.sqr_rmax && s1 > R.sqr_rmin)) continue;
        } else {
          const double dz = q1.z - q2.z;
          pi1 = dz * dz;
          if (!(pi1 < R.sqr_pimax)) continue;
          rp1 = rp_sum(R.rp_pat, q1.x - q2.x, q1.y - q2.y);
          if (!(rp1 < R.sqr_rpmax && rp1 > R.sqr_rpmin)) continue;
        }
        for (int s3 = 0; s3 < 27; ++s3) {
          double sh3[3];
          long c3 = neighbour_cell(g, home, s3, sh3);
          if (c3 < 0) continue;
          for (long l = g3.start[c3]; l < g3.start[c3] + g3.count[c3]; ++l) {
            Pt q3;
            if (g.survey) {
              q3 = g3.pts[l];
              const double s2v = sqr_sep<P>(q1, q3);
              const double s3v = sqr_sep<P>(q2, q3);
              if (s2v < R.sqr_rmax && s3v < R.sqr_rmax && s2v > R.sqr_rmin && s3v > R.sqr_rmin) {
                long t = survey_rppi_body(R, q1, q2, q3, s1, s2v, s3v);
                if (t != -1) rppi_add(h, t, q1.w * q2.w * q3.w);
              }
            } else {
              shifted(g3.pts[l], sh3, &q3);
              double dz2 = q1.z - q3.z, dz3 = q2.z - q3.z;
              const double pi2 = dz2 * dz2, pi3 = dz3 * dz3;
              if (pi2 < R.sqr_pimax && pi3 < R.sqr_pimax) {
                const double rp2 = rp_sum(R.rp_pat, q1.x - q3.x, q1.y - q3.y);
                const double rp3 = rp_sum(R.rp_pat, q2.x - q3.x, q2.y - q3.y);
                if (rp2 < R.sqr_rpmax && rp3 < R.sqr_rpmax && rp2 > R.sqr_rpmin && rp3 > R.sqr_rpmin) {
                  long t = rppi_index(rp1, rp2, rp3, pi1, pi2, pi3, g.sqr_bins, g.nb, R.npi);
                  if (t != -1) rppi_add(h, t, q1.w * q2.w * q3.w);
                }
              }
            }
          }
        }
      }
    }
  }
  out->bins.assign(nbin, Acc());
  out->overflow = Acc();
  for (int t = 0; t < nthreads; ++t) {
    for (long b = 0; b < nbin; ++b) {
      out->bins[b].add(part[t].bins[b].s);
      out->bins[b].add(part[t].bins[b].c);
    }
    out->overflow.add(part[t].overflow.s);
    out->overflow.add(part[t].overflow.c);
  }
}

struct RNbr {
  Pt p;            // neighbour (its periodic image in a box)
  double a, b;     // box: rp^2, pi^2 to the anchor; survey: sqrS, unused
};

// The anchor's neighbours that pass the reference's p2 cut. The p3 cuts
// against the anchor are the same tests (pi^2 < piMax^2 and rp^2 in range in
// a box, sqrS in range in a survey), so one list serves both roles.
template <int P>
inline void gather_rppi(const RppiGeometry& R, const Pt& q1, const int home[3], const Grid& gr,
                        std::vector<RNbr>* lst) {
  const Geometry& g = R.g;
  lst->clear();
  for (int s = 0; s < 27; ++s) {
    double sh[3];
    long c = neighbour_cell(g, home, s, sh);
    if (c < 0) continue;
    for (long j = gr.start[c]; j < gr.start[c] + gr.count[c]; ++j) {
      if (g.survey) {
        const Pt& q = gr.pts[j];
        const double s1 = sqr_sep<P>(q1, q);
        if (s1 < R.sqr_rmax && s1 > R.sqr_rmin) lst->push_back({q, s1, 0.0});
      } else {
        Pt q;
        shifted(gr.pts[j], sh, &q);
        const double dz = q1.z - q.z;
        const double pi = dz * dz;
        if (!(pi < R.sqr_pimax)) continue;
        const double rp = rp_sum(R.rp_pat, q1.x - q.x, q1.y - q.y);
        if (rp < R.sqr_rpmax && rp > R.sqr_rpmin) lst->push_back({q, rp, pi});
      }
    }
  }
}

// Same arithmetic as count_rppi_literal with each anchor's lists gathered
// once (the reference's inner walk recomputes the anchor-p3 terms for every
// p2 and gets the same values).
template <int P>
void count_rppi_lists(const RppiGeometry& R, const Pt* p1, long n1, const Grid& g2, const Grid& g3,
                      bool same23, int nthreads, RppiHist* out) {
  const Geometry& g = R.g;
  const long nbin = static_cast<long>(g.nb) * g.nb * g.nb * R.npi * R.npi;
  std::vector<RppiHist> part(nthreads);
  for (auto& h : part) h.bins.assign(nbin, Acc());
#pragma omp parallel num_threads(nthreads)
  {
    std::vector<RNbr> l2, l3;
    RppiHist& h = part[omp_get_thread_num()];
#pragma omp for schedule(dynamic, 4)
    for (long a = 0; a < n1; ++a) {
      const Pt q1 = p1[a];
      int home[3];
      anchor_cell(g, q1, home);
      gather_rppi<P>(R, q1, home, g2, &l2);
      const std::vector<RNbr>* pl3 = &l2;
      if (!same23) {
        gather_rppi<P>(R, q1, home, g3, &l3);
        pl3 = &l3;
      }
      const std::vector<RNbr>& L3 = *pl3;
      for (const RNbr& b : l2) {
        for (const RNbr& c : L3) {
          long t = -1;
          if (g.survey) {
            const double s3 = sqr_sep<P>(b.p, c.p);
            if (s3 < R.sqr_rmax && s3 > R.sqr_rmin) t = survey_rppi_body(R, q1, b.p, c.p, b.a, c.a, s3);
          } else {
            const double dz = b.p.z - c.p.z;
            const double pi3 = dz * dz;
            if (pi3 < R.sqr_pimax) {
              const double rp3 = rp_sum(R.rp_pat, b.p.x - c.p.x, b.p.y - c.p.y);
              if (rp3 < R.sqr_rpmax && rp3 > R.sqr_rpmin)
                t = rppi_index(b.a, c.a, rp3, b.b, c.b, pi3, g.sqr_bins, g.nb, R.npi);
            }
          }
          if (t != -1) rppi_add(h, t, q1.w * b.p.w * c.p.w);
        }
      }
    }
  }
  out->bins.assign(nbin, Acc());
  out->overflow = Acc();
  for (int t = 0; t < nthreads; ++t) {
    for (long b = 0; b < nbin; ++b) {
      out->bins[b].add(part[t].bins[b].s);
      out->bins[b].add(part[t].bins[b].c);
    }
    out->overflow.add(part[t].overflow.s);
    out->overflow.add(part[t].overflow.c);
  }
}

template <int P>
int run_rppi(const RppiGeometry& R, const Pt* p1, long n1, const Pt* p2, long n2, const Pt* p3, long n3,
             int nthreads, int variant, double* hist, double* overflow) {
  const Geometry& g = R.g;
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
  RppiHist acc;
  if (variant == 0)
    count_rppi_literal<P>(R, p1, n1, g2, G3, nthreads, &acc);
  else
    count_rppi_lists<P>(R, p1, n1, g2, G3, same23, nthreads, &acc);
  for (size_t b = 0; b < acc.bins.size(); ++b) hist[b] = acc.bins[b].value();
  if (overflow) *overflow = acc.overflow.value();
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

// Full (rp, pi) histogram of the reference's calculateD1D2D3 for the rppi bin
// type (source/cudaNcorr.cu:159-216, :220-430 with source/device.cu:317-379
// or :434-505): nb^3 * nPi^2 doubles in the reference's triCountsAll_ layout
// (rppi_index above). *overflow receives the total weight of triangles whose
// index falls past the end of that array, where the reference writes out of
// bounds. rp_pattern / dot_pattern select the contraction of sqrRpBox and of
// dotProduct_d3; fma_pattern that of sqrSep. Returns 0, -1 (bad edges, box
// or nPi), -2 (grid too large), -3 (a point outside the cell grid),
// -4 (bad args).
int oracle_count_rppi(const double* box, const double* edges, int n_edges, int num_pi_bins,
                      int is_survey, const double* ori, const double* p1, long n1, const double* p2,
                      long n2, const double* p3, long n3, int fma_pattern, int rp_pattern,
                      int dot_pattern, int nthreads, int variant, double* hist_out, double* overflow) {
  RppiGeometry R;
  int rc = make_rppi_geometry(box, edges, n_edges, num_pi_bins, is_survey, ori, &R);
  if (rc) return rc;
  const double nbin = std::pow(static_cast<double>(R.g.nb), 3) * R.npi * R.npi;
  if (nbin + R.npi >= 2147483647.0) return -2;  // the reference indexes with int
  if (n1 < 0 || n2 < 0 || n3 < 0 || !hist_out) return -4;
  if (rp_pattern < 0 || rp_pattern > 2 || dot_pattern < 0 || dot_pattern > 5) return -4;
  R.rp_pat = rp_pattern;
  R.dot_pat = dot_pattern;
  if (nthreads <= 0) nthreads = omp_get_max_threads();
  const Pt* a = reinterpret_cast<const Pt*>(p1);
  const Pt* b = reinterpret_cast<const Pt*>(p2);
  const Pt* c = reinterpret_cast<const Pt*>(p3);
  switch (fma_pattern) {
    case 0: return run_rppi<0>(R, a, n1, b, n2, c, n3, nthreads, variant, hist_out, overflow);
    case 1: return run_rppi<1>(R, a, n1, b, n2, c, n3, nthreads, variant, hist_out, overflow);
    case 2: return run_rppi<2>(R, a, n1, b, n2, c, n3, nthreads, variant, hist_out, overflow);
    case 3: return run_rppi<3>(R, a, n1, b, n2, c, n3, nthreads, variant, hist_out, overflow);
    case 4: return run_rppi<4>(R, a, n1, b, n2, c, n3, nthreads, variant, hist_out, overflow);
    case 5: return run_rppi<5>(R, a, n1, b, n2, c, n3, nthreads, variant, hist_out, overflow);
    default: return -4;
  }
}

// getTriangleIndexRppi (source/device.cu:203-255) on three (rp^2, pi^2) sides.
long oracle_rppi_index(double rp1, double rp2, double rp3, double pi1, double pi2, double pi3,
                       const double* edges, int n_edges, int num_pi_bins) {
  std::vector<double> sb(n_edges);
  for (int i = 0; i < n_edges; ++i) sb[i] = edges[i] * edges[i];
  return rppi_index(rp1, rp2, rp3, pi1, pi2, pi3, sb, n_edges - 1, num_pi_bins);
}

// Cell grid of the rppi constructor (source/cudaNcorr.cu:182-193):
// cell[3] and nc[3]. Returns make_rppi_geometry's status.
int oracle_rppi_grid(const double* box, const double* edges, int n_edges, int num_pi_bins, int is_survey,
                     double* cell, int* nc) {
  RppiGeometry R;
  int rc = make_rppi_geometry(box, edges, n_edges, num_pi_bins, is_survey, nullptr, &R);
  if (rc) return rc;
  for (int d = 0; d < 3; ++d) {
    cell[d] = R.cellv[d];
    nc[d] = R.g.nc[d];
  }
  return 0;
}

// prepTriCountsOutRppi (source/cudaNcorr.cu:88-105) and the triBinsOut_ /
// piBinsOut_ tables of the rppi constructor (source/cudaNcorr.cu:195-213):
// for every compacted (i <= j <= k, mid[k] <= mid[i] + mid[j]) and every pi
// pair (l, m): counts, rp mids (3 per entry) and pi bins (l, m) as doubles.
// Any output may be null; returns the number of entries.
long oracle_compact_rppi(const double* edges, int n_edges, int num_pi_bins, const double* hist_all,
                         double* counts_out, double* bins_out, double* pi_out) {
  const int nb = n_edges - 1;
  const long P = num_pi_bins;
  std::vector<double> mid(nb);
  for (int i = 1; i < n_edges; ++i) mid[i - 1] = (edges[i] + edges[i - 1]) / 2.0;
  long n = 0;
  for (int i = 0; i < nb; ++i)
    for (int j = i; j < nb; ++j)
      for (int k = j; k < nb; ++k)
        if (mid[k] <= mid[i] + mid[j])
          for (long l = 0; l < P; ++l)
            for (long m = 0; m < P; ++m) {
              const long idx = m + l * P + k * P * P + j * P * P * nb + static_cast<long>(i) * P * P * nb * nb;
              if (counts_out) counts_out[n] = hist_all[idx];
              if (bins_out) {
                bins_out[3 * n] = mid[i];
                bins_out[3 * n + 1] = mid[j];
                bins_out[3 * n + 2] = mid[k];
              }
              if (pi_out) {
                pi_out[2 * n] = static_cast<double>(l);
                pi_out[2 * n + 1] = static_cast<double>(m);
              }
              ++n;
            }
  return n;
}

// The six (rp^2, pi^2) values countTrianglesRppiSurvey derives for the
// triangle (p1, p2, p3) before its cuts (source/device.cu:446-488):
// out = {rp1, rp2, rp3, pi1, pi2, pi3}. Used to build inputs that separate
// the contraction candidates of dotProduct_d3.
void oracle_survey_rppi_sides(const double* p1, const double* p2, const double* p3, const double* ori,
                              int fma_pattern, int dot_pattern, double* out) {
  const Pt& a = *reinterpret_cast<const Pt*>(p1);
  const Pt& b = *reinterpret_cast<const Pt*>(p2);
  const Pt& c = *reinterpret_cast<const Pt*>(p3);
  const double o[3] = {ori[0], 0.0, 0.0};
  const double A[3] = {a.x - o[0], a.y - o[1], a.z - o[2]};
  const double B[3] = {b.x - o[0], b.y - o[1], b.z - o[2]};
  const double C[3] = {c.x - o[0], c.y - o[1], c.z - o[2]};
  const double los[3] = {A[0] + B[0] + C[0], A[1] + B[1] + C[1], A[2] + B[2] + C[2]};
  const double sqrL = dot3(dot_pattern, los, los);
  const Pt* pr[3][2] = {{&a, &b}, {&a, &c}, {&b, &c}};
  for (int k = 0; k < 3; ++k) {
    const Pt& u = *pr[k][0];
    const Pt& v = *pr[k][1];
    const double d[3] = {u.x - v.x, u.y - v.y, u.z - v.z};
    const double t = dot3(dot_pattern, los, d);
    const double pi = (t * t) / sqrL;
    const double s = oracle_sqr_sep(reinterpret_cast<const double*>(&u), reinterpret_cast<const double*>(&v),
                                    fma_pattern);
    out[k] = s - pi;
    out[3 + k] = pi;
  }
}

// sqrRpBox (source/device.cu:38-43) under a given contraction pattern.
double oracle_sqr_rp(const double* a, const double* b, int rp_pattern) {
  return rp_sum(rp_pattern, a[0] - b[0], a[1] - b[1]);
}

}  // extern "C"
