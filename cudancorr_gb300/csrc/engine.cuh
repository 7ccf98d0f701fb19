// Internal definitions shared by the engine's CUDA translation units.
//
// Data layout in HBM (one "catalogue" = one std::vector<double4> argument of
// the reference's calculateD1D2D3):
//   pd[n]    double4  exact (x, y, z, w), grouped by cell          32 B/point
//   pq[n]    float4   (x - o_c, y - o_c, z - o_c, w) in FP32, o_c = the
//                     cell's lower corner (cell-local coordinates)    16 B/point
//   pc[n]    int      flat cell id of each sorted point               4 B/point
//   start/count[ncell] int   cell offsets of the cell list
// The cell grid is the reference's: cell edge = r_max, nc = ceil(box/r_max),
// flat id z + nc.z*(y + nc.y*x) (source/cudaNcorr.cu:50-58, :137-140).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace ncorr_gb300 {

constexpr int kMaxEdges = 128;   // nb <= 127
constexpr int kThreads = 512;    // triangle kernel CTA (one per SM)
constexpr int kWarps = kThreads / 32;
constexpr int kReg = 4;          // list entries per lane held in registers
constexpr int kTile = 32 * kReg; // column tile of the pair loop
constexpr int kQueueCap = 256;   // per-warp queue of careful/exact-path candidates
#ifndef NCORR_TABLE_SIZE
#define NCORR_TABLE_SIZE 65536
#endif
constexpr int kTableSize = NCORR_TABLE_SIZE;  // bin table entries (u8)

// Bin codes returned by the FP32 classifiers.
constexpr unsigned kCodeReject = 0xFEu;
constexpr unsigned kCodeCareful = 0xFFu;

// The CTA histogram of the triangle kernel holds, for every (bin_j, bin_l),
// a row of nb + 2 bins: the nb real ones, then two sinks that rejected and
// careful candidates add into (the bin table's codes for them), so the
// candidate bodies need not test the code. Nothing reads the sinks.
__host__ __device__ inline int hist_row(int nb) { return nb + 2; }
__host__ __device__ inline int hist_words(int nb) { return nb * nb * hist_row(nb); }
// Bin-table codes of "reject" and "careful": with a CTA histogram (code
// scale = the byte stride of a bin, > 1) the two sink bins of the row; with
// the global histogram (code scale 1) the plain markers above.
__host__ __device__ inline unsigned table_code_reject(int nb, int cs) {
  return cs > 1 ? static_cast<unsigned>(nb * cs) : kCodeReject;
}
__host__ __device__ inline unsigned table_code_careful(int nb, int cs) {
  return cs > 1 ? static_cast<unsigned>((nb + 1) * cs) : kCodeCareful;
}

// One neighbour-list entry of the triangle kernel (32 bytes): the offset d
// from the anchor and rho^2 (rho = sqrt_rn of the r1^2 estimate), then what
// the pair loop needs when the entry is a row, computed once when the list is
// built: 2 rho and bin * (the histogram stride of bin_j); then bin | slot << 8
// and the point's index in its catalogue.
struct __align__(16) ListEnt {
  float4 e;
  float a2r;
  unsigned key;
  unsigned m;
  int p;
};
// Padding records after each list: a row loop that runs up to this many rows
// past the list's end reads padding rows, which add into sink bins only.
constexpr int kListPad = 8;

// Error flags written by kernels.
constexpr int kFlagOutOfGrid = 1;     // a point the reference would index out of bounds
constexpr int kFlagNonFinite = 2;
constexpr int kFlagSurveyFace = 4;    // survey anchor whose unclamped cell index is nc
constexpr int kFlagListOverflow = 8;  // neighbour list exceeded its slab (host bug)
constexpr int kFlagWeighted = 16;     // some weight != 1.0 (informational)
constexpr int kFlagNoSym6 = 32;       // a point near a cell face or with an inexact +-box image
constexpr int kFlagSchedStall = 128;  // a warp waited too long for the CTA histogram (never expected)

struct Geom {
  int nb;                 // bins per side
  int nc[3];              // cells per axis
  int survey;             // 1: clipped neighbours, no image shift
  int fma_pattern;        // contraction of the reference's sqrSep
  double box[3];
  double cell;            // = r_max
  double sqr_rmin, sqr_rmax;
  double sqr_bins[kMaxEdges];  // edges^2 as the reference computes them (double)
  float e2lo[kMaxEdges];       // largest float <= edges^2
  float e2hi[kMaxEdges];       // smallest float >= edges^2
  // FP32 error model: |v - V| <= ka*v + kb for every FP32 r^2 estimate v of
  // the reference's double r^2 V (pair and triangle stage alike).
  float ka, kb;
  // Prefilter of the pair stage on cell-local FP32 estimates.
  float pre_lo, pre_hi;
  // Triangle-test margin: with list values rho_j, rho_l (square roots of the
  // r1^2 and r2^2 estimates) and third side v, the reference's FP32 sqrtf
  // test certainly keeps the triangle when
  // |v - (rho_j^2 + rho_l^2)| < 2 rho_j rho_l + hm  (hm = -M < 0).
  float hm;
  // Bin table: code of r^2 = table[rint(v*tab_scale)], clamped to the last entry.
  float tab_scale;
  int tab_n;
};

struct Catalog {
  const double4_16a* pd;
  const float4* pq;
  const int* pc;
  const int* start;
  const int* count;
  int n;
};

// A candidate triangle whose FP32 classification stays uncertain, deferred to
// the exact FP64 kernel: the anchor's position in the work queue (which names
// the batch item and the anchor's sorted index in its catalogue 1), the two
// neighbours (sorted indices in catalogues 2 and 3), and
// meta = slot_j | slot_l << 5 | bin_j << 10 | bin_l << 18.
struct ExactEntry {
  int ai, pj, pl;
  unsigned meta;
};

// Fixed-point weighted sums are kept as signed 128-bit integers in two u64
// words per bin: lo at [2*b], hi at [2*b+1].
struct HistOut {
  unsigned long long* counts;  // nb^3 unsorted keys (count mode)
  unsigned long long* wsum;    // 2*nb^3 (weighted mode)
};

// One catalogue triple (p1, p2, p3) counted into its own histogram; a single
// calculateD1D2D3 is a batch of one item. Items of one launch share the
// geometry, the bins and the kernel variant (survey, p2 == p3, weighted).
struct BatchItem {
  Catalog c1, c2, c3;
  HistOut hist;
  double* out;                // folded nb^3 result (triCountsAll_ layout)
  unsigned long long* total;  // sum of the folded unweighted counts
  const int* flags1;          // grid flags of catalogue 1, read on the device
  int sym6_ok;                // the host-side conditions of the six-fold loop hold
  int cell_base;              // offset of this item's cells in per-cell arrays
};

// The six-fold loop runs for an item when the host allowed it and no point of
// catalogue 1 broke the per-point conditions while it was gridded.
__device__ __forceinline__ bool item_sym6(const BatchItem& it) {
  return it.sym6_ok && !(*it.flags1 & kFlagNoSym6);
}

// Sum of squares of the reference's sqrSep (source/device.cu:30-36) under
// the contraction pattern the CUDA compiler applied to it; the explicit
// intrinsics keep this code from being contracted differently.
__device__ __forceinline__ double sqr_sum_exact(double dx, double dy, double dz, int pattern) {
  switch (pattern) {
    case 0:
      return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
    case 1:
      return __fma_rn(dz, dz, __fma_rn(dy, dy, __dmul_rn(dx, dx)));
    case 2:
      return __fma_rn(dz, dz, __fma_rn(dx, dx, __dmul_rn(dy, dy)));
    case 3:
      return __fma_rn(dz, dz, __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
    case 4:
      return __dadd_rn(__fma_rn(dy, dy, __dmul_rn(dx, dx)), __dmul_rn(dz, dz));
    default:
      return __dadd_rn(__fma_rn(dx, dx, __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
  }
}

__device__ __forceinline__ double sqr_sep_exact(double ax, double ay, double az, double bx,
                                                double by, double bz, int pattern) {
  return sqr_sum_exact(__dsub_rn(ax, bx), __dsub_rn(ay, by), __dsub_rn(az, bz), pattern);
}

// Bin of an exact r^2 already known to lie in (rmin^2, rmax^2): the unique b
// with sqr_bins[b] <= r < sqr_bins[b+1] (source/device.cu:181-191).
__device__ __forceinline__ int exact_bin(double r, const double* sqr_bins, int nb) {
  int lo = 0, hi = nb - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (r >= sqr_bins[mid])
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// The reference's FP32 triangle test (source/device.cu:163-175) on three
// exact r^2 values: true when the triangle is kept.
__device__ __forceinline__ bool exact_triangle_ok(double r1, double r2, double r3) {
  double t;
  if (r1 > r2) { t = r1; r1 = r2; r2 = t; }
  if (r1 > r3) { t = r1; r1 = r3; r3 = t; }
  if (r2 > r3) { t = r2; r2 = r3; r3 = t; }
  float s1 = __fsqrt_rn(__double2float_rn(r1));
  float s2 = __fsqrt_rn(__double2float_rn(r2));
  float s3 = __fsqrt_rn(__double2float_rn(r3));
  return !(__fadd_rn(s1, s2) <= s3);
}

}  // namespace ncorr_gb300
