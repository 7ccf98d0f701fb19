// The (rp, pi) bin type: geometry and kernel arguments shared by rppi.cu and
// the C ABI. The reference's second constructor (source/cudaNcorr.cu:159-216)
// bins each side by its projected separation rp (nb bins, the given edges)
// and, for the two shortest sides, by its line-of-sight separation pi (nPi
// unit bins); its kernels are countTrianglesRppiBox (source/device.cu:317-379,
// line of sight = z) and countTrianglesRppiSurvey (source/device.cu:434-505,
// line of sight = the sum of the three position vectors).
#pragma once
#include "engine.cuh"
#include "rppi_fast.cuh"

namespace ncorr_gb300 {

struct RppiGeom {
  int nb;            // rp bins
  int npi;           // unit pi bins (numPiBins_)
  int survey;
  int fma_pattern;   // contraction of sqrSep (survey)
  int rp_pattern;    // contraction of sqrRpBox: 0 none, 1 fma(dy,dy,dx*dx), 2 fma(dx,dx,dy*dy)
  int dot_pattern;   // contraction of dotProduct_d3 (sqrSep numbering)
  int nc[3];
  double box[3];
  double cell[3];    // box: (rpMax, rpMax, piMax); survey: rMax = sqrtf(rpMax^2 + piMax^2) per axis
  double ori_x;      // d_ori as the survey kernel sees it: (ori.x, 0, 0)
  double sqr_rpmax, sqr_rpmin, sqr_pimax;
  double sqr_rmax, sqr_rmin;  // survey pair cut: rpMax^2 + piMax^2 and 0
  double sqr_bins[kMaxEdges];
  // FP32 prefilter on anchor-relative offsets: a candidate whose estimate
  // passes one of these thresholds is certainly cut by the reference.
  float f_pi_hi;     // box: dz^2 estimate > f_pi_hi  => pi^2 >= piMax^2
  float f_rp_hi;     // box: rp^2 estimate > f_rp_hi  => rp^2 >= rpMax^2
  float f_rp_lo;     // box: rp^2 estimate < f_rp_lo  => rp^2 <= rpMin^2
  float f_s_hi;      // survey: s^2 estimate > f_s_hi => s^2 >= sqrRMax
  // FP32 prefilter of the neighbour gather, on the points' FP32 copies (each
  // coordinate rounded once) and FP32 image shifts: a point whose estimate
  // passes one of these thresholds is certainly cut against the anchor.
  float fbox[3];     // fl32(box)
  float a_pi_hi;     // box: dz^2 estimate > a_pi_hi  => pi^2 >= piMax^2
  float a_rp_hi;     // box: rp^2 estimate > a_rp_hi  => rp^2 >= rpMax^2
  float a_rp_lo;     // box: rp^2 estimate < a_rp_lo  => rp^2 <= rpMin^2 (-1: never)
  float a_s_hi;      // survey: s^2 estimate > a_s_hi => s^2 >= sqrRMax
  float los_smax;    // survey: smallest float >= sqrt(sqrRMax), for rppi_los_cut
  long long nbins;   // nb^3 * nPi^2
  // Box mode: the FP32 classifier (rppi_fast.cuh) and its bin-edge bounds.
  RppiFast fast;
  float fe2lo[kMaxEdges];  // largest float <= edges^2
  float fe2hi[kMaxEdges];  // smallest float >= edges^2
};

struct RppiArgs {
  RppiGeom g;
  const double4_16a* a_pd;  // anchors (cell order)
  const float4* a_pq;       // their FP32 copies; .w = cell id (int bits)
  int n1;
  const double4_16a* pd2;
  const float4* pq2;
  const int* start2;
  const int* count2;
  const double4_16a* pd3;
  const float4* pq3;
  const int* start3;
  const int* count3;
  // Per-warp neighbour lists: one list of `cap` entries per warp when p2 and
  // p3 are one catalogue, two otherwise.
  double4_16a* l_pos;  // neighbour (its image in a box), weight
  double2* l_ab;       // box: (rp^2, pi^2) to the anchor; survey: (sqrS, 0)
  float4* l_rel;       // FP32 anchor-relative offset; box: .w = sqrt_rn(fl32(rp^2))
  unsigned* l_meta;    // box: exact rp bin | pi bin << 16 of the anchor side
  double* l_pw;        // weighted: fl(w_anchor * w_neighbour); else null
  const unsigned char* tab;  // box: the classifier's rp3 table (kRppiTab entries)
  int cap;
  unsigned long long* hist_u;  // hist_copies x (nbins + 1) counts; [nbins] collects indices past the end
  double* hist_w;              // the same for weighted sums
  int hist_copies;             // CTA b adds to copy b % hist_copies
  int* work;
  int* flags;
  unsigned long long* stats;   // [0] anchors, [1] scanned, [2] candidate pairs, [3] FP64 evaluations,
                               // [4] pairs settled by the FP32 classifier
};

}  // namespace ncorr_gb300
