// FP32 classification of a box-mode rppi candidate, with rigorous error
// bands: it returns the reference's flat index (or "not counted") only when
// every decision of countTrianglesRppiBox / getTriangleIndexRppi
// (source/device.cu:203-255, :317-379 of cudaNcorr) is certain from the
// estimates, and "uncertain" otherwise, which sends the candidate to the FP64
// restatement. Host and device code, so that a host program can check the
// logic against the exact computation on adversarial inputs.
//
// Inputs per side (list entry of an anchor): the FP32 anchor-relative offset
// d = fl32(D) of the neighbour (its periodic image), rho = sqrt_rn(fl32(rp^2))
// of its exact rp^2 to the anchor, and meta = rp bin | pi bin << 16, both
// exact (computed from the FP64 values as the reference computes them).
// Error bounds (u = 2^-24; |D_xy| < rpMax and |D_z| < piMax for list
// entries, so the third side has |dz3| < 2 piMax and |dx3|, |dy3| < 2 rpMax):
//   pi3:   |fl(dz^2) - pi3| <= 20u piMax^2             band epi = 64u piMax^2
//   rp3:   |fma(dx,dx,dy*dy) - rp3| <= 48u rpMax^2,
//          |rho^2 - rp^2| <= 4u rpMax^2                 band erp = 128u rpMax^2
//   triangle: Q = 2 sqrt(AB) - |C - A - B| (A, B the anchor sides, C the
//          third, all projected) is estimated by 2 rho_j rho_l - |p| with
//          p = -2 (d_j.d_l)_xy within 20u rpMax^2; Q > 19.8u rpMax^2 proves
//          the reference's FP32 sqrtf test keeps the triangle (the same
//          argument as for the threeD bin type); margin M = 128u rpMax^2.
//   pi bin k of pi3: certain when pi3 lies farther than pmarg = 16u piMax^2
//          from k^2 and (k+1)^2, which covers the FP32 rounding of the
//          reference's floor(sqrtf(pi3)).
// Ties (rp3 equal to an anchor side, or the anchor sides equal) are never
// certain, so the reference's swap order is never guessed.
#pragma once
#include <cuda_runtime.h>

#include <cmath>

namespace ncorr_gb300 {

struct RppiFast {
  float epi, erp;              // band half-widths of the pi3 and rp3 estimates
  float pimax2;                // piMax^2 = nPi^2, exact in FP32
  float rpmax2_lo, rpmax2_hi;  // FP32 neighbours below / above rpMax^2
  float rpmin2_lo, rpmin2_hi;  // and rpMin^2
  float hm;                    // -M of the triangle margin
  float pmarg;                 // pi-bin margin
  float tab_scale;             // 2^k: entry of the rp3 table for an estimate rf
  float tab_band;              // the table's band: erp in a box, 4 erp in a survey
  int nb, npi;
};

constexpr int kRppiUncertain = -2;

// The rp3 table: kRppiTab entries over the estimate rf of the third side's
// rp^2, entry c for rf in [c, c + 1) / tab_scale (the last one for everything
// above). With the band e = tab_band, an entry holds the bin b when every rf
// of its cell has rf - e > fl32 up(edge_b^2) and rf + e < fl32
// down(edge_{b+1}^2): an rp^2 within e of rf then lies in bin b, and so
// within (rpMin^2, rpMax^2). It holds kRppiTabReject when every rf of the
// cell has rf - e >= rpmax2_hi or rf + e < rpmin2_lo (certainly cut), else
// kRppiTabUncertain. The bounds are evaluated exactly (in FP64, from FP32
// inputs), and tab_scale is a power of two, so the kernel's cell index
// floor(rf * tab_scale) is exact.
constexpr int kRppiTab = 1 << 14;
constexpr unsigned char kRppiTabReject = 0xFE, kRppiTabUncertain = 0xFF;

inline float rppi_tab_scale(float rpmax2_hi, float band) {
  // The largest power of two with (kRppiTab - 1) / scale >= rpmax2_hi + band,
  // so that the last (clamped) entry is a reject.
  const double need = (static_cast<double>(rpmax2_hi) + band) / (kRppiTab - 1);
  return static_cast<float>(std::ldexp(1.0, -static_cast<int>(std::ceil(std::log2(need)))));
}

inline void rppi_build_table(const RppiFast& f, const float* e2lo, const float* e2hi, unsigned char* tab) {
  const double inv = 1.0 / f.tab_scale;
  for (int c = 0; c < kRppiTab; ++c) {
    const double lo = c * inv - f.tab_band;  // infimum of rf - band over the cell
    const double hi = c == kRppiTab - 1 ? INFINITY : (c + 1) * inv + f.tab_band;  // supremum of rf + band
    unsigned char code = kRppiTabUncertain;
    if (lo >= f.rpmax2_hi || hi <= f.rpmin2_lo) {
      code = kRppiTabReject;
    } else {
      for (int b = 0; b < f.nb; ++b)
        if (lo > e2hi[b] && hi <= e2lo[b + 1]) code = static_cast<unsigned char>(b);
    }
    tab[c] = code;
  }
}

// Thresholds of the neighbour gather's FP32 prefilter, which drops the
// points that the reference certainly cuts against the anchor before the
// FP64 test. A valid point has |coordinate| < X = (nc + 1) cell per axis
// (the cell list clamps the upper face into the last cell), and box <= nc
// cell, so an offset D = q + shift - p1 has |D| < 3X. The kernel's FP32
// offset of a neighbour in a box is fl(fl(fl(q) + fl(shift)) - fl(p1)):
// roundings of at most uX, uX, 2uX, uX and u|D| (u = 2^-24) put it within
// 8uX of D; in a survey fl(fl(q) - fl(p1)) is within 4uX. The reference's
// own FP64 offset lies within 2^-50 X of D. With E the per-axis bound, the FP32 rp (pi, s) estimate is
// within |E_xy| (E_z, |E|) of the reference's, and the FP32 squares err by
// at most (1 + u)^2 (1 + u, (1 + u)^3) relatively; each threshold adds
// those, plus a relative 2^-40 that covers the reference's FP64 rounding of
// the squares, so an estimate past it proves the reference cuts the point:
// box rp^2 > rp_hi or < rp_lo (-1: no lower cut) or dz^2 > pi_hi, survey
// s^2 > s_hi.
struct RppiGatherCut {
  float rp_hi, rp_lo, pi_hi, s_hi;
};

inline RppiGatherCut rppi_gather_cut(const int nc[3], const double cell[3], bool survey, double rpmin, double rpmax,
                                     double pimax) {
  auto up = [](double x) {
    float f = static_cast<float>(x);
    return static_cast<double>(f) < x ? std::nextafter(f, INFINITY) : f;
  };
  auto down = [](double x) {
    float f = static_cast<float>(x);
    return static_cast<double>(f) > x ? std::nextafter(f, -INFINITY) : f;
  };
  const double u = std::ldexp(1.0, -24), r40 = std::ldexp(1.0, -40);
  double e[3];
  for (int d = 0; d < 3; ++d) {
    const double X = (nc[d] + 1.0) * cell[d];
    e[d] = u * (survey ? 4.0 : 8.0) * X * (1.0 + 1e-6) + std::ldexp(X, -50);
  }
  const double smax = std::sqrt(rpmax * rpmax + pimax * pimax);
  const double er = std::sqrt(e[0] * e[0] + e[1] * e[1]) + rpmax * r40;
  const double ez = e[2] + pimax * r40;
  const double es = std::sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]) + smax * r40;
  RppiGatherCut c;
  c.rp_hi = up((rpmax + er) * (rpmax + er) * (1.0 + u) * (1.0 + u) * (1.0 + r40));
  c.rp_lo = rpmin > er ? down((rpmin - er) * (rpmin - er) * (1.0 - u) * (1.0 - u) * (1.0 - r40)) : -1.0f;
  c.pi_hi = up((pimax + ez) * (pimax + ez) * (1.0 + u) * (1.0 + r40));
  c.s_hi = up((smax + es) * (smax + es) * (1.0 + u) * (1.0 + u) * (1.0 + u) * (1.0 + r40));
  return c;
}

// Survey mode: whether the anchor side (p1, q), with FP32 offset d = p1 - q
// and s^2 = s2, is certainly cut for every partner of the list. The
// reference's line of sight for a pair is L = 3A + (pj - p1) + (pl - p1),
// A = (p1.x - ori.x, p1.y, p1.z) (source/device.cu:45-56); both partners
// lie within sMax of p1, so L is within the angle phi of A, sin(phi) <=
// (s + sMax) / (3 |A|). With theta_A the angle between d and A, the side's
// |cos(theta)| against L lies between cos(theta_A + phi) (0 past pi/2) and
// cos(theta_A - phi) (1 below 0), so pi^2 = s^2 cos^2 and rp^2 = s^2 sin^2
// are bounded for every partner; the side is cut when pi^2 >= piMax^2, rp^2
// >= rpMax^2 or rp^2 <= rpMin^2 over the whole range (the reference keeps
// rpMin^2 < rp^2 < rpMax^2 and pi^2 < piMax^2 for both anchor sides,
// source/device.cu:483-490). The FP32 evaluation errs by a few 2^-24
// relatively; the margins (1e-5 on cos, 1e-4 on sin(phi), 1e-5 on the
// squares) exceed that and the reference's FP64 rounding by far.
// los = (A in FP32, |A|); smax >= sMax; pimax2, rpmax2 >= and rpmin2 <= the
// squared limits.
__host__ __device__ inline bool rppi_los_cut(float dx, float dy, float dz, float s2, float4 los, float smax,
                                             float pimax2, float rpmax2, float rpmin2) {
  const float s = sqrtf(s2);
  const float sp = (s + smax) / (3.0f * los.w) * 1.0001f + 1e-6f;
  if (!(sp < 0.999f) || !(s2 > 0.0f)) return false;
  const float cp = sqrtf(1.0f - sp * sp);
  const float c = fabsf(dx * los.x + dy * los.y + dz * los.z) / (s * los.w);
  const float cl = fmaxf(c - 1e-5f, 0.0f), ch = fminf(c + 1e-5f, 1.0f);
  const float sah = sqrtf(fmaxf(1.0f - cl * cl, 0.0f));
  const float cmin = fmaxf(cl * cp - sah * sp - 1e-6f, 0.0f);
  const float cmax = ch >= cp ? 1.0f : fminf(ch + sah * sp + 1e-6f, 1.0f);
  const float lo = s2 * (1.0f - 1e-5f), hi = s2 * (1.0f + 1e-5f);
  return (lo * cmin * cmin >= pimax2 * (1.0f + 1e-5f)) |
         (lo * (1.0f - cmax * cmax) - 1e-5f * hi >= rpmax2 * (1.0f + 1e-5f)) |
         (hi * (1.0f - cmin * cmin) + 1e-5f * hi <= rpmin2 * (1.0f - 1e-5f));
}

// An estimate of sqrt(x) for x >= 0; its error only costs certainty (the
// pi-bin test below checks the bin it gives against margins).
__host__ __device__ inline float rppi_sqrt_est(float x) {
#ifdef __CUDA_ARCH__
  float r;
  asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
#else
  return std::sqrt(x);
#endif
}

// Survey mode: the FP32 classification of a pair (j, l) of an anchor's list:
// the flat index when every decision of the reference (source/device.cu:
// 455-490 and getTriangleIndexRppi, :203-255) is certain, -1 when it
// certainly does not count the pair, and kRppiUncertain otherwise. Inputs:
// the FP32 offsets dj = pj - p1 and dl = pl - p1 with their FP32 s^2 in .w,
// and A = (p1.x - ori.x, p1.y, p1.z) in FP32. The reference's line of sight
// (getLOS, getSqrSdotL, getSqrRpSqrPi, :45-68) is L = 3A + dj + dl; tau_k =
// L.d_k / |L| is side k's projection (d1 = dj, d2 = dl, d3 = dj - dl), pi_k
// = tau_k^2 and rp_k = s_k^2 - pi_k. With u = 2^-24, each offset errs by
// u|d| and each A component by u|A|; the FP32 L = fl(fma(3, A, fl(dj + dl)))
// is then within EL = u(2|L| + 6 sMax) of the true one (3|A| <= |L| + 2
// sMax), its direction within 2 EL / |L|, and tau_k within |d_k| (2 EL / |L|
// + 8u) + u sMax (4u sMax for d3 = fl(dj - dl)), the 8u covering the FP32
// dot product and normalisation; s3^2 from the FP32 d3 is within 30u
// sMax^2. The bounds carry 1% on these, 4u for the FP32 rounding of their
// own evaluation, a factor 2 on EL and on the offset errors over this
// derivation, and a relative 1e-6 on the limits that covers the reference's
// FP64 rounding. Side k's rp^2 and pi^2 thus lie in intervals
// [R_lo, R_hi] and [P_lo, P_hi]. The pair is certainly not counted when a
// pi^2 exceeds piMax^2 or an rp^2 leaves (rpMin^2, rpMax^2) over its whole
// interval. The decisions are certain when: s3^2 is inside
// (0, sMax^2); every pi^2 is below piMax^2 and every rp^2 inside (rpMin^2,
// rpMax^2); the three rp^2 intervals are disjoint (their order is the
// reference's sort; ties are never certain); sqrt(R_lo) of the two shortest
// sides exceed sqrt(R_hi) of the longest by a relative 1e-6 (the FP32 sqrtf
// test keeps the triangle); every rp^2 interval lies in one bin of the rp^2
// table, whose cells decide a bin only for all values within f.tab_band of
// them (so the interval's half-width must not exceed it); and the pi^2
// intervals of the two shortest sides lie farther than f.pmarg from the
// squares k^2, (k+1)^2 around their pi bin k, which covers the FP32 rounding
// of the reference's floor(sqrtf(pi^2)).
__host__ __device__ inline int rppi_survey_index(float4 dj, float4 dl, float4 los, float smax, const RppiFast& f,
                                                 const unsigned char* tab) {
  const float u = 5.9604645e-8f;  // 2^-24
  const float lx = fmaf(3.0f, los.x, dj.x + dl.x), ly = fmaf(3.0f, los.y, dj.y + dl.y),
              lz = fmaf(3.0f, los.z, dj.z + dl.z);
  const float ln = sqrtf(fmaf(lz, lz, fmaf(ly, ly, lx * lx)));
  const float el = 2.02f * u * (2.0f * ln + 6.0f * smax);
  if (!(ln > 2.0f * el)) return kRppiUncertain;
  const float inv = 1.0f / ln, ang = 2.02f * el / (ln - el) + 8.0f * u, ed = 2.02f * u * smax;
  const float d3x = dj.x - dl.x, d3y = dj.y - dl.y, d3z = dj.z - dl.z;
  const float s3 = fmaf(d3z, d3z, fmaf(d3y, d3y, d3x * d3x));
  const float t[3] = {fabsf(fmaf(lz, dj.z, fmaf(ly, dj.y, lx * dj.x))) * inv,
                      fabsf(fmaf(lz, dl.z, fmaf(ly, dl.y, lx * dl.x))) * inv,
                      fabsf(fmaf(lz, d3z, fmaf(ly, d3y, lx * d3x))) * inv};
  const float ss[3] = {dj.w, dl.w, s3};
  const float es3 = 30.3f * u * smax * smax;
  const float pm = f.pimax2 * (1.0f + 1e-6f), pml = f.pimax2 * (1.0f - 1e-6f);
  const float rhi = f.rpmax2_hi * (1.0f + 1e-6f), rhl = f.rpmax2_lo * (1.0f - 1e-6f);
  const float rlo = f.rpmin2_lo * (1.0f - 1e-6f), rll = f.rpmin2_hi * (1.0f + 1e-6f);
  float plo[3], phi[3], rl[3], rh[3];
  bool reject = false, ok = true;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float e = sqrtf(ss[k]) * ang + (k == 2 ? 4.0f : 1.0f) * ed;
    const float a = fmaxf(t[k] - e, 0.0f), b = t[k] + e;
    const float sl = k == 2 ? ss[k] - es3 : ss[k] * (1.0f - 4.0f * u);
    const float sh = k == 2 ? ss[k] + es3 : ss[k] * (1.0f + 4.0f * u);
    plo[k] = a * a * (1.0f - 4.0f * u);
    phi[k] = b * b * (1.0f + 4.0f * u);
    rl[k] = sl - phi[k] - 4.0f * u * (fabsf(sl) + phi[k]);
    rh[k] = sh - plo[k] + 4.0f * u * (sh + plo[k]);
    reject |= (plo[k] > pm) | (rl[k] > rhi) | (rh[k] < rlo);
    ok &= (phi[k] < pml) & (rh[k] < rhl) & (rl[k] > rll);
  }
  ok &= (s3 + es3 < f.rpmax2_lo + f.pimax2 * (1.0f - 1e-6f)) & (s3 - es3 > 0.0f);
  // The reference's sort of (rp1, rp2, rp3): certain when the intervals are
  // disjoint. o[i] = the side in sorted position i.
  const bool g01 = rl[0] > rh[1], l01 = rh[0] < rl[1];
  const bool g02 = rl[0] > rh[2], l02 = rh[0] < rl[2];
  const bool g12 = rl[1] > rh[2], l12 = rh[1] < rl[2];
  ok &= (g01 | l01) & (g02 | l02) & (g12 | l12);
  // Rank of sides 0 and 1 (number of sides below; side 2 takes the rest).
  const int rk0 = (g01 ? 1 : 0) + (g02 ? 1 : 0), rk1 = (l01 ? 1 : 0) + (g12 ? 1 : 0);
  auto side_at = [&](int r) { return rk0 == r ? 0 : (rk1 == r ? 1 : 2); };
  const int oa = side_at(0), ob = side_at(1), oc = side_at(2);
  // Side k's values by selects (no indexed register arrays).
  auto pick = [](const float* v, int k) { return k == 0 ? v[0] : (k == 1 ? v[1] : v[2]); };
  // FP32 triangle test of the sorted sides: keep certain.
  ok &= (sqrtf(fmaxf(pick(rl, oa), 0.0f)) + sqrtf(fmaxf(pick(rl, ob), 0.0f))) * (1.0f - 1e-6f) >
        sqrtf(fmaxf(pick(rh, oc), 0.0f)) * (1.0f + 1e-6f);
  // rp bins from the table, pi bins of the two shortest sides.
  int bin[3], pib[2];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const int k = i == 0 ? oa : (i == 1 ? ob : oc);
    const float rlk = pick(rl, k), rhk = pick(rh, k), plk = pick(plo, k), phk = pick(phi, k);
    const float mid = 0.5f * (rlk + rhk), hw = 0.5f * (rhk - rlk);
    const int code = tab[static_cast<int>(fminf(fmaxf(mid, 0.0f) * f.tab_scale, static_cast<float>(kRppiTab - 1)))];
    ok &= (code < kRppiTabReject) & (hw + 4.0f * u * fabsf(mid) <= f.tab_band);
    bin[i] = code;
    if (i < 2) {
      const float pmid = 0.5f * (plk + phk);
      const int q = static_cast<int>(fminf(rppi_sqrt_est(pmid), 4095.0f));
      const float q2 = static_cast<float>(q * q), q3 = static_cast<float>((q + 1) * (q + 1));
      ok &= ((q == 0) | (plk - f.pmarg > q2)) & (phk + f.pmarg < q3);
      pib[i] = q;
    }
  }
  const unsigned P = static_cast<unsigned>(f.npi), B = static_cast<unsigned>(f.nb);
  const unsigned idx = static_cast<unsigned>(pib[1]) +
                       P * (static_cast<unsigned>(pib[0]) +
                            P * (static_cast<unsigned>(bin[2]) +
                                 B * (static_cast<unsigned>(bin[1]) + B * static_cast<unsigned>(bin[0]))));
  return reject ? -1 : (ok ? static_cast<int>(idx) : kRppiUncertain);
}

// The flat index (below 2^31: the constructor checks nb^3 nPi^2 + nPi), -1
// (the reference certainly does not count it), or kRppiUncertain. `tab` is
// the rp3 table. Every test is evaluated and combined with selects (no early
// return), so a warp classifying 32 pairs runs a single path.
__host__ __device__ inline int rppi_fast_index(float xj, float yj, float zj, float rj, unsigned mj, float xl,
                                               float yl, float zl, float rl, unsigned ml, const RppiFast& f,
                                               const unsigned char* tab) {
  const float dz = zj - zl, dx = xj - xl, dy = yj - yl;
  const float pf = dz * dz;
  const float rf = fmaf(dx, dx, dy * dy);
  const float lo = rf - f.erp, hi = rf + f.erp;
  const int b3 = tab[static_cast<int>(fminf(rf * f.tab_scale, static_cast<float>(kRppiTab - 1)))];
  // The tests below combine with & and | (no short-circuit): one path.
  // Certainly cut: pi3 >= piMax^2, or rp3 outside (rpMin^2, rpMax^2).
  const bool reject = (pf - f.epi >= f.pimax2) | (b3 == kRppiTabReject);
  // rp3 certainly in range and in bin b3; pi3 certainly below piMax^2.
  bool ok = (pf + f.epi < f.pimax2) & (b3 < kRppiTabReject);
  // Order of the three rp^2: rho is monotone in rp^2, so rho_j < rho_l
  // proves A < B; equal rho leaves the order open.
  ok &= rj != rl;
  const bool jfirst = rj < rl;
  const float a = rj * rj, b = rl * rl;
  const float mn = jfirst ? a : b, mx = jfirst ? b : a;
  const bool below = hi < mn, above = lo > mx, between = (lo > mn) & (hi < mx);
  ok &= below | above | between;
  const int pos = below ? 0 : (above ? 2 : 1);  // anchor sides below rp3
  // Triangle test: |p| < 2 rho_j rho_l - M with p = -2 (d_j.d_l)_xy, as
  // |(d_j.d_l)_xy| < fma(rho_j, rho_l, -M/2) (both sides halved exactly).
  ok &= fabsf(fmaf(xj, xl, yj * yl)) < fmaf(rj, rl, 0.5f * f.hm);
  // pi bin of the third side, needed when it is one of the two shortest.
  const int k = static_cast<int>(fminf(rppi_sqrt_est(pf), 4095.0f));
  const float k2 = static_cast<float>(k * k), k3 = static_cast<float>((k + 1) * (k + 1));
  const float w = f.epi + f.pmarg;
  ok &= (pos == 2) | (((k == 0) | (pf - w > k2)) & (pf + w < k3));
  const unsigned ms = jfirst ? mj : ml, mL = jfirst ? ml : mj;
  const int rs = static_cast<int>(ms & 0xffffu), ps = static_cast<int>(ms >> 16);
  const int rL = static_cast<int>(mL & 0xffffu), pL = static_cast<int>(mL >> 16);
  // Sorted ascending: rp bins r1 <= r2 <= r3, pi bins q1, q2 of the two shortest.
  const int r1 = pos == 0 ? b3 : rs;
  const int q1 = pos == 0 ? k : ps;
  const int r2 = pos == 0 ? rs : (pos == 1 ? b3 : rL);
  const int q2 = pos == 0 ? ps : (pos == 1 ? k : pL);
  const int r3 = pos == 2 ? b3 : rL;
  // Unsigned: the discarded values of uncertain pairs may wrap.
  const unsigned P = static_cast<unsigned>(f.npi), B = static_cast<unsigned>(f.nb);
  const unsigned idx = q2 + P * (q1 + P * (r3 + B * (r2 + B * static_cast<unsigned>(r1))));
  return reject ? -1 : (ok ? static_cast<int>(idx) : kRppiUncertain);
}

}  // namespace ncorr_gb300
