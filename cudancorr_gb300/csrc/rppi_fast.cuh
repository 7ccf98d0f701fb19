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
  int nb, npi;
};

constexpr long long kRppiUncertain = -2;

// The flat index, -1 (the reference certainly does not count it), or
// kRppiUncertain. e2lo/e2hi: FP32 neighbours below / above each bin edge^2.
__host__ __device__ inline long long rppi_fast_index(float xj, float yj, float zj, float rj, unsigned mj, float xl,
                                                     float yl, float zl, float rl, unsigned ml, const RppiFast& f,
                                                     const float* e2lo, const float* e2hi) {
  const float dz = zj - zl, dx = xj - xl, dy = yj - yl;
  const float pf = dz * dz;
  if (!(pf + f.epi < f.pimax2)) return (pf - f.epi >= f.pimax2) ? -1 : kRppiUncertain;
  const float rf = fmaf(dx, dx, dy * dy);
  const float lo = rf - f.erp, hi = rf + f.erp;
  if (lo >= f.rpmax2_hi || hi < f.rpmin2_lo) return -1;
  if (!(lo > f.rpmin2_hi && hi < f.rpmax2_lo)) return kRppiUncertain;
  // Order of the three rp^2: rho is monotone in rp^2, so rho_j < rho_l
  // proves A < B; equal rho leaves the order open.
  if (rj == rl) return kRppiUncertain;
  const bool jfirst = rj < rl;
  const float a = rj * rj, b = rl * rl;
  const float mn = jfirst ? a : b, mx = jfirst ? b : a;
  int pos;  // anchor sides below rp3
  if (hi < mn)
    pos = 0;
  else if (lo > mx)
    pos = 2;
  else if (lo > mn && hi < mx)
    pos = 1;
  else
    return kRppiUncertain;
  // Triangle test.
  const float p = -2.0f * fmaf(xj, xl, yj * yl);
  if (!(fabsf(p) < fmaf(2.0f * rj, rl, f.hm))) return kRppiUncertain;
  // rp bin of the third side.
  int b3 = 0, bh = f.nb - 1;
  while (b3 < bh) {
    const int mid = (b3 + bh + 1) >> 1;
    if (rf >= e2lo[mid])
      b3 = mid;
    else
      bh = mid - 1;
  }
  if (!(lo > e2hi[b3] && hi < e2lo[b3 + 1])) return kRppiUncertain;
  // pi bin of the third side, needed when it is one of the two shortest.
  int p3 = 0;
  if (pos < 2) {
    const int k = static_cast<int>(floorf(sqrtf(pf)));
    const float k2 = static_cast<float>(k * k), k3 = static_cast<float>((k + 1) * (k + 1));
    const float w = f.epi + f.pmarg;
    if (!((k == 0 || pf - w > k2) && pf + w < k3)) return kRppiUncertain;
    p3 = k;
  }
  const int rs = static_cast<int>((jfirst ? mj : ml) & 0xffffu), ps = static_cast<int>((jfirst ? mj : ml) >> 16);
  const int rL = static_cast<int>((jfirst ? ml : mj) & 0xffffu), pL = static_cast<int>((jfirst ? ml : mj) >> 16);
  int r1, r2, r3, q1, q2;  // sorted ascending: rp bins and pi bins of the two shortest
  if (pos == 0) {
    r1 = b3; q1 = p3; r2 = rs; q2 = ps; r3 = rL;
  } else if (pos == 1) {
    r1 = rs; q1 = ps; r2 = b3; q2 = p3; r3 = rL;
  } else {
    r1 = rs; q1 = ps; r2 = rL; q2 = pL; r3 = b3;
  }
  const long long P = f.npi, B = f.nb;
  return q2 + q1 * P + r3 * P * P + r2 * B * P * P + static_cast<long long>(r1) * B * B * P * P;
}

}  // namespace ncorr_gb300
