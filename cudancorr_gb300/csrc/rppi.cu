// The (rp, pi) bin type on the GPU: cell lists with the rppi constructor's
// anisotropic (box) or cubic (survey) cells, and a triangle kernel that
// restates countTrianglesRppiBox / countTrianglesRppiSurvey
// (source/device.cu:317-379, :434-505 of cudaNcorr) operation for operation.
//
// One warp owns one anchor at a time; warps take anchors four at a time, in
// cell order, from a global counter, so consecutive anchors of a warp share
// their 27 (cell, image) slots. The GPU's FP64 pipe is a small fraction of
// its FP32 rate, so FP64 work only ever runs 32 lanes wide: FP32 estimates
// with rigorous bounds decide what they can, and what they leave waits in a
// per-warp ring in shared memory until 32 items are ready.
// Phase A walks the slots' points (FP32 copies, 32 per round); points that
// the FP32 estimate does not certainly cut are settled in FP64 against the
// reference's cut: box pi^2 < piMax^2 and rpMin^2 < rp^2 < rpMax^2, survey
// 0 < s^2 < rpMax^2 + piMax^2. That cut is the same test for the kernel's p2
// and p3 roles, so a list per distinct catalogue serves both.
// Phase B enumerates the list pairs flattened over the lanes (pairs j < l
// when p2 == p3 in a box, all ordered pairs otherwise). In a box, the FP32
// classifier of rppi_fast.cuh settles almost every pair with rigorous error
// bands; the pairs it leaves uncertain, and every survey pair that an FP32
// estimate does not certainly cut, are evaluated in FP64 with the
// reference's operations and contractions, sorted and binned as
// getTriangleIndexRppi does (source/device.cu:203-255). Each counted
// triangle is added to the global histogram with one atomic. With p2 == p3
// in a box, each unordered pair is visited once: its two orderings give the
// same index unless two sides tie in rp^2 (the reference's swap order then
// decides which pi goes with which side), and the tie case computes both.
#include "host.cuh"

namespace ncorr_gb300 {

__device__ __forceinline__ double rp_exact(double dx, double dy, int pat) {
  if (pat == 0) return __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
  if (pat == 1) return __fma_rn(dy, dy, __dmul_rn(dx, dx));
  return __fma_rn(dx, dx, __dmul_rn(dy, dy));
}

// dotProduct_d3 (source/device.cu:23-25) under a contraction pattern.
__device__ __forceinline__ double dot3_exact(double ax, double ay, double az, double bx, double by, double bz,
                                             int pat) {
  switch (pat) {
    case 0:
      return __dadd_rn(__dadd_rn(__dmul_rn(ax, bx), __dmul_rn(ay, by)), __dmul_rn(az, bz));
    case 1:
      return __fma_rn(az, bz, __fma_rn(ay, by, __dmul_rn(ax, bx)));
    case 2:
      return __fma_rn(az, bz, __fma_rn(ax, bx, __dmul_rn(ay, by)));
    case 3:
      return __fma_rn(az, bz, __dadd_rn(__dmul_rn(ax, bx), __dmul_rn(ay, by)));
    case 4:
      return __dadd_rn(__fma_rn(ay, by, __dmul_rn(ax, bx)), __dmul_rn(az, bz));
    default:
      return __dadd_rn(__fma_rn(ax, bx, __dmul_rn(ay, by)), __dmul_rn(az, bz));
  }
}

// a < b for doubles a, b >= +0: the IEEE order of non-negative values is
// the integer order of their bits. Integer compares keep the FP64 pipe,
// a small fraction of the FP32 rate on this GPU, for arithmetic.
__device__ __forceinline__ bool dlt_pos(double a, double b) {
  return __double_as_longlong(a) < __double_as_longlong(b);
}

// exact_bin for r >= +0 with integer compares (sqr_bins are >= +0).
__device__ __forceinline__ int exact_bin_pos(double r, const double* sb, int nb) {
  const long long rb = __double_as_longlong(r);
  int lo = 0, hi = nb - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (rb >= __double_as_longlong(sb[mid]))
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// The same integer compare against a limit, for any non-NaN a: a < T when
// T > +0, and a > T when T >= +0 (a negative a, or -0, has a negative
// integer image, below every non-negative one).
__device__ __forceinline__ bool dlt_lim(double a, double t) {
  return __double_as_longlong(a) < __double_as_longlong(t);
}
__device__ __forceinline__ bool dgt_lim(double a, double t) {
  return __double_as_longlong(a) > __double_as_longlong(t);
}
__device__ __forceinline__ bool deq_pos(double a, double b) {
  return __double_as_longlong(a) == __double_as_longlong(b);
}

// getTriangleIndexRppi (source/device.cu:203-255). Returns -1 when the FP32
// triangle test rejects; the index may reach nbins + nPi - 1 (pi bin nPi).
// Every caller has checked r1, r2, r3 > rpMin^2 >= 0, so the sort and the bin
// searches compare the values' bits.
__device__ __forceinline__ long long rppi_index(double r1, double r2, double r3, double q1, double q2, double q3,
                                                const double* sb, int nb, int npi) {
  double t;
  if (dlt_pos(r2, r1)) {
    t = r1; r1 = r2; r2 = t;
    t = q1; q1 = q2; q2 = t;
  }
  if (dlt_pos(r3, r1)) {
    t = r1; r1 = r3; r3 = t;
    t = q1; q1 = q3; q3 = t;
  }
  if (dlt_pos(r3, r2)) {
    t = r2; r2 = r3; r3 = t;
    t = q2; q2 = q3; q3 = t;
  }
  const float s1 = __fsqrt_rn(__double2float_rn(r1));
  const float s2 = __fsqrt_rn(__double2float_rn(r2));
  const float s3 = __fsqrt_rn(__double2float_rn(r3));
  if (__fadd_rn(s1, s2) <= s3) return -1;
  const long long i1 = exact_bin_pos(r1, sb, nb);
  const long long i2 = exact_bin_pos(r2, sb, nb);
  const long long i3 = exact_bin_pos(r3, sb, nb);
  const long long p1 = static_cast<long long>(floorf(__fsqrt_rn(__double2float_rn(q1))));
  const long long p2 = static_cast<long long>(floorf(__fsqrt_rn(__double2float_rn(q2))));
  const long long P = npi, B = nb;
  return p2 + p1 * P + i3 * P * P + i2 * B * P * P + i1 * B * B * P * P;
}

// The CTA's copy of the histogram (nbins + 1 bins; [nbins] collects indices
// past the reference's array).
struct RppiOut {
  unsigned long long* u;
  double* w;
  long long nbins;
};

template <bool WEIGHTED>
__device__ __forceinline__ void rppi_add(const RppiOut& o, long long idx, double w, unsigned long long n) {
  if (idx < 0) return;
  if (idx > o.nbins) idx = o.nbins;  // past the reference's array: one overflow slot
  if (WEIGHTED)
    atomicAdd(&o.w[idx], w);
  else
    atomicAdd(&o.u[idx], n);
}

// `*addr += v` when p, as one predicated reduction (no branch around it).
__device__ __forceinline__ void rppi_red_u64(bool p, unsigned long long* addr, unsigned long long v) {
  asm volatile(
      "{\n\t.reg .pred q;\n\tsetp.ne.u32 q, %0, 0;\n\t@q red.relaxed.gpu.global.add.u64 [%1], %2;\n\t}"
      :
      : "r"(static_cast<unsigned>(p)), "l"(addr), "l"(v)
      : "memory");
}

// Per point: the reference's host cell (clamped, source/cudaNcorr.cu:50-58),
// validation, per-cell counts. The survey anchor cell is not clamped
// (source/device.cu:84-87): a point on the upper face raises kFlagSurveyFace.
__global__ void k_rp_assign(const double4_16a* __restrict__ in, int n, RppiGeom g, int* __restrict__ cid,
                            int* __restrict__ count, int* __restrict__ flags) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  int f = 0;
  if (i < n) {
    const double4_16a p = in[i];
    const double c3[3] = {p.x, p.y, p.z};
    int ijk[3] = {0, 0, 0};
    if (!isfinite(p.x) || !isfinite(p.y) || !isfinite(p.z) || !isfinite(p.w)) f |= kFlagNonFinite;
    for (int d = 0; d < 3 && !(f & (kFlagNonFinite | kFlagOutOfGrid)); ++d) {
      const double q = __ddiv_rn(c3[d], g.cell[d]);
      if (!(q > -2.0e9 && q < 2.0e9)) {
        f |= kFlagOutOfGrid;
        break;
      }
      int c = static_cast<int>(q);
      if (g.survey && c == g.nc[d]) f |= kFlagSurveyFace;
      if (c == g.nc[d]) --c;
      if (c < 0 || c >= g.nc[d]) f |= kFlagOutOfGrid;
      ijk[d] = c;
    }
    if (p.w != 1.0) f |= kFlagWeighted;
    if (f & (kFlagNonFinite | kFlagOutOfGrid)) {
      cid[i] = -1;
    } else {
      const int c = ijk[2] + g.nc[2] * (ijk[1] + g.nc[1] * ijk[0]);
      cid[i] = c;
      atomicAdd(&count[c], 1);
    }
  }
  f = __reduce_or_sync(0xffffffffu, f);
  if ((threadIdx.x & 31) == 0 && f) atomicOr(flags, f);
}

// Cell-ordered copy of the points, and an FP32 copy (each coordinate rounded
// once) carrying the point's cell id.
__global__ void k_rp_scatter(const double4_16a* __restrict__ in, int n, const int* __restrict__ cid,
                             int* __restrict__ cursor, double4_16a* __restrict__ pd, float4* __restrict__ pq) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int c = cid[i];
  if (c < 0) return;
  const double4_16a p = in[i];
  const int k = atomicAdd(&cursor[c], 1);
  pd[k] = p;
  pq[k] = make_float4(__double2float_rn(p.x), __double2float_rn(p.y), __double2float_rn(p.z), __int_as_float(c));
}

constexpr int kRppiThreads = 256;
constexpr int kRppiWarps = kRppiThreads / 32;
constexpr int kRppiChunk = 4;  // consecutive anchors a warp takes per counter increment
constexpr int kRppiRing = 64;  // per-warp ring of points or pairs awaiting FP64
constexpr unsigned kRppiFull = 0xffffffffu;
constexpr int kRppiNoShift = 0x15;  // shift code of the unshifted image (sign + 1 = 1 on each axis)

// One catalogue's 27 (cell, image) slots around a home cell, slot s in lane
// s: the FP32 image shift (x, y, z) and, in .w (int bits), the slot's first
// point less its offset in the flattened walk; `code` the shift's signs
// (two bits per axis, sign + 1).
struct RppiSlots {
  float4 f[32];
  int code[32];
};

struct RppiWarpSm {
  RppiSlots s2, s3;
  int2 ring[kRppiRing];
};

// One per-warp list (per-catalogue neighbours of the current anchor).
struct RppiList {
  double4_16a* pos;
  double2* ab;
  float4* rel;
  unsigned* meta;
  double* pw;
};

__device__ __forceinline__ double rppi_shift(int code, int d, double box) {
  const int s = ((code >> (2 * d)) & 3) - 1;
  return s == 0 ? 0.0 : (s > 0 ? box : -box);
}

// Anchor cell (initCellIndexBox / initCellIndexSurvey, source/device.cu:75-87:
// the cell id k_rp_assign gave the anchor, which is clamped in a box and
// never on the upper face in a survey) and its 27 slots (shiftCellIndexBox /
// Survey, :89-153) in the reference's i, j, k order. Returns the slots'
// total point count; `excl` gets the lane's exclusive offset (0x7fffffff
// past slot 26, so that rppi_slot_of never picks those lanes).
template <bool SURVEY>
__device__ __forceinline__ int rppi_slots(const RppiGeom& g, int hc, const int* count, const int* start,
                                          RppiSlots& sl, int lane, int& excl) {
  const int h[3] = {hc / (g.nc[1] * g.nc[2]), (hc / g.nc[2]) % g.nc[1], hc % g.nc[2]};
  int cnt = 0, first = 0, code = 0;
  float sh[3] = {0.0f, 0.0f, 0.0f};
  if (lane < 27) {
    const int sd[3] = {lane / 9 - 1, (lane / 3) % 3 - 1, lane % 3 - 1};
    int c[3];
    bool ok = true;
    for (int d = 0; d < 3; ++d) {
      c[d] = h[d] + sd[d];
      int s = 0;
      if (SURVEY) {
        if (c[d] == g.nc[d] || c[d] == -1) ok = false;
      } else if (c[d] == g.nc[d]) {
        c[d] = 0;
        s = 1;
      } else if (c[d] == -1) {
        c[d] = g.nc[d] - 1;
        s = -1;
      }
      code |= (s + 1) << (2 * d);
      sh[d] = s == 0 ? 0.0f : (s > 0 ? g.fbox[d] : -g.fbox[d]);
    }
    if (ok) {
      const int cell = c[2] + g.nc[2] * (c[1] + g.nc[1] * c[0]);
      cnt = count[cell];
      first = start[cell];
    }
  }
  int incl = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(kRppiFull, incl, o);
    if (lane >= o) incl += v;
  }
  excl = lane < 27 ? incl - cnt : 0x7fffffff;
  __syncwarp();  // the previous table is no longer read
  sl.f[lane] = make_float4(sh[0], sh[1], sh[2], __int_as_float(first - (incl - cnt)));
  sl.code[lane] = code;
  __syncwarp();
  return __shfl_sync(kRppiFull, incl, 26);
}

// The slot of flattened position t: the largest s with excl[s] <= t.
__device__ __forceinline__ int rppi_slot_of(int excl, int t) {
  int s = 0;
#pragma unroll
  for (int step = 16; step; step >>= 1)
    if (__shfl_sync(kRppiFull, excl, s + step) <= t) s += step;
  return s;
}

// FP64 settling of up to 32 ring entries (point index, shift code), one per
// lane, against the reference's cut. Kept points are appended to the list
// from position n on; returns the new count (entries past `cap` are not
// written and raise `overflow`).
template <bool SURVEY, bool WEIGHTED>
__device__ __forceinline__ int rppi_settle(const RppiArgs& a, const double4_16a& p1, const double4_16a* pd,
                                           int2 e, bool act, const RppiList& L, int n, const double* sb, int lane,
                                           bool& overflow) {
  const RppiGeom& g = a.g;
  double4_16a q = {0.0, 0.0, 0.0, 0.0};
  double x, y = 0.0;
  if (act) q = pd[e.x];
  if (!SURVEY) {
    // particle2.x += rShift2.x (source/device.cu:334-336). Slots of interior
    // cells have no image shift, and adding +0 changes at most the sign of
    // a zero coordinate, which no later result depends on, so the adds run
    // only when a lane of the warp has a shift.
    if (__any_sync(kRppiFull, act && e.y != kRppiNoShift)) {
      q.x = __dadd_rn(q.x, rppi_shift(e.y, 0, g.box[0]));
      q.y = __dadd_rn(q.y, rppi_shift(e.y, 1, g.box[1]));
      q.z = __dadd_rn(q.z, rppi_shift(e.y, 2, g.box[2]));
    }
  }
  const double dx = __dsub_rn(p1.x, q.x), dy = __dsub_rn(p1.y, q.y), dz = __dsub_rn(p1.z, q.z);
  bool keep;
  if (SURVEY) {
    x = sqr_sum_exact(dx, dy, dz, g.fma_pattern);  // sqrSep(p1, q), >= +0
    keep = act && dlt_pos(x, g.sqr_rmax) && dlt_pos(g.sqr_rmin, x);
    // A side outside the rp and pi ranges for every partner's line of sight
    // takes part in no counted triangle: it is not kept.
    const float ax = __double2float_rn(__dsub_rn(p1.x, g.ori_x)), ay = __double2float_rn(p1.y),
                az = __double2float_rn(p1.z);
    const float4 los = make_float4(ax, ay, az, sqrtf(fmaf(az, az, fmaf(ay, ay, ax * ax))));
    keep = keep && !rppi_los_cut(__double2float_rn(dx), __double2float_rn(dy), __double2float_rn(dz),
                                 __double2float_rn(x), los, g.los_smax, g.fast.pimax2, g.fast.rpmax2_hi,
                                 g.fast.rpmin2_lo);
  } else {
    y = __dmul_rn(dz, dz);
    x = rp_exact(dx, dy, g.rp_pattern);  // >= +0
    keep = act && dlt_pos(y, g.sqr_pimax) && dlt_pos(x, g.sqr_rpmax) && dlt_pos(g.sqr_rpmin, x);
  }
  const unsigned km = __ballot_sync(kRppiFull, keep);
  if (keep) {
    const int k = n + __popc(km & ((1u << lane) - 1u));
    if (k < a.cap) {
      L.pos[k] = q;
      L.ab[k] = make_double2(x, y);
      // The anchor-relative offset fl32(q - p1) = -fl32(p1 - q) and, in a
      // box, the classifier's per-side inputs: sqrt_rn(fl32(rp^2)) and the
      // exact rp and pi bins (floor(sqrtf(pi^2)) as the reference forms it).
      // (Survey: .w holds fl32(s^2) for rppi_survey_index.)
      const float rho = SURVEY ? __double2float_rn(x) : __fsqrt_rn(__double2float_rn(x));
      L.rel[k] = make_float4(-__double2float_rn(dx), -__double2float_rn(dy), -__double2float_rn(dz), rho);
      if (!SURVEY)
        L.meta[k] = static_cast<unsigned>(exact_bin_pos(x, sb, g.nb)) |
                    (static_cast<unsigned>(floorf(__fsqrt_rn(__double2float_rn(y)))) << 16);
      if (WEIGHTED) L.pw[k] = __dmul_rn(p1.w, q.w);
    } else {
      overflow = true;
    }
  }
  return n + __popc(km);
}

// Phase A for one catalogue: the warp walks the slots' points 32 at a time.
// The FP32 estimate drops the points the reference certainly cuts (the a_*
// thresholds); the rest wait in the ring and are settled 32 at a time.
// Returns the number of points kept.
template <bool SURVEY, bool WEIGHTED>
__device__ __forceinline__ int rppi_gather(const RppiArgs& a, const double4_16a& p1, const float4& p1f,
                                           const double4_16a* pd, const float4* pq, const RppiSlots& sl, int excl,
                                           int total, int2* ring, const RppiList& L, const double* sb, int lane,
                                           bool& overflow) {
  const RppiGeom& g = a.g;
  const unsigned lt = (1u << lane) - 1u;
  int n = 0, head = 0, tail = 0;
  for (int t0 = 0; t0 < total; t0 += 32) {
    const int t = t0 + lane;
    const int s = rppi_slot_of(excl, t);
    bool cand = false;
    int idx = 0;
    if (t < total) {
      const float4 f = sl.f[s];
      idx = __float_as_int(f.w) + t;
      const float4 q = pq[idx];
      if (SURVEY) {
        const float dx = q.x - p1f.x, dy = q.y - p1f.y, dz = q.z - p1f.z;
        cand = fmaf(dz, dz, fmaf(dx, dx, dy * dy)) <= g.a_s_hi;
      } else {
        const float dx = (q.x + f.x) - p1f.x, dy = (q.y + f.y) - p1f.y, dz = (q.z + f.z) - p1f.z;
        const float rp = fmaf(dx, dx, dy * dy);
        cand = dz * dz <= g.a_pi_hi && rp <= g.a_rp_hi && rp >= g.a_rp_lo;
      }
    }
    const unsigned m = __ballot_sync(kRppiFull, cand);
    if (cand) ring[(tail + __popc(m & lt)) & (kRppiRing - 1)] = make_int2(idx, sl.code[s]);
    tail += __popc(m);
    if (tail - head >= 32) {
      __syncwarp();
      n = rppi_settle<SURVEY, WEIGHTED>(a, p1, pd, ring[(head + lane) & (kRppiRing - 1)], true, L, n, sb, lane,
                                        overflow);
      head += 32;
      __syncwarp();  // these entries may be overwritten
    }
  }
  if (tail > head) {
    __syncwarp();
    n = rppi_settle<SURVEY, WEIGHTED>(a, p1, pd, ring[(head + lane) & (kRppiRing - 1)], lane < tail - head, L, n,
                                      sb, lane, overflow);
    __syncwarp();
  }
  return n;
}

template <bool SURVEY, bool SYM, bool WEIGHTED>
__device__ __forceinline__ void rppi_count(const RppiOut& o, long long idx, long long idx2, double w, double w2) {
  if (SYM && !SURVEY) {
    if (idx2 == idx && !WEIGHTED) {
      rppi_add<false>(o, idx, 0.0, 2ull);
    } else {
      rppi_add<WEIGHTED>(o, idx, w, 1ull);
      rppi_add<WEIGHTED>(o, idx2, w2, 1ull);
    }
  } else {
    rppi_add<WEIGHTED>(o, idx, w, 1ull);
  }
}

// FP64 evaluation of one list pair (j of list 2, l of list 3) with the
// reference's operations, and its histogram update.
template <bool SURVEY, bool SYM, bool WEIGHTED>
__device__ __forceinline__ void rppi_exact_pair(const RppiArgs& a, const RppiOut& o, const double4_16a& p1, double o1x,
                                                int2 e, const RppiList& L2, const RppiList& L3, const double* sb) {
  const RppiGeom& g = a.g;
  const double4_16a pj = L2.pos[e.x], pl = L3.pos[e.y];
  const double2 abj = L2.ab[e.x], abl = L3.ab[e.y];
  long long idx = -1, idx2 = -1;
  double w = 1.0, w2 = 1.0;
  if (!SURVEY) {
    const double dz = __dsub_rn(pj.z, pl.z);
    const double pi3 = __dmul_rn(dz, dz);
    if (!dlt_pos(pi3, g.sqr_pimax)) return;
    const double rp3 = rp_exact(__dsub_rn(pj.x, pl.x), __dsub_rn(pj.y, pl.y), g.rp_pattern);
    if (!(dlt_pos(rp3, g.sqr_rpmax) && dlt_pos(g.sqr_rpmin, rp3))) return;
    idx = rppi_index(abj.x, abl.x, rp3, abj.y, abl.y, pi3, sb, g.nb, g.npi);
    if (idx < 0) return;
    if (WEIGHTED) w = __dmul_rn(__dmul_rn(p1.w, pj.w), pl.w);
    if (SYM) {
      // The (l, j) ordering: same sides, anchor sides swapped.
      if (deq_pos(abj.x, abl.x) || deq_pos(abj.x, rp3) || deq_pos(abl.x, rp3))
        idx2 = rppi_index(abl.x, abj.x, rp3, abl.y, abj.y, pi3, sb, g.nb, g.npi);
      else
        idx2 = idx;
      if (WEIGHTED) w2 = __dmul_rn(__dmul_rn(p1.w, pl.w), pj.w);
    }
  } else {
    const double s3 = sqr_sep_exact(pj.x, pj.y, pj.z, pl.x, pl.y, pl.z, g.fma_pattern);
    if (!(dlt_pos(s3, g.sqr_rmax) && dlt_pos(g.sqr_rmin, s3))) return;
    // getLOS (source/device.cu:45-56): positions relative to d_ori, summed
    // left to right.
    const double lx = __dadd_rn(__dadd_rn(o1x, __dsub_rn(pj.x, g.ori_x)), __dsub_rn(pl.x, g.ori_x));
    const double ly = __dadd_rn(__dadd_rn(p1.y, pj.y), pl.y);
    const double lz = __dadd_rn(__dadd_rn(p1.z, pj.z), pl.z);
    const double sqrL = dot3_exact(lx, ly, lz, lx, ly, lz, g.dot_pattern);
    const double pm = __dmul_rn(g.sqr_pimax, sqrL);
    // getSqrSdotL (source/device.cu:58-63) for (p1,p2), (p1,p3), (p2,p3).
    double t = dot3_exact(lx, ly, lz, __dsub_rn(p1.x, pj.x), __dsub_rn(p1.y, pj.y), __dsub_rn(p1.z, pj.z),
                          g.dot_pattern);
    const double q1 = __dmul_rn(t, t);
    if (dlt_pos(pm, q1)) return;
    t = dot3_exact(lx, ly, lz, __dsub_rn(p1.x, pl.x), __dsub_rn(p1.y, pl.y), __dsub_rn(p1.z, pl.z), g.dot_pattern);
    const double q2 = __dmul_rn(t, t);
    if (dlt_pos(pm, q2)) return;
    t = dot3_exact(lx, ly, lz, __dsub_rn(pj.x, pl.x), __dsub_rn(pj.y, pl.y), __dsub_rn(pj.z, pl.z), g.dot_pattern);
    const double q3 = __dmul_rn(t, t);
    if (dlt_pos(pm, q3)) return;
    // getSqrRpSqrPi (source/device.cu:65-68).
    const double pi1 = __ddiv_rn(q1, sqrL), pi2 = __ddiv_rn(q2, sqrL), pi3 = __ddiv_rn(q3, sqrL);
    const double rp1 = __dsub_rn(abj.x, pi1), rp2 = __dsub_rn(abl.x, pi2), rp3 = __dsub_rn(s3, pi3);
    // rp may round below zero; the limits are rpMax^2 > 0 and rpMin^2 >= 0.
    if (!(dlt_lim(rp1, g.sqr_rpmax) && dlt_lim(rp2, g.sqr_rpmax) && dlt_lim(rp3, g.sqr_rpmax) &&
          dgt_lim(rp1, g.sqr_rpmin) && dgt_lim(rp2, g.sqr_rpmin) && dgt_lim(rp3, g.sqr_rpmin) &&
          dlt_pos(pi1, g.sqr_pimax) && dlt_pos(pi2, g.sqr_pimax)))
      return;
    idx = rppi_index(rp1, rp2, rp3, pi1, pi2, pi3, sb, g.nb, g.npi);
    if (WEIGHTED) w = __dmul_rn(__dmul_rn(p1.w, pj.w), pl.w);
  }
  rppi_count<SURVEY, SYM, WEIGHTED>(o, idx, idx2, w, w2);
}

// Next pair of a lane after its flattened position moved on: rows j of the
// pairs j < l < n (TRI), or of all (j, l) in n2 x n3.
template <bool TRI>
__device__ __forceinline__ void rppi_norm(int& j, int& l, int n2, int n3) {
  if (TRI) {
    while (l >= n2 && j < n2 - 1) {
      ++j;
      l += j + 1 - n2;
    }
  } else {
    while (l >= n3 && j < n2) {
      l -= n3;
      ++j;
    }
  }
}

template <bool SURVEY, bool SYM, bool WEIGHTED>
__global__ void __launch_bounds__(kRppiThreads) k_rppi(const __grid_constant__ RppiArgs a) {
  const RppiGeom& g = a.g;
  __shared__ double s_sb[kMaxEdges];
  __shared__ __align__(16) unsigned char s_tab[kRppiTab];
  __shared__ RppiWarpSm s_w[kRppiWarps];
  for (int i = threadIdx.x; i <= g.nb; i += blockDim.x) s_sb[i] = g.sqr_bins[i];
  for (int i = threadIdx.x; i < kRppiTab / 16; i += blockDim.x)
    reinterpret_cast<uint4*>(s_tab)[i] = reinterpret_cast<const uint4*>(a.tab)[i];
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned lt = (1u << lane) - 1u;
  RppiWarpSm& ws = s_w[warp];
  // Copies of the histogram spread the adds to its most frequent bins,
  // which the SMs would otherwise serialise on in L2.
  const long long copy_off = static_cast<long long>(blockIdx.x % a.hist_copies) * (g.nbins + 1);
  const RppiOut out = {WEIGHTED ? nullptr : a.hist_u + copy_off, WEIGHTED ? a.hist_w + copy_off : nullptr, g.nbins};
  const size_t wl0 = (static_cast<size_t>(blockIdx.x) * kRppiWarps + warp) * (SYM ? 1 : 2) * a.cap;
  const size_t wl1 = SYM ? wl0 : wl0 + a.cap;
  const RppiList L2 = {a.l_pos + wl0, a.l_ab + wl0, a.l_rel + wl0, a.l_meta + wl0, WEIGHTED ? a.l_pw + wl0 : nullptr};
  const RppiList L3 = {a.l_pos + wl1, a.l_ab + wl1, a.l_rel + wl1, a.l_meta + wl1, WEIGHTED ? a.l_pw + wl1 : nullptr};
  unsigned long long n_anchor = 0, n_scan = 0, n_pairs = 0, n_exact = 0, n_fast = 0;
  bool overflow = false;
  int cell = -1, excl2 = 0x7fffffff, excl3 = 0x7fffffff, tot2 = 0, tot3 = 0;
  for (int ai = 0, last = 0;; ++ai) {
    if (ai >= last) {
      int first = 0;
      if (lane == 0) first = atomicAdd(a.work, kRppiChunk);
      first = __shfl_sync(kRppiFull, first, 0);
      if (first >= a.n1) break;
      ai = first;
      last = min(first + kRppiChunk, a.n1);
    }
    const double4_16a p1 = a.a_pd[ai];
    const float4 p1f = a.a_pq[ai];
    const int hc = __float_as_int(p1f.w);
    if (hc != cell) {
      cell = hc;
      tot2 = rppi_slots<SURVEY>(g, hc, a.count2, a.start2, ws.s2, lane, excl2);
      if (!SYM) tot3 = rppi_slots<SURVEY>(g, hc, a.count3, a.start3, ws.s3, lane, excl3);
    }
    int n2 = rppi_gather<SURVEY, WEIGHTED>(a, p1, p1f, a.pd2, a.pq2, ws.s2, excl2, tot2, ws.ring, L2, s_sb, lane,
                                           overflow);
    int n3 = n2;
    if (!SYM)
      n3 = rppi_gather<SURVEY, WEIGHTED>(a, p1, p1f, a.pd3, a.pq3, ws.s3, excl3, tot3, ws.ring, L3, s_sb, lane,
                                         overflow);
    n2 = min(n2, a.cap);
    n3 = min(n3, a.cap);
    ++n_anchor;
    n_scan += static_cast<unsigned long long>(tot2 + (SYM ? 0 : tot3));
    n_pairs += (SYM && !SURVEY) ? static_cast<unsigned long long>(n2) * (n2 - 1) / 2
                                : static_cast<unsigned long long>(n2) * n3;
    __syncwarp();  // the lists are complete
    // Phase B.
    double o1x = 0.0;
    float4 los = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (SURVEY) {
      o1x = __dsub_rn(p1.x, g.ori_x);  // pos1 = p1 - d_ori, d_ori = (ori.x, 0, 0)
      los = make_float4(__double2float_rn(o1x), __double2float_rn(p1.y), __double2float_rn(p1.z), 0.0f);
    }
    constexpr bool kTri = SYM && !SURVEY;  // pairs j < l
    int j = 0, l = kTri ? 1 + lane : lane;
    rppi_norm<kTri>(j, l, n2, n3);
    int head = 0, tail = 0;
    const int nbins32 = static_cast<int>(g.nbins);  // below 2^31
    // Lanes past the end read entry 0 (the lists are not empty while a lane
    // is valid) and discard the result.
    bool valid = kTri ? j < n2 - 1 : j < n2;
    int jj = valid ? j : 0, ll = valid ? l : 0;
    float4 rj = L2.rel[jj], rl = L3.rel[ll];
    unsigned mj = SURVEY ? 0u : L2.meta[jj], ml = SURVEY ? 0u : L3.meta[ll];
    for (;;) {
      if (!__any_sync(kRppiFull, valid)) break;
      const bool vc = (SYM && SURVEY) ? valid && j != l : valid;
      // FP32 classification (rppi_fast_index in a box, rppi_survey_index in a
      // survey after the FP32 s^2 prefilter); the FP64 restatement settles
      // what it leaves uncertain.
      bool pre = vc;
      int fi;
      if (!SURVEY) {
        fi = rppi_fast_index(rj.x, rj.y, rj.z, rj.w, mj, rl.x, rl.y, rl.z, rl.w, ml, g.fast, s_tab);
      } else {
        const float dxf = rj.x - rl.x, dyf = rj.y - rl.y, dzf = rj.z - rl.z;
        pre = pre && fmaf(dzf, dzf, fmaf(dxf, dxf, dyf * dyf)) <= g.f_s_hi;
        fi = rppi_survey_index(rj, rl, los, g.los_smax, g.fast, s_tab);
      }
      const bool hit = pre && fi >= 0;
      n_fast += hit ? 1u : 0u;
      if (WEIGHTED) {
        if (hit) {
          const double w = __dmul_rn(L2.pw[jj], L3.pos[ll].w);   // (w1 w2) w3
          const double w2 = __dmul_rn(L3.pw[ll], L2.pos[jj].w);  // (w1 w3) w2, box with p2 == p3
          rppi_count<SURVEY, SYM, WEIGHTED>(out, fi, fi, w, w2);  // no rp^2 ties when certain
        }
      } else {
        // One count per ordering (two for a box pair when p2 == p3: no rp^2
        // ties when certain); indices past the histogram go to its overflow
        // slot.
        rppi_red_u64(hit, out.u + min(max(fi, 0), nbins32), (SYM && !SURVEY) ? 2ull : 1ull);
      }
      const bool unc = pre && fi == kRppiUncertain;
      const unsigned m = __ballot_sync(kRppiFull, unc);
      if (unc) ws.ring[(tail + __popc(m & lt)) & (kRppiRing - 1)] = make_int2(j, l);
      tail += __popc(m);
      if (tail - head >= 32) {
        __syncwarp();
        rppi_exact_pair<SURVEY, SYM, WEIGHTED>(a, out, p1, o1x, ws.ring[(head + lane) & (kRppiRing - 1)], L2, L3, s_sb);
        head += 32;
        __syncwarp();
      }
      l += 32;
      rppi_norm<kTri>(j, l, n2, n3);
      valid = kTri ? j < n2 - 1 : j < n2;
      jj = valid ? j : 0;
      ll = valid ? l : 0;
      rj = L2.rel[jj];
      rl = L3.rel[ll];
      if (!SURVEY) {
        mj = L2.meta[jj];
        ml = L3.meta[ll];
      }
    }
    if (tail > head) {
      __syncwarp();
      if (lane < tail - head)
        rppi_exact_pair<SURVEY, SYM, WEIGHTED>(a, out, p1, o1x, ws.ring[(head + lane) & (kRppiRing - 1)], L2, L3, s_sb);
    }
    n_exact += static_cast<unsigned long long>(tail);
    __syncwarp();  // the ring and the lists are no longer read
  }
  if (__any_sync(kRppiFull, overflow) && lane == 0) atomicOr(a.flags, kFlagListOverflow);
  for (int o = 16; o; o >>= 1) n_fast += __shfl_xor_sync(kRppiFull, n_fast, o);
  if (lane == 0 && n_anchor) {
    atomicAdd(&a.stats[0], n_anchor);
    atomicAdd(&a.stats[1], n_scan);
    atomicAdd(&a.stats[2], n_pairs);
    atomicAdd(&a.stats[3], n_exact);
    atomicAdd(&a.stats[4], n_fast);
  }
}

// Sums the histogram copies (n bins each) into copy 0.
template <bool WEIGHTED>
__global__ void k_rp_fold(unsigned long long* __restrict__ hu, double* __restrict__ hw, long long n, int copies) {
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    if (WEIGHTED) {
      double s = hw[i];
      for (int c = 1; c < copies; ++c) s += hw[c * n + i];
      hw[i] = s;
    } else {
      unsigned long long s = hu[i];
      for (int c = 1; c < copies; ++c) s += hu[c * n + i];
      hu[i] = s;
    }
  }
}

// Histogram copies for a histogram of `bytes`: as many as fit a 64 MiB
// budget, at most 4 (on the 2M-point clustered box, 12.4 MB of bins: 26.9 ms
// with one copy, 20.6 with two, 20.0 with four, no gain beyond).
constexpr long kRppiHistBudget = 64L << 20;
constexpr int kRppiHistCopiesMax = 4;
// Device memory for the per-warp neighbour lists; dense catalogues (long
// lists) get fewer CTAs rather than a failed allocation.
constexpr size_t kRppiSlabBudget = size_t{16} << 30;
static int rppi_hist_copies(size_t bytes) {
  return static_cast<int>(std::max<long>(1, std::min<long>(kRppiHistCopiesMax, kRppiHistBudget / static_cast<long>(bytes))));
}

template <bool SURVEY, bool SYM, bool WEIGHTED>
static cudaError_t rppi_launch_one(const RppiArgs& a, int grid, cudaStream_t st) {
  k_rppi<SURVEY, SYM, WEIGHTED><<<grid, kRppiThreads, 0, st>>>(a);
  return cudaGetLastError();
}

template <bool SURVEY, bool SYM, bool WEIGHTED>
static int rppi_occupancy_one() {
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_rppi<SURVEY, SYM, WEIGHTED>, kRppiThreads, 0) !=
      cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

static cudaError_t rppi_launch(const RppiArgs& a, bool survey, bool sym, bool weighted, int grid, cudaStream_t st) {
  if (survey) {
    if (sym) return weighted ? rppi_launch_one<true, true, true>(a, grid, st)
                             : rppi_launch_one<true, true, false>(a, grid, st);
    return weighted ? rppi_launch_one<true, false, true>(a, grid, st) : rppi_launch_one<true, false, false>(a, grid, st);
  }
  if (sym) return weighted ? rppi_launch_one<false, true, true>(a, grid, st)
                           : rppi_launch_one<false, true, false>(a, grid, st);
  return weighted ? rppi_launch_one<false, false, true>(a, grid, st) : rppi_launch_one<false, false, false>(a, grid, st);
}

static int rppi_occupancy(bool survey, bool sym, bool weighted) {
  if (survey) {
    if (sym) return weighted ? rppi_occupancy_one<true, true, true>() : rppi_occupancy_one<true, true, false>();
    return weighted ? rppi_occupancy_one<true, false, true>() : rppi_occupancy_one<true, false, false>();
  }
  if (sym) return weighted ? rppi_occupancy_one<false, true, true>() : rppi_occupancy_one<false, true, false>();
  return weighted ? rppi_occupancy_one<false, false, true>() : rppi_occupancy_one<false, false, false>();
}

}  // namespace ncorr_gb300

namespace ncorr_host {

// Largest float <= x and smallest float >= x are in host.cuh (f32_down/up).

int rppi_init(ncorr_handle* h, const double box[3], const double* edges, int n_edges, int num_minor_bins,
              int is_survey, const double ori[3]) {
  RppiGeom& g = h->rg;
  std::memset(&g, 0, sizeof(g));
  const int nb = n_edges - 1;
  g.nb = nb;
  g.npi = num_minor_bins;
  g.survey = is_survey ? 1 : 0;
  g.fma_pattern = kDefaultFmaPattern;
  g.rp_pattern = kDefaultRpPattern;
  g.dot_pattern = kDefaultDotPattern;
  const double rpmax = edges[n_edges - 1], rpmin = edges[0];
  const double pimax = static_cast<double>(num_minor_bins);  // piBins_.back() (source/cudaNcorr.cu:174-180)
  g.sqr_rpmax = rpmax * rpmax;
  g.sqr_rpmin = rpmin * rpmin;
  g.sqr_pimax = pimax * pimax;
  g.sqr_rmax = rpmax * rpmax + pimax * pimax;
  // sqrRMin_ is never set by the rppi constructor; every value in
  // [0, rpMin^2] gives the same counts (a side that counts has
  // s^2 >= rp^2 > rpMin^2), so 0 stands for it.
  g.sqr_rmin = 0.0;
  const double rmax = static_cast<double>(sqrtf(static_cast<float>(g.sqr_rmax)));
  for (int d = 0; d < 3; ++d) {
    g.box[d] = box[d];
    g.cell[d] = is_survey ? rmax : (d < 2 ? rpmax : pimax);
    const double n = std::ceil(box[d] / g.cell[d]);
    if (n > 4096.0) return fail(NCORR_ERR_INVALID_ARGUMENT, "cell grid too large (more than 4096 cells per axis)");
    g.nc[d] = static_cast<int>(n);
  }
  const long ncell = static_cast<long>(g.nc[0]) * g.nc[1] * g.nc[2];
  if (ncell > (1L << 26)) return fail(NCORR_ERR_INVALID_ARGUMENT, "cell grid too large (more than 2^26 cells)");
  h->ncell = ncell;
  g.ori_x = (is_survey && ori) ? ori[0] : 0.0;  // only d_ori.x is uploaded (source/cudaNcorr.cu:253-255)
  for (int i = 0; i < n_edges; ++i) g.sqr_bins[i] = edges[i] * edges[i];
  const double nbins = std::pow(static_cast<double>(nb), 3) * num_minor_bins * num_minor_bins;
  if (nbins + num_minor_bins >= 2147483647.0)
    return fail(NCORR_ERR_INVALID_ARGUMENT, "nb^3 * numMinorBins^2 exceeds the reference's int index range");
  g.nbins = static_cast<long long>(nbins);
  // FP32 prefilter. Every list offset is the exact FP64 offset rounded once
  // to FP32, and every neighbour lies within two cells of the anchor, so each
  // estimated component errs by at most 2^-24 * 4 * cell; with the FP32
  // difference and squares, far less than the slack of 2^-14 * 4 * cell used
  // here, so a candidate past a threshold is certainly cut.
  const double cmax = std::max(g.cell[0], std::max(g.cell[1], g.cell[2]));
  const double slack = std::ldexp(4.0 * cmax, -14);
  g.f_pi_hi = f32_up((pimax + slack) * (pimax + slack));
  g.f_rp_hi = f32_up((rpmax + 2.0 * slack) * (rpmax + 2.0 * slack));
  g.f_rp_lo = rpmin > 2.0 * slack ? f32_down((rpmin - 2.0 * slack) * (rpmin - 2.0 * slack)) : 0.0f;
  const double smax = std::sqrt(g.sqr_rmax);
  g.f_s_hi = f32_up((smax + 2.0 * slack) * (smax + 2.0 * slack));
  // Gather prefilter (thresholds derived at rppi_gather_cut).
  {
    const RppiGatherCut gc = rppi_gather_cut(g.nc, g.cell, is_survey != 0, rpmin, rpmax, pimax);
    g.a_rp_hi = gc.rp_hi;
    g.a_rp_lo = gc.rp_lo;
    g.a_pi_hi = gc.pi_hi;
    g.a_s_hi = gc.s_hi;
    for (int d = 0; d < 3; ++d) g.fbox[d] = static_cast<float>(box[d]);
    g.los_smax = f32_up(std::sqrt(g.sqr_rmax));
  }
  // The box-mode FP32 classifier: its bands and margins, derived in
  // rppi_fast.cuh (u = 2^-24).
  const double u = std::ldexp(1.0, -24);
  RppiFast& f = g.fast;
  f.epi = f32_up(64.0 * u * g.sqr_pimax);
  f.erp = f32_up(128.0 * u * g.sqr_rpmax);
  f.pimax2 = static_cast<float>(g.sqr_pimax);  // nPi^2 <= 2^24: exact
  f.rpmax2_lo = f32_down(g.sqr_rpmax);
  f.rpmax2_hi = f32_up(g.sqr_rpmax);
  f.rpmin2_lo = f32_down(g.sqr_rpmin);
  f.rpmin2_hi = f32_up(g.sqr_rpmin);
  f.hm = -f32_up(128.0 * u * g.sqr_rpmax);
  f.pmarg = f32_up(16.0 * u * g.sqr_pimax);
  f.nb = nb;
  f.npi = num_minor_bins;
  f.tab_band = is_survey ? 4.0f * f.erp : f.erp;  // survey pairs carry wider bands than a box's third side
  f.tab_scale = rppi_tab_scale(f.rpmax2_hi, f.tab_band);
  for (int i = 0; i < n_edges; ++i) {
    g.fe2lo[i] = f32_down(g.sqr_bins[i]);
    g.fe2hi[i] = f32_up(g.sqr_bins[i]);
  }
  h->rp_tab_host.resize(kRppiTab);
  rppi_build_table(f, g.fe2lo, g.fe2hi, h->rp_tab_host.data());
  // Output tables (source/cudaNcorr.cu:195-213).
  for (int i = 0; i < nb; ++i)
    for (int j = i; j < nb; ++j)
      for (int k = j; k < nb; ++k)
        if (h->mids[k] <= h->mids[i] + h->mids[j])
          for (int l = 0; l < num_minor_bins; ++l)
            for (int m = 0; m < num_minor_bins; ++m) {
              h->tri_bins_out.push_back(h->mids[i]);
              h->tri_bins_out.push_back(h->mids[j]);
              h->tri_bins_out.push_back(h->mids[k]);
              h->pi_bins_out.push_back(static_cast<double>(l));
              h->pi_bins_out.push_back(static_cast<double>(m));
              h->counts_out.push_back(0.0);
            }
  h->counts_all.assign(static_cast<size_t>(g.nbins), 0.0);
  return NCORR_OK;
}

// prepTriCountsOutRppi (source/cudaNcorr.cu:88-105).
static void rppi_compact(ncorr_handle* h) {
  const long nb = h->nb, P = h->rg.npi;
  h->counts_out.clear();
  for (long i = 0; i < nb; ++i)
    for (long j = i; j < nb; ++j)
      for (long k = j; k < nb; ++k)
        if (h->mids[k] <= h->mids[i] + h->mids[j])
          for (long l = 0; l < P; ++l)
            for (long m = 0; m < P; ++m)
              h->counts_out.push_back(h->counts_all[m + l * P + k * P * P + j * P * P * nb + i * P * P * nb * nb]);
}

static int rppi_grid_catalog(ncorr_handle* h, int ci, const double4_16a* d_in, int n, cudaStream_t st) {
  CatDev& c = h->cat[ci];
  c.n = n;
  const size_t nn = static_cast<size_t>(std::max(n, 1));
  CU(c.cid.ensure(nn * sizeof(int)));
  CU(c.count.ensure(h->ncell * sizeof(int)));
  CU(c.start.ensure((h->ncell + 1) * sizeof(int)));
  CU(c.cursor.ensure(h->ncell * sizeof(int)));
  CU(c.pd.ensure(nn * sizeof(double4_16a)));
  CU(c.pq.ensure(nn * sizeof(float4)));
  CU(cudaMemsetAsync(c.count.p, 0, h->ncell * sizeof(int), st));
  if (n > 0)
    k_rp_assign<<<(n + 255) / 256, 256, 0, st>>>(d_in, n, h->rg, c.cid.as<int>(), c.count.as<int>(),
                                                 h->d_flags.as<int>() + ci);
  launch_scan(c.count.as<int>(), static_cast<int>(h->ncell), c.start.as<int>(), c.cursor.as<int>(), st);
  if (n > 0)
    k_rp_scatter<<<(n + 255) / 256, 256, 0, st>>>(d_in, n, c.cid.as<int>(), c.cursor.as<int>(),
                                                  c.pd.as<double4_16a>(), c.pq.as<float4>());
  CU(cudaGetLastError());
  return NCORR_OK;
}

int rppi_run(ncorr_handle* h, const double4_16a* d1, int n1, const double4_16a* d2, int n2, const double4_16a* d3,
             int n3, cudaStream_t st, const void* key1, const void* key2, const void* key3) {
  auto t0 = std::chrono::steady_clock::now();
  cudaGetLastError();
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
  const RppiGeom& g = h->rg;

  CU(h->d_flags.ensure(8 * sizeof(int)));
  CU(h->d_work.ensure(sizeof(int)));
  CU(h->d_bound.ensure(2 * sizeof(int)));
  CU(h->d_stats.ensure(8 * sizeof(unsigned long long)));
  CU(cudaMemsetAsync(h->d_flags.p, 0, 8 * sizeof(int), st));
  CU(cudaMemsetAsync(h->d_bound.p, 0, 2 * sizeof(int), st));
  CU(cudaMemsetAsync(h->d_stats.p, 0, 8 * sizeof(unsigned long long), st));
  CU(cudaMemsetAsync(h->d_work.p, 0, sizeof(int), st));
  CU(cudaEventRecord(h->ev[0], st));
  bool done[3] = {false, false, false};
  for (int r = 0; r < 3; ++r) {
    const int ci = role[r];
    if (done[ci]) continue;
    done[ci] = true;
    const int rc = rppi_grid_catalog(h, ci, src[r], ns[r], st);
    if (rc) return rc;
  }
  // Longest possible list: the largest 27-slot occupancy.
  Geom gb;
  std::memset(&gb, 0, sizeof(gb));
  for (int d = 0; d < 3; ++d) gb.nc[d] = g.nc[d];
  gb.survey = g.survey;
  launch_nbr_bound(h->cat[role[1]].count.as<int>(), gb, h->d_bound.as<int>(), st);
  if (!sym) launch_nbr_bound(h->cat[role[2]].count.as<int>(), gb, h->d_bound.as<int>() + 1, st);
  CU(cudaGetLastError());
  CU(cudaEventRecord(h->ev[1], st));
  int flags[8];
  int bound[2] = {0, 0};
  CU(cudaMemcpyAsync(flags, h->d_flags.p, sizeof(flags), cudaMemcpyDeviceToHost, st));
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
  if (g.survey && (flags[role[0]] & kFlagSurveyFace))
    return fail(NCORR_ERR_OUT_OF_GRID,
                "survey anchor on the upper face of the cell grid (unclamped cell index == nc)");

  const int cap = std::max(1, std::max(bound[0], bound[1]));
  if (cap > kListMax)
    return fail(NCORR_ERR_CAPACITY, "rppi: a 27-cell neighbourhood holds more than 2^24 points");
  const int occ = rppi_occupancy(g.survey != 0, sym, weighted);
  if (occ <= 0) return fail(NCORR_ERR_CUDA, "rppi kernel does not fit on the device");
  int nsm = 0;
  CU(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, h->device));
  // Warps take kRppiChunk anchors at a time: no more CTAs than that needs,
  // and no more than keep the per-warp lists within kRppiSlabBudget.
  const long per_cta = static_cast<long>(kRppiWarps) * kRppiChunk;
  const size_t entry_bytes =
      sizeof(double4_16a) + sizeof(double2) + sizeof(float4) + sizeof(unsigned) + (weighted ? sizeof(double) : 0);
  const size_t cta_bytes = static_cast<size_t>(kRppiWarps) * (sym ? 1 : 2) * cap * entry_bytes;
  const long fit = std::max<long>(1, static_cast<long>(kRppiSlabBudget / cta_bytes));
  const int grid = static_cast<int>(
      std::max(1L, std::min({(n1 + per_cta - 1) / per_cta, static_cast<long>(nsm) * occ, fit})));
  const size_t slab_n = static_cast<size_t>(grid) * kRppiWarps * (sym ? 1 : 2) * cap;
  CU(h->rp_pos.ensure(slab_n * sizeof(double4_16a)));
  CU(h->rp_ab.ensure(slab_n * sizeof(double2)));
  CU(h->rp_rel.ensure(slab_n * sizeof(float4)));
  CU(h->rp_meta.ensure(slab_n * sizeof(unsigned)));
  if (weighted) CU(h->rp_pw.ensure(slab_n * sizeof(double)));
  CU(h->rp_tab.ensure(kRppiTab));
  CU(cudaMemcpyAsync(h->rp_tab.p, h->rp_tab_host.data(), kRppiTab, cudaMemcpyHostToDevice, st));
  const size_t hist_n = static_cast<size_t>(g.nbins) + 1;
  const int copies = rppi_hist_copies(hist_n * sizeof(double));
  CU(h->d_hist.ensure(hist_n * copies * sizeof(double)));
  CU(cudaMemsetAsync(h->d_hist.p, 0, hist_n * copies * sizeof(double), st));

  RppiArgs a;
  std::memset(&a, 0, sizeof(a));
  a.g = g;
  a.a_pd = h->cat[role[0]].pd.as<double4_16a>();
  a.a_pq = h->cat[role[0]].pq.as<float4>();
  a.n1 = n1;
  a.pd2 = h->cat[role[1]].pd.as<double4_16a>();
  a.pq2 = h->cat[role[1]].pq.as<float4>();
  a.start2 = h->cat[role[1]].start.as<int>();
  a.count2 = h->cat[role[1]].count.as<int>();
  a.pd3 = h->cat[role[2]].pd.as<double4_16a>();
  a.pq3 = h->cat[role[2]].pq.as<float4>();
  a.start3 = h->cat[role[2]].start.as<int>();
  a.count3 = h->cat[role[2]].count.as<int>();
  a.l_pos = h->rp_pos.as<double4_16a>();
  a.l_ab = h->rp_ab.as<double2>();
  a.l_rel = h->rp_rel.as<float4>();
  a.l_meta = h->rp_meta.as<unsigned>();
  a.l_pw = weighted ? h->rp_pw.as<double>() : nullptr;
  a.tab = h->rp_tab.as<unsigned char>();
  a.cap = cap;
  a.hist_u = weighted ? nullptr : h->d_hist.as<unsigned long long>();
  a.hist_w = weighted ? h->d_hist.as<double>() : nullptr;
  a.hist_copies = copies;
  a.work = h->d_work.as<int>();
  a.flags = h->d_flags.as<int>() + 4;
  a.stats = h->d_stats.as<unsigned long long>();
  CU(cudaEventRecord(h->ev[2], st));
  if (n1 > 0) CU(rppi_launch(a, g.survey != 0, sym, weighted, grid, st));
  if (n1 > 0 && copies > 1) {
    const int fb = static_cast<int>(std::min<size_t>((hist_n + 255) / 256, static_cast<size_t>(nsm) * 8));
    if (weighted)
      k_rp_fold<true><<<fb, 256, 0, st>>>(nullptr, a.hist_w, static_cast<long long>(hist_n), copies);
    else
      k_rp_fold<false><<<fb, 256, 0, st>>>(a.hist_u, nullptr, static_cast<long long>(hist_n), copies);
    CU(cudaGetLastError());
  }
  CU(cudaEventRecord(h->ev[3], st));

  std::vector<unsigned long long> raw(hist_n);
  unsigned long long st_host[8];
  int kflags = 0;
  CU(cudaMemcpyAsync(raw.data(), h->d_hist.p, hist_n * sizeof(double), cudaMemcpyDeviceToHost, st));
  CU(cudaMemcpyAsync(st_host, h->d_stats.p, sizeof(st_host), cudaMemcpyDeviceToHost, st));
  CU(cudaMemcpyAsync(&kflags, h->d_flags.as<int>() + 4, sizeof(int), cudaMemcpyDeviceToHost, st));
  CU(cudaStreamSynchronize(st));
  if (kflags & kFlagListOverflow) return fail(NCORR_ERR_CAPACITY, "neighbour list overflow");
  h->counts_all.resize(static_cast<size_t>(g.nbins));
  unsigned long long total = 0;
  for (size_t i = 0; i < static_cast<size_t>(g.nbins); ++i) {
    if (weighted) {
      double v;
      std::memcpy(&v, &raw[i], sizeof(double));
      h->counts_all[i] = v;
    } else {
      h->counts_all[i] = static_cast<double>(raw[i]);
      total += raw[i];
    }
  }
  if (weighted)
    std::memcpy(&h->rppi_overflow, &raw[g.nbins], sizeof(double));
  else
    h->rppi_overflow = static_cast<double>(raw[g.nbins]);
  rppi_compact(h);
  float ms0 = 0, ms1 = 0;
  cudaEventElapsedTime(&ms0, h->ev[0], h->ev[1]);
  cudaEventElapsedTime(&ms1, h->ev[2], h->ev[3]);
  auto t1 = std::chrono::steady_clock::now();
  ncorr_stats& s = h->stats;
  std::memset(&s, 0, sizeof(s));
  s.ms_grid = ms0;
  s.ms_count = ms1;
  s.ms_total = std::chrono::duration<double, std::milli>(t1 - t0).count();
  s.n_anchors = st_host[0];
  s.n_pair_evals = st_host[1];
  s.n_pairs = st_host[2];
  s.n_exact_tris = st_host[3];
  s.n_queued = st_host[4];
  s.triangles = weighted ? 0 : total;
  s.weighted = weighted ? 1 : 0;
  s.symmetric = (sym && !g.survey) ? 2 : 1;
  s.grid_ctas = grid;
  s.list_capacity = cap;
  s.overflow = h->rppi_overflow;
  return NCORR_OK;
}

}  // namespace ncorr_host
