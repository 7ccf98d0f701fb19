// The (rp, pi) bin type on the GPU: cell lists with the rppi constructor's
// anisotropic (box) or cubic (survey) cells, and a triangle kernel that
// restates countTrianglesRppiBox / countTrianglesRppiSurvey
// (source/device.cu:317-379, :434-505 of cudaNcorr) operation for operation.
//
// One CTA of 256 threads owns one anchor at a time (taken from a global
// counter). Phase A walks the 27 (cell, image) slots of the anchor's home
// cell, flattened over the CTA's threads, and keeps the points that pass the
// reference's cut against the anchor: box pi^2 < piMax^2 and rpMin^2 < rp^2 <
// rpMax^2, survey 0 < s^2 < rpMax^2 + piMax^2. That cut is the same test for
// the kernel's p2 and p3 roles, so a list per distinct catalogue serves both.
// Phase B takes the list pairs (one row per warp, lanes over the row). An
// FP32 estimate from anchor-relative offsets drops pairs that are certainly
// cut. In a box, the FP32 classifier of rppi_fast.cuh then settles almost
// every pair with rigorous error bands; the pairs it leaves uncertain, and
// every survey pair, are evaluated in FP64 with the reference's operations
// and contractions, sorted and binned as getTriangleIndexRppi does
// (source/device.cu:203-255). Each counted triangle is added to the global
// histogram with one atomic. With p2 == p3 in a box, each unordered pair is visited once: its
// two orderings give the same index unless two sides tie in rp^2 (the
// reference's swap order then decides which pi goes with which side), and
// the tie case computes both.
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

// getTriangleIndexRppi (source/device.cu:203-255). Returns -1 when the FP32
// triangle test rejects; the index may reach nbins + nPi - 1 (pi bin nPi).
__device__ __forceinline__ long long rppi_index(double r1, double r2, double r3, double q1, double q2, double q3,
                                                const double* sb, int nb, int npi) {
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
  const float s1 = __fsqrt_rn(__double2float_rn(r1));
  const float s2 = __fsqrt_rn(__double2float_rn(r2));
  const float s3 = __fsqrt_rn(__double2float_rn(r3));
  if (__fadd_rn(s1, s2) <= s3) return -1;
  const long long i1 = exact_bin(r1, sb, nb);
  const long long i2 = exact_bin(r2, sb, nb);
  const long long i3 = exact_bin(r3, sb, nb);
  const long long p1 = static_cast<long long>(floorf(__fsqrt_rn(__double2float_rn(q1))));
  const long long p2 = static_cast<long long>(floorf(__fsqrt_rn(__double2float_rn(q2))));
  const long long P = npi, B = nb;
  return p2 + p1 * P + i3 * P * P + i2 * B * P * P + i1 * B * B * P * P;
}

template <bool WEIGHTED>
__device__ __forceinline__ void rppi_add(const RppiArgs& a, long long idx, double w, unsigned long long n) {
  if (idx < 0) return;
  if (idx > a.g.nbins) idx = a.g.nbins;  // past the reference's array: one overflow slot
  if (WEIGHTED)
    atomicAdd(&a.hist_w[idx], w);
  else
    atomicAdd(&a.hist_u[idx], n);
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

__global__ void k_rp_scatter(const double4_16a* __restrict__ in, int n, const int* __restrict__ cid,
                             int* __restrict__ cursor, double4_16a* __restrict__ pd) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int c = cid[i];
  if (c < 0) return;
  pd[atomicAdd(&cursor[c], 1)] = in[i];
}

constexpr int kRppiThreads = 256;

// Phase A for one catalogue: the 27 slots flattened over the CTA's threads.
// s_off[27] holds the slots' prefix sums, s_cell/s_sh their cell ids and
// image shifts (box).
__device__ __forceinline__ void rppi_gather(const RppiArgs& a, const double4_16a& p1, const double4_16a* pd,
                                            const int* start, const int* s_off, const int* s_cell,
                                            const double (*s_sh)[3], int total, int* s_n, double4_16a* pos,
                                            double2* ab, float4* rel, unsigned* meta, const double* sb, int cap) {
  const RppiGeom& g = a.g;
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    int s = 0;
    while (s < 26 && t >= s_off[s + 1]) ++s;
    double4_16a q = pd[start[s_cell[s]] + (t - s_off[s])];
    double x, y;
    bool keep;
    if (g.survey) {
      x = sqr_sep_exact(p1.x, p1.y, p1.z, q.x, q.y, q.z, g.fma_pattern);
      y = 0.0;
      keep = x < g.sqr_rmax && x > g.sqr_rmin;
    } else {
      // particle2.x += rShift2.x (source/device.cu:334-336)
      q.x = __dadd_rn(q.x, s_sh[s][0]);
      q.y = __dadd_rn(q.y, s_sh[s][1]);
      q.z = __dadd_rn(q.z, s_sh[s][2]);
      const double dz = __dsub_rn(p1.z, q.z);
      y = __dmul_rn(dz, dz);
      x = rp_exact(__dsub_rn(p1.x, q.x), __dsub_rn(p1.y, q.y), g.rp_pattern);
      keep = y < g.sqr_pimax && x < g.sqr_rpmax && x > g.sqr_rpmin;
    }
    if (keep) {
      const int k = atomicAdd(s_n, 1);
      if (k < cap) {
        pos[k] = q;
        ab[k] = make_double2(x, y);
        // Box: the classifier's per-side inputs, sqrt_rn(fl32(rp^2)) and the
        // exact rp and pi bins (floor(sqrtf(pi^2)) as the reference forms it).
        const float rho = g.survey ? 0.0f : __fsqrt_rn(__double2float_rn(x));
        rel[k] = make_float4(__double2float_rn(__dsub_rn(q.x, p1.x)), __double2float_rn(__dsub_rn(q.y, p1.y)),
                             __double2float_rn(__dsub_rn(q.z, p1.z)), rho);
        if (!g.survey)
          meta[k] = static_cast<unsigned>(exact_bin(x, sb, g.nb)) |
                    (static_cast<unsigned>(floorf(__fsqrt_rn(__double2float_rn(y)))) << 16);
      } else {
        atomicOr(a.flags, kFlagListOverflow);
      }
    }
  }
}

template <bool SURVEY, bool SYM, bool WEIGHTED>
__global__ void __launch_bounds__(kRppiThreads) k_rppi(const __grid_constant__ RppiArgs a) {
  const RppiGeom& g = a.g;
  __shared__ double s_sb[kMaxEdges];
  __shared__ int s_off2[28], s_off3[28], s_cell[27];
  __shared__ double s_sh[27][3];
  __shared__ float s_e2lo[kMaxEdges], s_e2hi[kMaxEdges];
  __shared__ int s_anchor, s_n2, s_n3;
  for (int i = threadIdx.x; i <= g.nb; i += blockDim.x) {
    s_sb[i] = g.sqr_bins[i];
    s_e2lo[i] = g.fe2lo[i];
    s_e2hi[i] = g.fe2hi[i];
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  double4_16a* pos2 = a.l_pos + static_cast<size_t>(blockIdx.x) * 2 * a.cap;
  double4_16a* pos3 = SYM ? pos2 : pos2 + a.cap;
  double2* ab2 = a.l_ab + static_cast<size_t>(blockIdx.x) * 2 * a.cap;
  double2* ab3 = SYM ? ab2 : ab2 + a.cap;
  float4* rel2 = a.l_rel + static_cast<size_t>(blockIdx.x) * 2 * a.cap;
  float4* rel3 = SYM ? rel2 : rel2 + a.cap;
  unsigned* meta2 = a.l_meta + static_cast<size_t>(blockIdx.x) * 2 * a.cap;
  unsigned* meta3 = SYM ? meta2 : meta2 + a.cap;
  unsigned long long n_exact = 0, n_fast = 0;
  for (;;) {
    __syncthreads();  // the previous anchor's lists are no longer read
    if (threadIdx.x == 0) {
      s_anchor = atomicAdd(a.work, 1);
      s_n2 = 0;
      s_n3 = 0;
    }
    __syncthreads();
    const int ai = s_anchor;
    if (ai >= a.n1) break;
    const double4_16a p1 = a.a_pd[ai];
    // Anchor cell (initCellIndexBox / initCellIndexSurvey, source/device.cu:75-87)
    // and its 27 slots (shiftCellIndexBox / Survey, :89-153) in the
    // reference's i, j, k order.
    if (threadIdx.x < 27) {
      const int s = threadIdx.x;
      const double c3[3] = {p1.x, p1.y, p1.z};
      const int sd[3] = {s / 9 - 1, (s / 3) % 3 - 1, s % 3 - 1};
      int c[3];
      bool ok = true;
      for (int d = 0; d < 3; ++d) {
        int h = static_cast<int>(__ddiv_rn(c3[d], g.cell[d]));
        if (!SURVEY && h == g.nc[d]) --h;
        c[d] = h + sd[d];
        s_sh[s][d] = 0.0;
        if (SURVEY) {
          if (c[d] == g.nc[d] || c[d] == -1) ok = false;
        } else if (c[d] == g.nc[d]) {
          c[d] = 0;
          s_sh[s][d] = g.box[d];
        } else if (c[d] == -1) {
          c[d] = g.nc[d] - 1;
          s_sh[s][d] = -g.box[d];
        }
      }
      const int cell = ok ? c[2] + g.nc[2] * (c[1] + g.nc[1] * c[0]) : -1;
      s_cell[s] = cell < 0 ? 0 : cell;
      s_off2[s + 1] = cell < 0 ? 0 : a.count2[cell];
      s_off3[s + 1] = cell < 0 ? 0 : a.count3[cell];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      s_off2[0] = 0;
      s_off3[0] = 0;
      for (int s = 0; s < 27; ++s) {
        s_off2[s + 1] += s_off2[s];
        s_off3[s + 1] += s_off3[s];
      }
    }
    __syncthreads();
    rppi_gather(a, p1, a.pd2, a.start2, s_off2, s_cell, s_sh, s_off2[27], &s_n2, pos2, ab2, rel2, meta2, s_sb,
                a.cap);
    if (!SYM)
      rppi_gather(a, p1, a.pd3, a.start3, s_off3, s_cell, s_sh, s_off3[27], &s_n3, pos3, ab3, rel3, meta3, s_sb,
                  a.cap);
    __syncthreads();
    const int n2 = min(s_n2, a.cap);
    const int n3 = SYM ? n2 : min(s_n3, a.cap);
    if (threadIdx.x == 0) {
      atomicAdd(&a.stats[0], 1ull);
      atomicAdd(&a.stats[1], static_cast<unsigned long long>(s_off2[27] + (SYM ? 0 : s_off3[27])));
      const unsigned long long pairs = (SYM && !SURVEY) ? static_cast<unsigned long long>(n2) * (n2 - 1) / 2
                                                        : static_cast<unsigned long long>(n2) * n3;
      atomicAdd(&a.stats[2], pairs);
    }
    // Phase B.
    double o1x = 0.0;
    if (SURVEY) o1x = __dsub_rn(p1.x, g.ori_x);  // pos1 = p1 - d_ori, d_ori = (ori.x, 0, 0)
    for (int j = warp; j < n2; j += nwarps) {
      const double4_16a pj = pos2[j];
      const double2 abj = ab2[j];
      const float4 rj = rel2[j];
      const unsigned mj = SURVEY ? 0u : meta2[j];
      const int l0 = (SYM && !SURVEY) ? j + 1 : 0;
      for (int l = l0 + lane; l < n3; l += 32) {
        if (SYM && l == j) continue;
        const float4 rl = rel3[l];
        const float dxf = rj.x - rl.x, dyf = rj.y - rl.y, dzf = rj.z - rl.z;
        long long idx = -1, idx2 = -1;
        double w = 1.0, w2 = 1.0;
        if (!SURVEY) {
          if (dzf * dzf > g.f_pi_hi) continue;
          const float rpf = fmaf(dxf, dxf, dyf * dyf);
          if (rpf > g.f_rp_hi || rpf < g.f_rp_lo) continue;
          // FP32 classification; the FP64 restatement below settles what it
          // leaves uncertain.
          const long long fi = rppi_fast_index(rj.x, rj.y, rj.z, rj.w, mj, rl.x, rl.y, rl.z, rl.w, meta3[l], g.fast,
                                               s_e2lo, s_e2hi);
          if (fi == -1) continue;
          if (fi >= 0) {
            ++n_fast;
            idx = fi;
            idx2 = fi;  // no rp^2 ties when the classifier is certain
            if (WEIGHTED) {
              const double wl = pos3[l].w;
              w = __dmul_rn(__dmul_rn(p1.w, pj.w), wl);
              w2 = __dmul_rn(__dmul_rn(p1.w, wl), pj.w);
            }
          } else {
            ++n_exact;
            const double4_16a pl = pos3[l];
            const double dz = __dsub_rn(pj.z, pl.z);
            const double pi3 = __dmul_rn(dz, dz);
            if (!(pi3 < g.sqr_pimax)) continue;
            const double rp3 = rp_exact(__dsub_rn(pj.x, pl.x), __dsub_rn(pj.y, pl.y), g.rp_pattern);
            if (!(rp3 < g.sqr_rpmax && rp3 > g.sqr_rpmin)) continue;
            const double2 abl = ab3[l];
            idx = rppi_index(abj.x, abl.x, rp3, abj.y, abl.y, pi3, s_sb, g.nb, g.npi);
            if (idx < 0) continue;
            if (WEIGHTED) w = __dmul_rn(__dmul_rn(p1.w, pj.w), pl.w);
            if (SYM) {
              // The (l, j) ordering: same sides, anchor sides swapped.
              if (abj.x == abl.x || abj.x == rp3 || abl.x == rp3)
                idx2 = rppi_index(abl.x, abj.x, rp3, abl.y, abj.y, pi3, s_sb, g.nb, g.npi);
              else
                idx2 = idx;
              if (WEIGHTED) w2 = __dmul_rn(__dmul_rn(p1.w, pl.w), pj.w);
            }
          }
        } else {
          if (fmaf(dzf, dzf, fmaf(dxf, dxf, dyf * dyf)) > g.f_s_hi) continue;
          ++n_exact;
          const double4_16a pl = pos3[l];
          const double s3 = sqr_sep_exact(pj.x, pj.y, pj.z, pl.x, pl.y, pl.z, g.fma_pattern);
          if (!(s3 < g.sqr_rmax && s3 > g.sqr_rmin)) continue;
          // getLOS (source/device.cu:45-56): positions relative to d_ori,
          // summed left to right.
          const double lx = __dadd_rn(__dadd_rn(o1x, __dsub_rn(pj.x, g.ori_x)), __dsub_rn(pl.x, g.ori_x));
          const double ly = __dadd_rn(__dadd_rn(p1.y, pj.y), pl.y);
          const double lz = __dadd_rn(__dadd_rn(p1.z, pj.z), pl.z);
          const double sqrL = dot3_exact(lx, ly, lz, lx, ly, lz, g.dot_pattern);
          const double pm = __dmul_rn(g.sqr_pimax, sqrL);
          // getSqrSdotL (source/device.cu:58-63) for (p1,p2), (p1,p3), (p2,p3).
          double t = dot3_exact(lx, ly, lz, __dsub_rn(p1.x, pj.x), __dsub_rn(p1.y, pj.y), __dsub_rn(p1.z, pj.z),
                                g.dot_pattern);
          const double q1 = __dmul_rn(t, t);
          if (pm < q1) continue;
          t = dot3_exact(lx, ly, lz, __dsub_rn(p1.x, pl.x), __dsub_rn(p1.y, pl.y), __dsub_rn(p1.z, pl.z),
                         g.dot_pattern);
          const double q2 = __dmul_rn(t, t);
          if (pm < q2) continue;
          t = dot3_exact(lx, ly, lz, __dsub_rn(pj.x, pl.x), __dsub_rn(pj.y, pl.y), __dsub_rn(pj.z, pl.z),
                         g.dot_pattern);
          const double q3 = __dmul_rn(t, t);
          if (pm < q3) continue;
          // getSqrRpSqrPi (source/device.cu:65-68).
          const double pi1 = __ddiv_rn(q1, sqrL), pi2 = __ddiv_rn(q2, sqrL), pi3 = __ddiv_rn(q3, sqrL);
          const double2 abl = ab3[l];
          const double rp1 = __dsub_rn(abj.x, pi1), rp2 = __dsub_rn(abl.x, pi2), rp3 = __dsub_rn(s3, pi3);
          if (!(rp1 < g.sqr_rpmax && rp2 < g.sqr_rpmax && rp3 < g.sqr_rpmax && rp1 > g.sqr_rpmin &&
                rp2 > g.sqr_rpmin && rp3 > g.sqr_rpmin && pi1 < g.sqr_pimax && pi2 < g.sqr_pimax))
            continue;
          idx = rppi_index(rp1, rp2, rp3, pi1, pi2, pi3, s_sb, g.nb, g.npi);
          if (WEIGHTED) w = __dmul_rn(__dmul_rn(p1.w, pj.w), pl.w);
        }
        if (SYM && !SURVEY) {
          if (idx2 == idx && !WEIGHTED) {
            rppi_add<false>(a, idx, 0.0, 2ull);
          } else {
            rppi_add<WEIGHTED>(a, idx, w, 1ull);
            rppi_add<WEIGHTED>(a, idx2, w2, 1ull);
          }
        } else {
          rppi_add<WEIGHTED>(a, idx, w, 1ull);
        }
      }
    }
  }
  if (n_exact) atomicAdd(&a.stats[3], n_exact);
  if (n_fast) atomicAdd(&a.stats[4], n_fast);
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
  for (int i = 0; i < n_edges; ++i) {
    g.fe2lo[i] = f32_down(g.sqr_bins[i]);
    g.fe2hi[i] = f32_up(g.sqr_bins[i]);
  }
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
  CU(cudaMemsetAsync(c.count.p, 0, h->ncell * sizeof(int), st));
  if (n > 0)
    k_rp_assign<<<(n + 255) / 256, 256, 0, st>>>(d_in, n, h->rg, c.cid.as<int>(), c.count.as<int>(),
                                                 h->d_flags.as<int>() + ci);
  launch_scan(c.count.as<int>(), static_cast<int>(h->ncell), c.start.as<int>(), c.cursor.as<int>(), st);
  if (n > 0)
    k_rp_scatter<<<(n + 255) / 256, 256, 0, st>>>(d_in, n, c.cid.as<int>(), c.cursor.as<int>(),
                                                  c.pd.as<double4_16a>());
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
  const int occ = rppi_occupancy(g.survey != 0, sym, weighted);
  if (occ <= 0) return fail(NCORR_ERR_CUDA, "rppi kernel does not fit on the device");
  int nsm = 0;
  CU(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, h->device));
  const int grid = std::max(1, std::min(n1, nsm * occ));
  const size_t slab_n = static_cast<size_t>(grid) * 2 * cap;
  CU(h->rp_pos.ensure(slab_n * sizeof(double4_16a)));
  CU(h->rp_ab.ensure(slab_n * sizeof(double2)));
  CU(h->rp_rel.ensure(slab_n * sizeof(float4)));
  CU(h->rp_meta.ensure(slab_n * sizeof(unsigned)));
  const size_t hist_n = static_cast<size_t>(g.nbins) + 1;
  CU(h->d_hist.ensure(hist_n * sizeof(double)));
  CU(cudaMemsetAsync(h->d_hist.p, 0, hist_n * sizeof(double), st));

  RppiArgs a;
  std::memset(&a, 0, sizeof(a));
  a.g = g;
  a.a_pd = h->cat[role[0]].pd.as<double4_16a>();
  a.n1 = n1;
  a.pd2 = h->cat[role[1]].pd.as<double4_16a>();
  a.start2 = h->cat[role[1]].start.as<int>();
  a.count2 = h->cat[role[1]].count.as<int>();
  a.pd3 = h->cat[role[2]].pd.as<double4_16a>();
  a.start3 = h->cat[role[2]].start.as<int>();
  a.count3 = h->cat[role[2]].count.as<int>();
  a.l_pos = h->rp_pos.as<double4_16a>();
  a.l_ab = h->rp_ab.as<double2>();
  a.l_rel = h->rp_rel.as<float4>();
  a.l_meta = h->rp_meta.as<unsigned>();
  a.cap = cap;
  a.hist_u = weighted ? nullptr : h->d_hist.as<unsigned long long>();
  a.hist_w = weighted ? h->d_hist.as<double>() : nullptr;
  a.work = h->d_work.as<int>();
  a.flags = h->d_flags.as<int>() + 4;
  a.stats = h->d_stats.as<unsigned long long>();
  CU(cudaEventRecord(h->ev[2], st));
  if (n1 > 0) CU(rppi_launch(a, g.survey != 0, sym, weighted, grid, st));
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
