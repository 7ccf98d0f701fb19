// Triangle-count kernel: the GB300 counterpart of the reference's
// countTrianglesThreeDBox / countTrianglesThreeDSurvey
// (source/device.cu:259-315, :381-431).
//
// One CTA of 256 threads owns one anchor (a point of catalogue 1) at a time;
// anchors come from a global counter, in cell order.
//  Phase A  the 27 (cell, image) slots around the anchor's home cell are
//           streamed from the cell list. A cell-local FP32 estimate of r1^2
//           drops candidates certainly out of range; for the others the
//           anchor-relative offset is formed exactly in FP64 and rounded once
//           to FP32, and r1^2 from it is classified against the bins
//           (rigorous error band; the rare undecided ones are recomputed in
//           FP64 exactly as the reference computes them). In-range neighbours
//           go to a list in shared memory (overflow: a per-CTA global slab):
//           offset d (float3), r1^2 estimate, exact bin, slot, point index,
//           weight.
//  Phase B  every neighbour pair (j, l) of the list(s) is a candidate
//           triangle. Work items are (l-tile of 128 entries, 32 j-entries);
//           warps take items from a shared counter. A warp holds its l-tile in
//           registers (4 per lane) and streams the j-entries as warp-wide
//           broadcasts. Per candidate: |d_j - d_l|^2 in FP32, its bin from a
//           shared-memory table, a Heron test proving the reference's FP32
//           triangle test, and one predicated shared atomic into the CTA's
//           (bin_j, bin_l, bin_3) histogram. Candidates whose FP32
//           classification is not certain are queued per warp and settled by
//           the exact FP64 restatement.
// Symmetry: with catalogues 2 and 3 identical (SYM), only pairs j < l are
// visited and count twice -- the reference's ordered double loop is symmetric
// in (p2, p3) because (a-b)^2 == (b-a)^2 bit for bit. With all three
// catalogues identical and the geometry checked to make every triangle's
// three vertices see each other through bit-identical images (SYM6, decided
// on the host), only neighbours after the anchor in cell order are listed and
// each counted triangle stands for all six orderings.
#pragma once
#include <type_traits>

#include "engine.cuh"

namespace ncorr_gb300 {

constexpr unsigned kCodeExact = 0xFDu;
constexpr int kSubJ = 32;                       // j-entries per work item
constexpr int kSubPerTile = kTile / kSubJ;      // work items per tile pair

// Shared-memory layout (dynamic part). The bin table sits at offset 0 and the
// CTA histogram right after it, so both are addressed with immediate offsets.
struct SmemLayout {
  int table, hist, e2, e3, m2, m3, p2, p3, w2, w3, queue, total;
};

__host__ __device__ inline int align16(int x) { return (x + 15) & ~15; }

__host__ __device__ inline SmemLayout make_layout(int nb, int ks, bool sym, bool weighted,
                                                  bool hist_global) {
  SmemLayout L;
  int o = 0;
  L.table = o;
  o += kTableSize;
  L.hist = o;
  if (!hist_global) o = align16(o + nb * nb * nb * (weighted ? 8 : 4));
  L.e2 = o;
  o += ks * 16;
  L.e3 = sym ? L.e2 : o;
  if (!sym) o += ks * 16;
  L.m2 = o;
  o += ks * 4;
  L.m3 = sym ? L.m2 : o;
  if (!sym) o += ks * 4;
  L.p2 = o;
  o += ks * 4;
  L.p3 = sym ? L.p2 : o;
  if (!sym) o += ks * 4;
  L.w2 = o;
  if (weighted) o += ks * 4;
  L.w3 = (sym || !weighted) ? L.w2 : o;
  if (weighted && !sym) o += ks * 4;
  o = align16(o);
  L.queue = o;
  o += kWarps * kQueueCap * 8;
  L.total = align16(o);
  return L;
}

struct KArgs {
  Geom g;
  Catalog c1, c2, c3;
  const unsigned char* table;
  int* work;
  int* flags;
  HistOut hist;
  // Per-CTA overflow slabs, two lists of kg entries each.
  float4* slab_e;
  unsigned* slab_m;
  int* slab_p;
  float* slab_w;
  int ks;  // shared-memory list capacity (multiple of kTile)
  int kg;  // slab capacity per list
  int sym6;
  float wscale;
  // Byte stride of one bin in the CTA histogram as encoded in the table
  // (4: u32 counts, 8: int64 sums, 1: global histogram, bins unscaled).
  int code_scale;
  unsigned long long* stats;  // exact tris, exact pairs, anchors, W, P
};

// Bin code of an FP32 r^2 estimate: table[rint(v * scale)], clamped.
__device__ __forceinline__ unsigned table_code(float v, const unsigned char* tab, float scale,
                                               int n) {
  const float y = fmaf(v, scale, 8388608.0f);
  const int idx = min(__float_as_int(y) - 0x4B000000, n - 1);
  return tab[idx];
}

// Slow FP32 classification with the explicit error band [v-E, v+E].
// Returns a plain bin index, kCodeReject or kCodeExact.
__device__ __forceinline__ unsigned careful_code(float v, const float* e2lo, const float* e2hi,
                                                 int nb, float ka, float kb) {
  const float e = fmaf(ka, v, kb);
  const float lo = v - e, hi = v + e;
  if (hi <= e2lo[0]) return kCodeReject;
  if (lo >= e2hi[nb]) return kCodeReject;
  if (!(lo > e2hi[0])) return kCodeExact;
  if (!(hi < e2lo[nb])) return kCodeExact;
  for (int b = 0; b < nb; ++b) {
    if (hi < e2lo[b + 1]) return (b == 0 || lo >= e2hi[b]) ? static_cast<unsigned>(b) : kCodeExact;
  }
  return kCodeExact;
}

struct ListView {
  float4* e;
  unsigned* m;
  int* p;
  float* w;
  float4* se;  // slab
  unsigned* sm;
  int* sp;
  float* sw;
  __device__ __forceinline__ float4 E(int i, int ks) const { return i < ks ? e[i] : se[i - ks]; }
  __device__ __forceinline__ unsigned M(int i, int ks) const { return i < ks ? m[i] : sm[i - ks]; }
  __device__ __forceinline__ int P(int i, int ks) const { return i < ks ? p[i] : sp[i - ks]; }
  __device__ __forceinline__ float W(int i, int ks) const { return i < ks ? w[i] : sw[i - ks]; }
};

// Signed 128-bit accumulate into (lo, hi) words of global memory.
__device__ __forceinline__ void add128(unsigned long long* w, long long v) {
  const unsigned long long lo = static_cast<unsigned long long>(v);
  const unsigned long long old = atomicAdd(&w[0], lo);
  const long long adj = ((old + lo) < old ? 1 : 0) - (v < 0 ? 1 : 0);
  if (adj) atomicAdd(&w[1], static_cast<unsigned long long>(adj));
}

// Shared-memory primitives on 32-bit shared-window addresses, so that base
// offsets fold into the keys and the histogram update is a predicated
// reduction rather than a branch around an atomic.
__device__ __forceinline__ unsigned lds_u8(unsigned addr) {
  unsigned v;
  asm volatile("ld.shared.u8 %0, [%1];" : "=r"(v) : "r"(addr));
  return v;
}

__device__ __forceinline__ void red_shared_u32_if(unsigned addr, bool pred) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %1, 0;\n\t@p red.shared.add.u32 [%0], 1;\n\t}"
      :
      : "r"(addr), "r"(static_cast<unsigned>(pred))
      : "memory");
}

__device__ __forceinline__ void red_shared_u64_if(unsigned addr, unsigned long long v, bool pred) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %2, 0;\n\t@p red.shared.add.u64 [%0], %1;\n\t}"
      :
      : "r"(addr), "l"(v), "r"(static_cast<unsigned>(pred))
      : "memory");
}

// Histogram update. The key is the table-scaled code: a byte offset into the
// shared histogram, or a plain bin index for the global histogram (HG).
template <bool WEIGHTED, bool HG>
__device__ __forceinline__ void hist_add(unsigned char* hist_s, const KArgs& a, unsigned key, float w) {
  if (HG) {
    if (WEIGHTED)
      add128(&a.hist.wsum[2 * key], __float2ll_rn(w));
    else
      atomicAdd(&a.hist.counts[key], 1ull);
  } else {
    if (WEIGHTED)
      atomicAdd(reinterpret_cast<unsigned long long*>(hist_s + key),
                static_cast<unsigned long long>(__float2ll_rn(w)));
    else
      atomicAdd(reinterpret_cast<unsigned*>(hist_s + key), 1u);
  }
}

template <bool SURVEY, bool SYM, bool WEIGHTED, bool HG>
__global__ void __launch_bounds__(kThreads, 2) k_triangles(KArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ double s_sqr_bins[kMaxEdges];
  __shared__ float s_e2lo[kMaxEdges], s_e2hi[kMaxEdges];
  __shared__ int s_start2[27], s_start3[27], s_pre2[28], s_pre3[28];
  __shared__ float s_do[27][3];
  __shared__ double s_shift[27][3];
  __shared__ int s_anchor, s_k2, s_k3, s_item;
  __shared__ unsigned long long s_since;

  const Geom& g = a.g;
  const int nb = g.nb;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const unsigned FULL = 0xffffffffu;
  const unsigned lt_mask = (1u << lane) - 1u;
  const SmemLayout L = make_layout(nb, a.ks, SYM, WEIGHTED, HG);
  unsigned char* tab = smem + L.table;
  unsigned char* hist_s = smem + L.hist;
  unsigned long long* queue = reinterpret_cast<unsigned long long*>(smem + L.queue) + warp * kQueueCap;
  const int nbin = nb * nb * nb;
  const int cs = a.code_scale;
  const unsigned nb_cs = static_cast<unsigned>(nb * cs);

  ListView l2, l3;
  l2.e = reinterpret_cast<float4*>(smem + L.e2);
  l2.m = reinterpret_cast<unsigned*>(smem + L.m2);
  l2.p = reinterpret_cast<int*>(smem + L.p2);
  l2.w = reinterpret_cast<float*>(smem + L.w2);
  l3.e = reinterpret_cast<float4*>(smem + L.e3);
  l3.m = reinterpret_cast<unsigned*>(smem + L.m3);
  l3.p = reinterpret_cast<int*>(smem + L.p3);
  l3.w = reinterpret_cast<float*>(smem + L.w3);
  {
    const size_t base2 = static_cast<size_t>(blockIdx.x) * 2 * static_cast<size_t>(a.kg);
    const size_t base3 = base2 + a.kg;
    l2.se = a.slab_e + base2;
    l2.sm = a.slab_m + base2;
    l2.sp = a.slab_p + base2;
    l2.sw = a.slab_w ? a.slab_w + base2 : nullptr;
    l3.se = a.slab_e + base3;
    l3.sm = a.slab_m + base3;
    l3.sp = a.slab_p + base3;
    l3.sw = a.slab_w ? a.slab_w + base3 : nullptr;
    if (SYM) l3 = l2;
  }

  for (int i = tid; i <= nb; i += kThreads) {
    s_sqr_bins[i] = g.sqr_bins[i];
    s_e2lo[i] = g.e2lo[i];
    s_e2hi[i] = g.e2hi[i];
  }
  for (int i = tid; i < g.tab_n; i += kThreads) tab[i] = a.table[i];
  if (!HG) {
    for (int i = tid; i < nbin; i += kThreads) {
      if (WEIGHTED)
        reinterpret_cast<long long*>(hist_s)[i] = 0;
      else
        reinterpret_cast<unsigned*>(hist_s)[i] = 0;
    }
  }
  if (tid == 0) s_since = 0;

  unsigned long long n_exact_tri = 0, n_exact_pair = 0, n_anchor = 0, n_pairs = 0, n_evals = 0;

  auto flush = [&]() {
    for (int i = tid; i < (HG ? 0 : nbin); i += kThreads) {
      if (WEIGHTED) {
        long long* h = reinterpret_cast<long long*>(hist_s);
        const long long v = h[i];
        if (v) {
          add128(&a.hist.wsum[2 * i], v);
          h[i] = 0;
        }
      } else {
        unsigned* h = reinterpret_cast<unsigned*>(hist_s);
        const unsigned v = h[i];
        if (v) {
          atomicAdd(&a.hist.counts[i], static_cast<unsigned long long>(v));
          h[i] = 0;
        }
      }
    }
  };

  for (;;) {
    __syncthreads();
    if (tid == 0) s_anchor = atomicAdd(a.work, 1);
    __syncthreads();
    const int ai = s_anchor;
    if (ai >= a.c1.n) break;
    ++n_anchor;
    const double4_16a pa = a.c1.pd[ai];
    const float4 qa = a.c1.pq[ai];
    const int hc = a.c1.pc[ai];
    const int hz = hc % g.nc[2];
    const int hy = (hc / g.nc[2]) % g.nc[1];
    const int hx = hc / (g.nc[2] * g.nc[1]);

    // ---- slots: 27 (cell, image) pairs, order of source/cudaNcorr.cu:37-48
    if (tid < 27) {
      const int s = tid;
      int c[3] = {hx + s / 9 - 1, hy + (s / 3) % 3 - 1, hz + s % 3 - 1};
      const int h[3] = {hx, hy, hz};
      double sh[3] = {0.0, 0.0, 0.0};
      bool ok = true;
      for (int d = 0; d < 3; ++d) {
        if (SURVEY) {
          if (c[d] == g.nc[d] || c[d] == -1) ok = false;
        } else {
          if (c[d] == g.nc[d]) {
            c[d] = 0;
            sh[d] = g.box[d];
          } else if (c[d] == -1) {
            c[d] = g.nc[d] - 1;
            sh[d] = -g.box[d];
          }
        }
      }
      const int cell = ok ? c[2] + g.nc[2] * (c[1] + g.nc[1] * c[0]) : -1;
      for (int d = 0; d < 3; ++d) {
        s_shift[s][d] = sh[d];
        if (ok) {
          const double o_n = __dmul_rn(static_cast<double>(c[d]), g.cell);
          const double o_h = __dmul_rn(static_cast<double>(h[d]), g.cell);
          s_do[s][d] = __double2float_rn(__dsub_rn(__dadd_rn(o_n, sh[d]), o_h));
        } else {
          s_do[s][d] = 0.0f;
        }
      }
      s_start2[s] = ok ? a.c2.start[cell] : 0;
      s_pre2[s + 1] = ok ? a.c2.count[cell] : 0;
      if (!SYM) {
        s_start3[s] = ok ? a.c3.start[cell] : 0;
        s_pre3[s + 1] = ok ? a.c3.count[cell] : 0;
      }
    }
    __syncthreads();
    if (tid == 0) {
      s_pre2[0] = 0;
      for (int s = 0; s < 27; ++s) s_pre2[s + 1] += s_pre2[s];
      if (!SYM) {
        s_pre3[0] = 0;
        for (int s = 0; s < 27; ++s) s_pre3[s + 1] += s_pre3[s];
      }
      s_k2 = 0;
      s_k3 = 0;
    }
    __syncthreads();

    // ---- Phase A: neighbour lists
    const bool after_only = SYM && a.sym6;
    auto build = [&](const Catalog& cat, const int* pre, const int* st, ListView& lv, int* counter) {
      const int total = pre[27];
      const int rounded = (total + 31) & ~31;
      int s = 0;
      for (int base = warp * 32; base < rounded; base += kThreads) {
        const int item = base + lane;
        bool acc = false;
        float4 ent;
        unsigned meta = 0;
        int pidx = 0;
        float w = 0.0f;
        if (item < total) {
          while (item >= pre[s + 1]) ++s;
          const int j = st[s] + (item - pre[s]);
          const float4 q = cat.pq[j];
          // Cell-local FP32 prefilter: skip candidates certainly out of range.
          const float fx = (q.x - qa.x) + s_do[s][0];
          const float fy = (q.y - qa.y) + s_do[s][1];
          const float fz = (q.z - qa.z) + s_do[s][2];
          const float vp = fmaf(fz, fz, fmaf(fy, fy, fx * fx));
          if (vp < g.pre_hi && vp > g.pre_lo && (!after_only || j > ai)) {
            // Exact anchor-relative offset of the image (FP64), rounded once.
            const double4_16a p = cat.pd[j];
            const double Dx = __dsub_rn(__dadd_rn(p.x, s_shift[s][0]), pa.x);
            const double Dy = __dsub_rn(__dadd_rn(p.y, s_shift[s][1]), pa.y);
            const double Dz = __dsub_rn(__dadd_rn(p.z, s_shift[s][2]), pa.z);
            const float dx = __double2float_rn(Dx), dy = __double2float_rn(Dy), dz = __double2float_rn(Dz);
            const float v = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
            unsigned code = table_code(v, tab, g.tab_scale, g.tab_n);
            if (code < nb_cs) {
              code /= cs;
            } else if (code == kCodeCareful) {
              code = careful_code(v, s_e2lo, s_e2hi, nb, g.ka, g.kb);
            }
            if (code == kCodeExact) {
              ++n_exact_pair;
              const double r = sqr_sep_exact(pa.x, pa.y, pa.z, __dadd_rn(p.x, s_shift[s][0]),
                                             __dadd_rn(p.y, s_shift[s][1]), __dadd_rn(p.z, s_shift[s][2]),
                                             g.fma_pattern);
              code = (r < g.sqr_rmax && r > g.sqr_rmin) ? static_cast<unsigned>(exact_bin(r, s_sqr_bins, nb))
                                                        : kCodeReject;
            }
            if (code < static_cast<unsigned>(nb)) {
              acc = true;
              ent = make_float4(dx, dy, dz, v);
              meta = code | (static_cast<unsigned>(s) << 8);
              pidx = j;
              w = q.w;
            }
          }
        }
        const unsigned bal = __ballot_sync(FULL, acc);
        if (bal) {
          int e0 = 0;
          if (lane == 0) e0 = atomicAdd(counter, __popc(bal));
          e0 = __shfl_sync(FULL, e0, 0);
          if (acc) {
            const int e = e0 + __popc(bal & lt_mask);
            if (e < a.ks) {
              lv.e[e] = ent;
              lv.m[e] = meta;
              lv.p[e] = pidx;
              if (WEIGHTED) lv.w[e] = w;
            } else if (e - a.ks < a.kg) {
              const int f = e - a.ks;
              lv.se[f] = ent;
              lv.sm[f] = meta;
              lv.sp[f] = pidx;
              if (WEIGHTED) lv.sw[f] = w;
            } else {
              atomicOr(a.flags, kFlagListOverflow);
            }
          }
        }
      }
    };
    build(a.c2, s_pre2, s_start2, l2, &s_k2);
    if (!SYM) build(a.c3, s_pre3, s_start3, l3, &s_k3);
    __syncthreads();
    const int cap = a.ks + a.kg;
    const int k2 = min(s_k2, cap);
    const int k3 = SYM ? k2 : min(s_k3, cap);
    if (tid == 0) {
      n_pairs += SYM ? static_cast<unsigned long long>(k2) * (k2 > 0 ? k2 - 1 : 0) / 2
                     : static_cast<unsigned long long>(k2) * k3;
      n_evals += static_cast<unsigned long long>(s_pre2[27]) +
                 (SYM ? 0ull : static_cast<unsigned long long>(s_pre3[27]));
    }
    const int nt2 = (k2 + kTile - 1) / kTile;
    const int nt3 = (k3 + kTile - 1) / kTile;
    const long long npairs_t = SYM ? static_cast<long long>(nt2) * (nt2 + 1) / 2
                                   : static_cast<long long>(nt2) * nt3;
    const long long nitems = npairs_t * kSubPerTile;
    // A CTA histogram bin grows by at most kSubJ*kTile per item; flush before
    // it could overflow its 32-bit counter (count mode) or 64-bit sum
    // (weighted mode, |term| <= 2^30).
    const long long kItemLimit = (1LL << 31) / (static_cast<long long>(kSubJ) * kTile);
    const float wa = static_cast<float>(pa.w);

    for (long long m0 = 0; m0 < nitems; m0 += kItemLimit) {
      const long long m1 = min(nitems, m0 + kItemLimit);
      if (!HG && s_since + static_cast<unsigned long long>(m1 - m0) > static_cast<unsigned long long>(kItemLimit)) {
        flush();
        __syncthreads();
        if (tid == 0) s_since = 0;
      }
      __syncthreads();
      if (tid == 0) {
        s_since += static_cast<unsigned long long>(m1 - m0);
        s_item = 0;
      }
      __syncthreads();

      int qn = 0;  // warp-uniform queue fill
      // Settles queued candidates, 32 per round.
      auto drain = [&]() {
        for (int q0 = 0; q0 < qn; q0 += 32) {
          const int qi = q0 + lane;
          if (qi < qn) {
            const unsigned long long pr = queue[qi];
            const int j = static_cast<int>(pr & 0xffffffffu);
            const int l = static_cast<int>(pr >> 32);
            const float4 ej = l2.E(j, a.ks);
            const unsigned mj = l2.M(j, a.ks);
            const float4 el = l3.E(l, a.ks);
            const unsigned ml = l3.M(l, a.ks);
            const float dx = ej.x - el.x, dy = ej.y - el.y, dz = ej.z - el.z;
            const float v = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
            const unsigned key_jl = ((mj & 0xffu) * nb * nb + (ml & 0xffu) * nb);
            unsigned code = careful_code(v, s_e2lo, s_e2hi, nb, g.ka, g.kb);
            if (code < static_cast<unsigned>(nb)) {
              const float s = ej.w + el.w, t = v - s;
              const float H = fmaf(-t, t, 4.0f * ej.w * el.w);
              const float S = s + v;
              if (!(H > S * fmaf(g.ha, S, g.hb))) code = kCodeExact;
            }
            if (code == kCodeExact) {
              ++n_exact_tri;
              const int pj = l2.P(j, a.ks);
              const int pl = l3.P(l, a.ks);
              const int sj = static_cast<int>(mj >> 8), sl = static_cast<int>(ml >> 8);
              const double4_16a dj = a.c2.pd[pj];
              const double4_16a dl = a.c3.pd[pl];
              const double jx = __dadd_rn(dj.x, s_shift[sj][0]), jy = __dadd_rn(dj.y, s_shift[sj][1]),
                           jz = __dadd_rn(dj.z, s_shift[sj][2]);
              const double lx = __dadd_rn(dl.x, s_shift[sl][0]), ly = __dadd_rn(dl.y, s_shift[sl][1]),
                           lz = __dadd_rn(dl.z, s_shift[sl][2]);
              const double r1 = sqr_sep_exact(pa.x, pa.y, pa.z, jx, jy, jz, g.fma_pattern);
              const double r2 = sqr_sep_exact(pa.x, pa.y, pa.z, lx, ly, lz, g.fma_pattern);
              const double r3 = sqr_sep_exact(jx, jy, jz, lx, ly, lz, g.fma_pattern);
              code = kCodeReject;
              if (r3 < g.sqr_rmax && r3 > g.sqr_rmin && exact_triangle_ok(r1, r2, r3))
                code = static_cast<unsigned>(exact_bin(r3, s_sqr_bins, nb));
            }
            if (code < static_cast<unsigned>(nb)) {
              const float wprod = WEIGHTED ? (wa * l2.W(j, a.ks)) * l3.W(l, a.ks) * a.wscale : 0.0f;
              hist_add<WEIGHTED, HG>(hist_s, a, (key_jl + code) * cs, wprod);
            }
          }
        }
        qn = 0;
        __syncwarp();
      };

      // One work item: l-tile lt (registers) against 32 j-entries of tile jt.
      auto item = [&](int jt, int lt, int sub, auto diag_tag) {
        constexpr bool DIAG = decltype(diag_tag)::value;
        float4 el[kReg];
        unsigned kl[kReg];
        float wl[kReg];
        const int lb = lt * kTile;
        const bool l_in_smem = lb < a.ks;
#pragma unroll
        for (int r = 0; r < kReg; ++r) {
          const int l = lb + r * 32 + lane;
          if (l < k3) {
            el[r] = l_in_smem ? l3.e[l] : l3.se[l - a.ks];
            const unsigned ml = l_in_smem ? l3.m[l] : l3.sm[l - a.ks];
            kl[r] = (ml & 0xffu) * nb_cs;
            wl[r] = WEIGHTED ? (l_in_smem ? l3.w[l] : l3.sw[l - a.ks]) : 0.0f;
          } else {
            el[r] = make_float4(1.0e18f, 1.0e18f, 1.0e18f, 0.0f);
            kl[r] = 0;
            wl[r] = 0.0f;
          }
        }
        const int jb = jt * kTile + sub * kSubJ;
        const int je = min(jb + kSubJ, k2);
        const bool j_in_smem = jb < a.ks;
        const float4* ej_base = j_in_smem ? l2.e + jb : l2.se + (jb - a.ks);
        const unsigned* mj_base = j_in_smem ? l2.m + jb : l2.sm + (jb - a.ks);
        const float* wj_base = WEIGHTED ? (j_in_smem ? l2.w + jb : l2.sw + (jb - a.ks)) : nullptr;
        const unsigned kj_mul = static_cast<unsigned>(nb * nb * cs);
        // Shared-window addresses: table entry = tab_adj + bits(y), clamped;
        // histogram byte address = hist_sh + kj + kl + code.
        const unsigned tab_sh = static_cast<unsigned>(__cvta_generic_to_shared(tab));
        const unsigned tab_adj = tab_sh - 0x4B000000u;
        const unsigned tab_last = tab_sh + static_cast<unsigned>(g.tab_n - 1);
        const unsigned hist_sh = static_cast<unsigned>(__cvta_generic_to_shared(hist_s));
        const float tscale = g.tab_scale, ha = g.ha, hb = g.hb;

        // One j-entry against the lane's kReg l-entries; returns true when a
        // candidate needs the careful/exact path.
        auto jrow = [&](int j) -> bool {
          const float4 ej = ej_base[j - jb];
          const unsigned kj = (mj_base[j - jb] & 0xffu) * kj_mul + (HG ? 0u : hist_sh);
          const float a4 = 4.0f * ej.w;
          const float wja = WEIGHTED ? wa * wj_base[j - jb] * a.wscale : 0.0f;
          bool q = false;
#pragma unroll
          for (int r = 0; r < kReg; ++r) {
            const float dx = ej.x - el[r].x;
            const float dy = ej.y - el[r].y;
            const float dz = ej.z - el[r].z;
            const float v = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
            const float y = fmaf(v, tscale, 8388608.0f);
            const unsigned code = lds_u8(min(__float_as_uint(y) + tab_adj, tab_last));
            const float b = el[r].w;
            const float s = ej.w + b;
            const float t = v - s;
            const float H = fmaf(-t, t, a4 * b);
            const float S = s + v;
            const bool clean = H > S * fmaf(ha, S, hb);
            bool ok = code < nb_cs;
            bool careful = code == kCodeCareful;
            if (DIAG) {
              const bool in = j < lb + r * 32 + lane;
              ok = ok && in;
              careful = careful && in;
            }
            const unsigned key = kj + kl[r] + code;
            if (HG) {
              if (ok && clean) hist_add<WEIGHTED, true>(hist_s, a, key, wja * wl[r]);
            } else if (WEIGHTED) {
              red_shared_u64_if(key, static_cast<unsigned long long>(__float2ll_rn(wja * wl[r])), ok && clean);
            } else {
              red_shared_u32_if(key, ok && clean);
            }
            q = q || careful || (ok && !clean);
          }
          return q;
        };

        // Queues the candidates of row j that need the careful/exact path.
        auto enqueue_row = [&](int j) {
          const float4 ej = ej_base[j - jb];
          const float a4 = 4.0f * ej.w;
#pragma unroll
          for (int r = 0; r < kReg; ++r) {
            const float dx = ej.x - el[r].x;
            const float dy = ej.y - el[r].y;
            const float dz = ej.z - el[r].z;
            const float v = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
            const unsigned code = table_code(v, tab, g.tab_scale, g.tab_n);
            const float b = el[r].w;
            const float s = ej.w + b;
            const float t = v - s;
            const float H = fmaf(-t, t, a4 * b);
            const float S = s + v;
            const bool clean = H > S * fmaf(g.ha, S, g.hb);
            bool want = code == kCodeCareful || (code < nb_cs && !clean);
            if (DIAG) want = want && (j < lb + r * 32 + lane);
            const unsigned bal = __ballot_sync(FULL, want);
            if (want) {
              queue[qn + __popc(bal & lt_mask)] =
                  static_cast<unsigned long long>(j) |
                  (static_cast<unsigned long long>(lb + r * 32 + lane) << 32);
            }
            qn += __popc(bal);
          }
        };

        int j = jb;
        for (; j + 1 < je; j += 2) {
          const bool q0 = jrow(j);
          const bool q1 = jrow(j + 1);
          const unsigned qm = __ballot_sync(FULL, q0) | (__ballot_sync(FULL, q1) ? 2u : 0u);
          if (qm) {
            if (qm & 1u) {
              enqueue_row(j);
              __syncwarp();
              if (qn > kQueueCap - kTile) drain();
            }
            if (qm & 2u) {
              enqueue_row(j + 1);
              __syncwarp();
              if (qn > kQueueCap - kTile) drain();
            }
          }
        }
        if (j < je) {
          if (__any_sync(FULL, jrow(j))) {
            enqueue_row(j);
            __syncwarp();
            if (qn > kQueueCap - kTile) drain();
          }
        }
      };

      for (;;) {
        int mi = 0;
        if (lane == 0) mi = atomicAdd(&s_item, 1);
        mi = __shfl_sync(FULL, mi, 0);
        const long long m = m0 + mi;
        if (m >= m1) break;
        const int sub = static_cast<int>(m % kSubPerTile);
        const long long tp = m / kSubPerTile;
        int jt, lt;
        if (SYM) {
          lt = static_cast<int>((sqrtf(8.0f * static_cast<float>(tp) + 1.0f) - 1.0f) * 0.5f);
          while (static_cast<long long>(lt) * (lt + 1) / 2 > tp) --lt;
          while (static_cast<long long>(lt + 1) * (lt + 2) / 2 <= tp) ++lt;
          jt = static_cast<int>(tp - static_cast<long long>(lt) * (lt + 1) / 2);
        } else {
          jt = static_cast<int>(tp % nt2);
          lt = static_cast<int>(tp / nt2);
        }
        if (jt * kTile + sub * kSubJ >= k2) continue;  // empty sub-range of the last tile
        if (SYM && jt == lt)
          item(jt, lt, sub, std::true_type());
        else
          item(jt, lt, sub, std::false_type());
      }
      __syncwarp();
      drain();
      __syncthreads();
    }
  }
  __syncthreads();
  flush();
  if (a.stats) {
    atomicAdd(&a.stats[0], n_exact_tri);
    atomicAdd(&a.stats[1], n_exact_pair);
    if (tid == 0) {
      atomicAdd(&a.stats[2], n_anchor);
      atomicAdd(&a.stats[3], n_pairs);
      atomicAdd(&a.stats[4], n_evals);
    }
  }
}

}  // namespace ncorr_gb300
