// Triangle-count kernel: the GB300 counterpart of the reference's
// countTrianglesThreeDBox / countTrianglesThreeDSurvey
// (source/device.cu:259-315, :381-431).
//
// One CTA of 256 threads owns one anchor (a point of catalogue 1) at a time.
// Anchors come from a work queue whose positions name (batch item, anchor):
// in cell order or in a learned order, taken from a shared counter (dynamic)
// or as one contiguous range per CTA (static). A CTA keeps one histogram for
// the item of its current anchor and adds it to that item's global histogram
// when the item changes.
//  Phase A  the 27 (cell, image) slots around the anchor's home cell are
//           streamed from the cell list. A cell-local FP32 estimate of r1^2
//           drops candidates certainly out of range; for the others the
//           anchor-relative offset is formed exactly in FP64 and rounded once
//           to FP32, and r1^2 from it is classified against the bins
//           (rigorous error band; the rare undecided ones are recomputed in
//           FP64 exactly as the reference computes them). In-range neighbours
//           go to a list in shared memory (overflow: a per-CTA global slab):
//           offset d (float3), the square root of the r1^2 estimate, exact
//           bin, slot, point index, weight.
//  Phase B  every neighbour pair (j, l) of the list(s) is a candidate
//           triangle. Work items are (l-tile of 128 entries, 32 j-entries);
//           warps take items from a shared counter. A warp holds its l-tile in
//           registers (4 per lane) and streams the j-entries as warp-wide
//           broadcasts. Per candidate: r3^2 in FP32 as
//           rho_j^2 + rho_l^2 - 2 d_j.d_l, its bin from a shared-memory
//           table, a margin test on d_j.d_l proving the reference's FP32
//           triangle test, and one shared atomic into the CTA's
//           (bin_j, bin_l, bin_3) histogram. Candidates whose FP32
//           classification is not certain are queued per warp and settled by
//           the exact FP64 restatement.
// Symmetry: with catalogues 2 and 3 identical (SYM), only pairs l < j are
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

// j-rows evaluated per iteration of the unweighted pair loop (1 or 2).
#ifndef NCORR_ROW_UNROLL
#define NCORR_ROW_UNROLL 2
#endif
// j-entries per work item: 8, 16 or 32 (a run-time choice, KArgs::sub_j).
constexpr int kSubJDefault = 32;

// Shared-memory layout (dynamic part). The bin table sits at offset 0 and the
// CTA histogram right after it, so both are addressed with immediate offsets.
struct SmemLayout {
  int table, hist, e2, e3, m2, m3, p2, p3, w2, w3, queue, xbuf, scratch, total;
};

__host__ __device__ inline int align16(int x) { return (x + 15) & ~15; }

__host__ __device__ inline SmemLayout make_layout(int nb, int ks, bool sym, bool weighted,
                                                  bool hist_global, int hist_copies = 1) {
  SmemLayout L;
  int o = 0;
  L.table = o;
  o += kTableSize;
  L.hist = o;
  if (!hist_global) o = align16(o + hist_copies * nb * nb * nb * (weighted ? 8 : 4));
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
  L.xbuf = o;  // per warp: 32 uncertain candidates awaiting the exact kernel
  o += kWarps * 32 * 16;
  L.scratch = o;  // 8 bytes per lane: sink of non-counting reductions
  o += 32 * 8;
  L.total = align16(o);
  return L;
}

struct KArgs {
  Geom g;
  const BatchItem* items;  // device array of n_items
  int n_items;
  // Work queue: position w stands for anchor q_anchor[w] (sorted index in
  // catalogue 1) of item q_item[w]; null arrays mean item 0 and anchor w.
  const int* q_item;
  const int* q_anchor;
  int n_work;
  // 1: CTA b takes positions [b*n/G, (b+1)*n/G) in order (static schedule);
  // 0: CTAs take positions from the shared counter `work`.
  int sched_static;
  int sub_j;        // j-entries per work item (8, 16 or 32)
  int hist_copies;  // copies of the CTA histogram, lane & (copies-1) picks one
  // Optional: candidate pairs of each anchor added to its home cell
  // (cell_base of the item + cell), the work the scheduler learns.
  unsigned long long* cell_work;
  const unsigned char* table;
  int* work;
  int* flags;
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
  unsigned long long* stats;  // exact tris, exact pairs, anchors, W, P, flagged rows, queued
  // Deferred exact candidates (null: settle them in place).
  ExactEntry* xq;
  unsigned* xq_count;
  unsigned xq_cap;
  // A copy of these arguments in global memory, used by the out-of-line
  // paths (taking the address of the kernel parameter would copy it to local
  // memory in every thread).
  const KArgs* self;
};

// Bin code of an FP32 r^2 estimate: table[rint(v * scale)], clamped.
__device__ __forceinline__ unsigned table_code(float v, const unsigned char* tab, float scale,
                                               int n) {
  const float y = fmaf(v, scale, 8388608.0f);
  // Unsigned, as in the PTX body: a slightly negative v (the estimate of a
  // side near zero) rounds to index 0; anything below that or beyond the
  // table wraps or clamps to the last entry.
  const unsigned idx = min(static_cast<unsigned>(__float_as_int(y) - 0x4B000000), static_cast<unsigned>(n - 1));
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

// The margin form of the triangle test. List entries keep rho = sqrt_rn of
// their r^2 estimate in .w; with a = rho_j^2 and b = rho_l^2 (the products
// formed inside the FMAs) a candidate of third side v is certainly kept by
// the reference's FP32 sqrtf test when |v - (a + b)| < 2 rho_j rho_l - M
// (hm = -M; the PTX body evaluates the same operations).
__device__ __forceinline__ bool heron_clean(float v, float aj, float a2r, float rl, float hm) {
  const float s = fmaf(rl, rl, aj);
  const float t = __fsub_rn(v, s);
  const float w = fmaf(a2r, rl, hm);
  return fabsf(t) < w;
}

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

// Classification of one candidate (j, l) in hand-written PTX, shared verbatim
// by the counting bodies and the flag-only body so that all take
// bit-identical decisions. Operands: %1-%3 the row's offset d_j, %4 rho_j^2,
// %5 2 rho_j, %6-%8 the column's offset scaled by -2, %9 rho_l, %12 `in`
// (diagonal tiles: l < j), %13 table scale, %14/%15 table address bias and
// last entry, %16 nb * code scale, %17 -M. With p = -2 d_j.d_l the third
// side is v = p + (rho_l^2 + rho_j^2): three products and two adds instead of
// three differences and three squares, and p itself is the quantity of the
// margin test, |p| < 2 rho_j rho_l - M (|C - A - B| = |2 D_j.D_l| for the
// exact sides). Every rounding is explicit (.rn), matching the error model.
// Results: `upd` (the candidate counts in bin `code`) and, OR-ed into %0,
// "needs the careful/exact path".
#define NCORR_CAND_CLASSIFY                    \
  "mul.rn.f32 pp, %1, %6;\n\t"                 \
  "fma.rn.f32 pp, %2, %7, pp;\n\t"             \
  "fma.rn.f32 pp, %3, %8, pp;\n\t"             \
  "fma.rn.f32 s, %9, %9, %4;\n\t"              \
  "add.rn.f32 v, pp, s;\n\t"                   \
  "fma.rn.f32 y, v, %13, 0f4B000000;\n\t"      \
  "mov.b32 ia, y;\n\t"                         \
  "add.u32 ia, ia, %14;\n\t"                   \
  "min.u32 ia, ia, %15;\n\t"                   \
  "ld.shared.u8 code, [ia];\n\t"               \
  "abs.f32 t, pp;\n\t"                         \
  "fma.rn.f32 H, %5, %9, %17;\n\t"             \
  "setp.lt.u32 ok, code, %16;\n\t"             \
  NCORR_CAND_MASK                              \
  "setp.lt.and.f32 upd, t, H, ok;\n\t"         \
  "setp.ge.and.f32 nco, t, H, ok;\n\t"         \
  NCORR_CAND_WQ                                \
  "@wq or.b32 %0, %0, 1;\n\t"

// Diagonal tiles mask the candidate with `in` (operand 12).
#define NCORR_CAND_MASK_ON           \
  "setp.ne.u32 inp, %12, 0;\n\t"     \
  "and.pred ok, ok, inp;\n\t"
#define NCORR_CAND_WQ_ON                      \
  "setp.eq.and.u32 car, code, 255, inp;\n\t"  \
  "or.pred wq, car, nco;\n\t"
#define NCORR_CAND_WQ_OFF "setp.eq.or.u32 wq, code, 255, nco;\n\t"

#define NCORR_CAND_DECLS                             \
  ".reg .f32 pp, s, v, y, t, H;\n\t"                 \
  ".reg .b32 ia, code, key, adr;\n\t"                \
  ".reg .pred ok, upd, nco, car, wq, inp;\n\t"

// One unweighted candidate: the classification, then the shared-memory
// histogram reduction at byte offset kj + kl + code (kj includes the
// histogram's base address). The reduction is unconditional: a candidate
// that does not count adds to the lane's own scratch word `dummy` instead,
// which keeps the loop free of the branch a predicated atomic compiles to.
template <bool DIAG>
__device__ __forceinline__ void cand_count(float ex, float ey, float ez, float a, float a2r, float lx, float ly,
                                           float lz, float b, unsigned kj, unsigned kl, unsigned in, float tscale,
                                           unsigned tab_adj, unsigned tab_last, unsigned nb_cs, float hm,
                                           unsigned dummy, unsigned& q) {
#define NCORR_CAND_COUNT_ASM                                                                          \
  asm volatile(                                                                                      \
      "{\n\t" NCORR_CAND_DECLS NCORR_CAND_CLASSIFY                                                     \
      "add.u32 key, %10, %11;\n\t"                                                                   \
      "add.u32 key, key, code;\n\t"                                                                  \
      "selp.b32 adr, key, %18, upd;\n\t"                                                             \
      "red.shared.add.u32 [adr], 1;\n\t"                                                             \
      "}"                                                                                            \
      : "+r"(q)                                                                                      \
      : "f"(ex), "f"(ey), "f"(ez), "f"(a), "f"(a2r), "f"(lx), "f"(ly), "f"(lz), "f"(b), "r"(kj), "r"(kl), \
        "r"(in), "f"(tscale), "r"(tab_adj), "r"(tab_last), "r"(nb_cs), "f"(hm), "r"(dummy)               \
      : "memory")
  if (DIAG) {
#define NCORR_CAND_MASK NCORR_CAND_MASK_ON
#define NCORR_CAND_WQ NCORR_CAND_WQ_ON
    NCORR_CAND_COUNT_ASM;
#undef NCORR_CAND_WQ
#undef NCORR_CAND_MASK
  } else {
#define NCORR_CAND_MASK ""
#define NCORR_CAND_WQ NCORR_CAND_WQ_OFF
    NCORR_CAND_COUNT_ASM;
#undef NCORR_CAND_WQ
#undef NCORR_CAND_MASK
  }
#undef NCORR_CAND_COUNT_ASM
}

// The weighted twin of cand_count: the same classification, then the
// fixed-point weight w_row * w_l (|value| <= 2^30 by the choice of the scale,
// so the 32-bit conversion is exact and equals the 64-bit one) added into the
// int64 bin, or into the lane's 8-byte scratch word when it does not count.
// A 64-bit shared-memory add is not a native atomic (it compiles to a
// compare-and-swap loop), so the add is split over the bin's two 32-bit
// words with native atomics: the low word by atom.add, whose old value gives
// the carry, then the high word by the sign extension plus that carry. Every
// thread's carry comes from its own atomic on the low word, so the 64-bit
// total is exact however the adds interleave.
template <bool DIAG>
__device__ __forceinline__ void cand_wsum(float ex, float ey, float ez, float a, float a2r, float lx, float ly,
                                          float lz, float b, unsigned kj, unsigned kl, unsigned in, float tscale,
                                          unsigned tab_adj, unsigned tab_last, unsigned nb_cs, float hm,
                                          unsigned dummy, float wrow, float wl, unsigned& q) {
#define NCORR_CAND_WSUM_ASM                                                                           \
  asm volatile(                                                                                      \
      "{\n\t" NCORR_CAND_DECLS                                                                        \
      ".reg .f32 wp;\n\t.reg .b32 wi, whi, wold, wnew, wcy, adrh;\n\t" NCORR_CAND_CLASSIFY              \
      "add.u32 key, %10, %11;\n\t"                                                                   \
      "add.u32 key, key, code;\n\t"                                                                  \
      "selp.b32 adr, key, %18, upd;\n\t"                                                             \
      "mul.rn.f32 wp, %19, %20;\n\t"                                                                 \
      "cvt.rni.s32.f32 wi, wp;\n\t"                                                                  \
      "shr.s32 whi, wi, 31;\n\t"                                                                     \
      "atom.shared.add.u32 wold, [adr], wi;\n\t"                                                     \
      "add.u32 wnew, wold, wi;\n\t"                                                                  \
      "set.lt.u32.u32 wcy, wnew, wold;\n\t"                                                          \
      "sub.u32 whi, whi, wcy;\n\t"                                                                   \
      "add.u32 adrh, adr, 4;\n\t"                                                                    \
      "red.shared.add.u32 [adrh], whi;\n\t"                                                          \
      "}"                                                                                            \
      : "+r"(q)                                                                                      \
      : "f"(ex), "f"(ey), "f"(ez), "f"(a), "f"(a2r), "f"(lx), "f"(ly), "f"(lz), "f"(b), "r"(kj), "r"(kl), \
        "r"(in), "f"(tscale), "r"(tab_adj), "r"(tab_last), "r"(nb_cs), "f"(hm), "r"(dummy), "f"(wrow),  \
        "f"(wl)                                                                                      \
      : "memory")
  if (DIAG) {
#define NCORR_CAND_MASK NCORR_CAND_MASK_ON
#define NCORR_CAND_WQ NCORR_CAND_WQ_ON
    NCORR_CAND_WSUM_ASM;
#undef NCORR_CAND_WQ
#undef NCORR_CAND_MASK
  } else {
#define NCORR_CAND_MASK ""
#define NCORR_CAND_WQ NCORR_CAND_WQ_OFF
    NCORR_CAND_WSUM_ASM;
#undef NCORR_CAND_WQ
#undef NCORR_CAND_MASK
  }
#undef NCORR_CAND_WSUM_ASM
}

// Counting body of the shared-histogram path: count or weighted sum.
template <bool WEIGHTED, bool DIAG>
__device__ __forceinline__ void cand_body(float ex, float ey, float ez, float a, float a2r, float lx, float ly,
                                          float lz, float b, unsigned kj, unsigned kl, unsigned in, float tscale,
                                          unsigned tab_adj, unsigned tab_last, unsigned nb_cs, float hm,
                                          unsigned dummy, float wrow, float wl, unsigned& q) {
  if (WEIGHTED)
    cand_wsum<DIAG>(ex, ey, ez, a, a2r, lx, ly, lz, b, kj, kl, in, tscale, tab_adj, tab_last, nb_cs, hm, dummy, wrow,
                    wl, q);
  else
    cand_count<DIAG>(ex, ey, ez, a, a2r, lx, ly, lz, b, kj, kl, in, tscale, tab_adj, tab_last, nb_cs, hm, dummy, q);
}

// The same classification without the histogram update: 1 when the
// candidate needs the careful/exact path.
__device__ __forceinline__ unsigned cand_flag(float ex, float ey, float ez, float a, float a2r, float lx,
                                              float ly, float lz, float b, unsigned in, float tscale,
                                              unsigned tab_adj, unsigned tab_last, unsigned nb_cs, float hm) {
  unsigned q = 0;
#define NCORR_CAND_MASK NCORR_CAND_MASK_ON
#define NCORR_CAND_WQ NCORR_CAND_WQ_ON
  asm volatile(
      "{\n\t" NCORR_CAND_DECLS NCORR_CAND_CLASSIFY "}"
      : "+r"(q)
      : "f"(ex), "f"(ey), "f"(ez), "f"(a), "f"(a2r), "f"(lx), "f"(ly), "f"(lz), "f"(b), "r"(0u), "r"(0u),
        "r"(in), "f"(tscale), "r"(tab_adj), "r"(tab_last), "r"(nb_cs), "f"(hm));
#undef NCORR_CAND_WQ
#undef NCORR_CAND_MASK
  return q;
}

// Four candidates of one row against one lane's four columns, unweighted and
// off the diagonal (full l-tiles, most of the work): the classification of
// NCORR_CAND_CLASSIFY operation for operation for each, then the four
// histogram reductions. A candidate that needs the careful/exact path ORs
// `rbit` (the row's bit in the work item) into q. One asm statement lets the four table loads issue
// before the first reduction; as four statements, each table load would wait
// behind the previous candidate's reduction, which may touch the same
// shared-memory word as far as the compiler can tell.
#define NCORR_ROW_CLS(C, LX, LY, LZ, B)                  \
  "mul.rn.f32 pp" #C ", %1, " LX ";\n\t"                 \
  "fma.rn.f32 pp" #C ", %2, " LY ", pp" #C ";\n\t"       \
  "fma.rn.f32 pp" #C ", %3, " LZ ", pp" #C ";\n\t"       \
  "fma.rn.f32 s" #C ", " B ", " B ", %4;\n\t"            \
  "add.rn.f32 v" #C ", pp" #C ", s" #C ";\n\t"           \
  "fma.rn.f32 y" #C ", v" #C ", %7, 0f4B000000;\n\t"     \
  "mov.b32 ia" #C ", y" #C ";\n\t"                       \
  "add.u32 ia" #C ", ia" #C ", %8;\n\t"                  \
  "min.u32 ia" #C ", ia" #C ", %9;\n\t"                  \
  "ld.shared.u8 code" #C ", [ia" #C "];\n\t"
#define NCORR_ROW_UPD(C, B, KL)                                      \
  "abs.f32 t" #C ", pp" #C ";\n\t"                                   \
  "fma.rn.f32 H" #C ", %5, " B ", %11;\n\t"                          \
  "setp.lt.u32 ok" #C ", code" #C ", %10;\n\t"                       \
  "setp.lt.and.f32 upd" #C ", t" #C ", H" #C ", ok" #C ";\n\t"       \
  "setp.ge.and.f32 nco" #C ", t" #C ", H" #C ", ok" #C ";\n\t"       \
  "setp.eq.or.u32 wq" #C ", code" #C ", 255, nco" #C ";\n\t"         \
  "@wq" #C " or.b32 %0, %0, %33;\n\t"                                \
  "add.u32 key" #C ", %6, " KL ";\n\t"                               \
  "add.u32 key" #C ", key" #C ", code" #C ";\n\t"                    \
  "selp.b32 adr" #C ", key" #C ", %12, upd" #C ";\n\t"
#define NCORR_ROW_DECL(C)                                                     \
  ".reg .f32 pp" #C ", s" #C ", v" #C ", y" #C ", t" #C ", H" #C ";\n\t"      \
  ".reg .b32 ia" #C ", code" #C ", key" #C ", adr" #C ";\n\t"                 \
  ".reg .pred ok" #C ", upd" #C ", nco" #C ", wq" #C ";\n\t"

__device__ __forceinline__ void row4_count(float ex, float ey, float ez, float a, float a2r, unsigned kj,
                                           float tscale, unsigned tab_adj, unsigned tab_last, unsigned nb_cs,
                                           float hm, unsigned dummy, const float4& l0, unsigned k0, const float4& l1,
                                           unsigned k1, const float4& l2, unsigned k2, const float4& l3, unsigned k3,
                                           unsigned rbit, unsigned& q) {
  asm volatile(
      "{\n\t" NCORR_ROW_DECL(0) NCORR_ROW_DECL(1) NCORR_ROW_DECL(2) NCORR_ROW_DECL(3)
      NCORR_ROW_CLS(0, "%13", "%14", "%15", "%16") NCORR_ROW_CLS(1, "%18", "%19", "%20", "%21")
      NCORR_ROW_CLS(2, "%23", "%24", "%25", "%26") NCORR_ROW_CLS(3, "%28", "%29", "%30", "%31")
      NCORR_ROW_UPD(0, "%16", "%17") NCORR_ROW_UPD(1, "%21", "%22") NCORR_ROW_UPD(2, "%26", "%27")
      NCORR_ROW_UPD(3, "%31", "%32")
      "red.shared.add.u32 [adr0], 1;\n\t"
      "red.shared.add.u32 [adr1], 1;\n\t"
      "red.shared.add.u32 [adr2], 1;\n\t"
      "red.shared.add.u32 [adr3], 1;\n\t"
      "}"
      : "+r"(q)
      : "f"(ex), "f"(ey), "f"(ez), "f"(a), "f"(a2r), "r"(kj), "f"(tscale), "r"(tab_adj), "r"(tab_last), "r"(nb_cs),
        "f"(hm), "r"(dummy), "f"(l0.x), "f"(l0.y), "f"(l0.z), "f"(l0.w), "r"(k0), "f"(l1.x), "f"(l1.y), "f"(l1.z),
        "f"(l1.w), "r"(k1), "f"(l2.x), "f"(l2.y), "f"(l2.z), "f"(l2.w), "r"(k2), "f"(l3.x), "f"(l3.y), "f"(l3.z),
        "f"(l3.w), "r"(k3), "r"(rbit)
      : "memory");
}
#undef NCORR_ROW_CLS
#undef NCORR_ROW_UPD
#undef NCORR_ROW_DECL

// The classification in C++ with the same operations, for the paths that do
// not run the PTX bodies (global histogram, weighted row re-examination).
// `l` is the column entry as the pair loop holds it: (-2 d_l, rho_l).
__device__ __forceinline__ void cand_classify(float ex, float ey, float ez, float a, float a2r, float4 l,
                                              const unsigned char* tab, float scale, int n, float hm,
                                              unsigned* code, bool* clean) {
  float pp = __fmul_rn(ex, l.x);
  pp = __fmaf_rn(ey, l.y, pp);
  pp = __fmaf_rn(ez, l.z, pp);
  const float s = __fmaf_rn(l.w, l.w, a);
  const float v = __fadd_rn(pp, s);
  *code = table_code(v, tab, scale, n);
  *clean = fabsf(pp) < __fmaf_rn(a2r, l.w, hm);
}

__device__ __forceinline__ float lds_f32(unsigned addr) {
  float v;
  asm volatile("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"(addr));
  return v;
}

__device__ __forceinline__ float4 lds_f4(unsigned addr) {
  float4 v;
  asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "r"(addr));
  return v;
}

__device__ __forceinline__ unsigned lds_u32(unsigned addr) {
  unsigned v;
  asm volatile("ld.shared.u32 %0, [%1];" : "=r"(v) : "r"(addr));
  return v;
}

// Histogram update. The key is the table-scaled code: a byte offset into the
// shared histogram, or a plain bin index for the global histogram (HG).
template <bool WEIGHTED, bool HG>
__device__ __forceinline__ void hist_add(unsigned char* hist_s, const HistOut& hist, unsigned key, float w) {
  if (HG) {
    if (WEIGHTED)
      add128(&hist.wsum[2 * key], __float2ll_rn(w));
    else
      atomicAdd(&hist.counts[key], 1ull);
  } else {
    if (WEIGHTED)
      atomicAdd(reinterpret_cast<unsigned long long*>(hist_s + key),
                static_cast<unsigned long long>(__float2ll_rn(w)));
    else
      atomicAdd(reinterpret_cast<unsigned*>(hist_s + key), 1u);
  }
}

// Settles one uncertain candidate exactly as the reference computes it
// (source/device.cu:154-201, :259-315 / :381-431): FP64 images and sides
// with the pinned sqrSep contraction, FP32 sqrtf triangle test, bin search;
// adds into the global unsorted histogram. Uses global data only.
template <bool SURVEY, bool WEIGHTED>
__device__ __forceinline__ void settle_exact(const KArgs& a, const ExactEntry& e) {
  const Geom& g = a.g;
  const int nb = g.nb;
  const int sj = static_cast<int>(e.meta & 31u), sl = static_cast<int>((e.meta >> 5) & 31u);
  const unsigned bj = (e.meta >> 10) & 0xffu, bl = (e.meta >> 18) & 0xffu;
  const BatchItem& it = a.items[a.q_item ? a.q_item[e.ai] : 0];
  const int ai = a.q_anchor ? a.q_anchor[e.ai] : e.ai;
  const double4_16a pa = it.c1.pd[ai];
  const int hc = it.c1.pc[ai];
  const int h[3] = {hc / (g.nc[2] * g.nc[1]), (hc / g.nc[2]) % g.nc[1], hc % g.nc[2]};
  double shj[3], shl[3];
  // Image shift of a slot (source/device.cu:89-122); zero in survey mode.
  const int dj3[3] = {sj / 9 - 1, (sj / 3) % 3 - 1, sj % 3 - 1};
  const int dl3[3] = {sl / 9 - 1, (sl / 3) % 3 - 1, sl % 3 - 1};
  for (int d = 0; d < 3; ++d) {
    shj[d] = 0.0;
    shl[d] = 0.0;
    if (!SURVEY) {
      const int cj = h[d] + dj3[d], cl = h[d] + dl3[d];
      if (cj == g.nc[d]) shj[d] = g.box[d]; else if (cj == -1) shj[d] = -g.box[d];
      if (cl == g.nc[d]) shl[d] = g.box[d]; else if (cl == -1) shl[d] = -g.box[d];
    }
  }
  const double4_16a dj = it.c2.pd[e.pj];
  const double4_16a dl = it.c3.pd[e.pl];
  const double jx = __dadd_rn(dj.x, shj[0]), jy = __dadd_rn(dj.y, shj[1]), jz = __dadd_rn(dj.z, shj[2]);
  const double lx = __dadd_rn(dl.x, shl[0]), ly = __dadd_rn(dl.y, shl[1]), lz = __dadd_rn(dl.z, shl[2]);
  const double r1 = sqr_sep_exact(pa.x, pa.y, pa.z, jx, jy, jz, g.fma_pattern);
  const double r2 = sqr_sep_exact(pa.x, pa.y, pa.z, lx, ly, lz, g.fma_pattern);
  const double r3 = sqr_sep_exact(jx, jy, jz, lx, ly, lz, g.fma_pattern);
  if (!(r3 < g.sqr_rmax && r3 > g.sqr_rmin) || !exact_triangle_ok(r1, r2, r3)) return;
  int lo = 0, hi = nb - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (r3 >= g.sqr_bins[mid]) lo = mid; else hi = mid - 1;
  }
  const unsigned key = (bj * nb + bl) * nb + static_cast<unsigned>(lo);
  if (WEIGHTED) {
    const float w = (static_cast<float>(pa.w) * static_cast<float>(dj.w)) * static_cast<float>(dl.w) * a.wscale;
    add128(&it.hist.wsum[2 * key], __float2ll_rn(w));
  } else {
    atomicAdd(&it.hist.counts[key], 1ull);
  }
}

// ---------------------------------------------------------------------------
// Rarely taken paths, kept out of line so that the hot pair loop stays small
// in the instruction cache. Cold holds one warp's state for them.
struct Cold {
  const KArgs* a;
  ListView l2, l3;
  unsigned long long* queue;  // this warp's (j, l) queue
  ExactEntry* xbuf;           // this warp's buffer of uncertain candidates
  const float* e2lo;
  const float* e2hi;
  const double* sqr_bins;
  unsigned char* tab;
  unsigned char* hist_s;  // this lane's copy of the CTA histogram
  HistOut hist;           // the current item's global histogram
  int qn, xn;
  int nb, cs, ai;  // ai: the anchor's position in the work queue
  float wa;
  unsigned lane, lt_mask;
  unsigned long long n_exact_tri, n_queued, n_flag_rows;
};

// Moves the warp's buffered uncertain candidates to the global queue (one
// atomic per 32), or settles them here when the queue is full.
template <bool SURVEY, bool WEIGHTED>
__device__ __noinline__ void cold_flush_exact(Cold& c) {
  const KArgs& a = *c.a;
  if (c.xn == 0) return;
  unsigned base = 0;
  if (c.lane == 0 && a.xq) base = atomicAdd(a.xq_count, static_cast<unsigned>(c.xn));
  base = __shfl_sync(0xffffffffu, base, 0);
  if (static_cast<int>(c.lane) < c.xn) {
    const ExactEntry e = c.xbuf[c.lane];
    if (a.xq && base + c.lane < a.xq_cap)
      a.xq[base + c.lane] = e;
    else
      settle_exact<SURVEY, WEIGHTED>(a, e);
  }
  c.xn = 0;
  __syncwarp();
}

// Settles the queued candidates, 32 per round: the explicit FP32 band and the
// margin test of the triangle decide most; the rest go to the exact buffer.
template <bool SURVEY, bool WEIGHTED, bool HG>
__device__ __noinline__ void cold_drain(Cold& c) {
  const KArgs& a = *c.a;
  const Geom& g = a.g;
  const int nb = c.nb;
  for (int q0 = 0; q0 < c.qn; q0 += 32) {
    const int qi = q0 + static_cast<int>(c.lane);
    bool exact = false;
    ExactEntry xe;
    if (qi < c.qn) {
      const unsigned long long pr = c.queue[qi];
      const int j = static_cast<int>(pr & 0xffffffffu);
      const int l = static_cast<int>(pr >> 32);
      const float4 ej = c.l2.E(j, a.ks);
      const unsigned mj = c.l2.M(j, a.ks);
      const float4 el = c.l3.E(l, a.ks);
      const unsigned ml = c.l3.M(l, a.ks);
      const float dx = ej.x - el.x, dy = ej.y - el.y, dz = ej.z - el.z;
      const float v = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
      const unsigned key_jl = ((mj & 0xffu) * nb * nb + (ml & 0xffu) * nb);
      unsigned code = careful_code(v, c.e2lo, c.e2hi, nb, g.ka, g.kb);
      if (code < static_cast<unsigned>(nb)) {
        if (!heron_clean(v, __fmul_rn(ej.w, ej.w), 2.0f * ej.w, el.w, g.hm)) code = kCodeExact;
      }
      if (code == kCodeExact) {
        ++c.n_exact_tri;
        exact = true;
        xe.ai = c.ai;
        xe.pj = c.l2.P(j, a.ks);
        xe.pl = c.l3.P(l, a.ks);
        xe.meta = (mj >> 8) | ((ml >> 8) << 5) | ((mj & 0xffu) << 10) | ((ml & 0xffu) << 18);
      } else if (code < static_cast<unsigned>(nb)) {
        const float wprod = WEIGHTED ? (c.wa * c.l2.W(j, a.ks)) * c.l3.W(l, a.ks) * a.wscale : 0.0f;
        hist_add<WEIGHTED, HG>(c.hist_s, c.hist, (key_jl + code) * c.cs, wprod);
      }
    }
    const unsigned xbal = __ballot_sync(0xffffffffu, exact);
    if (c.xn + __popc(xbal) > 32) cold_flush_exact<SURVEY, WEIGHTED>(c);
    if (exact) c.xbuf[c.xn + __popc(xbal & c.lt_mask)] = xe;
    c.xn += __popc(xbal);
    __syncwarp();
  }
  c.qn = 0;
  __syncwarp();
}

// Re-examines row j of a work item (lane's l-entries el[r] at lb + 32r + lane)
// and queues the candidates that need the careful/exact path, with the same
// decisions the counting body took. Inline: it only recomputes flags.
template <bool WEIGHTED, bool HG, int MODE>
__device__ __forceinline__ void enqueue_row(Cold& c, const Geom& g, int j, float4 ej, const float4 (&el)[kReg],
                                            int lb, int rhi, unsigned tab_adj, unsigned tab_last,
                                            unsigned nb_cs) {
  constexpr bool DIAG = MODE == 2;
  const float aj = __fmul_rn(ej.w, ej.w), a2r = 2.0f * ej.w;
  ++c.n_flag_rows;
#pragma unroll
  for (int r = 0; r < kReg; ++r) {
    const int lr = lb + r * 32 + static_cast<int>(c.lane);
    bool want = false;
    if (MODE == 0 || r < rhi) {
      if (!WEIGHTED && !HG) {
        want = cand_flag(ej.x, ej.y, ej.z, aj, a2r, el[r].x, el[r].y, el[r].z, el[r].w,
                         DIAG ? static_cast<unsigned>(j > lr) : 1u, g.tab_scale, tab_adj, tab_last, nb_cs,
                         g.hm) != 0;
      } else {
        unsigned code;
        bool clean;
        cand_classify(ej.x, ej.y, ej.z, aj, a2r, el[r], c.tab, g.tab_scale, g.tab_n, g.hm, &code, &clean);
        want = code == kCodeCareful || (code < nb_cs && !clean);
        if (DIAG) want = want && (j > lr);
      }
    }
    const unsigned bal = __ballot_sync(0xffffffffu, want);
    if (want)
      c.queue[c.qn + __popc(bal & c.lt_mask)] =
          static_cast<unsigned long long>(j) | (static_cast<unsigned long long>(lr) << 32);
    c.qn += __popc(bal);
    if (c.lane == 0) c.n_queued += __popc(bal);
  }
  __syncwarp();
}

// Exact r1^2 of a pair-stage candidate and its bin (or kCodeReject).
static __device__ __noinline__ unsigned cold_pair_exact(const Geom* g, const double* sqr_bins, double4_16a pa,
                                                        double px, double py, double pz) {
  const double r = sqr_sep_exact(pa.x, pa.y, pa.z, px, py, pz, g->fma_pattern);
  return (r < g->sqr_rmax && r > g->sqr_rmin) ? static_cast<unsigned>(exact_bin(r, sqr_bins, g->nb)) : kCodeReject;
}

template <bool SURVEY, bool SYM, bool WEIGHTED, bool HG>
__global__ void __launch_bounds__(kThreads, 2) k_triangles(KArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ double s_sqr_bins[kMaxEdges];
  __shared__ float s_e2lo[kMaxEdges], s_e2hi[kMaxEdges];
  __shared__ int s_start2[27], s_start3[27], s_pre2[28], s_pre3[28];
  __shared__ float s_do[27][3];
  __shared__ double s_shift[27][3];
  __shared__ int s_w, s_k2, s_k3, s_item, s_cur, s_sym6;
  __shared__ long long s_next, s_end;
  __shared__ unsigned long long s_since;
  __shared__ BatchItem s_it;  // the item of the current anchor

  const Geom& g = a.g;
  const int nb = g.nb;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const unsigned FULL = 0xffffffffu;
  const unsigned lt_mask = (1u << lane) - 1u;
  const SmemLayout L = make_layout(nb, a.ks, SYM, WEIGHTED, HG, a.hist_copies);
  unsigned char* tab = smem + L.table;
  unsigned char* hist_s = smem + L.hist;
  const int nbin = nb * nb * nb;
  const int copies = HG ? 1 : a.hist_copies;
  // This lane's copy of the CTA histogram: lanes that hit one bin in the same
  // instruction spread over the copies.
  const unsigned copy_off = static_cast<unsigned>((lane & (copies - 1)) * nbin * (WEIGHTED ? 8 : 4));
  const int sub_j = a.sub_j;
  const int spt = kTile / sub_j;  // work items per tile pair
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
    for (int i = tid; i < nbin * copies; i += kThreads) {
      if (WEIGHTED)
        reinterpret_cast<long long*>(hist_s)[i] = 0;
      else
        reinterpret_cast<unsigned*>(hist_s)[i] = 0;
    }
  }
  if (tid == 0) {
    s_since = 0;
    s_cur = -1;
    const long long n = a.n_work, G = gridDim.x, b = blockIdx.x;
    s_next = b * n / G;
    s_end = (b + 1) * n / G;
  }

  Cold c;
  c.a = a.self;
  c.l2 = l2;
  c.l3 = l3;
  c.queue = reinterpret_cast<unsigned long long*>(smem + L.queue) + warp * kQueueCap;
  c.xbuf = reinterpret_cast<ExactEntry*>(smem + L.xbuf) + warp * 32;
  c.e2lo = s_e2lo;
  c.e2hi = s_e2hi;
  c.sqr_bins = s_sqr_bins;
  c.tab = tab;
  c.hist_s = hist_s + copy_off;
  c.hist.counts = nullptr;
  c.hist.wsum = nullptr;
  c.qn = 0;
  c.xn = 0;
  c.nb = nb;
  c.cs = cs;
  c.ai = 0;
  c.wa = 0.0f;
  c.lane = static_cast<unsigned>(lane);
  c.lt_mask = lt_mask;
  c.n_exact_tri = 0;
  c.n_queued = 0;
  c.n_flag_rows = 0;

  unsigned long long n_exact_pair = 0, n_anchor = 0, n_pairs = 0, n_evals = 0;

  // Adds the CTA histogram (all copies) into the current item's histogram.
  auto flush = [&]() {
    for (int i = tid; i < (HG ? 0 : nbin); i += kThreads) {
      if (WEIGHTED) {
        long long* h = reinterpret_cast<long long*>(hist_s);
        long long v = 0;
        for (int cp = 0; cp < copies; ++cp) {
          v += h[cp * nbin + i];
          h[cp * nbin + i] = 0;
        }
        if (v) add128(&s_it.hist.wsum[2 * i], v);
      } else {
        unsigned* h = reinterpret_cast<unsigned*>(hist_s);
        unsigned long long v = 0;
        for (int cp = 0; cp < copies; ++cp) {
          v += h[cp * nbin + i];
          h[cp * nbin + i] = 0;
        }
        if (v) atomicAdd(&s_it.hist.counts[i], v);
      }
    }
  };

  // Addresses in the shared window, for the PTX candidate body.
  const unsigned tab_sh = static_cast<unsigned>(__cvta_generic_to_shared(tab));
  const unsigned tab_adj = tab_sh - 0x4B000000u;
  const unsigned tab_last = tab_sh + static_cast<unsigned>(g.tab_n - 1);
  const unsigned hist_sh = static_cast<unsigned>(__cvta_generic_to_shared(hist_s)) + copy_off;
  const unsigned dummy = static_cast<unsigned>(__cvta_generic_to_shared(smem + L.scratch)) + 8u * lane;
  const float tscale = g.tab_scale, hm = g.hm;

  for (;;) {
    __syncthreads();
    if (tid == 0) {
      if (a.sched_static)
        s_w = s_next < s_end ? static_cast<int>(s_next++) : a.n_work;
      else
        s_w = atomicAdd(a.work, 1);
    }
    __syncthreads();
    const int w = s_w;
    if (static_cast<unsigned>(w) >= static_cast<unsigned>(a.n_work)) break;
    const int item = a.q_item ? a.q_item[w] : 0;
    if (item != s_cur) {
      // New item: its predecessor's counts go to the predecessor's histogram.
      if (s_cur >= 0) flush();
      __syncthreads();
      if (tid == 0) {
        s_it = a.items[item];
        s_sym6 = item_sym6(a.items[item]) ? 1 : 0;
        s_cur = item;
        s_since = 0;
      }
      __syncthreads();
    }
    c.hist = s_it.hist;
    const int ai = a.q_anchor ? a.q_anchor[w] : w;
    ++n_anchor;
    const double4_16a pa = s_it.c1.pd[ai];
    const float4 qa = s_it.c1.pq[ai];
    const int hc = s_it.c1.pc[ai];
    const int hz = hc % g.nc[2];
    const int hy = (hc / g.nc[2]) % g.nc[1];
    const int hx = hc / (g.nc[2] * g.nc[1]);

    // ---- slots: 27 (cell, image) pairs, order of source/cudaNcorr.cu:37-48
    if (tid < 27) {
      const int s = tid;
      int cc[3] = {hx + s / 9 - 1, hy + (s / 3) % 3 - 1, hz + s % 3 - 1};
      const int h[3] = {hx, hy, hz};
      double sh[3] = {0.0, 0.0, 0.0};
      bool ok = true;
      for (int d = 0; d < 3; ++d) {
        if (SURVEY) {
          if (cc[d] == g.nc[d] || cc[d] == -1) ok = false;
        } else {
          if (cc[d] == g.nc[d]) {
            cc[d] = 0;
            sh[d] = g.box[d];
          } else if (cc[d] == -1) {
            cc[d] = g.nc[d] - 1;
            sh[d] = -g.box[d];
          }
        }
      }
      const int cell = ok ? cc[2] + g.nc[2] * (cc[1] + g.nc[1] * cc[0]) : -1;
      for (int d = 0; d < 3; ++d) {
        s_shift[s][d] = sh[d];
        if (ok) {
          const double o_n = __dmul_rn(static_cast<double>(cc[d]), g.cell);
          const double o_h = __dmul_rn(static_cast<double>(h[d]), g.cell);
          s_do[s][d] = __double2float_rn(__dsub_rn(__dadd_rn(o_n, sh[d]), o_h));
        } else {
          s_do[s][d] = 0.0f;
        }
      }
      int st2 = ok ? s_it.c2.start[cell] : 0;
      int n2 = ok ? s_it.c2.count[cell] : 0;
      if (SYM && s_sym6) {
        // Six-fold loop: only neighbours after the anchor in cell order,
        // so the slot's range starts past the anchor's sorted index.
        const int lo = max(st2, ai + 1);
        n2 = max(0, st2 + n2 - lo);
        st2 = lo;
      }
      s_start2[s] = st2;
      s_pre2[s + 1] = n2;
      if (!SYM) {
        s_start3[s] = ok ? s_it.c3.start[cell] : 0;
        s_pre3[s + 1] = ok ? s_it.c3.count[cell] : 0;
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
    const bool after_only = SYM && s_sym6;
    auto build = [&](const Catalog& cat, const int* pre, const int* st, ListView& lv, int* counter) {
      const int total = pre[27];
      const int rounded = (total + 31) & ~31;
      // Software pipeline: the next round's point is loaded before this
      // round's is classified, so two loads are in flight per thread.
      int sn = 0, jn = 0;
      float4 qn = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      if (warp * 32 + lane < total) {
        const int first = warp * 32 + lane;
        while (first >= pre[sn + 1]) ++sn;
        jn = st[sn] + (first - pre[sn]);
        qn = cat.pq[jn];
      }
      for (int base = warp * 32; base < rounded; base += kThreads) {
        const int item = base + lane;
        const int s = sn, j = jn;
        const float4 q = qn;
        const int next = item + kThreads;
        if (next < total) {
          while (next >= pre[sn + 1]) ++sn;
          jn = st[sn] + (next - pre[sn]);
          qn = cat.pq[jn];
        }
        bool acc = false;
        float4 ent;
        unsigned meta = 0;
        int pidx = 0;
        float w = 0.0f;
        if (item < total) {
          // Cell-local FP32 prefilter: skip candidates certainly out of range.
          const float fx = (q.x - qa.x) + s_do[s][0];
          const float fy = (q.y - qa.y) + s_do[s][1];
          const float fz = (q.z - qa.z) + s_do[s][2];
          const float vp = fmaf(fz, fz, fmaf(fy, fy, fx * fx));
          if (vp < g.pre_hi && vp > g.pre_lo && (!after_only || j > ai)) {
            // Exact anchor-relative offset of the image (FP64), rounded once.
            const double4_16a p = cat.pd[j];
            const double px = __dadd_rn(p.x, s_shift[s][0]);
            const double py = __dadd_rn(p.y, s_shift[s][1]);
            const double pz = __dadd_rn(p.z, s_shift[s][2]);
            const float dx = __double2float_rn(__dsub_rn(px, pa.x));
            const float dy = __double2float_rn(__dsub_rn(py, pa.y));
            const float dz = __double2float_rn(__dsub_rn(pz, pa.z));
            const float v = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
            unsigned code = table_code(v, tab, g.tab_scale, g.tab_n);
            if (code < nb_cs) {
              code /= cs;
            } else if (code == kCodeCareful) {
              code = careful_code(v, s_e2lo, s_e2hi, nb, g.ka, g.kb);
            }
            if (code == kCodeExact) {
              ++n_exact_pair;
              code = cold_pair_exact(&a.self->g, s_sqr_bins, pa, px, py, pz);
            }
            if (code < static_cast<unsigned>(nb)) {
              acc = true;
              ent = make_float4(dx, dy, dz, __fsqrt_rn(v));
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
    build(s_it.c2, s_pre2, s_start2, l2, &s_k2);
    if (!SYM) build(s_it.c3, s_pre3, s_start3, l3, &s_k3);
    __syncthreads();
    const int cap = a.ks + a.kg;
    const int k2 = min(s_k2, cap);
    const int k3 = SYM ? k2 : min(s_k3, cap);
    if (tid == 0) {
      const unsigned long long pairs_here = SYM ? static_cast<unsigned long long>(k2) * (k2 > 0 ? k2 - 1 : 0) / 2
                                                : static_cast<unsigned long long>(k2) * k3;
      n_pairs += pairs_here;
      if (a.cell_work) atomicAdd(&a.cell_work[s_it.cell_base + hc], pairs_here);
      n_evals += static_cast<unsigned long long>(s_pre2[27]) +
                 (SYM ? 0ull : static_cast<unsigned long long>(s_pre3[27]));
    }
    const int nt2 = (k2 + kTile - 1) / kTile;
    const int nt3 = (k3 + kTile - 1) / kTile;
    const long long npairs_t = SYM ? static_cast<long long>(nt2) * (nt2 + 1) / 2
                                   : static_cast<long long>(nt2) * nt3;
    const long long nitems = npairs_t * spt;
    // A CTA histogram bin grows by at most sub_j*kTile per item; flush before
    // it could overflow its 32-bit counter (count mode) or 64-bit sum
    // (weighted mode, |term| <= 2^30).
    const long long kItemLimit = (1LL << 31) / (static_cast<long long>(sub_j) * kTile);
    const float wa = static_cast<float>(pa.w);
    c.ai = w;
    c.wa = wa;

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

      // One work item: l-tile lt (registers) against 32 j-entries of tile jt.
      // MODE 0: full l-tile; 1: the list's partial last l-tile; 2: diagonal
      // tile pair (identical catalogues, pairs j > l only).
      auto item = [&](int jt, int lt, int sub, auto mode_tag) {
        constexpr int MODE = decltype(mode_tag)::value;
        constexpr bool DIAG = MODE == 2;
        float4 el[kReg];
        unsigned kl[kReg];
        float wl[kReg];
        const int lb = lt * kTile;
        const bool l_in_smem = lb < a.ks;
#pragma unroll
        for (int r = 0; r < kReg; ++r) {
          const int l = lb + r * 32 + lane;
          // Columns are held as (-2 d_l, rho_l); the padding (0, rho = 1e18)
          // gives v = 1e36 and is rejected by the table for every row.
          if (l < k3) {
            const float4 e = l_in_smem ? l3.e[l] : l3.se[l - a.ks];
            el[r] = make_float4(-2.0f * e.x, -2.0f * e.y, -2.0f * e.z, e.w);
            const unsigned ml = l_in_smem ? l3.m[l] : l3.sm[l - a.ks];
            kl[r] = (ml & 0xffu) * nb_cs;
            wl[r] = WEIGHTED ? (l_in_smem ? l3.w[l] : l3.sw[l - a.ks]) : 0.0f;
          } else {
            el[r] = make_float4(0.0f, 0.0f, 0.0f, 1.0e18f);
            kl[r] = 0;
            wl[r] = 0.0f;
          }
        }
        const int jb = jt * kTile + sub * sub_j;
        const int je = min(jb + sub_j, k2);
        const bool j_in_smem = jb < a.ks;
        const float4* ej_base = j_in_smem ? l2.e + jb : l2.se + (jb - a.ks);
        const unsigned* mj_base = j_in_smem ? l2.m + jb : l2.sm + (jb - a.ks);
        const float* wj_base = WEIGHTED ? (j_in_smem ? l2.w + jb : l2.sw + (jb - a.ks)) : nullptr;
        const unsigned kj_mul = static_cast<unsigned>(nb * nb * cs);
        // l-slices r >= rhi hold no candidate of these rows: they lie past
        // the end of the list or, on the diagonal, at or above the rows.
        const int rhi = MODE == 0 ? kReg : min(kReg, (min(k3, DIAG ? je : k3) - lb + 31) >> 5);
        // Rows with a candidate needing the careful/exact path are flagged
        // here and re-examined out of line after the loop.
        unsigned rowmask = 0;

        if (!HG) {
          // Shared histogram: the PTX candidate body, counts or weighted
          // sums. The lane's four l-entries are explicit scalars; slices
          // without candidates are skipped with a warp-uniform test. A row's
          // weight is (w_anchor * w_j) * scale, the order of the exact path.
          const float4 L0 = el[0], L1 = el[1], L2 = el[2], L3 = el[3];
          const unsigned K0 = kl[0], K1 = kl[1], K2 = kl[2], K3 = kl[3];
          const float W0 = wl[0], W1 = wl[1], W2 = wl[2], W3 = wl[3];
          const int lr0 = lb + lane, lr1 = lr0 + 32, lr2 = lr0 + 64, lr3 = lr0 + 96;
          const float wsc = a.wscale;
          auto row = [&](float4 e, unsigned k, int jj, float wr) -> unsigned {
            const float aj = __fmul_rn(e.w, e.w), a2r = 2.0f * e.w;
            unsigned q = 0;
            if (MODE == 0 && !WEIGHTED) {
              row4_count(e.x, e.y, e.z, aj, a2r, k, tscale, tab_adj, tab_last, nb_cs, hm, dummy, L0, K0, L1, K1, L2,
                         K2, L3, K3, 1u, q);
              return __any_sync(FULL, q != 0) ? 1u : 0u;
            }
            cand_body<WEIGHTED, DIAG>(e.x, e.y, e.z, aj, a2r, L0.x, L0.y, L0.z, L0.w, k, K0, jj > lr0, tscale,
                                      tab_adj, tab_last, nb_cs, hm, dummy, wr, W0, q);
            if (MODE == 0 || rhi > 1)
              cand_body<WEIGHTED, DIAG>(e.x, e.y, e.z, aj, a2r, L1.x, L1.y, L1.z, L1.w, k, K1, jj > lr1,
                                        tscale, tab_adj, tab_last, nb_cs, hm, dummy, wr, W1, q);
            if (MODE == 0 || rhi > 2)
              cand_body<WEIGHTED, DIAG>(e.x, e.y, e.z, aj, a2r, L2.x, L2.y, L2.z, L2.w, k, K2, jj > lr2,
                                        tscale, tab_adj, tab_last, nb_cs, hm, dummy, wr, W2, q);
            if (MODE == 0 || rhi > 3)
              cand_body<WEIGHTED, DIAG>(e.x, e.y, e.z, aj, a2r, L3.x, L3.y, L3.z, L3.w, k, K3, jj > lr3,
                                        tscale, tab_adj, tab_last, nb_cs, hm, dummy, wr, W3, q);
            return __any_sync(FULL, q != 0) ? 1u : 0u;
          };
          int j = jb;
          if (j_in_smem) {
            const unsigned e_sh = static_cast<unsigned>(__cvta_generic_to_shared(l2.e + jb));
            const unsigned m_sh = static_cast<unsigned>(__cvta_generic_to_shared(l2.m + jb));
            const unsigned w_sh = WEIGHTED ? static_cast<unsigned>(__cvta_generic_to_shared(l2.w + jb)) : 0u;
            if (MODE == 0 && !WEIGHTED) {
              // Full tile, counts: each row ORs its bit into the lane's flag
              // word, and one warp reduction per work item gives the rows to
              // re-examine.
              unsigned qbits = 0;
#pragma unroll 2
              for (; j < je; ++j) {
                const unsigned o = static_cast<unsigned>(j - jb);
                const float4 e0 = lds_f4(e_sh + 16u * o);
                const unsigned k0 = (lds_u32(m_sh + 4u * o) & 0xffu) * kj_mul + hist_sh;
                row4_count(e0.x, e0.y, e0.z, __fmul_rn(e0.w, e0.w), 2.0f * e0.w, k0, tscale, tab_adj, tab_last, nb_cs,
                           hm, dummy, L0, K0, L1, K1, L2, K2, L3, K3, 1u << o, qbits);
              }
              rowmask |= __reduce_or_sync(FULL, qbits);
            }
#if NCORR_ROW_UNROLL == 2
            for (; j + 1 < je; j += 2) {
              const unsigned o = static_cast<unsigned>(j - jb);
              const float4 e0 = lds_f4(e_sh + 16u * o);
              const float4 e1 = lds_f4(e_sh + 16u * o + 16u);
              const unsigned k0 = (lds_u32(m_sh + 4u * o) & 0xffu) * kj_mul + hist_sh;
              const unsigned k1 = (lds_u32(m_sh + 4u * o + 4u) & 0xffu) * kj_mul + hist_sh;
              const float w0 = WEIGHTED ? wa * lds_f32(w_sh + 4u * o) * wsc : 0.0f;
              const float w1 = WEIGHTED ? wa * lds_f32(w_sh + 4u * o + 4u) * wsc : 0.0f;
              const unsigned f0 = row(e0, k0, j, w0);
              const unsigned f1 = row(e1, k1, j + 1, w1);
              rowmask |= (f0 | (f1 << 1)) << o;
            }
#endif
            for (; j < je; ++j) {
              const unsigned o = static_cast<unsigned>(j - jb);
              const float4 e0 = lds_f4(e_sh + 16u * o);
              const unsigned k0 = (lds_u32(m_sh + 4u * o) & 0xffu) * kj_mul + hist_sh;
              const float w0 = WEIGHTED ? wa * lds_f32(w_sh + 4u * o) * wsc : 0.0f;
              rowmask |= row(e0, k0, j, w0) << o;
            }
          } else {
            for (; j < je; ++j) {
              const unsigned o = static_cast<unsigned>(j - jb);
              const float w0 = WEIGHTED ? wa * wj_base[o] * wsc : 0.0f;
              rowmask |= row(ej_base[o], (mj_base[o] & 0xffu) * kj_mul + hist_sh, j, w0) << o;
            }
          }
        } else {
          // Global histogram (too many bins for shared memory): the same
          // decisions in C++.
          for (int j = jb; j < je; ++j) {
            const unsigned o = static_cast<unsigned>(j - jb);
            const float4 ej = ej_base[o];
            const unsigned kj = (mj_base[o] & 0xffu) * kj_mul + (HG ? 0u : hist_sh);
            const float aj = __fmul_rn(ej.w, ej.w), a2r = 2.0f * ej.w;
            const float wja = WEIGHTED ? wa * wj_base[o] * a.wscale : 0.0f;
            bool q = false;
#pragma unroll
            for (int r = 0; r < kReg; ++r) {
              if (MODE != 0 && r >= rhi) continue;
              unsigned code;
              bool clean;
              cand_classify(ej.x, ej.y, ej.z, aj, a2r, el[r], tab, g.tab_scale, g.tab_n, hm, &code, &clean);
              bool ok = code < nb_cs;
              bool careful = code == kCodeCareful;
              if (DIAG) {
                const bool in = j > lb + r * 32 + lane;
                ok = ok && in;
                careful = careful && in;
              }
              const unsigned key = kj + kl[r] + code;
              if (HG) {
                if (ok && clean) hist_add<WEIGHTED, true>(hist_s, c.hist, key, wja * wl[r]);
              } else {
                red_shared_u64_if(key, static_cast<unsigned long long>(__float2ll_rn(wja * wl[r])), ok && clean);
              }
              q = q || careful || (ok && !clean);
            }
            rowmask |= (__any_sync(FULL, q) ? 1u : 0u) << o;
          }
        }
        while (rowmask) {
          const int bit = __ffs(rowmask) - 1;
          rowmask &= rowmask - 1u;
          if (c.qn > kQueueCap - kTile) cold_drain<SURVEY, WEIGHTED, HG>(c);
          enqueue_row<WEIGHTED, HG, MODE>(c, g, jb + bit, ej_base[bit], el, lb, rhi, tab_adj, tab_last, nb_cs);
        }
      };

      for (;;) {
        int mi = 0;
        if (lane == 0) mi = atomicAdd(&s_item, 1);
        mi = __shfl_sync(FULL, mi, 0);
        const long long m = m0 + mi;
        if (m >= m1) break;
        const int sub = static_cast<int>(m % spt);
        const long long tp = m / spt;
        int jt, lt;
        if (SYM) {
          // Tile pairs lt <= jt: the list's partial last tile is a j-tile
          // (rows stop at the list end) except on its own diagonal.
          jt = static_cast<int>((sqrtf(8.0f * static_cast<float>(tp) + 1.0f) - 1.0f) * 0.5f);
          while (static_cast<long long>(jt) * (jt + 1) / 2 > tp) --jt;
          while (static_cast<long long>(jt + 1) * (jt + 2) / 2 <= tp) ++jt;
          lt = static_cast<int>(tp - static_cast<long long>(jt) * (jt + 1) / 2);
        } else {
          jt = static_cast<int>(tp % nt2);
          lt = static_cast<int>(tp / nt2);
        }
        if (jt * kTile + sub * sub_j >= k2) continue;  // empty sub-range of the last tile
        if (SYM && jt == lt)
          item(jt, lt, sub, std::integral_constant<int, 2>());
        else if ((lt + 1) * kTile > k3)
          item(jt, lt, sub, std::integral_constant<int, 1>());
        else
          item(jt, lt, sub, std::integral_constant<int, 0>());
      }
      // Queue entries refer to this anchor's lists: settle them now.
      if (c.qn > 0) cold_drain<SURVEY, WEIGHTED, HG>(c);
      __syncthreads();
    }
  }
  cold_flush_exact<SURVEY, WEIGHTED>(c);
  __syncthreads();
  if (s_cur >= 0) flush();
  if (a.stats) {
    atomicAdd(&a.stats[0], c.n_exact_tri);
    atomicAdd(&a.stats[1], n_exact_pair);
    if (tid == 0) {
      atomicAdd(&a.stats[2], n_anchor);
      atomicAdd(&a.stats[3], n_pairs);
      atomicAdd(&a.stats[4], n_evals);
    }
    if (lane == 0) {
      atomicAdd(&a.stats[5], c.n_flag_rows);
      atomicAdd(&a.stats[6], c.n_queued);
    }
  }
}

}  // namespace ncorr_gb300
