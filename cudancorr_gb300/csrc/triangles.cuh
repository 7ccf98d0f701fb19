// Triangle-count kernel: the GB300 counterpart of the reference's
// countTrianglesThreeDBox / countTrianglesThreeDSurvey
// (source/device.cu:259-315, :381-431).
//
// A persistent grid of one CTA of 16 warps per SM. Each WARP owns one anchor
// (a point of catalogue 1) at a time, start to finish, so warps never wait on
// one another: there is no CTA-wide barrier between anchors. Anchors come
// from a work queue whose positions name (batch item, anchor): in cell order
// or in a learned order, taken one at a time from a global counter (dynamic)
// or from one contiguous range per CTA (static).
//  Phase A  the warp streams the 27 (cell, image) slots around the anchor's
//           home cell from the cell list. A cell-local FP32 estimate of r1^2
//           drops candidates certainly out of range; for the others the
//           anchor-relative offset is formed exactly in FP64 and rounded once
//           to FP32, and r1^2 from it is classified against the bins
//           (rigorous error band; the rare undecided ones are recomputed in
//           FP64 exactly as the reference computes them). In-range neighbours
//           are appended to the warp's list in global memory (cached in L1):
//           offset d (float3), the square root of the r1^2 estimate, exact
//           bin, slot, point index, weight.
//  Phase B  every neighbour pair (j, l) of the list(s) is a candidate
//           triangle. The warp holds a tile of 128 columns in registers (four
//           per lane) and streams the rows past it, one row ahead in flight.
//           Per candidate: r3^2 in FP32 as rho_j^2 + rho_l^2 - 2 d_j.d_l, its
//           bin from a shared-memory table, a margin test on d_j.d_l proving
//           the reference's FP32 triangle test, and one shared-memory
//           reduction into the CTA's (bin_j, bin_l, bin_3) histogram.
//           Candidates whose FP32 classification is not certain set their
//           (row, column slot) bit in a per-lane flag word; after each group
//           of rows exactly those candidates are queued and settled by the
//           careful band or the exact FP64 restatement.
// Symmetry: with catalogues 2 and 3 identical (SYM), only pairs l < j are
// visited and count twice -- the reference's ordered double loop is symmetric
// in (p2, p3) because (a-b)^2 == (b-a)^2 bit for bit. With all three
// catalogues identical and the geometry checked to make every triangle's
// three vertices see each other through bit-identical images (six-fold,
// decided on the host and per point), only neighbours after the anchor in
// cell order are listed and each counted triangle stands for all six
// orderings.
// The CTA histogram is shared by all 16 warps. It is bound to one batch item
// at a time through a small ownership word: a warp whose anchor belongs to
// another item waits until no warp uses the histogram, adds it to the old
// item's global histogram and rebinds it (the queue keeps each item's anchors
// together, so this happens about once per item and CTA). To keep its 32-bit
// counts (64-bit fixed-point sums) from overflowing, warps reserve every
// tile's candidates in a shared counter, and the warp whose reservation
// crosses a multiple of 2^30 drains the histogram into the global one with
// atomic exchanges, which is exact while other warps keep adding.
#pragma once
#include <type_traits>

#include "engine.cuh"

namespace ncorr_gb300 {

constexpr unsigned kCodeExact = 0xFDu;

// Rows per careful-flag group (8, 16 or 32; a run-time choice, KArgs::sub_j).
constexpr int kSubJDefault = 32;
// Slot word of the CTA histogram: owner = batch item + 1 (0: unbound,
// kSlotLocked: being rebound) in the high half, warps using it in the low.
constexpr unsigned kSlotLocked = 0xFFFFFFFFu;
// Reservation counter unit (candidates) and the drain period (units).
constexpr int kSinceShift = 10;
constexpr unsigned kSinceDrainBits = 20;  // 2^20 units = 2^30 candidates
// Upper bound of the waits for the histogram slot (iterations of ~0.5 us).
constexpr int kSlotSpinLimit = 1 << 22;

// Per-warp slot table of the anchor being listed (shared memory).
struct SlotTab {
  double shift[27][3];  // image shift of the slot (0 or +-box per axis)
  float dof[27][3];     // FP32 offset of the slot's cell origin from the home cell's
  int start2[27], pre2[28], start3[27], pre3[28];
};

// Shared-memory layout (dynamic part). The bin table sits at offset 0 and the
// CTA histogram right after it, so both are addressed with immediate offsets.
struct SmemLayout {
  int table, hist, slots, scratch, total;
};

__host__ __device__ inline int align16(int x) { return (x + 15) & ~15; }

__host__ __device__ inline SmemLayout make_layout(int nb, bool weighted, bool hist_global, int hist_copies = 1) {
  SmemLayout L;
  int o = 0;
  L.table = o;
  o += kTableSize;
  L.hist = o;
  if (!hist_global) o = align16(o + hist_copies * nb * nb * nb * (weighted ? 8 : 4));
  L.slots = o;
  o += kWarps * static_cast<int>(sizeof(SlotTab));
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
  // 1: CTA b takes positions [b*n/G, (b+1)*n/G), its warps one at a time in
  // order (static schedule); 0: warps take positions from the global counter
  // `work`.
  int sched_static;
  int sub_j;        // rows per careful-flag group (8, 16 or 32)
  int hist_copies;  // copies of the CTA histogram, lane & (copies-1) picks one
  // Optional: candidate pairs of each anchor added to its home cell
  // (cell_base of the item + cell), the work the scheduler learns.
  unsigned long long* cell_work;
  const unsigned char* table;
  int* work;
  int* flags;
  // Per-warp global slabs: neighbour lists (kcap2 entries for p2, then kcap3
  // for p3; kcap3 = 0 when p2 == p3), careful queue, exact buffer.
  float4* slab_e;
  unsigned* slab_m;
  int* slab_p;
  float* slab_w;
  unsigned long long* slab_q;
  ExactEntry* slab_x;
  int kcap2, kcap3;
  float wscale;
  // Byte stride of one bin in the CTA histogram as encoded in the table
  // (4: u32 counts, 8: int64 sums, 1: global histogram, bins unscaled).
  int code_scale;
  unsigned long long* stats;  // exact tris, exact pairs, anchors, W, P, flagged rows, queued
  // Optional: per CTA, its start and end time (globaltimer, ns), from which
  // the host measures how long CTAs sat idle at the end of the launch.
  unsigned long long* cta_time;
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
  // Unsigned, as in the PTX bodies: a slightly negative v (the estimate of a
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

// A neighbour list in global memory.
struct ListView {
  float4* e;
  unsigned* m;
  int* p;
  float* w;
};

// The margin form of the triangle test. List entries keep rho = sqrt_rn of
// their r^2 estimate in .w; with a = rho_j^2 and b = rho_l^2 (the products
// formed inside the FMAs) a candidate of third side v is certainly kept by
// the reference's FP32 sqrtf test when |v - (a + b)| < 2 rho_j rho_l - M
// (hm = -M; the PTX bodies evaluate the same operations).
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

// ---------------------------------------------------------------------------
// Candidate bodies in hand-written PTX. Every rounding is explicit (.rn),
// matching the error model. With p = -2 d_j.d_l the third side is
// v = p + (rho_l^2 + rho_j^2): three products and two adds instead of three
// differences and three squares, and p itself is the quantity of the margin
// test, |p| < 2 rho_j rho_l - M (|C - A - B| = |2 D_j.D_l| for the exact
// sides). A candidate counts in bin `code` of the table when the margin test
// holds; one that needs the careful or exact path ORs `rbit` (its row's bit
// in the flag group) into the flag word of its column slot. The histogram
// reduction is unconditional: a candidate that does not count adds to the
// lane's own scratch word `dummy` instead, which keeps the loop free of the
// branch a predicated atomic compiles to.
//
// Operands of the row bodies:
//   %0-%3  flag words of column slots 0-3 (in/out)
//   %4-%6  the row's offset d_j, %7 rho_j^2, %8 2 rho_j, %9 the row's key
//          (histogram base + bin_j * nb^2 * code scale)
//   %10 table scale, %11/%12 table address bias and last entry, %13 nb * code
//   scale, %14 -M, %15 dummy address, %16 rbit, %17-%20 masks of column
//   slots 0-3 (diagonal rows: 1 below the row's slot, l < j in it, 0 above)
//   column c: %(21+5c)-%(23+5c) its offset scaled by -2, %(24+5c) rho_l,
//   %(25+5c) its key (bin_l * nb * code scale)
// One asm statement per row lets all table loads issue before the first
// reduction; in separate statements each load would wait behind the previous
// candidate's reduction, which may touch the same shared-memory word as far
// as the compiler can tell.
#define NCORR_DECL(C)                                                     \
  ".reg .f32 pp" #C ", s" #C ", v" #C ", t" #C ", H" #C ";\n\t"           \
  ".reg .b32 y" #C ", ia" #C ", code" #C ", key" #C ", adr" #C ";\n\t"     \
  ".reg .pred ok" #C ", upd" #C ", nco" #C ", wq" #C ";\n\t"
#define NCORR_CLS(C, LX, LY, LZ, B)                  \
  "mul.rn.f32 pp" #C ", %4, " LX ";\n\t"             \
  "fma.rn.f32 pp" #C ", %5, " LY ", pp" #C ";\n\t"   \
  "fma.rn.f32 pp" #C ", %6, " LZ ", pp" #C ";\n\t"   \
  "fma.rn.f32 s" #C ", " B ", " B ", %7;\n\t"        \
  "add.rn.f32 v" #C ", pp" #C ", s" #C ";\n\t"       \
  "fma.rn.f32 y" #C ", v" #C ", %10, 0f4B000000;\n\t" \
  "add.u32 ia" #C ", y" #C ", %11;\n\t"              \
  "min.u32 ia" #C ", ia" #C ", %12;\n\t"             \
  "ld.shared.u8 code" #C ", [ia" #C "];\n\t"
// Column operand groups, expanded through NCORR_CLSX so that a group fills
// the four column arguments of NCORR_CLS.
#define NCORR_CLS_I(C, ...) NCORR_CLS(C, __VA_ARGS__)
#define NCORR_CLSX(C, COLS) NCORR_CLS_I(C, COLS)
#define NCORR_KEY(C, KL)                               \
  "add.u32 key" #C ", %9, " KL ";\n\t"                 \
  "add.u32 key" #C ", key" #C ", code" #C ";\n\t"      \
  "selp.b32 adr" #C ", key" #C ", %15, upd" #C ";\n\t"
#define NCORR_UPD(C, B, KL, Q)                                     \
  "abs.f32 t" #C ", pp" #C ";\n\t"                                 \
  "fma.rn.f32 H" #C ", %8, " B ", %14;\n\t"                        \
  "setp.lt.u32 ok" #C ", code" #C ", %13;\n\t"                     \
  "setp.lt.and.f32 upd" #C ", t" #C ", H" #C ", ok" #C ";\n\t"     \
  "setp.ge.and.f32 nco" #C ", t" #C ", H" #C ", ok" #C ";\n\t"     \
  "setp.eq.or.u32 wq" #C ", code" #C ", 255, nco" #C ";\n\t"       \
  "@wq" #C " or.b32 " Q ", " Q ", %16;\n\t" NCORR_KEY(C, KL)
#define NCORR_UPD_MASKED(C, B, KL, Q, M)                           \
  "abs.f32 t" #C ", pp" #C ";\n\t"                                 \
  "fma.rn.f32 H" #C ", %8, " B ", %14;\n\t"                        \
  "setp.ne.u32 inp" #C ", " M ", 0;\n\t"                           \
  "setp.lt.u32 ok" #C ", code" #C ", %13;\n\t"                     \
  "and.pred ok" #C ", ok" #C ", inp" #C ";\n\t"                    \
  "setp.lt.and.f32 upd" #C ", t" #C ", H" #C ", ok" #C ";\n\t"     \
  "setp.ge.and.f32 nco" #C ", t" #C ", H" #C ", ok" #C ";\n\t"     \
  "setp.eq.and.u32 car" #C ", code" #C ", 255, inp" #C ";\n\t"     \
  "or.pred wq" #C ", car" #C ", nco" #C ";\n\t"                    \
  "@wq" #C " or.b32 " Q ", " Q ", %16;\n\t" NCORR_KEY(C, KL)
#define NCORR_RED(C) "red.shared.add.u32 [adr" #C "], 1;\n\t"
#define NCORR_C0 "%21", "%22", "%23", "%24"
#define NCORR_C1 "%26", "%27", "%28", "%29"
#define NCORR_C2 "%31", "%32", "%33", "%34"
#define NCORR_C3 "%36", "%37", "%38", "%39"
#define NCORR_ROW_OPERANDS                                                                                      \
  : "+r"(q0), "+r"(q1), "+r"(q2), "+r"(q3)                                                                     \
  : "f"(r.x), "f"(r.y), "f"(r.z), "f"(r.a), "f"(r.a2r), "r"(r.key), "f"(k.tscale), "r"(k.tab_adj),             \
    "r"(k.tab_last), "r"(k.nb_cs), "f"(k.hm), "r"(k.dummy), "r"(rbit), "r"(m0), "r"(m1), "r"(m2), "r"(m3),     \
    "f"(c.l[0].x), "f"(c.l[0].y), \
    "f"(c.l[0].z), "f"(c.l[0].w), "r"(c.k[0]), "f"(c.l[1].x), "f"(c.l[1].y), "f"(c.l[1].z), "f"(c.l[1].w),    \
    "r"(c.k[1]), "f"(c.l[2].x), "f"(c.l[2].y), "f"(c.l[2].z), "f"(c.l[2].w), "r"(c.k[2]), "f"(c.l[3].x),        \
    "f"(c.l[3].y), "f"(c.l[3].z), "f"(c.l[3].w), "r"(c.k[3])                                                   \
  : "memory"

// Constants of the candidate bodies, fixed per launch.
struct BodyK {
  float tscale, hm;
  unsigned tab_adj, tab_last, nb_cs, dummy;
};
// One row: offset, rho^2, 2 rho, key.
struct RowV {
  float x, y, z, a, a2r;
  unsigned key;
};
// The lane's four columns: (-2 d_l, rho_l) and keys.
struct ColV {
  float4 l[kReg];
  unsigned k[kReg];
};

// Four full candidates (column slots 0-3).
__device__ __forceinline__ void row_full4(const RowV& r, const ColV& c, const BodyK& k, unsigned rbit, unsigned& q0,
                                          unsigned& q1, unsigned& q2, unsigned& q3) {
  const unsigned m0 = 1u, m1 = 1u, m2 = 1u, m3 = 1u;
  asm volatile("{\n\t" NCORR_DECL(0) NCORR_DECL(1) NCORR_DECL(2) NCORR_DECL(3)
               NCORR_CLSX(0, NCORR_C0) NCORR_CLSX(1, NCORR_C1) NCORR_CLSX(2, NCORR_C2) NCORR_CLSX(3, NCORR_C3)
               NCORR_UPD(0, "%24", "%25", "%0") NCORR_UPD(1, "%29", "%30", "%1") NCORR_UPD(2, "%34", "%35", "%2")
               NCORR_UPD(3, "%39", "%40", "%3")
               NCORR_RED(0) NCORR_RED(1) NCORR_RED(2) NCORR_RED(3) "}" NCORR_ROW_OPERANDS);
}

// Four candidates with a mask each (diagonal rows of identical lists, pairs
// l < j): masked-out candidates neither count nor flag.
__device__ __forceinline__ void row_mask4(const RowV& r, const ColV& c, const BodyK& k, unsigned rbit, unsigned m0,
                                          unsigned m1, unsigned m2, unsigned m3, unsigned& q0, unsigned& q1,
                                          unsigned& q2, unsigned& q3) {
  asm volatile("{\n\t.reg .pred inp0, inp1, inp2, inp3, car0, car1, car2, car3;\n\t"
               NCORR_DECL(0) NCORR_DECL(1) NCORR_DECL(2) NCORR_DECL(3)
               NCORR_CLSX(0, NCORR_C0) NCORR_CLSX(1, NCORR_C1) NCORR_CLSX(2, NCORR_C2) NCORR_CLSX(3, NCORR_C3)
               NCORR_UPD_MASKED(0, "%24", "%25", "%0", "%17") NCORR_UPD_MASKED(1, "%29", "%30", "%1", "%18")
               NCORR_UPD_MASKED(2, "%34", "%35", "%2", "%19") NCORR_UPD_MASKED(3, "%39", "%40", "%3", "%20")
               NCORR_RED(0) NCORR_RED(1) NCORR_RED(2) NCORR_RED(3) "}" NCORR_ROW_OPERANDS);
}

// Two candidates with masks (column slots 0-1; diagonal rows of the first two
// 32-row groups of a tile, where slots 2-3 hold no pair).
__device__ __forceinline__ void row_mask2(const RowV& r, const ColV& c, const BodyK& k, unsigned rbit, unsigned m0,
                                          unsigned m1, unsigned& q0, unsigned& q1, unsigned& q2, unsigned& q3) {
  const unsigned m2 = 0u, m3 = 0u;
  asm volatile("{\n\t.reg .pred inp0, inp1, car0, car1;\n\t" NCORR_DECL(0) NCORR_DECL(1)
               NCORR_CLSX(0, NCORR_C0) NCORR_CLSX(1, NCORR_C1)
               NCORR_UPD_MASKED(0, "%24", "%25", "%0", "%17") NCORR_UPD_MASKED(1, "%29", "%30", "%1", "%18")
               NCORR_RED(0) NCORR_RED(1) "}" NCORR_ROW_OPERANDS);
}

// The weighted twin of one candidate: the same classification, then the
// fixed-point weight w_row * w_l (|value| <= 2^30 by the choice of the scale,
// so the 32-bit conversion is exact and equals the 64-bit one) added into the
// int64 bin, or into the lane's 8-byte scratch word when it does not count.
// A 64-bit shared-memory add is not a native atomic (it compiles to a
// compare-and-swap loop), so the add is split over the bin's two 32-bit
// words with native atomics: the low word by atom.add, whose old value gives
// the carry, then the high word by the sign extension plus that carry. Every
// thread's carry comes from its own atomic on the low word, so the 64-bit
// total is exact however the adds interleave. Operands: %0 flag word,
// %1-%3 d_j, %4 rho_j^2, %5 2 rho_j, %6-%8 -2 d_l, %9 rho_l, %10 row key,
// %11 column key, %12 mask, %13 table scale, %14/%15 table bias and last
// entry, %16 nb * code scale, %17 -M, %18 dummy, %19 row weight, %20 column
// weight, %21 rbit.
template <bool MASKED>
__device__ __forceinline__ void cand_wsum(const RowV& r, const float4& l, unsigned kl, unsigned in, const BodyK& k,
                                          float wrow, float wl, unsigned rbit, unsigned& q) {
#define NCORR_WSUM_ASM(UPD)                                                                                  \
  asm volatile("{\n\t.reg .pred inp, car;\n\t" NCORR_DECL(0)                                                 \
               ".reg .f32 wp;\n\t.reg .b32 wi, whi, wold, wnew, wcy, adrh;\n\t"                             \
               "mul.rn.f32 pp0, %1, %6;\n\t"                                                                 \
               "fma.rn.f32 pp0, %2, %7, pp0;\n\t"                                                            \
               "fma.rn.f32 pp0, %3, %8, pp0;\n\t"                                                            \
               "fma.rn.f32 s0, %9, %9, %4;\n\t"                                                              \
               "add.rn.f32 v0, pp0, s0;\n\t"                                                                 \
               "fma.rn.f32 y0, v0, %13, 0f4B000000;\n\t"                                                     \
               "add.u32 ia0, y0, %14;\n\t"                                                                   \
               "min.u32 ia0, ia0, %15;\n\t"                                                                  \
               "ld.shared.u8 code0, [ia0];\n\t" UPD                                                          \
               "mul.rn.f32 wp, %19, %20;\n\t"                                                                \
               "cvt.rni.s32.f32 wi, wp;\n\t"                                                                 \
               "shr.s32 whi, wi, 31;\n\t"                                                                    \
               "atom.shared.add.u32 wold, [adr0], wi;\n\t"                                                   \
               "add.u32 wnew, wold, wi;\n\t"                                                                 \
               "set.lt.u32.u32 wcy, wnew, wold;\n\t"                                                         \
               "sub.u32 whi, whi, wcy;\n\t"                                                                  \
               "add.u32 adrh, adr0, 4;\n\t"                                                                  \
               "red.shared.add.u32 [adrh], whi;\n\t"                                                         \
               "}"                                                                                           \
               : "+r"(q)                                                                                     \
               : "f"(r.x), "f"(r.y), "f"(r.z), "f"(r.a), "f"(r.a2r), "f"(l.x), "f"(l.y), "f"(l.z), "f"(l.w), \
                 "r"(r.key), "r"(kl), "r"(in), "f"(k.tscale), "r"(k.tab_adj), "r"(k.tab_last), "r"(k.nb_cs), \
                 "f"(k.hm), "r"(k.dummy), "f"(wrow), "f"(wl), "r"(rbit)                                      \
               : "memory")
#define NCORR_W_UPD                                                 \
  "abs.f32 t0, pp0;\n\t"                                            \
  "fma.rn.f32 H0, %5, %9, %17;\n\t"                                 \
  "setp.lt.u32 ok0, code0, %16;\n\t"                                \
  "setp.lt.and.f32 upd0, t0, H0, ok0;\n\t"                          \
  "setp.ge.and.f32 nco0, t0, H0, ok0;\n\t"                          \
  "setp.eq.or.u32 wq0, code0, 255, nco0;\n\t"                       \
  "@wq0 or.b32 %0, %0, %21;\n\t"                                    \
  "add.u32 key0, %10, %11;\n\t"                                     \
  "add.u32 key0, key0, code0;\n\t"                                  \
  "selp.b32 adr0, key0, %18, upd0;\n\t"
#define NCORR_W_UPD_MASKED                                          \
  "abs.f32 t0, pp0;\n\t"                                            \
  "fma.rn.f32 H0, %5, %9, %17;\n\t"                                 \
  "setp.ne.u32 inp, %12, 0;\n\t"                                    \
  "setp.lt.u32 ok0, code0, %16;\n\t"                                \
  "and.pred ok0, ok0, inp;\n\t"                                     \
  "setp.lt.and.f32 upd0, t0, H0, ok0;\n\t"                          \
  "setp.ge.and.f32 nco0, t0, H0, ok0;\n\t"                          \
  "setp.eq.and.u32 car, code0, 255, inp;\n\t"                       \
  "or.pred wq0, car, nco0;\n\t"                                     \
  "@wq0 or.b32 %0, %0, %21;\n\t"                                    \
  "add.u32 key0, %10, %11;\n\t"                                     \
  "add.u32 key0, key0, code0;\n\t"                                  \
  "selp.b32 adr0, key0, %18, upd0;\n\t"
  if (MASKED) {
    NCORR_WSUM_ASM(NCORR_W_UPD_MASKED);
  } else {
    NCORR_WSUM_ASM(NCORR_W_UPD);
  }
#undef NCORR_W_UPD_MASKED
#undef NCORR_W_UPD
#undef NCORR_WSUM_ASM
}

#undef NCORR_ROW_OPERANDS
#undef NCORR_C0
#undef NCORR_C1
#undef NCORR_C2
#undef NCORR_C3
#undef NCORR_RED
#undef NCORR_UPD_MASKED
#undef NCORR_UPD
#undef NCORR_KEY
#undef NCORR_CLSX
#undef NCORR_CLS_I
#undef NCORR_CLS
#undef NCORR_DECL

// The classification in C++ with the same operations, for the global
// histogram path. `l` is the column entry as the pair loop holds it:
// (-2 d_l, rho_l).
__device__ __forceinline__ void cand_classify(const RowV& r, float4 l, const unsigned char* tab, float scale, int n,
                                              float hm, unsigned* code, bool* clean) {
  float pp = __fmul_rn(r.x, l.x);
  pp = __fmaf_rn(r.y, l.y, pp);
  pp = __fmaf_rn(r.z, l.z, pp);
  const float s = __fmaf_rn(l.w, l.w, r.a);
  const float v = __fadd_rn(pp, s);
  *code = table_code(v, tab, scale, n);
  *clean = fabsf(pp) < __fmaf_rn(r.a2r, l.w, hm);
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
  unsigned long long* queue;  // this warp's (j, l) queue (global)
  ExactEntry* xbuf;           // this warp's buffer of uncertain candidates (global)
  const float* e2lo;
  const float* e2hi;
  unsigned char* hist_s;  // this lane's copy of the CTA histogram
  HistOut hist;           // the current item's global histogram
  int qn, xn;
  int nb, cs, ai;  // ai: the anchor's position in the work queue
  float wa;
  unsigned lane, lt_mask;
  unsigned long long n_exact_tri, n_queued, n_flag_rows;
  // Per-anchor bookkeeping, kept here (local memory) rather than in
  // registers the pair loop needs.
  unsigned long long n_exact_pair, n_anchor, n_pairs, n_evals;
};

// Moves the warp's buffered uncertain candidates to the global queue (one
// atomic per 32), or settles them here when the queue is full.
template <bool SURVEY, bool WEIGHTED>
__device__ __noinline__ void cold_flush_exact(Cold& c) {
  const KArgs& a = *c.a;
  if (c.xn == 0) return;
  __syncwarp();
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

// Histogram update of the careful path. The key is the table-scaled code: a
// byte offset into the shared histogram, or a plain bin index for the global
// histogram (HG).
template <bool WEIGHTED, bool HG>
__device__ __forceinline__ void hist_add(unsigned char* hist_s, const HistOut& hist, unsigned key, float w) {
  if (HG) {
    if (WEIGHTED)
      add128(&hist.wsum[2 * key], __float2ll_rn(w));
    else
      atomicAdd(&hist.counts[key], 1ull);
  } else {
    if (WEIGHTED) {
      // The split 64-bit add of the weighted body, in C++.
      unsigned* w32 = reinterpret_cast<unsigned*>(hist_s + key);
      const int wi = __float2int_rn(w);
      const unsigned old = atomicAdd(&w32[0], static_cast<unsigned>(wi));
      const unsigned cy = (old + static_cast<unsigned>(wi)) < old ? 1u : 0u;
      atomicAdd(&w32[1], static_cast<unsigned>(wi >> 31) + cy);
    } else {
      atomicAdd(reinterpret_cast<unsigned*>(hist_s + key), 1u);
    }
  }
}

// Settles the queued candidates, 32 per round: the explicit FP32 band and the
// margin test of the triangle decide most; the rest go to the exact buffer.
template <bool SURVEY, bool WEIGHTED, bool HG>
__device__ __noinline__ void cold_drain(Cold& c) {
  const KArgs& a = *c.a;
  const Geom& g = a.g;
  const int nb = c.nb;
  __syncwarp();
  for (int q0 = 0; q0 < c.qn; q0 += 32) {
    const int qi = q0 + static_cast<int>(c.lane);
    bool exact = false;
    ExactEntry xe;
    if (qi < c.qn) {
      const unsigned long long pr = c.queue[qi];
      const int j = static_cast<int>(pr & 0xffffffffu);
      const int l = static_cast<int>(pr >> 32);
      const float4 ej = c.l2.e[j];
      const unsigned mj = c.l2.m[j];
      const float4 el = c.l3.e[l];
      const unsigned ml = c.l3.m[l];
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
        xe.pj = c.l2.p[j];
        xe.pl = c.l3.p[l];
        xe.meta = (mj >> 8) | ((ml >> 8) << 5) | ((mj & 0xffu) << 10) | ((ml & 0xffu) << 18);
      } else if (code < static_cast<unsigned>(nb)) {
        const float wprod = WEIGHTED ? (c.wa * c.l2.w[j]) * c.l3.w[l] * a.wscale : 0.0f;
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

// Queues the candidates flagged in a group of rows: bit o of the flag word of
// column slot s stands for row jb + o against column lb + 32 s + lane.
template <bool SURVEY, bool WEIGHTED, bool HG>
__device__ __noinline__ void cold_enqueue(Cold& c, int jb, int lb, unsigned q0, unsigned q1, unsigned q2,
                                          unsigned q3) {
  unsigned rows = __reduce_or_sync(0xffffffffu, q0 | q1 | q2 | q3);
  const unsigned q[4] = {q0, q1, q2, q3};
  while (rows) {
    const int o = __ffs(rows) - 1;
    rows &= rows - 1u;
    if (c.qn > kQueueCap - kTile) cold_drain<SURVEY, WEIGHTED, HG>(c);
    ++c.n_flag_rows;
#pragma unroll
    for (int s = 0; s < kReg; ++s) {
      const bool want = (q[s] >> o) & 1u;
      const unsigned bal = __ballot_sync(0xffffffffu, want);
      if (want)
        c.queue[c.qn + __popc(bal & c.lt_mask)] =
            static_cast<unsigned long long>(jb + o) |
            (static_cast<unsigned long long>(lb + 32 * s + static_cast<int>(c.lane)) << 32);
      c.qn += __popc(bal);
      c.n_queued += __popc(bal);
    }
  }
  __syncwarp();
}

// Exact r1^2 of a pair-stage candidate and its bin (or kCodeReject).
static __device__ __noinline__ unsigned cold_pair_exact(const Geom* g, const double* sqr_bins, double4_16a pa,
                                                        double px, double py, double pz) {
  const double r = sqr_sep_exact(pa.x, pa.y, pa.z, px, py, pz, g->fma_pattern);
  return (r < g->sqr_rmax && r > g->sqr_rmin) ? static_cast<unsigned>(exact_bin(r, sqr_bins, g->nb)) : kCodeReject;
}

// Drains the CTA histogram into item `owner - 1`'s global histogram while
// other warps may still be adding to it: each 32-bit word is exchanged with
// zero atomically, so no addition is lost or counted twice. A weighted bin is
// two 32-bit words; taking them one at a time can split one thread's
// low-word and high-word additions between this drain and a later one, but
// the sum over all drains plus what remains is still exact (every carry is
// added to the high word by the thread that caused it).
template <bool WEIGHTED>
__device__ __noinline__ void drain_hist(const KArgs* a, unsigned char* hist_s, int nbin, int copies, unsigned owner,
                                        int t0, int stride) {
  if (owner == 0 || owner == kSlotLocked) return;
  const HistOut out = a->items[owner - 1].hist;
  for (int i = t0; i < nbin; i += stride) {
    if (WEIGHTED) {
      unsigned* h = reinterpret_cast<unsigned*>(hist_s);
      long long v = 0;
      for (int cp = 0; cp < copies; ++cp) {
        const unsigned lo = atomicExch(&h[2 * (cp * nbin + i)], 0u);
        const unsigned hi = atomicExch(&h[2 * (cp * nbin + i) + 1], 0u);
        v += static_cast<long long>((static_cast<unsigned long long>(hi) << 32) | lo);
      }
      if (v) add128(&out.wsum[2 * i], v);
    } else {
      unsigned* h = reinterpret_cast<unsigned*>(hist_s);
      unsigned long long v = 0;
      for (int cp = 0; cp < copies; ++cp) v += atomicExch(&h[cp * nbin + i], 0u);
      if (v) atomicAdd(&out.counts[i], v);
    }
  }
}

template <bool SURVEY, bool SYM, bool WEIGHTED, bool HG>
__global__ void __launch_bounds__(kThreads, 1) k_triangles(KArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ double s_sqr_bins[kMaxEdges];
  __shared__ float s_e2lo[kMaxEdges], s_e2hi[kMaxEdges];
  __shared__ unsigned long long s_slot;  // (owner << 32) | users
  __shared__ unsigned s_since;           // reserved candidates since binding, in units of 2^kSinceShift
  __shared__ int s_next, s_end;          // static schedule: the CTA's remaining range

  const Geom& g = a.g;
  const int nb = g.nb;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const unsigned FULL = 0xffffffffu;
  const unsigned lt_mask = (1u << lane) - 1u;
  if (a.cta_time && tid == 0) {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    a.cta_time[2 * blockIdx.x] = t;
  }
  const SmemLayout L = make_layout(nb, WEIGHTED, HG, a.hist_copies);
  unsigned char* tab = smem + L.table;
  unsigned char* hist_s = smem + L.hist;
  SlotTab& st = reinterpret_cast<SlotTab*>(smem + L.slots)[warp];
  const int nbin = nb * nb * nb;
  const int copies = HG ? 1 : a.hist_copies;
  // This lane's copy of the CTA histogram: lanes that hit one bin in the same
  // instruction spread over the copies.
  const unsigned copy_off = static_cast<unsigned>((lane & (copies - 1)) * nbin * (WEIGHTED ? 8 : 4));
  const int cs = a.code_scale;
  const unsigned nb_cs = static_cast<unsigned>(nb * cs);
  const int group = a.sub_j;

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
    s_slot = 0ull;
    s_since = 0u;
    const long long n = a.n_work, G = gridDim.x, b = blockIdx.x;
    s_next = static_cast<int>(b * n / G);
    s_end = static_cast<int>((b + 1) * n / G);
  }
  __syncthreads();

  // This warp's global slabs.
  const size_t gw = static_cast<size_t>(blockIdx.x) * kWarps + warp;
  ListView l2, l3;
  {
    const size_t stride = static_cast<size_t>(a.kcap2) + a.kcap3;
    const size_t b2 = gw * stride, b3 = b2 + a.kcap2;
    l2.e = a.slab_e + b2;
    l2.m = a.slab_m + b2;
    l2.p = a.slab_p + b2;
    l2.w = a.slab_w ? a.slab_w + b2 : nullptr;
    l3 = l2;
    if (!SYM) {
      l3.e = a.slab_e + b3;
      l3.m = a.slab_m + b3;
      l3.p = a.slab_p + b3;
      l3.w = a.slab_w ? a.slab_w + b3 : nullptr;
    }
  }

  Cold c;
  c.a = a.self;
  c.l2 = l2;
  c.l3 = l3;
  c.queue = a.slab_q + gw * kQueueCap;
  c.xbuf = a.slab_x + gw * 32;
  c.e2lo = s_e2lo;
  c.e2hi = s_e2hi;
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
  c.n_exact_pair = 0;
  c.n_anchor = 0;
  c.n_pairs = 0;
  c.n_evals = 0;

  // Constants of the PTX bodies (addresses in the shared window).
  BodyK bk;
  {
    const unsigned tab_sh = static_cast<unsigned>(__cvta_generic_to_shared(tab));
    bk.tab_adj = tab_sh - 0x4B000000u;
    bk.tab_last = tab_sh + static_cast<unsigned>(g.tab_n - 1);
    bk.nb_cs = nb_cs;
    bk.dummy = static_cast<unsigned>(__cvta_generic_to_shared(smem + L.scratch)) + 8u * lane;
    bk.tscale = g.tab_scale;
    bk.hm = g.hm;
  }
  const unsigned hist_sh = static_cast<unsigned>(__cvta_generic_to_shared(hist_s)) + copy_off;
  const unsigned kj_mul = static_cast<unsigned>(nb * nb * cs);
  unsigned held = 0;  // owner code of the histogram binding this warp holds (0: none)

  for (;;) {
    int w = 0;
    if (lane == 0) {
      if (a.sched_static) {
        w = atomicAdd(&s_next, 1);
        if (w >= s_end) w = a.n_work;
      } else {
        w = atomicAdd(a.work, 1);
      }
    }
    w = __shfl_sync(FULL, w, 0);
    if (static_cast<unsigned>(w) >= static_cast<unsigned>(a.n_work)) break;
    const int item = a.q_item ? a.q_item[w] : 0;
    const unsigned want = static_cast<unsigned>(item) + 1u;
    if (want != held) {
      // Release the old binding, then bind the CTA histogram to this item:
      // join it when it is bound to the item already; rebind it (draining
      // it into its old item) when no warp uses it; otherwise wait.
      if (lane == 0 && held) atomicAdd(&s_slot, ~0ull);
      int got = 0;
      for (int spin = 0; spin < kSlotSpinLimit; ++spin) {
        unsigned old_owner = 0;
        int r = 0;  // 0 wait, 1 joined, 2 locked for rebinding
        if (lane == 0) {
          const unsigned long long cur = atomicAdd(&s_slot, 0ull);
          const unsigned owner = static_cast<unsigned>(cur >> 32), users = static_cast<unsigned>(cur);
          if (owner == want) {
            if (atomicCAS(&s_slot, cur, cur + 1ull) == cur) r = 1;
          } else if (users == 0 && owner != kSlotLocked) {
            if (atomicCAS(&s_slot, cur, static_cast<unsigned long long>(kSlotLocked) << 32) == cur) {
              r = 2;
              old_owner = owner;
            }
          }
        }
        r = __shfl_sync(FULL, r, 0);
        if (r == 1) {
          got = 1;
          break;
        }
        if (r == 2) {
          old_owner = __shfl_sync(FULL, old_owner, 0);
          if (!HG) drain_hist<WEIGHTED>(a.self, hist_s, nbin, copies, old_owner, lane, 32);
          __syncwarp();
          if (lane == 0) {
            s_since = 0u;
            __threadfence_block();
            atomicExch(&s_slot, (static_cast<unsigned long long>(want) << 32) | 1ull);
          }
          got = 1;
          break;
        }
        __nanosleep(512);
      }
      if (!got) {
        // The binding never came free: report and stop this warp.
        if (lane == 0) atomicOr(a.flags, kFlagSchedStall);
        held = 0;
        break;
      }
      held = want;
    }
    const BatchItem& it = a.items[item];
    c.hist = it.hist;
    const bool sym6 = SYM && item_sym6(it);
    const int ai = a.q_anchor ? a.q_anchor[w] : w;
    ++c.n_anchor;
    const double4_16a pa = it.c1.pd[ai];
    const float4 qa = it.c1.pq[ai];
    const int hc = it.c1.pc[ai];
    const int hz = hc % g.nc[2];
    const int hy = (hc / g.nc[2]) % g.nc[1];
    const int hx = hc / (g.nc[2] * g.nc[1]);

    // ---- slots: 27 (cell, image) pairs, order of source/cudaNcorr.cu:37-48
    __syncwarp();  // the previous anchor's readers of the slot table are done
    {
      int n2 = 0, n3 = 0;
      if (lane < 27) {
        const int s = lane;
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
          st.shift[s][d] = sh[d];
          if (ok) {
            const double o_n = __dmul_rn(static_cast<double>(cc[d]), g.cell);
            const double o_h = __dmul_rn(static_cast<double>(h[d]), g.cell);
            st.dof[s][d] = __double2float_rn(__dsub_rn(__dadd_rn(o_n, sh[d]), o_h));
          } else {
            st.dof[s][d] = 0.0f;
          }
        }
        int st2 = ok ? it.c2.start[cell] : 0;
        n2 = ok ? it.c2.count[cell] : 0;
        if (sym6) {
          // Six-fold loop: only neighbours after the anchor in cell order,
          // so the slot's range starts past the anchor's sorted index.
          const int lo = max(st2, ai + 1);
          n2 = max(0, st2 + n2 - lo);
          st2 = lo;
        }
        st.start2[s] = st2;
        if (!SYM) {
          st.start3[s] = ok ? it.c3.start[cell] : 0;
          n3 = ok ? it.c3.count[cell] : 0;
        }
      }
      // Inclusive warp scans of the slot counts give the prefix tables.
      int p2 = n2, p3 = n3;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int t2 = __shfl_up_sync(FULL, p2, o);
        const int t3 = __shfl_up_sync(FULL, p3, o);
        if (lane >= o) {
          p2 += t2;
          p3 += t3;
        }
      }
      if (lane < 27) {
        st.pre2[lane + 1] = p2;
        if (!SYM) st.pre3[lane + 1] = p3;
      }
      if (lane == 0) {
        st.pre2[0] = 0;
        st.pre3[0] = 0;
      }
      __syncwarp();
    }

    // ---- Phase A: neighbour lists (in global memory, this warp's slab)
    auto build = [&](const Catalog& cat, const int* pre, const int* stt, ListView& lv, int cap) -> int {
      const int total = pre[27];
      const int rounded = (total + 31) & ~31;
      int cnt = 0;
      // Software pipeline: the next round's point is loaded before this
      // round's is classified, so two loads are in flight per thread.
      int sn = 0, jn = 0;
      float4 qn = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      if (lane < total) {
        while (lane >= pre[sn + 1]) ++sn;
        jn = stt[sn] + (lane - pre[sn]);
        qn = cat.pq[jn];
      }
      for (int base = 0; base < rounded; base += 32) {
        const int item_i = base + lane;
        const int s = sn, j = jn;
        const float4 q = qn;
        const int next = item_i + 32;
        if (next < total) {
          while (next >= pre[sn + 1]) ++sn;
          jn = stt[sn] + (next - pre[sn]);
          qn = cat.pq[jn];
        }
        bool acc = false;
        float4 ent;
        unsigned meta = 0;
        float wv = 0.0f;
        if (item_i < total) {
          // Cell-local FP32 prefilter: skip candidates certainly out of range.
          const float fx = (q.x - qa.x) + st.dof[s][0];
          const float fy = (q.y - qa.y) + st.dof[s][1];
          const float fz = (q.z - qa.z) + st.dof[s][2];
          const float vp = fmaf(fz, fz, fmaf(fy, fy, fx * fx));
          if (vp < g.pre_hi && vp > g.pre_lo && (!sym6 || j > ai)) {
            // Exact anchor-relative offset of the image (FP64), rounded once.
            const double4_16a p = cat.pd[j];
            const double px = __dadd_rn(p.x, st.shift[s][0]);
            const double py = __dadd_rn(p.y, st.shift[s][1]);
            const double pz = __dadd_rn(p.z, st.shift[s][2]);
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
              ++c.n_exact_pair;
              code = cold_pair_exact(&a.self->g, s_sqr_bins, pa, px, py, pz);
            }
            if (code < static_cast<unsigned>(nb)) {
              acc = true;
              ent = make_float4(dx, dy, dz, __fsqrt_rn(v));
              meta = code | (static_cast<unsigned>(s) << 8);
              wv = q.w;
            }
          }
        }
        const unsigned bal = __ballot_sync(FULL, acc);
        if (acc) {
          const int e = cnt + __popc(bal & lt_mask);
          if (e < cap) {
            lv.e[e] = ent;
            lv.m[e] = meta;
            lv.p[e] = j;
            if (WEIGHTED) lv.w[e] = wv;
          } else {
            atomicOr(a.flags, kFlagListOverflow);
          }
        }
        cnt += __popc(bal);
      }
      return min(cnt, cap);
    };
    const int k2 = build(it.c2, st.pre2, st.start2, l2, a.kcap2);
    const int k3 = SYM ? k2 : build(it.c3, st.pre3, st.start3, l3, a.kcap3);
    __syncwarp();  // the lists written by all lanes are visible to all lanes
    {
      const unsigned long long pairs_here = SYM ? static_cast<unsigned long long>(k2) * (k2 > 0 ? k2 - 1 : 0) / 2
                                                : static_cast<unsigned long long>(k2) * k3;
      if (lane == 0) {
        c.n_pairs += pairs_here;
        if (a.cell_work) atomicAdd(&a.cell_work[it.cell_base + hc], pairs_here);
        c.n_evals += static_cast<unsigned long long>(st.pre2[27]) +
                     (SYM ? 0ull : static_cast<unsigned long long>(st.pre3[27]));
      }
    }
    const float wa = static_cast<float>(pa.w);
    c.ai = w;
    c.wa = wa;
    const float wsc = a.wscale;

    // ---- Phase B: column tiles of 128 against every row that pairs with them
    const int nt = (k3 + kTile - 1) / kTile;
    for (int lt = 0; lt < nt; ++lt) {
      const int lb = lt * kTile;
      // Rows of this tile: SYM pairs l < j (rows from the tile start on),
      // otherwise all rows.
      const int jfirst = SYM ? lb : 0;
      if (jfirst >= k2) break;
      // Reserve this tile's candidates; the warp that crosses a multiple of
      // 2^30 drains the histogram (its 32-bit counts stay below 2^32).
      {
        const unsigned long long slots = static_cast<unsigned long long>(k2 - jfirst) * kTile;
        const unsigned units = static_cast<unsigned>((slots >> kSinceShift) + 1);
        unsigned old = 0;
        if (lane == 0) old = atomicAdd(&s_since, units);
        old = __shfl_sync(FULL, old, 0);
        if (!HG && (old >> kSinceDrainBits) != ((old + units) >> kSinceDrainBits))
          drain_hist<WEIGHTED>(a.self, hist_s, nbin, copies, held, lane, 32);
      }
      // Columns are held as (-2 d_l, rho_l); the padding (0, rho = 1e18)
      // gives v = 1e36 and is rejected by the table for every row.
      ColV col;
      float wl[kReg];
#pragma unroll
      for (int r = 0; r < kReg; ++r) {
        const int l = lb + r * 32 + lane;
        if (l < k3) {
          const float4 e = l3.e[l];
          col.l[r] = make_float4(-2.0f * e.x, -2.0f * e.y, -2.0f * e.z, e.w);
          col.k[r] = (l3.m[l] & 0xffu) * nb_cs;
          wl[r] = WEIGHTED ? l3.w[l] : 0.0f;
        } else {
          col.l[r] = make_float4(0.0f, 0.0f, 0.0f, 1.0e18f);
          col.k[r] = 0;
          wl[r] = 0.0f;
        }
      }
      auto make_row = [&](float4 e, unsigned m) {
        RowV r;
        r.x = e.x;
        r.y = e.y;
        r.z = e.z;
        r.a = __fmul_rn(e.w, e.w);
        r.a2r = 2.0f * e.w;
        r.key = HG ? (m & 0xffu) * kj_mul : (m & 0xffu) * kj_mul + hist_sh;
        return r;
      };
      // Weighted and global-histogram rows: one candidate at a time, each
      // with its mask (diagonal rows; 1 elsewhere).
      auto row_slow = [&](const RowV& r, float wj, unsigned rbit, const unsigned (&m)[kReg], unsigned& q0,
                          unsigned& q1, unsigned& q2, unsigned& q3) {
        auto one = [&](auto s_tag, unsigned& q) {
          constexpr int S = decltype(s_tag)::value;
          const unsigned ins = m[S];
          if (HG) {
            unsigned code;
            bool clean;
            cand_classify(r, col.l[S], tab, g.tab_scale, g.tab_n, bk.hm, &code, &clean);
            const bool ok = code < nb_cs && ins;
            const bool careful = (code == kCodeCareful || (code < nb_cs && !clean)) && ins;
            if (ok && clean)
              hist_add<WEIGHTED, true>(hist_s, c.hist, r.key + col.k[S] + code, (wa * wj * wsc) * wl[S]);
            if (careful) q |= rbit;
          } else if (WEIGHTED) {
            cand_wsum<true>(r, col.l[S], col.k[S], ins, bk, wa * wj * wsc, wl[S], rbit, q);
          }
        };
        one(std::integral_constant<int, 0>(), q0);
        one(std::integral_constant<int, 1>(), q1);
        one(std::integral_constant<int, 2>(), q2);
        one(std::integral_constant<int, 3>(), q3);
      };
      // Rows [jb, je) of one flag group, all of one kind: full rows, or
      // diagonal rows (SYM: rows of the column tile itself, whose slot
      // S = (j - lb) / 32 is masked by l < j and the slots above it empty).
      auto rows = [&](int jb, int je, auto diag_tag, unsigned& q0, unsigned& q1, unsigned& q2, unsigned& q3) {
        constexpr bool DIAG = decltype(diag_tag)::value;
        const int S = (jb - lb) >> 5;  // diagonal rows: the row's own slot (uniform in the group)
        float4 en = l2.e[jb];
        unsigned mn = l2.m[jb];
#pragma unroll(DIAG ? 1 : 2)
        for (int j = jb; j < je; ++j) {
          const float4 e = en;
          const unsigned m = mn;
          const int jn = min(j + 1, k2 - 1);
          en = l2.e[jn];
          mn = l2.m[jn];
          const RowV r = make_row(e, m);
          const unsigned rbit = 1u << (j - jb);
          unsigned mk[kReg] = {1u, 1u, 1u, 1u};
          if (DIAG) {
            const unsigned in = ((j - lb) & 31) > lane ? 1u : 0u;
#pragma unroll
            for (int s = 0; s < kReg; ++s) mk[s] = s < S ? 1u : (s == S ? in : 0u);
          }
          if (WEIGHTED || HG) {
            const float wj = WEIGHTED ? l2.w[j] : 0.0f;
            row_slow(r, wj, rbit, mk, q0, q1, q2, q3);
          } else if (!DIAG) {
            row_full4(r, col, bk, rbit, q0, q1, q2, q3);
          } else if (S < 2) {
            row_mask2(r, col, bk, rbit, mk[0], mk[1], q0, q1, q2, q3);
          } else {
            row_mask4(r, col, bk, rbit, mk[0], mk[1], mk[2], mk[3], q0, q1, q2, q3);
          }
        }
      };
      // Groups of `group` rows (8, 16 or 32, so a group never straddles a
      // 32-row slot boundary of the diagonal); after each, the flagged
      // candidates are queued.
#pragma unroll 1
      for (int jb = jfirst; jb < k2; jb += group) {
        const int je = min(jb + group, k2);
        unsigned q0 = 0, q1 = 0, q2 = 0, q3 = 0;
        if (!SYM || jb >= lb + kTile)
          rows(jb, je, std::false_type(), q0, q1, q2, q3);
        else
          rows(jb, je, std::true_type(), q0, q1, q2, q3);
        if (__any_sync(FULL, (q0 | q1 | q2 | q3) != 0))
          cold_enqueue<SURVEY, WEIGHTED, HG>(c, jb, lb, q0, q1, q2, q3);
      }
    }
    // Queue entries refer to this anchor's lists: settle them now.
    if (c.qn > 0) cold_drain<SURVEY, WEIGHTED, HG>(c);
  }
  if (lane == 0 && held) atomicAdd(&s_slot, ~0ull);
  cold_flush_exact<SURVEY, WEIGHTED>(c);
  __syncthreads();
  if (a.cta_time && tid == 0) {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    a.cta_time[2 * blockIdx.x + 1] = t;
  }
  if (!HG) {
    // Every warp has left: drain what the CTA histogram holds.
    const unsigned owner = static_cast<unsigned>(s_slot >> 32);
    drain_hist<WEIGHTED>(a.self, hist_s, nbin, copies, owner, tid, kThreads);
  }
  if (a.stats) {
    atomicAdd(&a.stats[0], c.n_exact_tri);
    atomicAdd(&a.stats[1], c.n_exact_pair);
    if (lane == 0) {
      atomicAdd(&a.stats[2], c.n_anchor);
      atomicAdd(&a.stats[3], c.n_pairs);
      atomicAdd(&a.stats[4], c.n_evals);
      atomicAdd(&a.stats[5], c.n_flag_rows);
      atomicAdd(&a.stats[6], c.n_queued);
    }
  }
}

}  // namespace ncorr_gb300
