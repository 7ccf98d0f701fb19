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

// Ring of points that passed the prefilter of the list build, per warp.
constexpr unsigned kRing = 64;

// Per-warp slot table of the anchor being listed (shared memory).
struct SlotTab {
  double shift[27][3];  // image shift of the slot (0 or +-box per axis)
  float dof[27][3];     // FP32 offset of the slot's cell origin from the home cell's
  int start2[27], pre2[28], start3[27], pre3[28];
  int ring_j[kRing];              // pending points: index in the catalogue
  unsigned char ring_s[kRing];    // and slot
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
  if (!hist_global) o = align16(o + hist_copies * hist_words(nb) * (weighted ? 8 : 4));
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
  // for p3; kcap3 = 0 when p2 == p3; the kListPad entries past a list hold
  // padding rows) with their weights, careful queue, exact buffer.
  ListEnt* slab_e;
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
  ListEnt* v;
  float* w;
};

// The margin form of the triangle test. List entries keep rho = sqrt_rn of
// their r^2 estimate (as rho^2 = fmul_rn(rho, rho) and 2 rho); with
// a = rho_j^2 and b = rho_l^2 (the product formed inside the FMA) a candidate
// of third side v is certainly kept by
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
// sides). Every candidate whose margin test holds is added at the address its
// table code gives: its bin when the code is one, else one of the two sink
// bins that end each (bin_j, bin_l) row of the CTA histogram (rejected,
// careful), which nothing reads. So the body never tests the code for
// "reject". A candidate whose code is "careful" or whose margin test fails
// sets `rbit` (its row's bit in the flag group) in the lane's flag word; a
// rejected one that fails the margin test (a nearly collinear triangle, rare)
// is flagged too and the careful path rejects it again. The histogram
// reduction is unconditional: a candidate that does not count adds to the
// lane's own scratch word `dummy` instead, which keeps the loop free of the
// branch a predicated atomic compiles to.
//
// Operands of the row bodies:
//   %0     the flag word of the row group (in/out)
//   %1-%3  the row's offset d_j, %4 rho_j^2, %5 2 rho_j, %6 the row's key
//          (histogram base + bin_j times its stride)
//   %7 table scale, %8/%9 table address bias and last entry, %10 the careful
//   code, %11 -M, %12 dummy address, %13 rbit
//   column c: %(14+5c)-%(16+5c) its offset scaled by -2, %(17+5c) rho_l,
//   %(18+5c) its key (bin_l times its stride)
//   %19 (one-column bodies) the mask: 0 for a pair that is not to be counted
// One asm statement per row lets all table loads issue before the first
// reduction; in separate statements each load would wait behind the previous
// candidate's reduction, which may touch the same shared-memory word as far
// as the compiler can tell.
#define NCORR_DECL(C)                                                     \
  ".reg .f32 pp" #C ", s" #C ", v" #C ", t" #C ", H" #C ";\n\t"           \
  ".reg .b32 y" #C ", ia" #C ", code" #C ", key" #C ", adr" #C ";\n\t"     \
  ".reg .pred upd" #C ", w" #C ";\n\t"
#define NCORR_CLS(C, LX, LY, LZ, B)                  \
  "mul.rn.f32 pp" #C ", %1, " LX ";\n\t"             \
  "fma.rn.f32 pp" #C ", %2, " LY ", pp" #C ";\n\t"   \
  "fma.rn.f32 pp" #C ", %3, " LZ ", pp" #C ";\n\t"   \
  "fma.rn.f32 s" #C ", " B ", " B ", %4;\n\t"        \
  "add.rn.f32 v" #C ", pp" #C ", s" #C ";\n\t"       \
  "fma.rn.f32 y" #C ", v" #C ", %7, 0f4B000000;\n\t" \
  "add.u32 ia" #C ", y" #C ", %8;\n\t"               \
  "min.u32 ia" #C ", ia" #C ", %9;\n\t"              \
  "ld.shared.u8 code" #C ", [ia" #C "];\n\t"
// Column operand groups, expanded through NCORR_CLSX so that a group fills
// the four column arguments of NCORR_CLS.
#define NCORR_CLS_I(C, ...) NCORR_CLS(C, __VA_ARGS__)
#define NCORR_CLSX(C, COLS) NCORR_CLS_I(C, COLS)
#define NCORR_KEY(C, KL)                               \
  "add.u32 key" #C ", %6, " KL ";\n\t"                 \
  "add.u32 key" #C ", key" #C ", code" #C ";\n\t"      \
  "selp.b32 adr" #C ", key" #C ", %12, upd" #C ";\n\t"
// upd: the margin test holds; w: careful code or failed margin test.
#define NCORR_UPD(C, B, KL)                                        \
  "abs.f32 t" #C ", pp" #C ";\n\t"                                 \
  "fma.rn.f32 H" #C ", %5, " B ", %11;\n\t"                        \
  "setp.lt.f32 upd" #C ", t" #C ", H" #C ";\n\t"                   \
  "setp.eq.or.u32 w" #C ", code" #C ", %10, !upd" #C ";\n\t" NCORR_KEY(C, KL)
// The same under a mask: a masked-out pair neither counts nor flags.
#define NCORR_UPD_MASKED(C, B, KL, M)                              \
  "abs.f32 t" #C ", pp" #C ";\n\t"                                 \
  "fma.rn.f32 H" #C ", %5, " B ", %11;\n\t"                        \
  "setp.ne.u32 inp, " M ", 0;\n\t"                                 \
  "setp.lt.and.f32 upd" #C ", t" #C ", H" #C ", inp;\n\t"          \
  "setp.eq.or.u32 w" #C ", code" #C ", %10, !upd" #C ";\n\t"       \
  "and.pred w" #C ", w" #C ", inp;\n\t" NCORR_KEY(C, KL)
#define NCORR_FLAG "@w0 or.b32 %0, %0, %13;\n\t"
#define NCORR_RED(C) "red.shared.add.u32 [adr" #C "], 1;\n\t"
#define NCORR_C0 "%14", "%15", "%16", "%17"
#define NCORR_C1 "%19", "%20", "%21", "%22"
#define NCORR_C2 "%24", "%25", "%26", "%27"
#define NCORR_C3 "%29", "%30", "%31", "%32"
#define NCORR_ROW_OPERANDS                                                                                      \
  : "+r"(q)                                                                                                    \
  : "f"(r.x), "f"(r.y), "f"(r.z), "f"(r.a), "f"(r.a2r), "r"(r.key), "f"(k.tscale), "r"(k.tab_adj),             \
    "r"(k.tab_last), "r"(k.car), "f"(k.hm), "r"(k.dummy), "r"(rbit), "f"(c.l[0].x), "f"(c.l[0].y),             \
    "f"(c.l[0].z), "f"(c.l[0].w), "r"(c.k[0]), "f"(c.l[1].x), "f"(c.l[1].y), "f"(c.l[1].z), "f"(c.l[1].w),    \
    "r"(c.k[1]), "f"(c.l[2].x), "f"(c.l[2].y), "f"(c.l[2].z), "f"(c.l[2].w), "r"(c.k[2]), "f"(c.l[3].x),        \
    "f"(c.l[3].y), "f"(c.l[3].z), "f"(c.l[3].w), "r"(c.k[3])                                                   \
  : "memory"

// Constants of the candidate bodies, fixed per launch.
struct BodyK {
  float tscale, hm;
  unsigned tab_adj, tab_last, car, dummy, nb_cs;
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

// Column slots 0..N-1 of one row, every pair one to count: N = 4 for the
// rows past the diagonal tile (and every row of distinct lists), N = 1..3 for
// the rows of the diagonal tile's block N against the blocks before it.
template <int N>
__device__ __forceinline__ void row_full(const RowV& r, const ColV& c, const BodyK& k, unsigned rbit, unsigned& q) {
  if constexpr (N == 4) {
    asm volatile("{\n\t" NCORR_DECL(0) NCORR_DECL(1) NCORR_DECL(2) NCORR_DECL(3)
                 NCORR_CLSX(0, NCORR_C0) NCORR_CLSX(1, NCORR_C1) NCORR_CLSX(2, NCORR_C2) NCORR_CLSX(3, NCORR_C3)
                 NCORR_UPD(0, "%17", "%18") NCORR_UPD(1, "%22", "%23") NCORR_UPD(2, "%27", "%28")
                 NCORR_UPD(3, "%32", "%33")
                 "or.pred w0, w0, w1;\n\tor.pred w2, w2, w3;\n\tor.pred w0, w0, w2;\n\t" NCORR_FLAG
                 NCORR_RED(0) NCORR_RED(1) NCORR_RED(2) NCORR_RED(3) "}" NCORR_ROW_OPERANDS);
  } else if constexpr (N == 3) {
    asm volatile("{\n\t" NCORR_DECL(0) NCORR_DECL(1) NCORR_DECL(2)
                 NCORR_CLSX(0, NCORR_C0) NCORR_CLSX(1, NCORR_C1) NCORR_CLSX(2, NCORR_C2)
                 NCORR_UPD(0, "%17", "%18") NCORR_UPD(1, "%22", "%23") NCORR_UPD(2, "%27", "%28")
                 "or.pred w0, w0, w1;\n\tor.pred w0, w0, w2;\n\t" NCORR_FLAG
                 NCORR_RED(0) NCORR_RED(1) NCORR_RED(2) "}" NCORR_ROW_OPERANDS);
  } else if constexpr (N == 2) {
    asm volatile("{\n\t" NCORR_DECL(0) NCORR_DECL(1) NCORR_CLSX(0, NCORR_C0) NCORR_CLSX(1, NCORR_C1)
                 NCORR_UPD(0, "%17", "%18") NCORR_UPD(1, "%22", "%23")
                 "or.pred w0, w0, w1;\n\t" NCORR_FLAG NCORR_RED(0) NCORR_RED(1) "}" NCORR_ROW_OPERANDS);
  } else {
    static_assert(N == 1, "one to four column slots");
    asm volatile("{\n\t" NCORR_DECL(0) NCORR_CLSX(0, NCORR_C0) NCORR_UPD(0, "%17", "%18") NCORR_FLAG
                 NCORR_RED(0) "}" NCORR_ROW_OPERANDS);
  }
}

// One candidate under a mask, with a row of its own per lane: the pairs of a
// diagonal 32-block, taken by rotation (column lane against row lane + d).
__device__ __forceinline__ void row_rot1(const RowV& r, const float4& l, unsigned kl, const BodyK& k, unsigned rbit,
                                         unsigned mask, unsigned& q) {
  asm volatile("{\n\t.reg .pred inp;\n\t" NCORR_DECL(0) NCORR_CLSX(0, NCORR_C0)
               NCORR_UPD_MASKED(0, "%17", "%18", "%19") NCORR_FLAG NCORR_RED(0) "}"
               : "+r"(q)
               : "f"(r.x), "f"(r.y), "f"(r.z), "f"(r.a), "f"(r.a2r), "r"(r.key), "f"(k.tscale), "r"(k.tab_adj),
                 "r"(k.tab_last), "r"(k.car), "f"(k.hm), "r"(k.dummy), "r"(rbit), "f"(l.x), "f"(l.y), "f"(l.z),
                 "f"(l.w), "r"(kl), "r"(mask)
               : "memory");
}

// The same without a mask (a full diagonal block, d < 16).
__device__ __forceinline__ void row_rot1_full(const RowV& r, const float4& l, unsigned kl, const BodyK& k,
                                              unsigned rbit, unsigned& q) {
  asm volatile("{\n\t" NCORR_DECL(0) NCORR_CLSX(0, NCORR_C0) NCORR_UPD(0, "%17", "%18") NCORR_FLAG NCORR_RED(0) "}"
               : "+r"(q)
               : "f"(r.x), "f"(r.y), "f"(r.z), "f"(r.a), "f"(r.a2r), "r"(r.key), "f"(k.tscale), "r"(k.tab_adj),
                 "r"(k.tab_last), "r"(k.car), "f"(k.hm), "r"(k.dummy), "r"(rbit), "f"(l.x), "f"(l.y), "f"(l.z),
                 "f"(l.w), "r"(kl)
               : "memory");
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
// entry, %16 the careful code, %17 -M, %18 dummy, %19 row weight, %20 column
// weight, %21 rbit, %22 nb * code scale. Unlike the count bodies, only a
// candidate with a bin code adds into the histogram; the others add to the
// lane's scratch word. Rejected candidates are common, and their returning,
// per-lane-valued atomics on the few reject-sink words would serialize.
__device__ __forceinline__ void cand_wsum(const RowV& r, const float4& l, unsigned kl, unsigned in, const BodyK& k,
                                          float wrow, float wl, unsigned rbit, unsigned& q) {
  asm volatile("{\n\t.reg .pred inp, ok, nmg;\n\t" NCORR_DECL(0)
               ".reg .f32 wp;\n\t.reg .b32 wi, whi, wold, wnew, wcy, adrh;\n\t"
               "mul.rn.f32 pp0, %1, %6;\n\t"
               "fma.rn.f32 pp0, %2, %7, pp0;\n\t"
               "fma.rn.f32 pp0, %3, %8, pp0;\n\t"
               "fma.rn.f32 s0, %9, %9, %4;\n\t"
               "add.rn.f32 v0, pp0, s0;\n\t"
               "fma.rn.f32 y0, v0, %13, 0f4B000000;\n\t"
               "add.u32 ia0, y0, %14;\n\t"
               "min.u32 ia0, ia0, %15;\n\t"
               "ld.shared.u8 code0, [ia0];\n\t"
               "abs.f32 t0, pp0;\n\t"
               "fma.rn.f32 H0, %5, %9, %17;\n\t"
               "setp.ne.u32 inp, %12, 0;\n\t"
               "setp.lt.u32 ok, code0, %22;\n\t"
               "and.pred ok, ok, inp;\n\t"
               "setp.lt.and.f32 upd0, t0, H0, ok;\n\t"
               "setp.ge.and.f32 nmg, t0, H0, ok;\n\t"
               "setp.eq.or.u32 w0, code0, %16, nmg;\n\t"
               "and.pred w0, w0, inp;\n\t"
               "@w0 or.b32 %0, %0, %21;\n\t"
               "add.u32 key0, %10, %11;\n\t"
               "add.u32 key0, key0, code0;\n\t"
               "selp.b32 adr0, key0, %18, upd0;\n\t"
               "mul.rn.f32 wp, %19, %20;\n\t"
               "cvt.rni.s32.f32 wi, wp;\n\t"
               "shr.s32 whi, wi, 31;\n\t"
               "atom.shared.add.u32 wold, [adr0], wi;\n\t"
               "add.u32 wnew, wold, wi;\n\t"
               "set.lt.u32.u32 wcy, wnew, wold;\n\t"
               "sub.u32 whi, whi, wcy;\n\t"
               "add.u32 adrh, adr0, 4;\n\t"
               "red.shared.add.u32 [adrh], whi;\n\t"
               "}"
               : "+r"(q)
               : "f"(r.x), "f"(r.y), "f"(r.z), "f"(r.a), "f"(r.a2r), "f"(l.x), "f"(l.y), "f"(l.z), "f"(l.w),
                 "r"(r.key), "r"(kl), "r"(in), "f"(k.tscale), "r"(k.tab_adj), "r"(k.tab_last), "r"(k.car),
                 "f"(k.hm), "r"(k.dummy), "f"(wrow), "f"(wl), "r"(rbit), "r"(k.nb_cs)
               : "memory");
}

#undef NCORR_ROW_OPERANDS
#undef NCORR_C0
#undef NCORR_C1
#undef NCORR_C2
#undef NCORR_C3
#undef NCORR_RED
#undef NCORR_FLAG
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
  unsigned long long* queue;  // this warp's careful queue (global)
  ExactEntry* xbuf;           // this warp's buffer of uncertain candidates (global)
  const float* e2lo;
  const float* e2hi;
  const unsigned char* tab;  // the bin table (shared memory)
  unsigned char* hist_s;     // this lane's copy of the CTA histogram
  HistOut hist;           // the current item's global histogram
  int xn;
  int nb, cs, ai;  // ai: the anchor's position in the work queue
  // Histogram strides of bin_j and bin_l: bytes in the CTA histogram (with
  // its sink bins), bins in the global one.
  unsigned kjm, klm;
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
// Drops the L2 lines of [p, p + bytes) without writing them back (the warp's
// lanes take a line each). A warp's lists are dead once its anchor is done
// and are rewritten before they are read again; left in L2, the next
// anchors' traffic evicts them and they are written back to DRAM for
// nothing. Skipped unless p is 128-byte aligned (the line size).
__device__ __forceinline__ void discard_l2(const void* p, size_t bytes, int lane) {
  const char* c = static_cast<const char*>(p);
  if (reinterpret_cast<uintptr_t>(c) & 127u) return;
  for (size_t off = static_cast<size_t>(lane) * 128; off < bytes; off += 32 * 128)
    asm volatile("discard.global.L2 [%0], 128;" ::"l"(c + off) : "memory");
}

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

// Careful queue entries: a lane's flag word of one row group in the high
// half, and in the low half  base << 8 | kind << 5 | lane.
//   kind n < 4: bit o is row base + o against column slots 0..n of the tile
//               at lb, that is columns lb + 32 s + lane;
//   kind 4:     the diagonal block at base; bit d - 1 is row
//               base + ((lane + d) & 31) against column base + lane.
constexpr unsigned kKindRot = 4;

// Settles the careful queue's entries of the tile at lb, one candidate per
// lane and round: the explicit FP32 band and the margin test of the triangle
// decide most; the rest go to the exact buffer. Flagged columns at or past
// k3 (the padding of the last tile) are skipped.
template <bool SURVEY, bool WEIGHTED, bool HG>
__device__ __noinline__ void cold_drain(Cold& c, int lb, int k3, int qn) {
  const KArgs& a = *c.a;
  const Geom& g = a.g;
  const int nb = c.nb;
  __syncwarp();
  for (int e0 = 0; e0 < qn; e0 += 32) {
    const int ei = e0 + static_cast<int>(c.lane);
    unsigned bits = 0, tag = 0;
    if (ei < qn) {
      const unsigned long long en = c.queue[ei];
      bits = static_cast<unsigned>(en >> 32);
      tag = static_cast<unsigned>(en);
      c.n_flag_rows += static_cast<unsigned>(__popc(bits));
    }
    const unsigned kind = (tag >> 5) & 7u, el_lane = tag & 31u;
    const int base = static_cast<int>(tag >> 8);
    const int nsl = kind == kKindRot ? 1 : static_cast<int>(kind) + 1;
    int s = 0;
    while (__any_sync(0xffffffffu, bits != 0u)) {
      bool exact = false;
      ExactEntry xe;
      if (bits) {
        const int o = __ffs(bits) - 1;
        int j, l;
        if (kind == kKindRot) {
          j = base + static_cast<int>((el_lane + static_cast<unsigned>(o) + 1u) & 31u);
          l = base + static_cast<int>(el_lane);
        } else {
          j = base + o;
          l = lb + 32 * s + static_cast<int>(el_lane);
        }
        if (++s == nsl) {
          s = 0;
          bits &= bits - 1u;
        }
        const ListEnt& ejv = c.l2.v[j];
        const ListEnt& elv = c.l3.v[min(l, k3 - 1)];
        const float4 ej = ejv.e, el = elv.e;
        const float a2rj = ejv.a2r;
        const float rhol = 0.5f * elv.a2r;
        // A row's bit stands for all its column slots: keep the candidates
        // the body itself flagged (its classification, recomputed with the
        // same operations), not the ones it counted or rejected.
        bool flagged = l < k3;
        if (flagged && kind != kKindRot) {
          RowV r;
          r.x = ej.x;
          r.y = ej.y;
          r.z = ej.z;
          r.a = ej.w;
          r.a2r = a2rj;
          r.key = 0;
          const float4 lc = make_float4(-2.0f * el.x, -2.0f * el.y, -2.0f * el.z, rhol);
          unsigned bc;
          bool clean;
          cand_classify(r, lc, c.tab, g.tab_scale, g.tab_n, g.hm, &bc, &clean);
          const unsigned car = table_code_careful(nb, c.cs);
          flagged = bc == car || (!clean && (!HG || bc < static_cast<unsigned>(nb * c.cs)));
        }
        if (flagged) {
          ++c.n_queued;
          const unsigned mj = ejv.m;
          const unsigned ml = elv.m;
          const float dx = ej.x - el.x, dy = ej.y - el.y, dz = ej.z - el.z;
          const float v = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
          unsigned code = careful_code(v, c.e2lo, c.e2hi, nb, g.ka, g.kb);
          if (code < static_cast<unsigned>(nb)) {
            if (!heron_clean(v, ej.w, a2rj, rhol, g.hm)) code = kCodeExact;
          }
          if (code == kCodeExact) {
            ++c.n_exact_tri;
            exact = true;
            xe.ai = c.ai;
            xe.pj = ejv.p;
            xe.pl = elv.p;
            xe.meta = (mj >> 8) | ((ml >> 8) << 5) | ((mj & 0xffu) << 10) | ((ml & 0xffu) << 18);
          } else if (code < static_cast<unsigned>(nb)) {
            const float wprod = WEIGHTED ? (c.wa * c.l2.w[j]) * c.l3.w[l] * a.wscale : 0.0f;
            const unsigned key = (mj & 0xffu) * c.kjm + (ml & 0xffu) * c.klm + code * static_cast<unsigned>(c.cs);
            hist_add<WEIGHTED, HG>(c.hist_s, c.hist, key, wprod);
          }
        }
      }
      const unsigned xbal = __ballot_sync(0xffffffffu, exact);
      if (c.xn + __popc(xbal) > 32) cold_flush_exact<SURVEY, WEIGHTED>(c);
      if (exact) c.xbuf[c.xn + __popc(xbal & c.lt_mask)] = xe;
      c.xn += __popc(xbal);
      __syncwarp();
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
// added to the high word by the thread that caused it). Bin i of the global
// histogram is word (i / nb) * (nb + 2) + i % nb of a copy; the sink bins are
// left alone (their values are never used, so wrapping is harmless).
template <bool WEIGHTED>
__device__ __noinline__ void drain_hist(const KArgs* a, unsigned char* hist_s, int nb, int copies, unsigned owner,
                                        int t0, int stride) {
  if (owner == 0 || owner == kSlotLocked) return;
  const HistOut out = a->items[owner - 1].hist;
  const int nbin = nb * nb * nb, nbp = hist_words(nb);
  for (int i = t0; i < nbin; i += stride) {
    const int pi = (i / nb) * hist_row(nb) + i % nb;
    if (WEIGHTED) {
      unsigned* h = reinterpret_cast<unsigned*>(hist_s);
      long long v = 0;
      for (int cp = 0; cp < copies; ++cp) {
        const unsigned lo = atomicExch(&h[2 * (cp * nbp + pi)], 0u);
        const unsigned hi = atomicExch(&h[2 * (cp * nbp + pi) + 1], 0u);
        v += static_cast<long long>((static_cast<unsigned long long>(hi) << 32) | lo);
      }
      if (v) add128(&out.wsum[2 * i], v);
    } else {
      unsigned* h = reinterpret_cast<unsigned*>(hist_s);
      unsigned long long v = 0;
      for (int cp = 0; cp < copies; ++cp) v += atomicExch(&h[cp * nbp + pi], 0u);
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
  const int nbp = hist_words(nb);  // words of one copy of the CTA histogram, sinks included
  const int copies = HG ? 1 : a.hist_copies;
  // This lane's copy of the CTA histogram: lanes that hit one bin in the same
  // instruction spread over the copies.
  const unsigned copy_off = static_cast<unsigned>((lane & (copies - 1)) * nbp * (WEIGHTED ? 8 : 4));
  const int cs = a.code_scale;
  const unsigned nb_cs = static_cast<unsigned>(nb * cs);
  const unsigned car = table_code_careful(nb, cs);
  const int group = a.sub_j;

  for (int i = tid; i <= nb; i += kThreads) {
    s_sqr_bins[i] = g.sqr_bins[i];
    s_e2lo[i] = g.e2lo[i];
    s_e2hi[i] = g.e2hi[i];
  }
  for (int i = tid; i < g.tab_n; i += kThreads) tab[i] = a.table[i];
  if (!HG) {
    for (int i = tid; i < nbp * copies; i += kThreads) {
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
    l2.v = a.slab_e + b2;
    l2.w = a.slab_w ? a.slab_w + b2 : nullptr;
    l3 = l2;
    if (!SYM) {
      l3.v = a.slab_e + b3;
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
  c.tab = tab;
  c.hist_s = hist_s + copy_off;
  c.hist.counts = nullptr;
  c.hist.wsum = nullptr;
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
    bk.car = car;
    bk.nb_cs = nb_cs;
    bk.dummy = static_cast<unsigned>(__cvta_generic_to_shared(smem + L.scratch)) + 8u * lane;
    bk.tscale = g.tab_scale;
    bk.hm = g.hm;
  }
  const unsigned hist_sh = static_cast<unsigned>(__cvta_generic_to_shared(hist_s)) + copy_off;
  // Strides of bin_l and bin_j: the CTA histogram's rows of nb + 2 bins
  // (bytes), or the global histogram's nb (bins).
  const unsigned kl_mul = HG ? static_cast<unsigned>(nb) : static_cast<unsigned>(hist_row(nb) * cs);
  const unsigned kj_mul = static_cast<unsigned>(nb) * kl_mul;
  c.kjm = kj_mul;
  c.klm = kl_mul;
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
          if (!HG) drain_hist<WEIGHTED>(a.self, hist_s, nb, copies, old_owner, lane, 32);
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

    // ---- Phase A: neighbour lists (in global memory, this warp's slab). A
    // list holds at most cap - kListPad entries; the kListPad entries after
    // its last one are padding rows. The slots' points stream past in rounds
    // of 32 (each round's cell-local FP32 points loaded two rounds ahead); a
    // prefilter drops those certainly out of range and puts the others in
    // the warp's ring of pending points. Whenever 32 are pending they are
    // settled one per lane: 32 independent FP64 position loads in flight at
    // once, then the exact offset, its classification and the append to the
    // list.
    auto build = [&](const Catalog& cat, const int* pre, const int* stt, ListView& lv, int cap) -> int {
      const int total = pre[27];
      const int rounded = (total + 31) & ~31;
      int cnt = 0;
      cap -= kListPad;
      unsigned head = 0, pend = 0;  // ring position of the oldest pending point; pending points
      auto settle = [&](int n) {
        __syncwarp();  // the ring entries written by all lanes are visible
        bool acc = false;
        ListEnt ent;
        float wv = 0.0f;
        if (lane < n) {
          const unsigned slot_i = (head + static_cast<unsigned>(lane)) & (kRing - 1);
          const int j = st.ring_j[slot_i];
          const int s = st.ring_s[slot_i];
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
          } else if (code == car) {
            code = careful_code(v, s_e2lo, s_e2hi, nb, g.ka, g.kb);
          }
          if (code == kCodeExact) {
            ++c.n_exact_pair;
            code = cold_pair_exact(&a.self->g, s_sqr_bins, pa, px, py, pz);
          }
          if (code < static_cast<unsigned>(nb)) {
            acc = true;
            const float rho = __fsqrt_rn(v);
            ent.e = make_float4(dx, dy, dz, __fmul_rn(rho, rho));
            ent.a2r = 2.0f * rho;
            ent.key = code * kj_mul;
            ent.m = code | (static_cast<unsigned>(s) << 8);
            ent.p = j;
            wv = __double2float_rn(p.w);
          }
        }
        const unsigned bal = __ballot_sync(FULL, acc);
        if (acc) {
          const int e = cnt + __popc(bal & lt_mask);
          if (e < cap) {
            lv.v[e] = ent;
            if (WEIGHTED) lv.w[e] = wv;
          } else {
            atomicOr(a.flags, kFlagListOverflow);
          }
        }
        cnt += __popc(bal);
        head += static_cast<unsigned>(n);
        pend -= static_cast<unsigned>(n);
        __syncwarp();  // the ring entries are read before the next round overwrites them
      };
      // Round r's point (slot, index, FP32 values) of this lane, rounds r
      // and r + 1 in flight.
      int sn = 0;
      auto fetch = [&](int item, int& s, int& j, float4& q) {
        if (item < total) {
          while (item >= pre[sn + 1]) ++sn;
          s = sn;
          j = stt[sn] + (item - pre[sn]);
          q = cat.pq[j];
        }
      };
      int s0 = 0, j0 = 0, s1 = 0, j1 = 0;
      float4 q0 = make_float4(0.0f, 0.0f, 0.0f, 0.0f), q1 = q0;
      fetch(lane, s0, j0, q0);
      fetch(lane + 32, s1, j1, q1);
      for (int base = 0; base < rounded; base += 32) {
        const int item_i = base + lane;
        const int s = s0, j = j0;
        const float4 q = q0;
        s0 = s1;
        j0 = j1;
        q0 = q1;
        fetch(item_i + 64, s1, j1, q1);
        bool pass = false;
        if (item_i < total) {
          // Cell-local FP32 prefilter: skip candidates certainly out of range.
          const float fx = (q.x - qa.x) + st.dof[s][0];
          const float fy = (q.y - qa.y) + st.dof[s][1];
          const float fz = (q.z - qa.z) + st.dof[s][2];
          const float vp = fmaf(fz, fz, fmaf(fy, fy, fx * fx));
          pass = vp < g.pre_hi && vp > g.pre_lo && (!sym6 || j > ai);
        }
        const unsigned bal = __ballot_sync(FULL, pass);
        if (pass) {
          const unsigned slot_i = (head + pend + static_cast<unsigned>(__popc(bal & lt_mask))) & (kRing - 1);
          st.ring_j[slot_i] = j;
          st.ring_s[slot_i] = static_cast<unsigned char>(s);
        }
        pend += static_cast<unsigned>(__popc(bal));
        if (pend >= 32u) settle(32);
      }
      if (pend > 0u) settle(static_cast<int>(pend));
      return min(cnt, cap);
    };
    const int k2 = build(it.c2, st.pre2, st.start2, l2, a.kcap2);
    const int k3 = SYM ? k2 : build(it.c3, st.pre3, st.start3, l3, a.kcap3);
    if (lane < kListPad) {
      // Padding rows after the rows: rho = 1e18 gives v >= 1e36 against
      // every column, rejected by the table, with a margin test that holds;
      // so they add into sink bins and are never flagged. Row loops that run
      // past their last row read them instead of testing for the end.
      ListEnt pad;
      pad.e = make_float4(0.0f, 0.0f, 0.0f, 1.0e36f);
      pad.a2r = 2.0e18f;
      pad.key = 0u;
      pad.m = 0u;
      pad.p = 0;
      l2.v[k2 + lane] = pad;
      if (WEIGHTED) l2.w[k2 + lane] = 0.0f;
    }
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
          drain_hist<WEIGHTED>(a.self, hist_s, nb, copies, held, lane, 32);
      }
      // Columns are held as (-2 d_l, rho_l) with the lane's histogram base in
      // their key; the padding (0, rho = 1e18) gives v = 1e36 and is
      // rejected by the table for every row.
      const unsigned col_base = HG ? 0u : hist_sh;
      ColV col;
      float wl[kReg];
#pragma unroll
      for (int r = 0; r < kReg; ++r) {
        const int l = lb + r * 32 + lane;
        if (l < k3) {
          const ListEnt& ce = l3.v[l];
          const float4 e = ce.e;
          col.l[r] = make_float4(-2.0f * e.x, -2.0f * e.y, -2.0f * e.z, 0.5f * ce.a2r);
          col.k[r] = (ce.m & 0xffu) * kl_mul + col_base;
          wl[r] = WEIGHTED ? l3.w[l] : 0.0f;
        } else {
          col.l[r] = make_float4(0.0f, 0.0f, 0.0f, 1.0e18f);
          col.k[r] = col_base;
          wl[r] = 0.0f;
        }
      }
      // A row in registers: offset and rho^2, then 2 rho and key (one 16-
      // and one 8-byte load), and the weight.
      struct RowReg {
        float4 e;
        uint2 fk;
        float w;
      };
      auto load_row = [&](const ListEnt* rp, const float* wp, RowReg& x) {
        x.e = rp->e;
        x.fk = *reinterpret_cast<const uint2*>(&rp->a2r);
        x.w = WEIGHTED ? *wp : 0.0f;
      };
      auto make_row = [&](const RowReg& x) {
        RowV r;
        r.x = x.e.x;
        r.y = x.e.y;
        r.z = x.e.z;
        r.a = x.e.w;
        r.a2r = __uint_as_float(x.fk.x);
        r.key = x.fk.y;
        return r;
      };
      // The careful queue: entries of this tile, settled when it fills and
      // at the end of the tile (format at kKindRot).
      // Every enqueue finds room for 32 entries: make_room settles the queue
      // when it has less, and it is called outside the row loops (a call
      // inside them would keep the rows in flight in local memory).
      int qn = 0;
      auto make_room = [&]() {
        if (qn + 32 > kQueueCap) {
          cold_drain<SURVEY, WEIGHTED, HG>(c, lb, k3, qn);
          qn = 0;
        }
      };
      auto enqueue = [&](unsigned q, unsigned tag) {
        const unsigned bal = __ballot_sync(FULL, q != 0u);
        if (q) c.queue[qn + __popc(bal & lt_mask)] = (static_cast<unsigned long long>(q) << 32) | tag;
        qn += __popc(bal);
      };
      // Weighted and global-histogram candidates, one at a time.
      auto cand_slow = [&](const RowV& r, const float4& cl, unsigned ck, float cw, unsigned in, float wj,
                           unsigned rbit, unsigned& q) {
        if (HG) {
          unsigned code;
          bool clean;
          cand_classify(r, cl, tab, g.tab_scale, g.tab_n, bk.hm, &code, &clean);
          const bool ok = code < nb_cs && in;
          const bool careful = (code == car || (code < nb_cs && !clean)) && in;
          if (ok && clean) hist_add<WEIGHTED, true>(hist_s, c.hist, r.key + ck + code, (wa * wj * wsc) * cw);
          if (careful) q |= rbit;
        } else if (WEIGHTED) {
          cand_wsum(r, cl, ck, in, bk, wa * wj * wsc, cw, rbit, q);
        }
      };
      // One row against column slots 0..N-1.
      auto row_at = [&](const RowReg& x, unsigned rbit, auto n_tag, unsigned& q) {
        constexpr int N = decltype(n_tag)::value;
        const RowV r = make_row(x);
        if (WEIGHTED || HG) {
#pragma unroll
          for (int s = 0; s < N; ++s) cand_slow(r, col.l[s], col.k[s], wl[s], 1u, x.w, rbit, q);
        } else {
          row_full<N>(r, col, bk, rbit, q);
        }
      };
      // Rows j0 .. j1 - 1 against column slots 0..N-1, R rows per iteration.
      // A range ends at k2 or holds a multiple of R rows, so the rows an
      // iteration takes past j1 are padding rows, which only add into sinks:
      // the loop has no remainder test. The bodies' "memory" clobber keeps
      // the compiler from hoisting loads above a body, so each row's
      // registers are reloaded with the row R positions ahead right after its
      // body (immediate offsets from one row pointer): the load has the next
      // R - 1 bodies' time to land, and no register is copied. The flag word
      // covers groups of `group` rows (8, 16 or 32, a multiple of R); after
      // each group it is queued, and when the queue is nearly full the loop
      // stops at that group boundary, the queue is settled and the loop
      // resumes there.
      auto run_rows = [&](int j0, int j1, auto n_tag) {
        constexpr int N = decltype(n_tag)::value;
        constexpr int R = N == kReg ? 4 : 2;
        int j = j0;
        while (j < j1) {
          make_room();
          const ListEnt* rp = l2.v + j;
          const float* wp = WEIGHTED ? l2.w + j : nullptr;
          RowReg x[R];
#pragma unroll
          for (int p = 0; p < R; ++p) load_row(rp + p, wp + p, x[p]);
          unsigned q = 0, rb = 1u;
          int jg = j;
#pragma unroll 1
          while (j < j1) {
#pragma unroll
            for (int p = 0; p < R; ++p) {
              row_at(x[p], rb << p, n_tag, q);
              load_row(rp + R + p, wp + R + p, x[p]);
            }
            rp += R;
            if (WEIGHTED) wp += R;
            j += R;
            rb <<= R;
            if (j - jg >= group || j >= j1) {
              enqueue(q, (static_cast<unsigned>(jg) << 8) | (static_cast<unsigned>(N - 1) << 5) |
                             static_cast<unsigned>(lane));
              q = 0;
              rb = 1u;
              jg = j;
              if (qn + 32 > kQueueCap) break;
            }
          }
        }
      };
      if (SYM) {
        // The diagonal tile, pairs l < j of its rows: block S (rows
        // lb + 32 S ..) against the column slots before it, then the pairs
        // inside the block by rotation, lane's column against row
        // lane + d (mod 32) for d = 1..16 (d = 16 in lanes 0-15 only), so
        // that no lane evaluates a pair that is not one.
        const int m = min(kTile, k2 - lb);
#pragma unroll 1
        for (int S = 0; S * 32 < m; ++S) {
          const int bb = lb + 32 * S, be = min(bb + 32, k2);
          if (S == 1) run_rows(bb, be, std::integral_constant<int, 1>());
          if (S == 2) run_rows(bb, be, std::integral_constant<int, 2>());
          if (S == 3) run_rows(bb, be, std::integral_constant<int, 3>());
          float4 cl = col.l[0];
          unsigned ck = col.k[0];
          float cw = wl[0];
#pragma unroll
          for (int s = 1; s < kReg; ++s) {
            if (S == s) {
              cl = col.l[s];
              ck = col.k[s];
              cw = wl[s];
            }
          }
          // Each lane's rows of steps d and d + 1 are in flight (block
          // positions past the list read stale entries of the slab, masked).
          const ListEnt* bp = l2.v + bb;
          const float* bw = WEIGHTED ? l2.w + bb : nullptr;
          auto rot_load = [&](int d, RowReg& x) {
            const int o = (lane + d) & 31;
            load_row(bp + o, bw + o, x);
          };
          auto rot_cand = [&](const RowReg& x, int d, unsigned in, bool masked, unsigned& q) {
            const RowV r = make_row(x);
            const unsigned rbit = 1u << (d - 1);
            if (WEIGHTED || HG)
              cand_slow(r, cl, ck, cw, in, x.w, rbit, q);
            else if (masked)
              row_rot1(r, cl, ck, bk, rbit, in, q);
            else
              row_rot1_full(r, cl, ck, bk, rbit, q);
          };
          unsigned qd = 0;
          RowReg x[2];
          rot_load(1, x[0]);
          rot_load(2, x[1]);
          if (be - bb == 32) {
            // A full block: every lane's pair is one to count, except that
            // d = 16 pairs lanes L and L + 16 twice.
#pragma unroll 1
            for (int d0 = 1; d0 < 15; d0 += 2) {
#pragma unroll
              for (int p = 0; p < 2; ++p) {
                rot_cand(x[p], d0 + p, 1u, false, qd);
                rot_load(d0 + p + 2, x[p]);
              }
            }
            rot_cand(x[0], 15, 1u, false, qd);
            rot_cand(x[1], 16, lane < 16 ? 1u : 0u, true, qd);
          } else {
            const bool cval = bb + lane < k2;
#pragma unroll 1
            for (int d0 = 1; d0 <= 16; d0 += 2) {
#pragma unroll
              for (int p = 0; p < 2; ++p) {
                const int d = d0 + p;
                const int rr = bb + ((lane + d) & 31);
                rot_cand(x[p], d, (cval && rr < k2 && (d < 16 || lane < 16)) ? 1u : 0u, true, qd);
                rot_load(d + 2, x[p]);
              }
            }
          }
          make_room();
          enqueue(qd, (static_cast<unsigned>(bb) << 8) | (kKindRot << 5) | static_cast<unsigned>(lane));
        }
        run_rows(lb + kTile, k2, std::integral_constant<int, kReg>());
      } else {
        run_rows(0, k2, std::integral_constant<int, kReg>());
      }
      if (qn > 0) cold_drain<SURVEY, WEIGHTED, HG>(c, lb, k3, qn);
    }
    __syncwarp();  // every lane has read the lists for the last time
    discard_l2(l2.v, static_cast<size_t>(k2 + kListPad) * sizeof(ListEnt), lane);
    if (WEIGHTED) discard_l2(l2.w, static_cast<size_t>(k2 + kListPad) * sizeof(float), lane);
    if (!SYM) {
      discard_l2(l3.v, static_cast<size_t>(k3) * sizeof(ListEnt), lane);
      if (WEIGHTED) discard_l2(l3.w, static_cast<size_t>(k3) * sizeof(float), lane);
    }
    __syncwarp();  // the discards precede the next anchor's list writes
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
    drain_hist<WEIGHTED>(a.self, hist_s, nb, copies, owner, tid, kThreads);
  }
  if (a.stats) {
    atomicAdd(&a.stats[0], c.n_exact_tri);
    atomicAdd(&a.stats[1], c.n_exact_pair);
    atomicAdd(&a.stats[5], c.n_flag_rows);
    atomicAdd(&a.stats[6], c.n_queued);
    if (lane == 0) {
      atomicAdd(&a.stats[2], c.n_anchor);
      atomicAdd(&a.stats[3], c.n_pairs);
      atomicAdd(&a.stats[4], c.n_evals);
    }
  }
}

}  // namespace ncorr_gb300
