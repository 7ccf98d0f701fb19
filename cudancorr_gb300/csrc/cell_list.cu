// GPU cell-list build: the device counterpart of the reference's host
// gridding (ncorr::getCellIndex / gridParticles, source/cudaNcorr.cu:50-70)
// and per-cell uploads (source/cudaNcorr.cu:279-295). One pass assigns each
// point its reference cell and counts cells, one scan gives the cell offsets,
// one pass scatters the points into cell order as exact double4_16a plus
// cell-local float4.
#include "engine.cuh"

namespace ncorr_gb300 {

// int(x / cell) exactly as the reference evaluates it (double division,
// truncation toward zero); returns false when the conversion itself would be
// undefined.
__device__ __forceinline__ bool axis_cell(double x, double cell, int* out) {
  double q = __ddiv_rn(x, cell);
  if (!(q > -2.0e9 && q < 2.0e9)) return false;
  *out = static_cast<int>(q);
  return true;
}

// True when the point lies exactly inside its cell [c*cell, (c+1)*cell)
// (the clamped face point x == nc*cell included) and, in box mode, its +-box
// images are exact in FP64. When every point passes and cells are exactly
// r_max wide, every pair closer than r_max is in adjacent cells and every
// triangle's three vertices see each other through bit-identical
// differences, which is what counting i < j < l once for all six orderings
// needs.
__device__ __forceinline__ bool sym6_point_ok(double x, int c, int d, const Geom& g) {
  const double lo = __fma_rn(-static_cast<double>(c), g.cell, x);
  const double hi = __fma_rn(-static_cast<double>(c + 1), g.cell, x);
  if (!(lo >= 0.0)) return false;
  if (!(hi < 0.0 || (hi == 0.0 && c == g.nc[d] - 1))) return false;
  if (!g.survey) {
    // Two-sum errors of x + box and x - box must vanish.
    const double L = g.box[d];
    const double s1 = __dadd_rn(x, L);
    const double b1 = __dsub_rn(s1, x);
    const double e1 = __dadd_rn(__dsub_rn(x, __dsub_rn(s1, b1)), __dsub_rn(L, b1));
    const double s2 = __dsub_rn(x, L);
    const double b2 = __dsub_rn(s2, x);
    const double e2 = __dadd_rn(__dsub_rn(x, __dsub_rn(s2, b2)), __dsub_rn(-L, b2));
    if (e1 != 0.0 || e2 != 0.0) return false;
  }
  return true;
}

// Per point: reference cell, validation, per-cell counts, weight summary.
__global__ void k_assign(const double4_16a* __restrict__ in, int n, Geom g, int* __restrict__ cid,
                         int* __restrict__ count, int* __restrict__ flags,
                         unsigned* __restrict__ wmax_bits) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  int f = 0;
  unsigned wb = 0;
  if (i < n) {
    const double4_16a p = in[i];
    const double c3[3] = {p.x, p.y, p.z};
    int ijk[3] = {0, 0, 0};
    if (!isfinite(p.x) || !isfinite(p.y) || !isfinite(p.z) || !isfinite(p.w)) f |= kFlagNonFinite;
    for (int d = 0; d < 3 && !(f & (kFlagNonFinite | kFlagOutOfGrid)); ++d) {
      int c;
      if (!axis_cell(c3[d], g.cell, &c)) {
        f |= kFlagOutOfGrid;
        break;
      }
      // The device anchor cell of the survey kernels is not clamped
      // (source/device.cu:84-87); only the host grid clamps (:50-58).
      if (g.survey && c == g.nc[d]) f |= kFlagSurveyFace;
      if (c == g.nc[d]) --c;
      if (c < 0 || c >= g.nc[d]) f |= kFlagOutOfGrid;
      ijk[d] = c;
      if (!sym6_point_ok(c3[d], c, d, g)) f |= kFlagNoSym6;
    }
    if (p.w != 1.0) f |= kFlagWeighted;
    const float aw = fabsf(static_cast<float>(p.w));
    if (isfinite(aw)) wb = __float_as_uint(aw);
    if (f & (kFlagNonFinite | kFlagOutOfGrid)) {
      cid[i] = -1;
    } else {
      const int c = ijk[2] + g.nc[2] * (ijk[1] + g.nc[1] * ijk[0]);
      cid[i] = c;
      atomicAdd(&count[c], 1);
    }
  }
  // One atomic per warp for the flags and the weight maximum.
  const unsigned FULL = 0xffffffffu;
  f = __reduce_or_sync(FULL, f);
  wb = __reduce_max_sync(FULL, wb);
  if ((threadIdx.x & 31) == 0) {
    if (f) atomicOr(flags, f);
    if (wb) atomicMax(wmax_bits, wb);
  }
}

// Exclusive scan of the cell counts by one CTA of 1024 threads: each thread
// owns a contiguous run of cells. Also initialises the scatter cursors.
__global__ void k_scan(const int* __restrict__ count, int ncell, int* __restrict__ start,
                       int* __restrict__ cursor) {
  __shared__ long long part[1024];
  const int t = threadIdx.x;
  const int per = (ncell + 1023) / 1024;
  const int b = t * per;
  const int e = min(ncell, b + per);
  long long s = 0;
  for (int c = b; c < e; ++c) s += count[c];
  part[t] = s;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    long long v = (t >= off) ? part[t - off] : 0;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  long long run = part[t] - s;
  for (int c = b; c < e; ++c) {
    start[c] = static_cast<int>(run);
    cursor[c] = static_cast<int>(run);
    run += count[c];
  }
  if (t == 1023) start[ncell] = static_cast<int>(part[1023]);
}

// Scatter into cell order. Order inside a cell is arbitrary (as in the
// reference, whose omp critical push_back also leaves it unspecified).
__global__ void k_scatter(const double4_16a* __restrict__ in, int n, Geom g,
                          const int* __restrict__ cid, int* __restrict__ cursor,
                          double4_16a* __restrict__ pd, float4* __restrict__ pq,
                          int* __restrict__ pc) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int c = cid[i];
  if (c < 0) return;
  int pos = atomicAdd(&cursor[c], 1);
  double4_16a p = in[i];
  int cz = c % g.nc[2];
  int cy = (c / g.nc[2]) % g.nc[1];
  int cx = c / (g.nc[2] * g.nc[1]);
  // Cell lower corner o = index * cell (double); q = fl32(x - o).
  double ox = __dmul_rn(static_cast<double>(cx), g.cell);
  double oy = __dmul_rn(static_cast<double>(cy), g.cell);
  double oz = __dmul_rn(static_cast<double>(cz), g.cell);
  pd[pos] = p;
  pq[pos] = make_float4(__double2float_rn(__dsub_rn(p.x, ox)), __double2float_rn(__dsub_rn(p.y, oy)),
                        __double2float_rn(__dsub_rn(p.z, oz)), __double2float_rn(p.w));
  pc[pos] = c;
}

// Upper bound of any anchor's neighbour-list length: the largest sum of the
// 27 (cell, image) slots the reference walks around a home cell.
__global__ void k_nbr_bound(const int* __restrict__ count, Geom g, int* __restrict__ out) {
  int ncell = g.nc[0] * g.nc[1] * g.nc[2];
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncell) return;
  int cz = c % g.nc[2];
  int cy = (c / g.nc[2]) % g.nc[1];
  int cx = c / (g.nc[2] * g.nc[1]);
  long long s = 0;
  for (int a = -1; a <= 1; ++a)
    for (int b = -1; b <= 1; ++b)
      for (int d = -1; d <= 1; ++d) {
        int x = cx + a, y = cy + b, z = cz + d;
        if (g.survey) {
          if (x < 0 || y < 0 || z < 0 || x >= g.nc[0] || y >= g.nc[1] || z >= g.nc[2]) continue;
        } else {
          x = (x == g.nc[0]) ? 0 : (x == -1 ? g.nc[0] - 1 : x);
          y = (y == g.nc[1]) ? 0 : (y == -1 ? g.nc[1] - 1 : y);
          z = (z == g.nc[2]) ? 0 : (z == -1 ? g.nc[2] - 1 : z);
        }
        s += count[z + g.nc[2] * (y + g.nc[1] * x)];
      }
  int v = s > 0x7fffffffLL ? 0x7fffffff : static_cast<int>(s);
  atomicMax(out, v);
}

void launch_assign(const double4_16a* in, int n, const Geom& g, int* cid, int* count, int* flags,
                   unsigned* wmax_bits, cudaStream_t st) {
  if (n <= 0) return;
  k_assign<<<(n + 255) / 256, 256, 0, st>>>(in, n, g, cid, count, flags, wmax_bits);
}

void launch_scan(const int* count, int ncell, int* start, int* cursor, cudaStream_t st) {
  k_scan<<<1, 1024, 0, st>>>(count, ncell, start, cursor);
}

void launch_scatter(const double4_16a* in, int n, const Geom& g, const int* cid, int* cursor,
                    double4_16a* pd, float4* pq, int* pc, cudaStream_t st) {
  if (n <= 0) return;
  k_scatter<<<(n + 255) / 256, 256, 0, st>>>(in, n, g, cid, cursor, pd, pq, pc);
}

void launch_nbr_bound(const int* count, const Geom& g, int* out, cudaStream_t st) {
  int ncell = g.nc[0] * g.nc[1] * g.nc[2];
  k_nbr_bound<<<(ncell + 255) / 256, 256, 0, st>>>(count, g, out);
}

}  // namespace ncorr_gb300
