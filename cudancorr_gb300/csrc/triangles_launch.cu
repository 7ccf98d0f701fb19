// Instantiations and launchers of the triangle kernel, plus the histogram fold.
#include "triangles.cuh"

namespace ncorr_gb300 {

// set_attr false: the shared-memory attribute was set by an earlier launch
// (inside a stream capture only kernel nodes are recorded).
template <bool SV, bool SYM, bool W, bool HG>
static cudaError_t launch_one(const KArgs& a, int grid, size_t smem, cudaStream_t st, bool set_attr) {
  if (set_attr) {
    cudaError_t e = cudaFuncSetAttribute(k_triangles<SV, SYM, W, HG>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem));
    if (e != cudaSuccess) return e;
  }
  k_triangles<SV, SYM, W, HG><<<grid, kThreads, smem, st>>>(a);
  return cudaGetLastError();
}

template <bool SV, bool SYM, bool W, bool HG>
static int occupancy_one(size_t smem) {
  if (cudaFuncSetAttribute(k_triangles<SV, SYM, W, HG>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           static_cast<int>(smem)) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_triangles<SV, SYM, W, HG>, kThreads, smem) !=
      cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

template <bool SV, bool SYM, bool W>
static cudaError_t launch_hg(const KArgs& a, bool hg, int grid, size_t smem, cudaStream_t st, bool set_attr) {
  return hg ? launch_one<SV, SYM, W, true>(a, grid, smem, st, set_attr)
            : launch_one<SV, SYM, W, false>(a, grid, smem, st, set_attr);
}

template <bool SV, bool SYM, bool W>
static int occupancy_hg(bool hg, size_t smem) {
  return hg ? occupancy_one<SV, SYM, W, true>(smem) : occupancy_one<SV, SYM, W, false>(smem);
}

cudaError_t launch_triangles(const KArgs& a, bool survey, bool sym, bool weighted, bool hg, int grid,
                             size_t smem, cudaStream_t st, bool set_attr) {
  const bool s = set_attr;
  if (survey) {
    if (sym) return weighted ? launch_hg<true, true, true>(a, hg, grid, smem, st, s)
                             : launch_hg<true, true, false>(a, hg, grid, smem, st, s);
    return weighted ? launch_hg<true, false, true>(a, hg, grid, smem, st, s)
                    : launch_hg<true, false, false>(a, hg, grid, smem, st, s);
  }
  if (sym) return weighted ? launch_hg<false, true, true>(a, hg, grid, smem, st, s)
                           : launch_hg<false, true, false>(a, hg, grid, smem, st, s);
  return weighted ? launch_hg<false, false, true>(a, hg, grid, smem, st, s)
                  : launch_hg<false, false, false>(a, hg, grid, smem, st, s);
}

int triangles_occupancy(bool survey, bool sym, bool weighted, bool hg, size_t smem) {
  if (survey) {
    if (sym) return weighted ? occupancy_hg<true, true, true>(hg, smem) : occupancy_hg<true, true, false>(hg, smem);
    return weighted ? occupancy_hg<true, false, true>(hg, smem) : occupancy_hg<true, false, false>(hg, smem);
  }
  if (sym) return weighted ? occupancy_hg<false, true, true>(hg, smem) : occupancy_hg<false, true, false>(hg, smem);
  return weighted ? occupancy_hg<false, false, true>(hg, smem) : occupancy_hg<false, false, false>(hg, smem);
}

template <bool SURVEY, bool WEIGHTED>
__global__ void __launch_bounds__(256) k_exact(KArgs a) {
  const unsigned n = min(*a.xq_count, a.xq_cap);
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    settle_exact<SURVEY, WEIGHTED>(a, a.xq[i]);
}

void launch_exact(const KArgs& a, bool survey, bool weighted, int grid, cudaStream_t st) {
  if (survey) {
    if (weighted) k_exact<true, true><<<grid, 256, 0, st>>>(a);
    else k_exact<true, false><<<grid, 256, 0, st>>>(a);
  } else {
    if (weighted) k_exact<false, true><<<grid, 256, 0, st>>>(a);
    else k_exact<false, false><<<grid, 256, 0, st>>>(a);
  }
}

// Folds each item's unsorted (bin_j, bin_l, bin_3) histogram into the
// reference's triCountsAll_ layout: out[hi + mid*nb + lo*nb^2] for
// lo <= mid <= hi sums the distinct permutations in a fixed order
// (deterministic), times 2 when only pairs j < l were visited (p2 == p3) or 6
// when only i < j < l were. blockIdx.y is the item.
__global__ void k_fold(const BatchItem* __restrict__ items, int nb, int weighted, int sym, double inv_scale) {
  const BatchItem& it = items[blockIdx.y];
  const int nbin = nb * nb * nb;
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nbin) return;
  const double factor = item_sym6(it) ? 6.0 : (sym ? 2.0 : 1.0);
  const int hi = f % nb, mid = (f / nb) % nb, lo = f / (nb * nb);
  if (!(lo <= mid && mid <= hi)) {
    it.out[f] = 0.0;
    return;
  }
  const int v[3] = {lo, mid, hi};
  const int perm[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
  int seen[6];
  int ns = 0;
  double acc = 0.0;
  unsigned long long cnt = 0;
  for (int p = 0; p < 6; ++p) {
    const int key = (v[perm[p][0]] * nb + v[perm[p][1]]) * nb + v[perm[p][2]];
    bool dup = false;
    for (int q = 0; q < ns; ++q) dup = dup || (seen[q] == key);
    if (dup) continue;
    seen[ns++] = key;
    if (weighted) {
      // Signed 128-bit (hi, lo) to double: negate negative values in integer
      // arithmetic first, so the conversion never cancels.
      unsigned long long wl = it.hist.wsum[2 * key];
      unsigned long long wh = it.hist.wsum[2 * key + 1];
      const bool neg = static_cast<long long>(wh) < 0;
      if (neg) {
        wl = ~wl + 1ull;
        wh = ~wh + (wl == 0ull ? 1ull : 0ull);
      }
      const double mag = static_cast<double>(wh) * 18446744073709551616.0 + static_cast<double>(wl);
      acc += (neg ? -mag : mag) * inv_scale;
    } else {
      cnt += it.hist.counts[key];
    }
  }
  if (weighted) {
    it.out[f] = acc * factor;
  } else {
    const unsigned long long c = cnt * static_cast<unsigned long long>(factor);
    it.out[f] = static_cast<double>(c);
    if (c) atomicAdd(it.total, c);
  }
}

void launch_fold(const BatchItem* items, int n_items, int nb, bool weighted, bool sym, double inv_scale,
                 cudaStream_t st) {
  const int nbin = nb * nb * nb;
  const dim3 grid((nbin + 255) / 256, n_items);
  k_fold<<<grid, 256, 0, st>>>(items, nb, weighted ? 1 : 0, sym ? 1 : 0, inv_scale);
}

}  // namespace ncorr_gb300
