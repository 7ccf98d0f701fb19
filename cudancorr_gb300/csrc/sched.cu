// Learned scheduling: per-cell features, the work-prediction MLP (inference,
// gradient and Adam kernels on the CUDA cores -- 6,081 parameters are far too
// few to feed a tensor core -- in FP32, or with a BF16 forward pass), and the
// construction of the triangle kernel's work queue.
#include <cmath>

#include <cuda_bf16.h>

#include "sched.cuh"

namespace ncorr_gb300 {

void launch_scan(const int* count, int ncell, int* start, int* cursor, cudaStream_t st);

// ---------------------------------------------------------------------------
// Features: log(1 + n) of the cell's catalogue-1 count and of the 27
// neighbour-slot counts of catalogue 2 (plus catalogue 3 when it differs),
// slots in the reference's order with the box wrap (survey: empty outside).
__global__ void k_cell_features(const BatchItem* __restrict__ items, int n_items, Geom g,
                                float* __restrict__ feats) {
  const int ncell = g.nc[0] * g.nc[1] * g.nc[2];
  const long long e = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= static_cast<long long>(n_items) * ncell) return;
  const int item = static_cast<int>(e / ncell), cell = static_cast<int>(e % ncell);
  const BatchItem& it = items[item];
  const bool two = it.c3.count != it.c2.count;
  const int h[3] = {cell / (g.nc[2] * g.nc[1]), (cell / g.nc[2]) % g.nc[1], cell % g.nc[2]};
  float* f = feats + e * kMlpIn;
  f[0] = log1pf(static_cast<float>(it.c1.count[cell]));
  for (int s = 0; s < 27; ++s) {
    int cc[3] = {h[0] + s / 9 - 1, h[1] + (s / 3) % 3 - 1, h[2] + s % 3 - 1};
    bool ok = true;
    for (int d = 0; d < 3; ++d) {
      if (cc[d] == g.nc[d]) {
        if (g.survey) ok = false; else cc[d] = 0;
      } else if (cc[d] == -1) {
        if (g.survey) ok = false; else cc[d] = g.nc[d] - 1;
      }
    }
    float occ = 0.0f;
    if (ok) {
      const int nbr = cc[2] + g.nc[2] * (cc[1] + g.nc[1] * cc[0]);
      occ = static_cast<float>(it.c2.count[nbr] + (two ? it.c3.count[nbr] : 0));
    }
    f[1 + s] = log1pf(occ);
  }
}

void launch_cell_features(const BatchItem* items, int n_items, const Geom& g, float* feats, cudaStream_t st) {
  const long long n = static_cast<long long>(n_items) * g.nc[0] * g.nc[1] * g.nc[2];
  if (n <= 0) return;
  k_cell_features<<<static_cast<unsigned>((n + 255) / 256), 256, 0, st>>>(items, n_items, g, feats);
}

// ---------------------------------------------------------------------------
// BF16 forward pass: weights, inputs and hidden activations are rounded to
// bfloat16 (round to nearest even); products of two bfloat16 values are exact
// in FP32 and are accumulated in FP32, as a BF16 tensor-core MMA accumulates;
// biases stay FP32. The FP32 variant uses the values unrounded.
template <bool BF16>
__device__ __forceinline__ float mlp_round(float x) {
  return BF16 ? __bfloat162float(__float2bfloat16_rn(x)) : x;
}

// Inference: one thread per sample, parameters in shared memory (bfloat16
// weights in the BF16 variant, half the bytes).
template <bool BF16>
__global__ void __launch_bounds__(128) k_mlp_predict(const float* __restrict__ params,
                                                     const float* __restrict__ feats, int n,
                                                     float* __restrict__ pred) {
  using W = typename std::conditional<BF16, __nv_bfloat16, float>::type;
  __shared__ W Pw[kMlpOffB3 + 1];
  __shared__ float Pb[kMlpParams];
  for (int i = threadIdx.x; i < kMlpParams; i += blockDim.x) {
    const float v = params[i];
    Pb[i] = v;
    if (BF16)
      Pw[i] = static_cast<W>(__float2bfloat16_rn(v));
    else
      Pw[i] = static_cast<W>(v);
  }
  __syncthreads();
  auto wt = [&](int i) -> float {
    if constexpr (BF16)
      return __bfloat162float(Pw[i]);
    else
      return Pw[i];
  };
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  float x[kMlpIn];
#pragma unroll
  for (int k = 0; k < kMlpIn; ++k) x[k] = mlp_round<BF16>(feats[static_cast<size_t>(s) * kMlpIn + k]);
  float h1[kMlpHidden];
#pragma unroll
  for (int i = 0; i < kMlpHidden; ++i) {
    float a = Pb[kMlpOffB1 + i];
#pragma unroll
    for (int k = 0; k < kMlpIn; ++k) a = fmaf(x[k], wt(kMlpOffW1 + k * kMlpHidden + i), a);
    h1[i] = mlp_round<BF16>(fmaxf(a, 0.0f));
  }
  float y = Pb[kMlpOffB3];
  for (int o = 0; o < kMlpHidden; ++o) {
    float a = Pb[kMlpOffB2 + o];
#pragma unroll
    for (int i = 0; i < kMlpHidden; ++i) a = fmaf(h1[i], wt(kMlpOffW2 + i * kMlpHidden + o), a);
    y = fmaf(wt(kMlpOffW3 + o), mlp_round<BF16>(fmaxf(a, 0.0f)), y);
  }
  pred[s] = y;
}

void launch_mlp_predict(const float* params, const float* feats, int n, float* pred, cudaStream_t st, bool bf16) {
  if (n <= 0) return;
  if (bf16)
    k_mlp_predict<true><<<(n + 127) / 128, 128, 0, st>>>(params, feats, n, pred);
  else
    k_mlp_predict<false><<<(n + 127) / 128, 128, 0, st>>>(params, feats, n, pred);
}

// ---------------------------------------------------------------------------
// Gradient of the mean squared error over a minibatch. Each CTA takes
// kMlpTile samples, runs forward and backward as small matrix products in
// shared memory, and writes its partial gradient; partials are summed in
// CTA order afterwards, so the result does not depend on timing. In the BF16
// variant the forward pass rounds weights, inputs and activations to
// bfloat16 (the backward pass uses those rounded values, in FP32); the master
// parameters and Adam stay FP32.
constexpr int kMlpParamsPad = (kMlpParams + 3) & ~3;
constexpr int kGradSmemFloats = kMlpParamsPad + kMlpTile * kMlpIn + 4 * kMlpTile * kMlpHidden + kMlpTile;

size_t mlp_grad_smem_bytes() { return static_cast<size_t>(kGradSmemFloats) * sizeof(float); }

template <bool BF16>
__global__ void __launch_bounds__(256) k_mlp_grad(const float* __restrict__ params,
                                                  const float* __restrict__ feats,
                                                  const float* __restrict__ target, const int* __restrict__ idx,
                                                  int n, float inv_n, float* __restrict__ partial,
                                                  float* __restrict__ partial_loss) {
  extern __shared__ float sm[];
  float* P = sm;
  float* X = P + kMlpParamsPad;            // [tile][in]
  float* H1 = X + kMlpTile * kMlpIn;       // [tile][hidden], after ReLU
  float* H2 = H1 + kMlpTile * kMlpHidden;  // [tile][hidden], after ReLU
  float* D2 = H2 + kMlpTile * kMlpHidden;  // dL/d(pre-activation 2)
  float* D1 = D2 + kMlpTile * kMlpHidden;  // dL/d(pre-activation 1)
  float* DY = D1 + kMlpTile * kMlpHidden;  // dL/dy
  __shared__ float s_loss[kMlpTile];
  const int t = threadIdx.x;
  const int b0 = blockIdx.x * kMlpTile;
  constexpr int TH = kMlpTile * kMlpHidden;

  for (int i = t; i < kMlpParams; i += blockDim.x) {
    const bool bias = (i >= kMlpOffB1 && i < kMlpOffW2) || (i >= kMlpOffB2 && i < kMlpOffW3) || i == kMlpOffB3;
    P[i] = bias ? params[i] : mlp_round<BF16>(params[i]);
  }
  for (int i = t; i < kMlpTile * kMlpIn; i += blockDim.x) {
    const int b = i / kMlpIn, k = i % kMlpIn, s = b0 + b;
    X[i] = s < n ? mlp_round<BF16>(feats[static_cast<size_t>(idx ? idx[s] : s) * kMlpIn + k]) : 0.0f;
  }
  __syncthreads();
  for (int i = t; i < TH; i += blockDim.x) {
    const int b = i / kMlpHidden, h = i % kMlpHidden;
    float a = P[kMlpOffB1 + h];
    for (int k = 0; k < kMlpIn; ++k) a = fmaf(X[b * kMlpIn + k], P[kMlpOffW1 + k * kMlpHidden + h], a);
    H1[i] = mlp_round<BF16>(fmaxf(a, 0.0f));
  }
  __syncthreads();
  for (int i = t; i < TH; i += blockDim.x) {
    const int b = i / kMlpHidden, o = i % kMlpHidden;
    float a = P[kMlpOffB2 + o];
    for (int h = 0; h < kMlpHidden; ++h) a = fmaf(H1[b * kMlpHidden + h], P[kMlpOffW2 + h * kMlpHidden + o], a);
    H2[i] = mlp_round<BF16>(fmaxf(a, 0.0f));
  }
  __syncthreads();
  if (t < kMlpTile) {
    const int s = b0 + t;
    float y = P[kMlpOffB3];
    for (int o = 0; o < kMlpHidden; ++o) y = fmaf(H2[t * kMlpHidden + o], P[kMlpOffW3 + o], y);
    const float r = s < n ? y - target[idx ? idx[s] : s] : 0.0f;
    DY[t] = 2.0f * r * inv_n;
    s_loss[t] = r * r;
  }
  __syncthreads();
  for (int i = t; i < TH; i += blockDim.x) {
    const int b = i / kMlpHidden, o = i % kMlpHidden;
    D2[i] = H2[i] > 0.0f ? DY[b] * P[kMlpOffW3 + o] : 0.0f;
  }
  __syncthreads();
  for (int i = t; i < TH; i += blockDim.x) {
    const int b = i / kMlpHidden, h = i % kMlpHidden;
    float a = 0.0f;
    for (int o = 0; o < kMlpHidden; ++o) a = fmaf(D2[b * kMlpHidden + o], P[kMlpOffW2 + h * kMlpHidden + o], a);
    D1[i] = H1[i] > 0.0f ? a : 0.0f;
  }
  __syncthreads();
  float* G = partial + static_cast<size_t>(blockIdx.x) * kMlpParams;
  for (int p = t; p < kMlpParams; p += blockDim.x) {
    float a = 0.0f;
    if (p < kMlpOffB1) {
      const int k = p / kMlpHidden, h = p % kMlpHidden;
      for (int b = 0; b < kMlpTile; ++b) a = fmaf(X[b * kMlpIn + k], D1[b * kMlpHidden + h], a);
    } else if (p < kMlpOffW2) {
      const int h = p - kMlpOffB1;
      for (int b = 0; b < kMlpTile; ++b) a += D1[b * kMlpHidden + h];
    } else if (p < kMlpOffB2) {
      const int q = p - kMlpOffW2, h = q / kMlpHidden, o = q % kMlpHidden;
      for (int b = 0; b < kMlpTile; ++b) a = fmaf(H1[b * kMlpHidden + h], D2[b * kMlpHidden + o], a);
    } else if (p < kMlpOffW3) {
      const int o = p - kMlpOffB2;
      for (int b = 0; b < kMlpTile; ++b) a += D2[b * kMlpHidden + o];
    } else if (p < kMlpOffB3) {
      const int o = p - kMlpOffW3;
      for (int b = 0; b < kMlpTile; ++b) a = fmaf(DY[b], H2[b * kMlpHidden + o], a);
    } else {
      for (int b = 0; b < kMlpTile; ++b) a += DY[b];
    }
    G[p] = a;
  }
  if (t == 0) {
    float l = 0.0f;
    for (int b = 0; b < kMlpTile; ++b) l += s_loss[b];
    partial_loss[blockIdx.x] = l;
  }
}

int launch_mlp_grad(const float* params, const float* feats, const float* target, const int* idx, int n,
                    float* partial, float* partial_loss, cudaStream_t st, bool bf16) {
  if (n <= 0) return 0;
  const int nblk = (n + kMlpTile - 1) / kMlpTile;
  const size_t smem = mlp_grad_smem_bytes();
  const float inv_n = 1.0f / static_cast<float>(n);
  if (bf16) {
    cudaFuncSetAttribute(k_mlp_grad<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    k_mlp_grad<true><<<nblk, 256, smem, st>>>(params, feats, target, idx, n, inv_n, partial, partial_loss);
  } else {
    cudaFuncSetAttribute(k_mlp_grad<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    k_mlp_grad<false><<<nblk, 256, smem, st>>>(params, feats, target, idx, n, inv_n, partial, partial_loss);
  }
  return nblk;
}

__global__ void k_mlp_reduce(const float* __restrict__ partial, const float* __restrict__ partial_loss, int nblk,
                             float* __restrict__ grad, float* __restrict__ loss) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < kMlpParams) {
    float a = 0.0f;
    for (int b = 0; b < nblk; ++b) a += partial[static_cast<size_t>(b) * kMlpParams + p];
    grad[p] = a;
  }
  if (p == 0 && loss) {
    float l = 0.0f;
    for (int b = 0; b < nblk; ++b) l += partial_loss[b];
    *loss = l;
  }
}

void launch_mlp_reduce(const float* partial, const float* partial_loss, int nblk, float* grad, float* loss,
                       cudaStream_t st) {
  k_mlp_reduce<<<(kMlpParams + 255) / 256, 256, 0, st>>>(partial, partial_loss, nblk, grad, loss);
}

// Adam (Kingma and Ba, 2015) on the summed partial gradients.
__global__ void k_adam(float* __restrict__ params, const float* __restrict__ partial, int nblk,
                       float* __restrict__ m, float* __restrict__ v, float lr, float c1, float c2) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= kMlpParams) return;
  const float beta1 = 0.9f, beta2 = 0.999f, eps = 1e-8f;
  float g = 0.0f;
  for (int b = 0; b < nblk; ++b) g += partial[static_cast<size_t>(b) * kMlpParams + p];
  const float mp = beta1 * m[p] + (1.0f - beta1) * g;
  const float vp = beta2 * v[p] + (1.0f - beta2) * g * g;
  m[p] = mp;
  v[p] = vp;
  params[p] -= lr * (mp * c1) / (sqrtf(vp * c2) + eps);
}

void launch_adam(float* params, const float* partial, int nblk, float* m, float* v, int step, float lr,
                 cudaStream_t st) {
  // Bias corrections 1 / (1 - beta^step), in double on the host.
  const float c1 = static_cast<float>(1.0 / (1.0 - std::pow(0.9, step)));
  const float c2 = static_cast<float>(1.0 / (1.0 - std::pow(0.999, step)));
  k_adam<<<(kMlpParams + 255) / 256, 256, 0, st>>>(params, partial, nblk, m, v, lr, c1, c2);
}

// ---------------------------------------------------------------------------
// Work queues.
__global__ void k_identity_queue(const int* __restrict__ item_off, int n_items, int* __restrict__ q_item,
                                 int* __restrict__ q_anchor, int n_work) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= n_work) return;
  int lo = 0, hi = n_items - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (item_off[mid] <= w) lo = mid; else hi = mid - 1;
  }
  q_item[w] = lo;
  q_anchor[w] = w - item_off[lo];
}

void launch_identity_queue(const int* item_off, int n_items, int* q_item, int* q_anchor, int n_work,
                           cudaStream_t st) {
  if (n_work <= 0) return;
  k_identity_queue<<<(n_work + 255) / 256, 256, 0, st>>>(item_off, n_items, q_item, q_anchor, n_work);
}

__device__ __forceinline__ float clamp_pred(float p) { return fminf(fmaxf(p, 0.0f), kSchedPredMax); }

__global__ void k_item_total(const BatchItem* __restrict__ items, int n_items, int ncell,
                             const float* __restrict__ pred, double* __restrict__ total) {
  const long long e = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= static_cast<long long>(n_items) * ncell) return;
  const int item = static_cast<int>(e / ncell), cell = static_cast<int>(e % ncell);
  if (items[item].c1.count[cell] > 0) atomicAdd(&total[item], expm1(static_cast<double>(clamp_pred(pred[e]))));
}

// Rank of each item by predicted total work, heaviest first (ties: lower index first).
__global__ void k_item_rank(const double* __restrict__ total, int n_items, int* __restrict__ rank) {
  for (int i = threadIdx.x; i < n_items; i += blockDim.x) {
    int r = 0;
    for (int j = 0; j < n_items; ++j) r += (total[j] > total[i] || (total[j] == total[i] && j < i)) ? 1 : 0;
    rank[i] = r;
  }
}

__global__ void k_entry_keys(const BatchItem* __restrict__ items, int n_items, int ncell,
                             const float* __restrict__ pred, const int* __restrict__ rank,
                             int* __restrict__ ekey, int* __restrict__ kcount) {
  const long long e = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= static_cast<long long>(n_items) * ncell) return;
  const int item = static_cast<int>(e / ncell), cell = static_cast<int>(e % ncell);
  if (items[item].c1.count[cell] == 0) {
    ekey[e] = -1;
    return;
  }
  const int bucket = min(kSchedBuckets - 1,
                         static_cast<int>(clamp_pred(pred[e]) * (kSchedBuckets / kSchedPredMax)));
  const int key = rank[item] * kSchedBuckets + (kSchedBuckets - 1 - bucket);
  ekey[e] = key;
  atomicAdd(&kcount[key], 1);
}

__global__ void k_entry_scatter(const BatchItem* __restrict__ items, int n_items, int ncell,
                                const int* __restrict__ ekey, int* __restrict__ kcursor, int* __restrict__ sorted,
                                int* __restrict__ acount) {
  const long long e = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= static_cast<long long>(n_items) * ncell) return;
  const int key = ekey[e];
  if (key < 0) return;
  const int pos = atomicAdd(&kcursor[key], 1);
  sorted[pos] = static_cast<int>(e);
  acount[pos] = items[e / ncell].c1.count[e % ncell];
}

// One warp per queued cell writes its anchors' positions.
__global__ void k_expand(const BatchItem* __restrict__ items, int ncell, const int* __restrict__ sorted,
                         const int* __restrict__ acount, const int* __restrict__ aoff,
                         const int* __restrict__ n_sorted, int* __restrict__ q_item, int* __restrict__ q_anchor) {
  const long long pos = (static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (pos >= *n_sorted) return;
  const int e = sorted[pos];
  const int item = e / ncell, cell = e % ncell;
  const int start = items[item].c1.start[cell];
  const int base = aoff[pos], cnt = acount[pos];
  for (int t = lane; t < cnt; t += 32) {
    q_item[base + t] = item;
    q_anchor[base + t] = start + t;
  }
}

void launch_learned_queue(const BatchItem* items, int n_items, int ncell, const OrderScratch& s, int* q_item,
                          int* q_anchor, cudaStream_t st) {
  const long long m = static_cast<long long>(n_items) * ncell;
  if (m <= 0) return;
  const int nkeys = n_items * kSchedBuckets;
  const unsigned g = static_cast<unsigned>((m + 255) / 256);
  cudaMemsetAsync(s.item_total, 0, n_items * sizeof(double), st);
  cudaMemsetAsync(s.kcount, 0, (nkeys + 1) * sizeof(int), st);
  cudaMemsetAsync(s.acount, 0, (m + 1) * sizeof(int), st);
  k_item_total<<<g, 256, 0, st>>>(items, n_items, ncell, s.pred, s.item_total);
  k_item_rank<<<1, 1024, 0, st>>>(s.item_total, n_items, s.item_rank);
  k_entry_keys<<<g, 256, 0, st>>>(items, n_items, ncell, s.pred, s.item_rank, s.ekey, s.kcount);
  launch_scan(s.kcount, nkeys, s.kstart, s.kcursor, st);
  k_entry_scatter<<<g, 256, 0, st>>>(items, n_items, ncell, s.ekey, s.kcursor, s.sorted, s.acount);
  launch_scan(s.acount, static_cast<int>(m), s.aoff, s.acursor, st);
  k_expand<<<static_cast<unsigned>((m * 32 + 255) / 256), 256, 0, st>>>(items, ncell, s.sorted, s.acount, s.aoff,
                                                                       s.kstart + nkeys, q_item, q_anchor);
}

}  // namespace ncorr_gb300
