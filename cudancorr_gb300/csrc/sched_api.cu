// C ABI of the scheduler's work model (include/ncorr_gb300.h): creation,
// parameters, inference, gradient and Adam training. All arithmetic runs in
// the kernels of sched.cu; the host only moves data and orders minibatches.
#include <numeric>
#include <random>

#include "host.cuh"

using namespace ncorr_gb300;
using namespace ncorr_host;

namespace {

// splitmix64 (Steele, Lea and Flood, 2014): the parameter initialiser's
// generator, fixed so that a seed gives the same model everywhere.
uint64_t splitmix64(uint64_t& x) {
  uint64_t z = (x += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

double uniform01(uint64_t& x) { return static_cast<double>(splitmix64(x) >> 11) * (1.0 / 9007199254740992.0); }

int check_sched(const ncorr_sched* s) {
  if (!s) return fail(NCORR_ERR_INVALID_ARGUMENT, "null scheduler model");
  int dev = -1;
  cudaGetDevice(&dev);
  if (dev != s->device) return fail(NCORR_ERR_INVALID_ARGUMENT, "scheduler model belongs to another device");
  return NCORR_OK;
}

// Uploads n rows of features (and targets) into the model's scratch.
int upload(ncorr_sched* s, const float* feats, const float* target, int64_t n) {
  CU(s->feats.ensure(static_cast<size_t>(n) * kMlpIn * sizeof(float)));
  CU(cudaMemcpyAsync(s->feats.p, feats, static_cast<size_t>(n) * kMlpIn * sizeof(float), cudaMemcpyHostToDevice,
                     s->stream));
  if (target) {
    CU(s->target.ensure(static_cast<size_t>(n) * sizeof(float)));
    CU(cudaMemcpyAsync(s->target.p, target, static_cast<size_t>(n) * sizeof(float), cudaMemcpyHostToDevice,
                       s->stream));
  }
  return NCORR_OK;
}

int ensure_partials(ncorr_sched* s, int64_t n) {
  const size_t nblk = static_cast<size_t>((n + kMlpTile - 1) / kMlpTile);
  CU(s->partial.ensure(nblk * kMlpParams * sizeof(float)));
  CU(s->partial_loss.ensure(nblk * sizeof(float)));
  return NCORR_OK;
}

}  // namespace

extern "C" {

int ncorr_sched_num_params(void) { return kMlpParams; }

int ncorr_sched_create(uint64_t seed, ncorr_sched** out) {
  if (!out) return fail(NCORR_ERR_INVALID_ARGUMENT, "null output pointer");
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return fail(NCORR_ERR_NO_DEVICE, "no CUDA device");
  }
  ncorr_sched* s = new ncorr_sched();
  cudaGetDevice(&s->device);
  auto bail = [&](int rc) {
    ncorr_sched_destroy(s);
    return rc;
  };
  if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess)
    return bail(fail(NCORR_ERR_CUDA, "cudaStreamCreate failed"));
  // He-uniform weights (bound sqrt(6 / fan_in)), zero biases.
  std::vector<float> p(kMlpParams, 0.0f);
  uint64_t x = seed;
  auto fill = [&](int off, int count, int fan_in) {
    const double b = std::sqrt(6.0 / fan_in);
    for (int i = 0; i < count; ++i) p[off + i] = static_cast<float>((2.0 * uniform01(x) - 1.0) * b);
  };
  fill(kMlpOffW1, kMlpIn * kMlpHidden, kMlpIn);
  fill(kMlpOffW2, kMlpHidden * kMlpHidden, kMlpHidden);
  fill(kMlpOffW3, kMlpHidden, kMlpHidden);
  for (DevBuf* b : {&s->params, &s->m, &s->v, &s->grad})
    if (b->ensure(kMlpParams * sizeof(float)) != cudaSuccess) return bail(fail(NCORR_ERR_CUDA, "cudaMalloc failed"));
  if (s->loss.ensure(sizeof(float)) != cudaSuccess) return bail(fail(NCORR_ERR_CUDA, "cudaMalloc failed"));
  if (cudaMemcpy(s->params.p, p.data(), kMlpParams * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemset(s->m.p, 0, kMlpParams * sizeof(float)) != cudaSuccess ||
      cudaMemset(s->v.p, 0, kMlpParams * sizeof(float)) != cudaSuccess)
    return bail(fail(NCORR_ERR_CUDA, "initialising the model failed"));
  *out = s;
  return NCORR_OK;
}

void ncorr_sched_destroy(ncorr_sched* s) {
  if (!s) return;
  if (s->stream) cudaStreamSynchronize(s->stream);
  for (DevBuf* b : {&s->params, &s->m, &s->v, &s->grad, &s->loss, &s->partial, &s->partial_loss, &s->feats,
                    &s->target, &s->idx, &s->pred})
    b->release();
  if (s->stream) cudaStreamDestroy(s->stream);
  delete s;
}

int ncorr_sched_get_params(const ncorr_sched* s, float* out, int64_t cap) {
  if (int rc = check_sched(s)) return rc;
  if (!out || cap < kMlpParams) return fail(NCORR_ERR_INVALID_ARGUMENT, "output too small");
  CU(cudaMemcpy(out, s->params.p, kMlpParams * sizeof(float), cudaMemcpyDeviceToHost));
  return NCORR_OK;
}

int ncorr_sched_set_params(ncorr_sched* s, const float* in, int64_t n) {
  if (int rc = check_sched(s)) return rc;
  if (!in || n != kMlpParams) return fail(NCORR_ERR_INVALID_ARGUMENT, "expected ncorr_sched_num_params() values");
  CU(cudaMemcpy(s->params.p, in, kMlpParams * sizeof(float), cudaMemcpyHostToDevice));
  CU(cudaMemset(s->m.p, 0, kMlpParams * sizeof(float)));
  CU(cudaMemset(s->v.p, 0, kMlpParams * sizeof(float)));
  s->step = 0;
  return NCORR_OK;
}

int ncorr_sched_set_precision(ncorr_sched* s, int precision) {
  if (int rc = check_sched(s)) return rc;
  if (precision != NCORR_MLP_FP32 && precision != NCORR_MLP_BF16)
    return fail(NCORR_ERR_INVALID_ARGUMENT, "precision must be NCORR_MLP_FP32 or NCORR_MLP_BF16");
  s->bf16 = precision == NCORR_MLP_BF16;
  return NCORR_OK;
}

int ncorr_sched_predict(ncorr_sched* s, const float* feats, int64_t n, float* out) {
  if (int rc = check_sched(s)) return rc;
  if (n < 0 || n > (int64_t(1) << 30) || (n > 0 && (!feats || !out)))
    return fail(NCORR_ERR_INVALID_ARGUMENT, "bad feature array");
  if (n == 0) return NCORR_OK;
  if (int rc = upload(s, feats, nullptr, n)) return rc;
  CU(s->pred.ensure(static_cast<size_t>(n) * sizeof(float)));
  launch_mlp_predict(s->params.as<float>(), s->feats.as<float>(), static_cast<int>(n), s->pred.as<float>(),
                     s->stream, s->bf16);
  CU(cudaGetLastError());
  CU(cudaMemcpyAsync(out, s->pred.p, static_cast<size_t>(n) * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
  CU(cudaStreamSynchronize(s->stream));
  return NCORR_OK;
}

int ncorr_sched_gradient(ncorr_sched* s, const float* feats, const float* target, int64_t n, float* grad,
                         float* loss) {
  if (int rc = check_sched(s)) return rc;
  if (n <= 0 || n > (int64_t(1) << 26) || !feats || !target || !grad)
    return fail(NCORR_ERR_INVALID_ARGUMENT, "bad gradient arguments");
  if (int rc = upload(s, feats, target, n)) return rc;
  if (int rc = ensure_partials(s, n)) return rc;
  const int nblk = launch_mlp_grad(s->params.as<float>(), s->feats.as<float>(), s->target.as<float>(), nullptr,
                                   static_cast<int>(n), s->partial.as<float>(), s->partial_loss.as<float>(),
                                   s->stream, s->bf16);
  launch_mlp_reduce(s->partial.as<float>(), s->partial_loss.as<float>(), nblk, s->grad.as<float>(),
                    s->loss.as<float>(), s->stream);
  CU(cudaGetLastError());
  CU(cudaMemcpyAsync(grad, s->grad.p, kMlpParams * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
  float l = 0.0f;
  CU(cudaMemcpyAsync(&l, s->loss.p, sizeof(float), cudaMemcpyDeviceToHost, s->stream));
  CU(cudaStreamSynchronize(s->stream));
  if (loss) *loss = l;
  return NCORR_OK;
}

int ncorr_sched_train(ncorr_sched* s, const float* feats, const float* target, int64_t n, int epochs, int batch,
                      float lr, uint64_t seed, float* last_epoch_loss) {
  if (int rc = check_sched(s)) return rc;
  if (n <= 0 || n > (int64_t(1) << 26) || !feats || !target)
    return fail(NCORR_ERR_INVALID_ARGUMENT, "bad training data");
  if (epochs < 1 || batch < kMlpTile || batch % kMlpTile || !(lr > 0.0f))
    return fail(NCORR_ERR_INVALID_ARGUMENT, "epochs >= 1, batch a positive multiple of 64, lr > 0");
  if (int rc = upload(s, feats, target, n)) return rc;
  if (int rc = ensure_partials(s, std::max<int64_t>(n, batch))) return rc;
  CU(s->idx.ensure(static_cast<size_t>(n) * sizeof(int)));
  if (s->step == 0) {
    // Start the output bias at the mean target (log-work is far from 0).
    double mean = 0.0;
    for (int64_t i = 0; i < n; ++i) mean += target[i];
    const float b3 = static_cast<float>(mean / static_cast<double>(n));
    CU(cudaMemcpyAsync(s->params.as<float>() + kMlpOffB3, &b3, sizeof(float), cudaMemcpyHostToDevice, s->stream));
  }
  std::vector<int> perm(n);
  std::iota(perm.begin(), perm.end(), 0);
  std::mt19937_64 rng(seed);
  for (int ep = 0; ep < epochs; ++ep) {
    std::shuffle(perm.begin(), perm.end(), rng);
    // The copy from pageable memory has completed when the call returns, so
    // the next epoch may overwrite perm.
    CU(cudaMemcpyAsync(s->idx.p, perm.data(), static_cast<size_t>(n) * sizeof(int), cudaMemcpyHostToDevice,
                       s->stream));
    for (int64_t b0 = 0; b0 < n; b0 += batch) {
      const int nb = static_cast<int>(std::min<int64_t>(batch, n - b0));
      const int nblk = launch_mlp_grad(s->params.as<float>(), s->feats.as<float>(), s->target.as<float>(),
                                       s->idx.as<int>() + b0, nb, s->partial.as<float>(),
                                       s->partial_loss.as<float>(), s->stream, s->bf16);
      launch_adam(s->params.as<float>(), s->partial.as<float>(), nblk, s->m.as<float>(), s->v.as<float>(),
                  ++s->step, lr, s->stream);
    }
    CU(cudaGetLastError());
  }
  if (last_epoch_loss) {
    // Mean squared error of the trained model over all n samples.
    const int nblk = launch_mlp_grad(s->params.as<float>(), s->feats.as<float>(), s->target.as<float>(), nullptr,
                                     static_cast<int>(n), s->partial.as<float>(), s->partial_loss.as<float>(),
                                     s->stream, s->bf16);
    launch_mlp_reduce(s->partial.as<float>(), s->partial_loss.as<float>(), nblk, s->grad.as<float>(),
                      s->loss.as<float>(), s->stream);
    float l = 0.0f;
    CU(cudaMemcpyAsync(&l, s->loss.p, sizeof(float), cudaMemcpyDeviceToHost, s->stream));
    CU(cudaStreamSynchronize(s->stream));
    *last_epoch_loss = l / static_cast<float>(n);
  }
  CU(cudaStreamSynchronize(s->stream));
  return NCORR_OK;
}

}  // extern "C"
