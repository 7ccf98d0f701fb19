// Runs the reference's own counting kernels, unmodified, on the GPU.
//
// TEST AND BASELINE INFRASTRUCTURE ONLY. The reference's device code
// (source/device.cu of cudaNcorr) is compiled, as it stands, into a cubin
// under oracle/_ref/ by oracle/Makefile. This file loads that cubin with the
// CUDA driver API and restates the host side of the reference's
// ncorr::calculateD1D2D3 (source/cudaNcorr.cu:220-430) around it: constants
// uploaded to the module's __constant__ symbols, the three catalogues
// gridded on the host into per-cell vectors, one device buffer per cell and
// catalogue, a pointer table per catalogue, the <<<ceil(N1/64), 64>>> launch,
// synchronise, copy-back. The only departures: every buffer is freed (the
// reference frees the pointer tables instead of the per-cell buffers,
// source/cudaNcorr.cu:397-405), gridding is serial (the reference's
// omp critical push_back, source/cudaNcorr.cu:60-70, only changes the order
// inside a cell), and the debug prints are omitted.
//
// It is used to pin the CPU oracle against the reference's real outputs (threeD
// and rppi) and as the reference arm of the benchmark. It is never part of
// the product.
#include <cuda.h>
#include <cuda_runtime.h>
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

struct RefModule {
  bool loaded = false;
  CUmodule mod = nullptr;
  CUfunction box = nullptr;
  CUfunction survey = nullptr;
  CUfunction rppi_box = nullptr;
  CUfunction rppi_survey = nullptr;
  std::string err;
};

RefModule g_ref;

void set_err(const char* what, CUresult r) {
  const char* s = nullptr;
  cuGetErrorString(r, &s);
  g_ref.err = std::string(what) + ": " + (s ? s : "?");
}

#define DRV(call)                 \
  do {                            \
    CUresult r_ = (call);         \
    if (r_ != CUDA_SUCCESS) {     \
      set_err(#call, r_);         \
      return -1;                  \
    }                             \
  } while (0)

#define RT(call)                                              \
  do {                                                        \
    cudaError_t e_ = (call);                                  \
    if (e_ != cudaSuccess) {                                  \
      g_ref.err = std::string(#call) + ": " + cudaGetErrorString(e_); \
      return -1;                                              \
    }                                                         \
  } while (0)

int upload(const char* name, const void* src, size_t bytes) {
  CUdeviceptr p;
  size_t sz;
  DRV(cuModuleGetGlobal(&p, &sz, g_ref.mod, name));
  if (sz < bytes) {
    g_ref.err = std::string("symbol too small: ") + name;
    return -1;
  }
  DRV(cuMemcpyHtoD(p, src, bytes));
  return 0;
}

struct D4 {
  double x, y, z, w;
};

}  // namespace

extern "C" {

const char* ref_runner_last_error() { return g_ref.err.c_str(); }

// Loads the reference cubin into the current device's primary context.
int ref_runner_load(const char* cubin_path) {
  if (g_ref.loaded) return 0;
  RT(cudaFree(nullptr));  // make the runtime's primary context current
  DRV(cuModuleLoad(&g_ref.mod, cubin_path));
  unsigned int n = 0;
  DRV(cuModuleGetFunctionCount(&n, g_ref.mod));
  std::vector<CUfunction> fns(n);
  DRV(cuModuleEnumerateFunctions(fns.data(), n, g_ref.mod));
  for (unsigned i = 0; i < n; ++i) {
    const char* name = nullptr;
    DRV(cuFuncGetName(&name, fns[i]));
    if (!name) continue;
    if (std::strstr(name, "countTrianglesThreeDBox")) g_ref.box = fns[i];
    if (std::strstr(name, "countTrianglesThreeDSurvey")) g_ref.survey = fns[i];
    if (std::strstr(name, "countTrianglesRppiBox")) g_ref.rppi_box = fns[i];
    if (std::strstr(name, "countTrianglesRppiSurvey")) g_ref.rppi_survey = fns[i];
  }
  if (!g_ref.box || !g_ref.survey || !g_ref.rppi_box || !g_ref.rppi_survey) {
    g_ref.err = "counting kernels not found in the reference cubin";
    return -1;
  }
  g_ref.loaded = true;
  return 0;
}

// One call of the reference's calculateD1D2D3 for the threeD bin type.
// Points are N x 4 doubles (x, y, z, w). hist_out receives the nb^3 doubles
// of triCountsAll_. kernel_ms: CUDA-event time of the launch alone;
// total_ms: host wall time of the whole call, gridding and copies included.
int ref_runner_count(const double* box, const double* edges, int n_edges, int is_survey,
                     const double* ori, const double* p1, long n1, const double* p2, long n2,
                     const double* p3, long n3, double* hist_out, double* kernel_ms,
                     double* total_ms) {
  if (!g_ref.loaded) {
    g_ref.err = "reference cubin not loaded";
    return -1;
  }
  auto t0 = std::chrono::steady_clock::now();
  // Constructor (source/cudaNcorr.cu:118-157).
  const int nb = n_edges - 1;
  std::vector<double> sqr_bins(n_edges);
  for (int i = 0; i < n_edges; ++i) sqr_bins[i] = edges[i] * edges[i];
  double rmax = edges[n_edges - 1], rmin = edges[0];
  double sqr_rmax = rmax * rmax, sqr_rmin = rmin * rmin;
  double cell[3] = {rmax, rmax, rmax};
  int nc[3];
  for (int d = 0; d < 3; ++d) nc[d] = static_cast<int>(std::ceil(box[d] / cell[d]));
  int shifts[27 * 3];
  int s = 0;
  for (int i = -1; i <= 1; ++i)
    for (int j = -1; j <= 1; ++j)
      for (int k = -1; k <= 1; ++k) {
        shifts[3 * s] = i;
        shifts[3 * s + 1] = j;
        shifts[3 * s + 2] = k;
        ++s;
      }
  // Constant upload (source/cudaNcorr.cu:228-233, :253-255: only d_ori.x is
  // written in survey mode; the threeD kernels do not read it).
  if (upload("d_sqrRMax", &sqr_rmax, sizeof(double))) return -1;
  if (upload("d_sqrRMin", &sqr_rmin, sizeof(double))) return -1;
  if (upload("d_cellSize", cell, 3 * sizeof(double))) return -1;
  if (upload("d_box", box, 3 * sizeof(double))) return -1;
  if (upload("d_numCells", nc, 3 * sizeof(int))) return -1;
  if (upload("d_shifts", shifts, sizeof(shifts))) return -1;
  if (is_survey && upload("d_ori", ori, sizeof(double))) return -1;

  // Host gridding (source/cudaNcorr.cu:50-70, :263-277).
  const long ncell = static_cast<long>(nc[0]) * nc[1] * nc[2];
  auto grid = [&](const double* p, long n, std::vector<std::vector<D4>>& cells) -> int {
    cells.assign(ncell, {});
    for (long i = 0; i < n; ++i) {
      const D4& q = reinterpret_cast<const D4*>(p)[i];
      const double c3[3] = {q.x, q.y, q.z};
      int ijk[3];
      for (int d = 0; d < 3; ++d) {
        double t = c3[d] / cell[d];
        if (!(t > -1.0e9 && t < 1.0e9)) return -1;
        int v = static_cast<int>(t);
        if (v == nc[d]) v--;
        if (v < 0 || v >= nc[d]) return -1;
        ijk[d] = v;
      }
      cells[ijk[2] + static_cast<long>(nc[2]) * (ijk[1] + static_cast<long>(nc[1]) * ijk[0])].push_back(q);
    }
    return 0;
  };
  std::vector<std::vector<D4>> c1, c2, c3;
  if (grid(p1, n1, c1) || grid(p2, n2, c2) || grid(p3, n3, c3)) {
    g_ref.err = "point outside the reference's cell grid";
    return -2;
  }
  // Per-cell device buffers (source/cudaNcorr.cu:279-295).
  std::vector<void*> h1(ncell, nullptr), h2(ncell, nullptr), h3(ncell, nullptr);
  std::vector<int> s2(ncell), s3(ncell);
  auto put = [&](std::vector<std::vector<D4>>& cells, std::vector<void*>& h, std::vector<int>* sz) -> int {
    for (long i = 0; i < ncell; ++i) {
      if (sz) (*sz)[i] = static_cast<int>(cells[i].size());
      RT(cudaMalloc(&h[i], cells[i].size() * sizeof(D4)));
      RT(cudaMemcpy(h[i], cells[i].data(), cells[i].size() * sizeof(D4), cudaMemcpyHostToDevice));
    }
    return 0;
  };
  int rc = put(c1, h1, nullptr) || put(c2, h2, &s2) || put(c3, h3, &s3);
  void *d_p1 = nullptr, *d_p2c = nullptr, *d_p3c = nullptr, *d_s2 = nullptr, *d_s3 = nullptr;
  void *d_sb = nullptr, *d_tc = nullptr;
  float kms = 0.0f;
  if (rc == 0) {
    // Flat anchors, pointer tables, sizes, bins, histogram (:299-325).
    RT(cudaMalloc(&d_p1, n1 * sizeof(D4)));
    RT(cudaMemcpy(d_p1, p1, n1 * sizeof(D4), cudaMemcpyHostToDevice));
    RT(cudaMalloc(&d_p2c, ncell * sizeof(void*)));
    RT(cudaMemcpy(d_p2c, h2.data(), ncell * sizeof(void*), cudaMemcpyHostToDevice));
    RT(cudaMalloc(&d_p3c, ncell * sizeof(void*)));
    RT(cudaMemcpy(d_p3c, h3.data(), ncell * sizeof(void*), cudaMemcpyHostToDevice));
    RT(cudaMalloc(&d_s2, ncell * sizeof(int)));
    RT(cudaMemcpy(d_s2, s2.data(), ncell * sizeof(int), cudaMemcpyHostToDevice));
    RT(cudaMalloc(&d_s3, ncell * sizeof(int)));
    RT(cudaMemcpy(d_s3, s3.data(), ncell * sizeof(int), cudaMemcpyHostToDevice));
    RT(cudaMalloc(&d_sb, n_edges * sizeof(double)));
    RT(cudaMemcpy(d_sb, sqr_bins.data(), n_edges * sizeof(double), cudaMemcpyHostToDevice));
    const long nbin = static_cast<long>(nb) * nb * nb;
    RT(cudaMalloc(&d_tc, nbin * sizeof(double)));
    RT(cudaMemset(d_tc, 0, nbin * sizeof(double)));
    // Launch (source/cudaNcorr.cu:327-355).
    int np1 = static_cast<int>(n1);
    int numBins = nb;
    void* args[] = {&d_p1, &np1, &d_p2c, &d_p3c, &d_s2, &d_s3, &d_sb, &numBins, &d_tc};
    unsigned grid_x = static_cast<unsigned>((n1 + 63) / 64);
    cudaEvent_t e0, e1;
    RT(cudaEventCreate(&e0));
    RT(cudaEventCreate(&e1));
    RT(cudaEventRecord(e0, 0));
    if (grid_x > 0)
      DRV(cuLaunchKernel(is_survey ? g_ref.survey : g_ref.box, grid_x, 1, 1, 64, 1, 1, 0, nullptr, args, nullptr));
    RT(cudaEventRecord(e1, 0));
    RT(cudaDeviceSynchronize());  // source/cudaNcorr.cu:389
    RT(cudaEventElapsedTime(&kms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    RT(cudaMemcpy(hist_out, d_tc, nbin * sizeof(double), cudaMemcpyDeviceToHost));
  }
  for (long i = 0; i < ncell; ++i) {
    cudaFree(h1[i]);
    cudaFree(h2[i]);
    cudaFree(h3[i]);
  }
  cudaFree(d_p1);
  cudaFree(d_p2c);
  cudaFree(d_p3c);
  cudaFree(d_s2);
  cudaFree(d_s3);
  cudaFree(d_sb);
  cudaFree(d_tc);
  if (rc) return -1;
  auto t1 = std::chrono::steady_clock::now();
  if (kernel_ms) *kernel_ms = kms;
  if (total_ms) *total_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
  return 0;
}

// One call of the reference's calculateD1D2D3 for the rppi bin type: the
// constructor of source/cudaNcorr.cu:159-216, the constant uploads of
// :228-255, the gridding and per-cell buffers of :263-325, and the
// countTrianglesRppiBox / countTrianglesRppiSurvey launch of :357-385.
// Departures, each on a value the reference leaves undefined: d_sqrRMin gets
// 0.0 (sqrRMin_ is never initialised by the rppi constructor; every value in
// [0, rpMin^2] yields the same counts), and the histogram buffer has
// nPi + 1 spare doubles after its nb^3 * nPi^2 bins, because the reference's
// pi index can reach nPi (floor(sqrtf(pi^2)) with pi^2 just below piMax^2)
// and then writes up to nPi elements past the end; their sum is returned in
// *overflow. Anchors are checked against the grid first (a survey anchor on
// the upper face would make the kernel read outside its cell tables).
int ref_runner_count_rppi(const double* box, const double* edges, int n_edges, int num_pi_bins,
                          int is_survey, const double* ori, const double* p1, long n1, const double* p2,
                          long n2, const double* p3, long n3, double* hist_out, double* overflow,
                          double* kernel_ms, double* total_ms) {
  if (!g_ref.loaded) {
    g_ref.err = "reference cubin not loaded";
    return -1;
  }
  if (num_pi_bins < 1 || n_edges < 2) {
    g_ref.err = "bad rppi binning";
    return -1;
  }
  auto t0 = std::chrono::steady_clock::now();
  const int nb = n_edges - 1;
  const int npi = num_pi_bins;
  std::vector<double> sqr_bins(n_edges);
  for (int i = 0; i < n_edges; ++i) sqr_bins[i] = edges[i] * edges[i];
  const double rpmax = edges[n_edges - 1], rpmin = edges[0];
  const double sqr_rpmax = rpmax * rpmax, sqr_rpmin = rpmin * rpmin;
  const double pimax = static_cast<double>(npi);
  const double sqr_pimax = pimax * pimax;
  const double sqr_rmax = rpmax * rpmax + pimax * pimax;
  const double rmax = static_cast<double>(sqrtf(static_cast<float>(sqr_rmax)));
  const double sqr_rmin = 0.0;
  double cell[3];
  if (is_survey) {
    cell[0] = cell[1] = cell[2] = rmax;
  } else {
    cell[0] = cell[1] = rpmax;
    cell[2] = pimax;
  }
  int nc[3];
  for (int d = 0; d < 3; ++d) nc[d] = static_cast<int>(std::ceil(box[d] / cell[d]));
  int shifts[27 * 3];
  int s = 0;
  for (int i = -1; i <= 1; ++i)
    for (int j = -1; j <= 1; ++j)
      for (int k = -1; k <= 1; ++k) {
        shifts[3 * s] = i;
        shifts[3 * s + 1] = j;
        shifts[3 * s + 2] = k;
        ++s;
      }
  if (upload("d_sqrRMax", &sqr_rmax, sizeof(double))) return -1;
  if (upload("d_sqrRMin", &sqr_rmin, sizeof(double))) return -1;
  if (upload("d_cellSize", cell, 3 * sizeof(double))) return -1;
  if (upload("d_box", box, 3 * sizeof(double))) return -1;
  if (upload("d_numCells", nc, 3 * sizeof(int))) return -1;
  if (upload("d_shifts", shifts, sizeof(shifts))) return -1;
  if (upload("d_sqrRpMax", &sqr_rpmax, sizeof(double))) return -1;
  if (upload("d_sqrRpMin", &sqr_rpmin, sizeof(double))) return -1;
  if (upload("d_sqrPiMax", &sqr_pimax, sizeof(double))) return -1;
  if (is_survey) {
    // source/cudaNcorr.cu:253-255 copies sizeof(double): only d_ori.x.
    const double zero3[3] = {0.0, 0.0, 0.0};
    if (upload("d_ori", zero3, 3 * sizeof(double))) return -1;
    if (upload("d_ori", ori, sizeof(double))) return -1;
  }

  const long ncell = static_cast<long>(nc[0]) * nc[1] * nc[2];
  auto cell_of = [&](const D4& q, bool clamp, int ijk[3]) -> bool {
    const double c3[3] = {q.x, q.y, q.z};
    for (int d = 0; d < 3; ++d) {
      double t = c3[d] / cell[d];
      if (!(t > -1.0e9 && t < 1.0e9)) return false;
      int v = static_cast<int>(t);
      if (clamp && v == nc[d]) v--;
      if (v < 0 || v >= nc[d]) return false;
      ijk[d] = v;
    }
    return true;
  };
  for (long i = 0; i < n1; ++i) {
    int ijk[3];
    const D4& q = reinterpret_cast<const D4*>(p1)[i];
    if (!cell_of(q, true, ijk) || !cell_of(q, !is_survey, ijk)) {
      g_ref.err = "anchor outside the reference's cell grid";
      return -2;
    }
  }
  auto grid = [&](const double* p, long n, std::vector<std::vector<D4>>& cells) -> int {
    cells.assign(ncell, {});
    for (long i = 0; i < n; ++i) {
      const D4& q = reinterpret_cast<const D4*>(p)[i];
      int ijk[3];
      if (!cell_of(q, true, ijk)) return -1;
      cells[ijk[2] + static_cast<long>(nc[2]) * (ijk[1] + static_cast<long>(nc[1]) * ijk[0])].push_back(q);
    }
    return 0;
  };
  // All three catalogues are gridded and uploaded per cell, as the
  // reference does (source/cudaNcorr.cu:273-295), although its kernels read
  // p1 from the flat copy.
  std::vector<std::vector<D4>> c1, c2, c3;
  if (grid(p1, n1, c1) || grid(p2, n2, c2) || grid(p3, n3, c3)) {
    g_ref.err = "point outside the reference's cell grid";
    return -2;
  }
  std::vector<void*> h1(ncell, nullptr), h2(ncell, nullptr), h3(ncell, nullptr);
  std::vector<int> s1(ncell), s2(ncell), s3(ncell);
  auto put = [&](std::vector<std::vector<D4>>& cells, std::vector<void*>& h, std::vector<int>* sz) -> int {
    for (long i = 0; i < ncell; ++i) {
      (*sz)[i] = static_cast<int>(cells[i].size());
      RT(cudaMalloc(&h[i], cells[i].size() * sizeof(D4)));
      RT(cudaMemcpy(h[i], cells[i].data(), cells[i].size() * sizeof(D4), cudaMemcpyHostToDevice));
    }
    return 0;
  };
  int rc = put(c1, h1, &s1) || put(c2, h2, &s2) || put(c3, h3, &s3);
  void *d_p1 = nullptr, *d_p2c = nullptr, *d_p3c = nullptr, *d_s2 = nullptr, *d_s3 = nullptr;
  void *d_sb = nullptr, *d_tc = nullptr;
  float kms = 0.0f;
  const long nbin = static_cast<long>(nb) * nb * nb * npi * npi;
  const long npad = npi + 1;
  if (rc == 0) {
    RT(cudaMalloc(&d_p1, std::max<long>(n1, 1) * sizeof(D4)));
    RT(cudaMemcpy(d_p1, p1, n1 * sizeof(D4), cudaMemcpyHostToDevice));
    RT(cudaMalloc(&d_p2c, ncell * sizeof(void*)));
    RT(cudaMemcpy(d_p2c, h2.data(), ncell * sizeof(void*), cudaMemcpyHostToDevice));
    RT(cudaMalloc(&d_p3c, ncell * sizeof(void*)));
    RT(cudaMemcpy(d_p3c, h3.data(), ncell * sizeof(void*), cudaMemcpyHostToDevice));
    RT(cudaMalloc(&d_s2, ncell * sizeof(int)));
    RT(cudaMemcpy(d_s2, s2.data(), ncell * sizeof(int), cudaMemcpyHostToDevice));
    RT(cudaMalloc(&d_s3, ncell * sizeof(int)));
    RT(cudaMemcpy(d_s3, s3.data(), ncell * sizeof(int), cudaMemcpyHostToDevice));
    RT(cudaMalloc(&d_sb, n_edges * sizeof(double)));
    RT(cudaMemcpy(d_sb, sqr_bins.data(), n_edges * sizeof(double), cudaMemcpyHostToDevice));
    RT(cudaMalloc(&d_tc, (nbin + npad) * sizeof(double)));
    RT(cudaMemset(d_tc, 0, (nbin + npad) * sizeof(double)));
    int np1 = static_cast<int>(n1);
    int numBins = nb;
    int numPiBins = npi;
    void* args[] = {&d_p1, &np1, &d_p2c, &d_p3c, &d_s2, &d_s3, &d_sb, &numBins, &numPiBins, &d_tc};
    unsigned grid_x = static_cast<unsigned>((n1 + 63) / 64);
    cudaEvent_t e0, e1;
    RT(cudaEventCreate(&e0));
    RT(cudaEventCreate(&e1));
    RT(cudaEventRecord(e0, 0));
    if (grid_x > 0)
      DRV(cuLaunchKernel(is_survey ? g_ref.rppi_survey : g_ref.rppi_box, grid_x, 1, 1, 64, 1, 1, 0, nullptr,
                         args, nullptr));
    RT(cudaEventRecord(e1, 0));
    RT(cudaDeviceSynchronize());
    RT(cudaEventElapsedTime(&kms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    std::vector<double> full(nbin + npad);
    RT(cudaMemcpy(full.data(), d_tc, (nbin + npad) * sizeof(double), cudaMemcpyDeviceToHost));
    std::memcpy(hist_out, full.data(), nbin * sizeof(double));
    double ov = 0.0;
    for (long i = nbin; i < nbin + npad; ++i) ov += full[i];
    if (overflow) *overflow = ov;
  }
  for (long i = 0; i < ncell; ++i) {
    cudaFree(h1[i]);
    cudaFree(h2[i]);
    cudaFree(h3[i]);
  }
  cudaFree(d_p1);
  cudaFree(d_p2c);
  cudaFree(d_p3c);
  cudaFree(d_s2);
  cudaFree(d_s3);
  cudaFree(d_sb);
  cudaFree(d_tc);
  if (rc) return -1;
  auto t1 = std::chrono::steady_clock::now();
  if (kernel_ms) *kernel_ms = kms;
  if (total_ms) *total_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
  return 0;
}

}  // extern "C"
