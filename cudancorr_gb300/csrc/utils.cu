// Catalogue input and result output of the C ABI (each entry point catches
// what the host code may throw, so nothing crosses the ABI): the counterparts of the
// reference's text reader, result writers and random catalogue
// (include/utils.hpp, source/utils.cu:29-52, :119-208 of cudaNcorr). Host
// code only; the engine's kernels never read files.
#include <cstdio>
#include <new>
#include <stdexcept>
#include <fstream>
#include <random>
#include <sstream>
#include <string>
#include <system_error>
#include <thread>

#include "host.cuh"

using namespace ncorr_host;

namespace {

// Buffered "%.6f" rows: the bytes the reference's std::fixed <<
// std::setprecision(6) stream writes (source/utils.cu:174-180, :199-205).
int write_rows(const char* filename, const double* const* cols, int ncols, int64_t n) {
  if (!filename) return fail(NCORR_ERR_INVALID_ARGUMENT, "null file name");
  if (n < 0) return fail(NCORR_ERR_INVALID_ARGUMENT, "negative row count");
  for (int c = 0; c < ncols; ++c)
    if (n > 0 && !cols[c]) return fail(NCORR_ERR_INVALID_ARGUMENT, "null column");
  FILE* f = std::fopen(filename, "w");
  if (!f) return fail(NCORR_ERR_INVALID_ARGUMENT, std::string("Unable to open file: ") + filename);
  std::vector<char> buf(1 << 20);
  size_t used = 0;
  char row[512];
  for (int64_t i = 0; i < n; ++i) {
    int len = 0;
    for (int c = 0; c < ncols; ++c)
      len += std::snprintf(row + len, sizeof(row) - len, c + 1 < ncols ? "%.6f " : "%.6f\n", cols[c][i]);
    if (used + len > buf.size()) {
      std::fwrite(buf.data(), 1, used, f);
      used = 0;
    }
    std::memcpy(buf.data() + used, row, len);
    used += len;
  }
  std::fwrite(buf.data(), 1, used, f);
  const bool bad = std::ferror(f) != 0;
  if (std::fclose(f) != 0 || bad) return fail(NCORR_ERR_INVALID_ARGUMENT, std::string("write failed: ") + filename);
  return NCORR_OK;
}

}  // namespace

extern "C" {

static int write_three_d_impl(const char* filename, const double* tri_bins, const double* counts, int64_t n) {
  if (n > 0 && (!tri_bins || !counts)) return fail(NCORR_ERR_INVALID_ARGUMENT, "null array");
  std::vector<double> r1(static_cast<size_t>(std::max<int64_t>(n, 0))), r2(r1.size()), r3(r1.size());
  for (int64_t i = 0; i < n; ++i) {
    r1[i] = tri_bins[3 * i];
    r2[i] = tri_bins[3 * i + 1];
    r3[i] = tri_bins[3 * i + 2];
  }
  const double* cols[4] = {r1.data(), r2.data(), r3.data(), counts};
  return write_rows(filename, cols, 4, n);
}

static int write_rppi_impl(const char* filename, const double* tri_bins, const double* pi_bins, const double* counts,
                     int64_t n) {
  if (n > 0 && (!tri_bins || !pi_bins || !counts)) return fail(NCORR_ERR_INVALID_ARGUMENT, "null array");
  const size_t m = static_cast<size_t>(std::max<int64_t>(n, 0));
  std::vector<double> r1(m), r2(m), r3(m), q1(m), q2(m);
  for (int64_t i = 0; i < n; ++i) {
    r1[i] = tri_bins[3 * i];
    r2[i] = tri_bins[3 * i + 1];
    r3[i] = tri_bins[3 * i + 2];
    q1[i] = pi_bins[2 * i];
    q2[i] = pi_bins[2 * i + 1];
  }
  const double* cols[6] = {r1.data(), r2.data(), r3.data(), q1.data(), q2.data(), counts};
  return write_rows(filename, cols, 6, n);
}

static int read_catalog_txt_impl(const char* filename, const double box[3], const int pos_columns[4], double* out,
                           int64_t cap, int64_t* n) {
  if (!filename || !box || !pos_columns || !n) return fail(NCORR_ERR_INVALID_ARGUMENT, "null argument");
  *n = 0;
  for (int k = 0; k < 4; ++k)
    if (pos_columns[k] < 0) return fail(NCORR_ERR_INVALID_ARGUMENT, "negative column index");
  std::ifstream in(filename);
  if (!in.is_open()) return fail(NCORR_ERR_INVALID_ARGUMENT, std::string("Unable to open file: ") + filename);
  std::string line;
  int64_t line_number = 0, count = 0;
  while (std::getline(in, line)) {
    ++line_number;
    // Whitespace-separated doubles, read until the first token that is not
    // one (the reference's `line_stream >> value` loop).
    std::istringstream ls(line);
    double v, q[4] = {0, 0, 0, 0};
    bool have[4] = {false, false, false, false};
    int column = 0;
    while (ls >> v) {
      for (int k = 0; k < 4; ++k)
        if (column == pos_columns[k] && !have[k]) {
          q[k] = v;
          have[k] = true;
          break;
        }
      ++column;
    }
    if (!(have[0] && have[1] && have[2] && have[3]))
      return fail(NCORR_ERR_INVALID_ARGUMENT,
                  "Error at line " + std::to_string(line_number) + ": missing column (x, y, z or w)");
    if (q[0] < 0 || q[1] < 0 || q[2] < 0 || q[0] > box[0] || q[1] > box[1] || q[2] > box[2])
      return fail(NCORR_ERR_OUT_OF_GRID,
                  "Error at line " + std::to_string(line_number) + ": double3 value is out of bounds.");
    if (out && count < cap)
      for (int k = 0; k < 4; ++k) out[4 * count + k] = q[k];
    ++count;
  }
  *n = count;
  if (out && count > cap) return fail(NCORR_ERR_CAPACITY, "output capacity too small");
  return NCORR_OK;
}

static int random_catalog_impl(int64_t n, const double box[3], uint64_t seed, double* out) {
  if (n < 0 || !box || (n > 0 && !out)) return fail(NCORR_ERR_INVALID_ARGUMENT, "bad argument");
  for (int d = 0; d < 3; ++d)
    if (!(box[d] > 0.0) || !std::isfinite(box[d])) return fail(NCORR_ERR_INVALID_ARGUMENT, "box sides must be positive");
  // Fixed chunks of 2^16 points, one mt19937 stream per chunk seeded from
  // (seed, chunk): the result depends on the seed only, not on the threads.
  const int64_t chunk = int64_t(1) << 16;
  const int64_t nchunk = (n + chunk - 1) / chunk;
  const unsigned nth = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  auto work = [&](unsigned t) {
    for (int64_t c = t; c < nchunk; c += nth) {
      std::seed_seq ss{static_cast<uint32_t>(seed), static_cast<uint32_t>(seed >> 32), static_cast<uint32_t>(c),
                       static_cast<uint32_t>(c >> 32)};
      std::mt19937 gen(ss);
      // generateRandomPosition (source/utils.cu:29-39): three uniform_real
      // distributions on [0, box), weight 1.
      std::uniform_real_distribution<double> dx(0, box[0]), dy(0, box[1]), dz(0, box[2]);
      const int64_t e = std::min(n, (c + 1) * chunk);
      for (int64_t i = c * chunk; i < e; ++i) {
        out[4 * i] = dx(gen);
        out[4 * i + 1] = dy(gen);
        out[4 * i + 2] = dz(gen);
        out[4 * i + 3] = 1.0;
      }
    }
  };
  std::vector<std::thread> pool;
  // Reserved up front, so that starting a thread never reallocates the
  // vector: a growth failure there would unwind past joinable threads.
  pool.reserve(nth);
  unsigned started = 1;  // stripes handed to threads (stripe 0 runs here)
  try {
    for (unsigned t = 1; t < nth; ++t) {
      pool.emplace_back(work, t);
      ++started;
    }
  } catch (const std::system_error&) {
    // Fewer threads than asked for: the remaining stripes run below.
  }
  for (unsigned t = started; t < nth; ++t) work(t);
  work(0);
  for (auto& th : pool) th.join();
  return NCORR_OK;
}

int ncorr_write_three_d(const char* filename, const double* tri_bins, const double* counts, int64_t n) {
  try {
    return write_three_d_impl(filename, tri_bins, counts, n);
  } catch (const std::bad_alloc&) {
    return fail(NCORR_ERR_CAPACITY, "host memory exhausted");
  } catch (const std::exception& e) {
    return fail(NCORR_ERR_INVALID_ARGUMENT, e.what());
  }
}

int ncorr_write_rppi(const char* filename, const double* tri_bins, const double* pi_bins, const double* counts,
                     int64_t n) {
  try {
    return write_rppi_impl(filename, tri_bins, pi_bins, counts, n);
  } catch (const std::bad_alloc&) {
    return fail(NCORR_ERR_CAPACITY, "host memory exhausted");
  } catch (const std::exception& e) {
    return fail(NCORR_ERR_INVALID_ARGUMENT, e.what());
  }
}

int ncorr_read_catalog_txt(const char* filename, const double box[3], const int pos_columns[4], double* out,
                           int64_t cap, int64_t* n) {
  try {
    return read_catalog_txt_impl(filename, box, pos_columns, out, cap, n);
  } catch (const std::bad_alloc&) {
    return fail(NCORR_ERR_CAPACITY, "host memory exhausted");
  } catch (const std::exception& e) {
    return fail(NCORR_ERR_INVALID_ARGUMENT, e.what());
  }
}

int ncorr_random_catalog(int64_t n, const double box[3], uint64_t seed, double* out) {
  try {
    return random_catalog_impl(n, box, seed, out);
  } catch (const std::bad_alloc&) {
    return fail(NCORR_ERR_CAPACITY, "host memory exhausted");
  } catch (const std::exception& e) {
    return fail(NCORR_ERR_INVALID_ARGUMENT, e.what());
  }
}

}  // extern "C"
