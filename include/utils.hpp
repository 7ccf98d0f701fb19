// Source-compatible replacement of cudaNcorr's include/utils.hpp: bin edges,
// random catalogues, the text catalogue reader and the result writers, as
// thin inline wrappers of the C ABI in ncorr_gb300.h. Failures throw
// std::runtime_error, as the reference's functions do.
//
// Differences from the reference: generateRandomCatalog draws a fresh seed
// from std::random_device (the reference seeds from the clock and the OpenMP
// thread number); generateRandomPosition keeps the reference's signature and
// distribution. readCatalogTxt rejects a line that lacks one of the four
// requested columns (the reference leaves that point uninitialised).
// readCatalogFits needs cfitsio, which this library does not link: it throws.
#ifndef _UTILS_HPP_
#define _UTILS_HPP_

#include <random>
#include <stdexcept>
#include <string>
#include <vector>
#include <vector_types.h>

#include "ncorr_gb300.h"

namespace ncorr_utils_detail {
inline void check(int rc) {
  if (rc != NCORR_OK) throw std::runtime_error(ncorr_last_error());
}
}  // namespace ncorr_utils_detail

// include/utils.hpp:9 of the reference.
inline std::vector<double> logspace(double start, double end, int Nedge) {
  std::vector<double> out(Nedge > 0 ? Nedge : 0);
  if (Nedge > 0) ncorr_utils_detail::check(ncorr_logspace(start, end, Nedge, out.data()));
  return out;
}

// include/utils.hpp:11 of the reference.
inline std::vector<double4> generateRandomCatalog(int Np, const double3& box) {
  std::vector<double4> p(Np > 0 ? Np : 0);
  const double b[3] = {box.x, box.y, box.z};
  std::random_device rd;
  const uint64_t seed = (static_cast<uint64_t>(rd()) << 32) ^ rd();
  ncorr_utils_detail::check(ncorr_random_catalog(static_cast<int64_t>(p.size()), b, seed,
                                                 reinterpret_cast<double*>(p.data())));
  return p;
}

// include/utils.hpp:13 of the reference.
inline double4 generateRandomPosition(std::mt19937& gen, const double3& box) {
  std::uniform_real_distribution<double> dx(0, box.x), dy(0, box.y), dz(0, box.z);
  double4 p;
  p.x = dx(gen);
  p.y = dy(gen);
  p.z = dz(gen);
  p.w = 1.0;
  return p;
}

// include/utils.hpp:15-19 of the reference.
inline void writeToFileThreeD(const std::string& filename, const std::vector<double3>& double3_vec,
                              const std::vector<double>& double_vec) {
  if (double3_vec.size() != double_vec.size()) throw std::runtime_error("Vectors have different sizes.");
  ncorr_utils_detail::check(ncorr_write_three_d(filename.c_str(), reinterpret_cast<const double*>(double3_vec.data()),
                                                double_vec.data(), static_cast<int64_t>(double_vec.size())));
}

// include/utils.hpp:21-26 of the reference.
inline void writeToFileRppi(const std::string& filename, const std::vector<double3>& double3_vec,
                            const std::vector<double2>& double2_vec, const std::vector<double>& double_vec) {
  if (double3_vec.size() != double_vec.size() || double3_vec.size() != double2_vec.size())
    throw std::runtime_error("Vectors have different sizes.");
  ncorr_utils_detail::check(ncorr_write_rppi(filename.c_str(), reinterpret_cast<const double*>(double3_vec.data()),
                                             reinterpret_cast<const double*>(double2_vec.data()), double_vec.data(),
                                             static_cast<int64_t>(double_vec.size())));
}

// include/utils.hpp:28-34 of the reference.
inline std::vector<double4> readCatalogFits(const std::string& filename, const std::vector<std::string>&, int,
                                            double, double) {
  throw std::runtime_error("readCatalogFits: FITS input needs cfitsio, which this library does not link (" +
                           filename + ")");
}

// include/utils.hpp:36-40 of the reference.
inline std::vector<double4> readCatalogTxt(const std::string& filename, const double3& box,
                                           const std::vector<int>& pos_columns) {
  if (pos_columns.size() < 4) throw std::runtime_error("readCatalogTxt: four column indices (x, y, z, w) needed");
  const double b[3] = {box.x, box.y, box.z};
  int64_t n = 0;
  ncorr_utils_detail::check(ncorr_read_catalog_txt(filename.c_str(), b, pos_columns.data(), nullptr, 0, &n));
  std::vector<double4> out(static_cast<size_t>(n));
  ncorr_utils_detail::check(
      ncorr_read_catalog_txt(filename.c_str(), b, pos_columns.data(), reinterpret_cast<double*>(out.data()), n, &n));
  return out;
}

#endif  // _UTILS_HPP_
