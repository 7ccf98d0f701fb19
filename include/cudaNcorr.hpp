// Source-compatible replacement of cudaNcorr's include/cudaNcorr.hpp.
//
// A program written against the reference's class `ncorr` (for example the
// box example of the reference's source/main.cu:20-45) compiles unchanged
// against this header and links against libcudancorr_gb300.so. The class is a
// thin inline wrapper of the C ABI in ncorr_gb300.h: every call maps to one C
// entry point, and failures throw std::runtime_error as the reference does
// (include/gpuerrchk.h:8-15 and source/cudaNcorr.cu:120-122 of cudaNcorr).
//
// Differences from the reference, all on inputs where the reference has
// undefined behaviour: points outside the reference's cell grid, non-finite
// values, and edges that are not strictly increasing and non-negative are
// rejected with std::runtime_error. Instances hold a device handle and are
// movable, not copyable.
#ifndef _CUDANCORR_HPP_
#define _CUDANCORR_HPP_

#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>
#include <vector_types.h>

#include "ncorr_gb300.h"

class ncorr {
 public:
  enum binType { threeD, rppi, smu };

  // include/cudaNcorr.hpp:14 of the reference.
  ncorr(double3 box, int bin_type, std::vector<double>& bins, bool isSurvey, double3 ori) {
    const double b[3] = {box.x, box.y, box.z};
    const double o[3] = {ori.x, ori.y, ori.z};
    check(ncorr_create(b, bin_type, bins.data(), static_cast<int>(bins.size()), isSurvey ? 1 : 0, o, &h_));
  }

  // include/cudaNcorr.hpp:15 of the reference (rppi).
  ncorr(double3 box, int bin_type, std::vector<double>& bins, int numMinorBins, bool isSurvey,
        double3 ori) {
    const double b[3] = {box.x, box.y, box.z};
    const double o[3] = {ori.x, ori.y, ori.z};
    check(ncorr_create_rppi(b, bin_type, bins.data(), static_cast<int>(bins.size()), numMinorBins,
                            isSurvey ? 1 : 0, o, &h_));
  }

  ~ncorr() { ncorr_destroy(h_); }
  ncorr(const ncorr&) = delete;
  ncorr& operator=(const ncorr&) = delete;
  ncorr(ncorr&& o) noexcept : h_(std::exchange(o.h_, nullptr)) {}
  ncorr& operator=(ncorr&& o) noexcept {
    if (this != &o) {
      ncorr_destroy(h_);
      h_ = std::exchange(o.h_, nullptr);
    }
    return *this;
  }

  // include/cudaNcorr.hpp:19 of the reference. Passing the same vector for
  // p2 and p3 (or for all three) lets the engine grid it once.
  void calculateD1D2D3(std::vector<double4>& p1, std::vector<double4>& p2, std::vector<double4>& p3) {
    check(ncorr_calculate_d1d2d3(h_, reinterpret_cast<const double*>(p1.data()),
                                 static_cast<int64_t>(p1.size()), reinterpret_cast<const double*>(p2.data()),
                                 static_cast<int64_t>(p2.size()), reinterpret_cast<const double*>(p3.data()),
                                 static_cast<int64_t>(p3.size())));
  }

  // include/cudaNcorr.hpp:21 of the reference.
  std::vector<double3> getTriBinsOut() const {
    const int64_t n = ncorr_num_out(h_);
    std::vector<double> flat(static_cast<size_t>(3 * n));
    check(ncorr_get_tri_bins_out(h_, flat.data(), 3 * n));
    std::vector<double3> out(static_cast<size_t>(n));
    for (int64_t i = 0; i < n; ++i) out[i] = double3{flat[3 * i], flat[3 * i + 1], flat[3 * i + 2]};
    return out;
  }

  // include/cudaNcorr.hpp:23 of the reference: (l, m) pi bins of every
  // output entry for rppi, empty for threeD.
  std::vector<double2> getPiBinsOut() const {
    int64_t n = 0;
    if (ncorr_num_pi_bins(h_) == 0) {
      double dummy = 0.0;
      check(ncorr_get_pi_bins_out(h_, &dummy, 0, &n));
      return std::vector<double2>(static_cast<size_t>(n));
    }
    const int64_t m = ncorr_num_out(h_);
    std::vector<double> flat(static_cast<size_t>(2 * m));
    check(ncorr_get_pi_bins_out(h_, flat.data(), 2 * m, &n));
    std::vector<double2> out(static_cast<size_t>(n));
    for (int64_t i = 0; i < n; ++i) out[i] = double2{flat[2 * i], flat[2 * i + 1]};
    return out;
  }

  // include/cudaNcorr.hpp:25 of the reference.
  std::vector<double> getTriCountsOut() const {
    std::vector<double> out(static_cast<size_t>(ncorr_num_out(h_)));
    check(ncorr_get_tri_counts_out(h_, out.data(), static_cast<int64_t>(out.size())));
    return out;
  }

  // The full histogram (the reference's private triCountsAll_): nb^3
  // entries, nb^3 * numPiBins^2 for rppi.
  std::vector<double> getTriCountsAll() const {
    const int nb = ncorr_num_bins(h_);
    const int npi = ncorr_num_pi_bins(h_);
    std::vector<double> out(static_cast<size_t>(nb) * nb * nb * (npi > 0 ? static_cast<size_t>(npi) * npi : 1));
    check(ncorr_get_tri_counts_all(h_, out.data(), static_cast<int64_t>(out.size())));
    return out;
  }

 private:
  static void check(int rc) {
    if (rc != NCORR_OK) throw std::runtime_error(std::string("ncorr: ") + ncorr_last_error());
  }
  ncorr_handle* h_ = nullptr;
};

#endif  // _CUDANCORR_HPP_
