// Source-compatible replacement of cudaNcorr's include/survey.hpp.
//
// `survey` prepares sky catalogues for the survey-mode count: RA/Dec/z to
// Cartesian comoving coordinates (source/survey.cu:39-57 of cudaNcorr) and
// the joint shift of data and randoms into a positive box
// (source/survey.cu:94-128). Thin inline wrappers of the C ABI in
// ncorr_gb300.h; failures throw std::runtime_error.
//
// comoving_distance differs in method: the reference integrates 1/E(z) with
// GSL's QAGS to a relative tolerance of 1e-7 (source/survey.cu:26-37); this
// engine uses its own Gauss-Legendre quadrature (converged to ~1e-13), so
// distances agree with the reference within GSL's tolerance, not bit for bit.
#ifndef SURVEY_HPP
#define SURVEY_HPP

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>
#include <vector_types.h>

#include "ncorr_gb300.h"

struct cosmology {
  double H0;
  double OmegaM;
  double OmegaLambda;
};

class survey {
 public:
  survey(const cosmology& cosmo) : cosmo_(cosmo) {}

  // (RA deg, Dec deg, z, w) -> (x, y, z, w) in Mpc/h.
  std::vector<double4> convert_coordinates(const std::vector<double4>& catalog) {
    std::vector<double4> out(catalog.size());
    const double c[3] = {cosmo_.H0, cosmo_.OmegaM, cosmo_.OmegaLambda};
    check(survey_convert_coordinates(c, reinterpret_cast<const double*>(catalog.data()),
                                     static_cast<int64_t>(catalog.size()), reinterpret_cast<double*>(out.data())));
    return out;
  }

  void prep_cat_survey(std::vector<double4>& catalog, double3& box, double3& ori) {
    double b[3], o[3];
    check(survey_prep_cat(reinterpret_cast<double*>(catalog.data()), static_cast<int64_t>(catalog.size()), b, o));
    box = double3{b[0], b[1], b[2]};
    ori = double3{o[0], o[1], o[2]};
  }

  void prep_cat_survey(std::vector<double4>& catalog1, std::vector<double4>& catalog2, double3& box,
                       double3& ori) {
    double b[3], o[3];
    check(survey_prep_cat2(reinterpret_cast<double*>(catalog1.data()), static_cast<int64_t>(catalog1.size()),
                           reinterpret_cast<double*>(catalog2.data()), static_cast<int64_t>(catalog2.size()), b, o));
    box = double3{b[0], b[1], b[2]};
    ori = double3{o[0], o[1], o[2]};
  }

 private:
  static void check(int rc) {
    if (rc != NCORR_OK) throw std::runtime_error(std::string("survey: ") + ncorr_last_error());
  }
  cosmology cosmo_;
};

#endif  // SURVEY_HPP
