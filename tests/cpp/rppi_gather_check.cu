// Host check of the rppi neighbour gather's FP32 prefilter
// (rppi_gather_cut in cudancorr_gb300/csrc/rppi_fast.cuh) against the
// reference's FP64 cut of countTrianglesRppiBox / countTrianglesRppiSurvey
// (source/device.cu:317-379, :434-505 of cudaNcorr): a point the prefilter
// drops must be one the reference cuts. The kernel's FP32 arithmetic is
// repeated operation for operation; the neighbours are placed on the cut
// surfaces (rp = rpMax, rp = rpMin, |dz| = piMax, s = sMax, to within a few
// 2^-20 relative), at coordinates up to the grid's far face and through the
// periodic images.
//   rppi_gather_check <n_per_kind> <seed>
// prints "checked <n> kept <k> dropped <d> near <m> violations <v>" and exits
// 1 on a violation (a kept point dropped).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>

#include "../../cudancorr_gb300/csrc/rppi_fast.cuh"

namespace {

struct Geo {
  bool survey;
  double box;  // periodic length (box mode), or the extent the points fill (survey)
  double rpmin, rpmax, pimax;
  double cell[3];
  int nc[3];
};

Geo make_geo(bool survey, double box, double rpmin, double rpmax, int npi) {
  Geo g;
  g.survey = survey;
  g.box = box;
  g.rpmin = rpmin;
  g.rpmax = rpmax;
  g.pimax = npi;
  const double rmax = static_cast<double>(std::sqrt(static_cast<float>(rpmax * rpmax + g.pimax * g.pimax)));
  for (int d = 0; d < 3; ++d) {
    g.cell[d] = survey ? rmax : (d < 2 ? rpmax : g.pimax);
    g.nc[d] = static_cast<int>(std::ceil(box / g.cell[d]));
  }
  return g;
}

}  // namespace

int main(int argc, char** argv) {
  const long n_per_kind = argc > 1 ? std::atol(argv[1]) : 200000;
  const unsigned seed = argc > 2 ? static_cast<unsigned>(std::atoi(argv[2])) : 1u;
  std::mt19937_64 rng(seed);
  std::uniform_real_distribution<double> U(0.0, 1.0);
  long checked = 0, kept = 0, dropped = 0, near = 0, violations = 0;
  // The rppi benchmark's box, a small non-divisible box, and a survey extent.
  const Geo geos[3] = {make_geo(false, 2000.0, 1.0, 30.0, 30), make_geo(false, 100.0, 0.5, 30.0, 12),
                       make_geo(true, 3000.0, 2.0, 30.0, 20)};
  for (const Geo& g : geos) {
    const ncorr_gb300::RppiGatherCut cut =
        ncorr_gb300::rppi_gather_cut(g.nc, g.cell, g.survey, g.rpmin, g.rpmax, g.pimax);
    const double sqr_rpmax = g.rpmax * g.rpmax, sqr_rpmin = g.rpmin * g.rpmin, sqr_pimax = g.pimax * g.pimax;
    const double sqr_rmax = sqr_rpmax + sqr_pimax;
    const double smax = std::sqrt(sqr_rmax);
    const float fbox = static_cast<float>(g.box);
    auto check = [&](const double p[3], const double D[3], bool edge) {
      // The neighbour and its image: q in the grid, q + shift = p + D.
      double q[3], sh[3];
      for (int d = 0; d < 3; ++d) {
        const double q0 = p[d] + D[d];
        sh[d] = 0.0;
        q[d] = q0;
        if (!g.survey) {
          if (q0 >= g.box) {
            q[d] = q0 - g.box;
            sh[d] = g.box;
          } else if (q0 < 0.0) {
            q[d] = q0 + g.box;
            sh[d] = -g.box;
          }
        }
        if (!(q[d] > -g.cell[d] && q[d] < (g.nc[d] + 1.0) * g.cell[d])) return;  // outside the cell grid
      }
      ++checked;
      // The reference: particle2 += rShift2, then its cut in FP64.
      bool keep;
      double dd[3];
      for (int d = 0; d < 3; ++d) dd[d] = p[d] - (q[d] + sh[d]);
      if (g.survey) {
        const double x = std::fma(dd[2], dd[2], std::fma(dd[0], dd[0], dd[1] * dd[1]));
        keep = x < sqr_rmax && x > 0.0;
      } else {
        const double x = std::fma(dd[0], dd[0], dd[1] * dd[1]), y = dd[2] * dd[2];
        keep = y < sqr_pimax && x < sqr_rpmax && x > sqr_rpmin;
      }
      // The kernel's FP32 estimate (rppi_gather).
      float f[3];
      for (int d = 0; d < 3; ++d) {
        const float qf = static_cast<float>(q[d]), pf = static_cast<float>(p[d]);
        const float sf = sh[d] == 0.0 ? 0.0f : (sh[d] > 0.0 ? fbox : -fbox);
        f[d] = g.survey ? qf - pf : (qf + sf) - pf;
      }
      bool cand;
      if (g.survey) {
        cand = std::fma(f[2], f[2], std::fma(f[0], f[0], f[1] * f[1])) <= cut.s_hi;
      } else {
        const float rp = std::fma(f[0], f[0], f[1] * f[1]);
        cand = f[2] * f[2] <= cut.pi_hi && rp <= cut.rp_hi && rp >= cut.rp_lo;
      }
      kept += keep;
      dropped += !cand;
      near += edge && !cand;
      if (keep && !cand) {
        if (violations < 10)
          std::printf("violation: p (%.17g %.17g %.17g) D (%.17g %.17g %.17g)\n", p[0], p[1], p[2], D[0], D[1],
                      D[2]);
        ++violations;
      }
    };
    for (long it = 0; it < n_per_kind; ++it) {
      // Anchors anywhere in the grid, a quarter of them within a cell of a face.
      double p[3];
      for (int d = 0; d < 3; ++d) {
        const double ext = g.survey ? g.nc[d] * g.cell[d] : g.box;
        const int k = static_cast<int>(U(rng) * 8.0);
        p[d] = k == 0 ? U(rng) * g.cell[d] : (k == 1 ? ext - U(rng) * g.cell[d] : U(rng) * ext);
      }
      const double eps = std::ldexp(std::round((U(rng) - 0.5) * 16.0), -20);  // a few 2^-20 either side
      const double t = 2.0 * M_PI * U(rng);
      double D[3];
      if (g.survey) {
        // On the sphere s = sMax, and at random inside two cells.
        const double z = 2.0 * U(rng) - 1.0, r = smax * (1.0 + eps), c = std::sqrt(1.0 - z * z);
        D[0] = r * c * std::cos(t);
        D[1] = r * c * std::sin(t);
        D[2] = r * z;
        check(p, D, true);
        for (int d = 0; d < 3; ++d) D[d] = (2.0 * U(rng) - 1.0) * 2.0 * g.cell[d];
        check(p, D, false);
        continue;
      }
      // rp = rpMax, rp = rpMin, |dz| = piMax, and at random inside two cells.
      for (int kind = 0; kind < 4; ++kind) {
        const double rxy = kind == 0 ? g.rpmax * (1.0 + eps)
                                     : (kind == 1 ? g.rpmin * (1.0 + eps) : g.rpmax * std::sqrt(U(rng)));
        D[0] = rxy * std::cos(t);
        D[1] = rxy * std::sin(t);
        D[2] = kind == 2 ? (U(rng) < 0.5 ? -1.0 : 1.0) * g.pimax * (1.0 + eps) : (2.0 * U(rng) - 1.0) * g.pimax;
        if (kind == 3)
          for (int d = 0; d < 3; ++d) D[d] = (2.0 * U(rng) - 1.0) * 2.0 * g.cell[d];
        check(p, D, kind < 3);
      }
    }
  }
  std::printf("checked %ld kept %ld dropped %ld near %ld violations %ld\n", checked, kept, dropped, near, violations);
  return violations ? 1 : 0;
}
