// Host check of the rppi neighbour gather's FP32 prefilter
// (rppi_gather_cut in cudancorr_gb300/csrc/rppi_fast.cuh) against the
// reference's FP64 cut of countTrianglesRppiBox / countTrianglesRppiSurvey
// (source/device.cu:317-379, :434-505 of cudaNcorr): a point the prefilter
// drops must be one the reference cuts. The kernel's FP32 arithmetic is
// repeated operation for operation; the neighbours are placed on the cut
// surfaces (rp = rpMax, rp = rpMin, |dz| = piMax, s = sMax, to within a few
// 2^-20 relative), at coordinates up to the grid's far face and through the
// periodic images.
// Survey mode also drops list entries that are outside the rp and pi ranges
// for every partner's line of sight (rppi_los_cut); each entry it drops is
// tested against the reference's anchor-side test with partners that tilt
// the line of sight as far as the list allows.
//   rppi_gather_check <n_per_kind> <seed>
// Survey pairs that rppi_survey_index rejects or indexes are checked against
// the reference's full pair test and index.
// prints the counts of each part ("... violations <v> ... los_violations <w>
// ... pair_violations <x>") and exits 1 on a violation.
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
  // The survey line-of-sight cut. The reference's dotProduct_d3 and sqrSep as
  // nvcc contracts them: fma(a.z, b.z, fma(a.x, b.x, a.y * b.y)).
  long los_checked = 0, los_cut = 0, los_partners = 0, los_violations = 0;
  {
    const double rpmin = 2.0, rpmax = 30.0, pimax = 20.0;
    const double sqr_rpmin = rpmin * rpmin, sqr_rpmax = rpmax * rpmax, sqr_pimax = pimax * pimax;
    const double sqr_rmax = sqr_rpmax + sqr_pimax, smax = std::sqrt(sqr_rmax);
    auto up = [](double x) {
      float f = static_cast<float>(x);
      return static_cast<double>(f) < x ? std::nextafter(f, INFINITY) : f;
    };
    auto down = [](double x) {
      float f = static_cast<float>(x);
      return static_cast<double>(f) > x ? std::nextafter(f, -INFINITY) : f;
    };
    const float smax_f = up(smax), pimax2_f = static_cast<float>(sqr_pimax), rpmax2_f = up(sqr_rpmax),
                rpmin2_f = down(sqr_rpmin);
    auto dot = [](const double a[3], const double b[3]) { return std::fma(a[2], b[2], std::fma(a[0], b[0], a[1] * b[1])); };
    auto unit = [&](double v[3]) {
      const double n = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
      for (int d = 0; d < 3; ++d) v[d] /= n;
    };
    std::normal_distribution<double> N(0.0, 1.0);
    for (long it = 0; it < n_per_kind; ++it) {
      // Anchor, observer offset (only ori.x enters the reference's line of
      // sight) and A; |A| from 60 (wide tilt) to 3000.
      const double ori_x = (U(rng) - 0.5) * 200.0;
      double dir[3] = {N(rng), N(rng), N(rng)};
      unit(dir);
      const double an = 60.0 * std::pow(50.0, U(rng));
      const double p1[3] = {ori_x + an * dir[0], an * dir[1], an * dir[2]};
      const double A[3] = {p1[0] - ori_x, p1[1], p1[2]};
      // Entry on the cylinder's surfaces as seen along A, or anywhere in the
      // sphere: offset d = p1 - pj at |d| < sMax.
      double e1[3] = {N(rng), N(rng), N(rng)};
      const double ad = dot(e1, dir);
      for (int d = 0; d < 3; ++d) e1[d] -= ad * dir[d];
      unit(e1);
      const int kind = static_cast<int>(U(rng) * 4.0);
      const double wig = 1.0 + (U(rng) - 0.5) * 0.2;
      double along = (2.0 * U(rng) - 1.0) * pimax, across = rpmax * std::sqrt(U(rng));
      if (kind == 0) along = (U(rng) < 0.5 ? -1.0 : 1.0) * pimax * wig;
      if (kind == 1) across = rpmax * wig;
      if (kind == 2) across = rpmin * wig;
      double dv[3];
      for (int d = 0; d < 3; ++d) dv[d] = along * dir[d] + across * e1[d];
      if (kind == 3)
        for (int d = 0; d < 3; ++d) dv[d] = (2.0 * U(rng) - 1.0) * smax;
      const double pj[3] = {p1[0] - dv[0], p1[1] - dv[1], p1[2] - dv[2]};
      double d64[3] = {p1[0] - pj[0], p1[1] - pj[1], p1[2] - pj[2]};
      const double s2 = dot(d64, d64);
      if (!(s2 < sqr_rmax && s2 > 0.0)) continue;
      ++los_checked;
      // The kernel's inputs: FP32 offset, s^2 and A.
      const float ax = static_cast<float>(A[0]), ay = static_cast<float>(A[1]), az = static_cast<float>(A[2]);
      const float4 los = {ax, ay, az, std::sqrt(std::fma(az, az, std::fma(ay, ay, ax * ax)))};
      if (!ncorr_gb300::rppi_los_cut(static_cast<float>(d64[0]), static_cast<float>(d64[1]),
                                     static_cast<float>(d64[2]), static_cast<float>(s2), los, smax_f, pimax2_f,
                                     rpmax2_f, rpmin2_f))
        continue;
      ++los_cut;
      // Partners within sMax: the directions that tilt L towards and away
      // from d and across, at the sphere's edge, and random ones.
      double perp[3] = {dv[1] * dir[2] - dv[2] * dir[1], dv[2] * dir[0] - dv[0] * dir[2],
                        dv[0] * dir[1] - dv[1] * dir[0]};
      double dperp[3];
      const double dd = dot(dv, dir);
      for (int d = 0; d < 3; ++d) dperp[d] = dv[d] - dd * dir[d];
      const bool has_perp = dot(perp, perp) > 1e-20 && dot(dperp, dperp) > 1e-20;
      if (has_perp) {
        unit(perp);
        unit(dperp);
      }
      for (int k = 0; k < 24; ++k) {
        double w[3];
        if (k < 6 && has_perp) {
          const double* b = k < 2 ? dperp : (k < 4 ? perp : dir);
          for (int d = 0; d < 3; ++d) w[d] = (k % 2 ? -1.0 : 1.0) * b[d];
        } else {
          w[0] = N(rng), w[1] = N(rng), w[2] = N(rng);
          unit(w);
        }
        const double r = smax * (k < 12 ? 0.999999 : U(rng));
        const double pl[3] = {p1[0] + r * w[0], p1[1] + r * w[1], p1[2] + r * w[2]};
        double dl[3] = {p1[0] - pl[0], p1[1] - pl[1], p1[2] - pl[2]};
        const double s2l = dot(dl, dl);
        if (!(s2l < sqr_rmax && s2l > 0.0)) continue;
        ++los_partners;
        // getLOS, getSqrSdotL, getSqrRpSqrPi (source/device.cu:45-68) for
        // the side (p1, pj).
        const double L[3] = {((p1[0] - ori_x) + (pj[0] - ori_x)) + (pl[0] - ori_x), (p1[1] + pj[1]) + pl[1],
                             (p1[2] + pj[2]) + pl[2]};
        const double sqrL = dot(L, L);
        const double t = dot(L, d64);
        const double q1 = t * t;
        const bool cut_here = sqr_pimax * sqrL < q1;
        const double pi1 = q1 / sqrL, rp1 = s2 - pi1;
        const bool side_ok = !cut_here && rp1 < sqr_rpmax && rp1 > sqr_rpmin && pi1 < sqr_pimax;
        if (side_ok) {
          if (los_violations < 10)
            std::printf("los violation: A %.6g d (%.9g %.9g %.9g) pl (%.9g %.9g %.9g) rp1 %.9g pi1 %.9g\n", an,
                        d64[0], d64[1], d64[2], dl[0], dl[1], dl[2], rp1, pi1);
          ++los_violations;
        }
      }
    }
  }
  // The survey pair classifier (rppi_survey_index): a pair it rejects must
  // not be counted by the reference (source/device.cu:455-490), and a pair
  // it indexes must be counted at that index (getTriangleIndexRppi,
  // :203-255, restated below in FP64).
  long pair_checked = 0, pair_cut = 0, pair_idx = 0, pair_near = 0, pair_violations = 0;
  {
    const double rpmin = 2.0, rpmax = 30.0, pimax = 20.0;
    const int nb = 8, npi = 20;
    const double sqr_rpmin = rpmin * rpmin, sqr_rpmax = rpmax * rpmax, sqr_pimax = pimax * pimax;
    const double sqr_rmax = sqr_rpmax + sqr_pimax, smax = std::sqrt(sqr_rmax);
    auto up = [](double x) {
      float f = static_cast<float>(x);
      return static_cast<double>(f) < x ? std::nextafter(f, INFINITY) : f;
    };
    auto down = [](double x) {
      float f = static_cast<float>(x);
      return static_cast<double>(f) > x ? std::nextafter(f, -INFINITY) : f;
    };
    double edges[nb + 1], sb[nb + 1];
    for (int i = 0; i <= nb; ++i) {
      edges[i] = std::pow(10.0, std::log10(rpmin) + i * (std::log10(rpmax) - std::log10(rpmin)) / nb);
      sb[i] = edges[i] * edges[i];
    }
    const double u = std::ldexp(1.0, -24);
    ncorr_gb300::RppiFast f;
    f.epi = up(64.0 * u * sqr_pimax);
    f.erp = up(128.0 * u * sqr_rpmax);
    f.pimax2 = static_cast<float>(sqr_pimax);
    f.rpmax2_lo = down(sqr_rpmax);
    f.rpmax2_hi = up(sqr_rpmax);
    f.rpmin2_lo = down(sqr_rpmin);
    f.rpmin2_hi = up(sqr_rpmin);
    f.hm = -up(128.0 * u * sqr_rpmax);
    f.pmarg = up(16.0 * u * sqr_pimax);
    f.nb = nb;
    f.npi = npi;
    float e2lo[nb + 1], e2hi[nb + 1];
    for (int i = 0; i <= nb; ++i) {
      e2lo[i] = down(sb[i]);
      e2hi[i] = up(sb[i]);
    }
    f.tab_band = 4.0f * f.erp;
    f.tab_scale = ncorr_gb300::rppi_tab_scale(f.rpmax2_hi, f.tab_band);
    static unsigned char tab[ncorr_gb300::kRppiTab];
    ncorr_gb300::rppi_build_table(f, e2lo, e2hi, tab);
    const float smax_f = up(smax);
    auto dot = [](const double a[3], const double b[3]) { return std::fma(a[2], b[2], std::fma(a[0], b[0], a[1] * b[1])); };
    auto sep = [&](const double a[3], const double b[3]) {
      const double d[3] = {a[0] - b[0], a[1] - b[1], a[2] - b[2]};
      return dot(d, d);
    };
    auto unit = [&](double v[3]) {
      const double n = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
      for (int d = 0; d < 3; ++d) v[d] /= n;
    };
    auto ebin = [&](double r) {
      int b = 0;
      for (int i = 1; i < nb; ++i)
        if (r >= sb[i]) b = i;
      return b;
    };
    std::normal_distribution<double> N(0.0, 1.0);
    for (long it = 0; it < n_per_kind; ++it) {
      const double ori_x = (U(rng) - 0.5) * 200.0;
      double dir[3] = {N(rng), N(rng), N(rng)};
      unit(dir);
      const double an = 60.0 * std::pow(50.0, U(rng));
      const double p1[3] = {ori_x + an * dir[0], an * dir[1], an * dir[2]};
      const double A[3] = {p1[0] - ori_x, p1[1], p1[2]};
      double e1[3] = {N(rng), N(rng), N(rng)};
      const double ad = dot(e1, dir);
      for (int d = 0; d < 3; ++d) e1[d] -= ad * dir[d];
      unit(e1);
      // pj and pl around p1; for kinds 0-6 a point is re-placed a few times
      // against the pair's own line of sight L (which depends on it) until
      // the chosen quantity sits on its limit to within 1e-6 relative: pi3,
      // rp3 or pi1 on the cut, rp1 or rp3 on a bin edge, pi1 on an integer,
      // or rp1 = rp2 exactly (pl the mirror image of pj across L).
      const int kind = static_cast<int>(U(rng) * 8.0);
      const double eps = (U(rng) - 0.5) * 2e-6;
      auto rnd = [&](double r) { return (2.0 * U(rng) - 1.0) * r; };
      double pj[3], pl[3];
      for (int d = 0; d < 3; ++d) {
        pj[d] = p1[d] + rnd(pimax) * dir[d] + rnd(rpmax * 0.7) * e1[d];
        pl[d] = p1[d] + rnd(smax * 0.57) * dir[d] + rnd(smax * 0.57) * e1[d];
      }
      const double sgn = U(rng) < 0.5 ? -1.0 : 1.0, side = rnd(10.0), t0 = 2.0 * M_PI * U(rng);
      const double edge = edges[1 + static_cast<int>(U(rng) * (nb - 1))];
      const double kpi = 1.0 + static_cast<int>(U(rng) * (pimax - 1.0));
      for (int iter = 0; kind < 7 && iter < 8; ++iter) {
        double Lh[3] = {((p1[0] - ori_x) + (pj[0] - ori_x)) + (pl[0] - ori_x), (p1[1] + pj[1]) + pl[1],
                        (p1[2] + pj[2]) + pl[2]};
        unit(Lh);
        double f1[3] = {e1[0], e1[1], e1[2]};
        const double fd = dot(f1, Lh);
        for (int d = 0; d < 3; ++d) f1[d] -= fd * Lh[d];
        unit(f1);
        const double f2[3] = {Lh[1] * f1[2] - Lh[2] * f1[1], Lh[2] * f1[0] - Lh[0] * f1[2],
                              Lh[0] * f1[1] - Lh[1] * f1[0]};
        const double cs = std::cos(t0), sn = std::sin(t0);
        double dj[3];
        for (int d = 0; d < 3; ++d) dj[d] = pj[d] - p1[d];
        const double tj = dot(dj, Lh);
        for (int d = 0; d < 3; ++d) {
          if (kind == 0) pl[d] = pj[d] + sgn * pimax * (1.0 + eps) * Lh[d] + side * f1[d];
          if (kind == 1) pl[d] = pj[d] + side * Lh[d] + rpmax * (1.0 + eps) * (cs * f1[d] + sn * f2[d]);
          if (kind == 2) pj[d] = p1[d] + sgn * pimax * (1.0 + eps) * Lh[d] + side * f1[d];
          if (kind == 3) pj[d] = p1[d] + side * Lh[d] + edge * (1.0 + eps) * (cs * f1[d] + sn * f2[d]);
          if (kind == 4) pl[d] = pj[d] + side * Lh[d] + edge * (1.0 + eps) * (cs * f1[d] + sn * f2[d]);
          if (kind == 5) pj[d] = p1[d] + sgn * kpi * (1.0 + eps) * Lh[d] + 0.5 * rpmax * (cs * f1[d] + sn * f2[d]);
          if (kind == 6) pl[d] = p1[d] + tj * Lh[d] - (dj[d] - tj * Lh[d]);
        }
      }
      const double s1 = sep(p1, pj), s2 = sep(p1, pl);
      if (!(s1 < sqr_rmax && s1 > 0.0 && s2 < sqr_rmax && s2 > 0.0)) continue;  // list entries only
      ++pair_checked;
      // The kernel's inputs: FP32 offsets q - p1 with fl32(s^2), and A.
      const float4 dj = {static_cast<float>(pj[0] - p1[0]), static_cast<float>(pj[1] - p1[1]),
                         static_cast<float>(pj[2] - p1[2]), static_cast<float>(s1)};
      const float4 dl = {static_cast<float>(pl[0] - p1[0]), static_cast<float>(pl[1] - p1[1]),
                         static_cast<float>(pl[2] - p1[2]), static_cast<float>(s2)};
      const float4 los = {static_cast<float>(A[0]), static_cast<float>(A[1]), static_cast<float>(A[2]), 0.0f};
      const int got = ncorr_gb300::rppi_survey_index(dj, dl, los, smax_f, f, tab);
      if (got == ncorr_gb300::kRppiUncertain) continue;
      if (got < 0)
        ++pair_cut;
      else
        ++pair_idx;
      pair_near += kind < 7;
      // The reference's decision and index for (p1, pj, pl).
      long long ref = -1;
      const double s3 = sep(pj, pl);
      if (s3 < sqr_rmax && s3 > 0.0) {
        const double L[3] = {((p1[0] - ori_x) + (pj[0] - ori_x)) + (pl[0] - ori_x), (p1[1] + pj[1]) + pl[1],
                             (p1[2] + pj[2]) + pl[2]};
        const double sqrL = dot(L, L), pm = sqr_pimax * sqrL;
        const double d1[3] = {p1[0] - pj[0], p1[1] - pj[1], p1[2] - pj[2]};
        const double d2[3] = {p1[0] - pl[0], p1[1] - pl[1], p1[2] - pl[2]};
        const double d3[3] = {pj[0] - pl[0], pj[1] - pl[1], pj[2] - pl[2]};
        const double q1 = dot(L, d1) * dot(L, d1), q2 = dot(L, d2) * dot(L, d2), q3 = dot(L, d3) * dot(L, d3);
        if (!(pm < q1) && !(pm < q2) && !(pm < q3)) {
          double qq[3] = {q1 / sqrL, q2 / sqrL, q3 / sqrL};
          double rr[3] = {s1 - qq[0], s2 - qq[1], s3 - qq[2]};
          if (rr[0] < sqr_rpmax && rr[1] < sqr_rpmax && rr[2] < sqr_rpmax && rr[0] > sqr_rpmin &&
              rr[1] > sqr_rpmin && rr[2] > sqr_rpmin && qq[0] < sqr_pimax && qq[1] < sqr_pimax) {
            double t;
            if (rr[0] > rr[1]) { t = rr[0]; rr[0] = rr[1]; rr[1] = t; t = qq[0]; qq[0] = qq[1]; qq[1] = t; }
            if (rr[0] > rr[2]) { t = rr[0]; rr[0] = rr[2]; rr[2] = t; t = qq[0]; qq[0] = qq[2]; qq[2] = t; }
            if (rr[1] > rr[2]) { t = rr[1]; rr[1] = rr[2]; rr[2] = t; t = qq[1]; qq[1] = qq[2]; qq[2] = t; }
            const float r1 = std::sqrt(static_cast<float>(rr[0])), r2 = std::sqrt(static_cast<float>(rr[1])),
                        r3 = std::sqrt(static_cast<float>(rr[2]));
            if (!(r1 + r2 <= r3)) {
              const long long P = npi, B = nb;
              const long long p1b = static_cast<long long>(std::floor(std::sqrt(static_cast<float>(qq[0]))));
              const long long p2b = static_cast<long long>(std::floor(std::sqrt(static_cast<float>(qq[1]))));
              ref = p2b + p1b * P + ebin(rr[2]) * P * P + ebin(rr[1]) * B * P * P + ebin(rr[0]) * B * B * P * P;
            }
          }
        }
      }
      if (static_cast<long long>(got) != ref) {
        if (pair_violations < 10)
          std::printf("pair violation: kind %d got %d ref %lld A %.6g pj-p1 (%.9g %.9g %.9g) pl-p1 (%.9g %.9g %.9g)\n",
                      kind, got, ref, an, pj[0] - p1[0], pj[1] - p1[1], pj[2] - p1[2], pl[0] - p1[0], pl[1] - p1[1],
                      pl[2] - p1[2]);
        ++pair_violations;
      }
    }
  }
  std::printf("checked %ld kept %ld dropped %ld near %ld violations %ld los_checked %ld los_cut %ld los_partners %ld "
              "los_violations %ld pair_checked %ld pair_cut %ld pair_idx %ld pair_near %ld pair_violations %ld\n",
              checked, kept, dropped, near, violations, los_checked, los_cut, los_partners, los_violations,
              pair_checked, pair_cut, pair_idx, pair_near, pair_violations);
  return violations || los_violations || pair_violations ? 1 : 0;
}
