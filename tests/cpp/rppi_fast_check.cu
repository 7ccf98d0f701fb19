// Host check of the FP32 rppi classifier (cudancorr_gb300/csrc/rppi_fast.cuh)
// against the exact computation of the reference's box kernel, restated here
// in FP64 (countTrianglesRppiBox / getTriangleIndexRppi, source/device.cu:
// 203-255, :317-379 of cudaNcorr): whenever the classifier answers, its
// answer must be the reference's. Random triangles plus adversarial ones
// (third side on a bin edge, equal to an anchor side, pi3 next to k^2, nearly
// collinear) are generated around random anchors.
//   rppi_fast_check <n_per_kind> <seed>
// prints "checked <n> certain <m> mismatches <k>" and exits 1 on a mismatch.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

#include "../../cudancorr_gb300/csrc/rppi_fast.cuh"

using ncorr_gb300::RppiFast;

namespace {

struct P3 {
  double x, y, z;
};

const double kU = std::ldexp(1.0, -24);

float f32_down(double x) {
  float f = static_cast<float>(x);
  if (static_cast<double>(f) > x) f = std::nextafter(f, -INFINITY);
  return f;
}
float f32_up(double x) {
  float f = static_cast<float>(x);
  if (static_cast<double>(f) < x) f = std::nextafter(f, INFINITY);
  return f;
}

// sqrRpBox as nvcc contracts it: fma(dx, dx, dy*dy).
double rp_of(const P3& a, const P3& b) {
  const double dx = a.x - b.x, dy = a.y - b.y;
  return std::fma(dx, dx, dy * dy);
}
double pi_of(const P3& a, const P3& b) {
  const double dz = a.z - b.z;
  return dz * dz;
}

int exact_bin(double r, const std::vector<double>& sb) {
  int idx = -1;
  for (size_t i = 0; i + 1 < sb.size(); ++i)
    if (r >= sb[i] && r < sb[i + 1]) idx = static_cast<int>(i);
  return idx;
}

// getTriangleIndexRppi on exact values.
long long ref_index(double r1, double r2, double r3, double q1, double q2, double q3, const std::vector<double>& sb,
                    int npi) {
  double t;
  if (r1 > r2) { t = r1; r1 = r2; r2 = t; t = q1; q1 = q2; q2 = t; }
  if (r1 > r3) { t = r1; r1 = r3; r3 = t; t = q1; q1 = q3; q3 = t; }
  if (r2 > r3) { t = r2; r2 = r3; r3 = t; t = q2; q2 = q3; q3 = t; }
  if (std::sqrt(static_cast<float>(r1)) + std::sqrt(static_cast<float>(r2)) <= std::sqrt(static_cast<float>(r3)))
    return -1;
  const long long i1 = exact_bin(r1, sb), i2 = exact_bin(r2, sb), i3 = exact_bin(r3, sb);
  const long long p1 = static_cast<long long>(std::floor(std::sqrt(static_cast<float>(q1))));
  const long long p2 = static_cast<long long>(std::floor(std::sqrt(static_cast<float>(q2))));
  const long long P = npi, B = static_cast<long long>(sb.size()) - 1;
  return p2 + p1 * P + i3 * P * P + i2 * B * P * P + i1 * B * B * P * P;
}

}  // namespace

int main(int argc, char** argv) {
  const long n_per_kind = argc > 1 ? std::atol(argv[1]) : 200000;
  const unsigned seed = argc > 2 ? static_cast<unsigned>(std::atoi(argv[2])) : 1u;
  // Binning of the rppi benchmark: 12 log rp bins in [1, 30), 30 unit pi bins.
  const int nb = 12, npi = 30;
  std::vector<double> edges(nb + 1);
  for (int i = 0; i <= nb; ++i) edges[i] = std::pow(10.0, std::log10(1.0) + i * (std::log10(30.0) / nb));
  std::vector<double> sb(nb + 1);
  for (int i = 0; i <= nb; ++i) sb[i] = edges[i] * edges[i];
  const double rpmax = edges[nb], rpmin = edges[0], pimax = npi;
  const double sqr_rpmax = rpmax * rpmax, sqr_rpmin = rpmin * rpmin, sqr_pimax = pimax * pimax;
  RppiFast f;
  f.epi = f32_up(64.0 * kU * sqr_pimax);
  f.erp = f32_up(128.0 * kU * sqr_rpmax);
  f.pimax2 = static_cast<float>(sqr_pimax);
  f.rpmax2_lo = f32_down(sqr_rpmax);
  f.rpmax2_hi = f32_up(sqr_rpmax);
  f.rpmin2_lo = f32_down(sqr_rpmin);
  f.rpmin2_hi = f32_up(sqr_rpmin);
  f.hm = -f32_up(128.0 * kU * sqr_rpmax);
  f.pmarg = f32_up(16.0 * kU * sqr_pimax);
  f.nb = nb;
  f.npi = npi;
  std::vector<float> e2lo(nb + 1), e2hi(nb + 1);
  for (int i = 0; i <= nb; ++i) {
    e2lo[i] = f32_down(sb[i]);
    e2hi[i] = f32_up(sb[i]);
  }
  f.tab_band = f.erp;
  f.tab_scale = ncorr_gb300::rppi_tab_scale(f.rpmax2_hi, f.tab_band);
  std::vector<unsigned char> tab(ncorr_gb300::kRppiTab);
  ncorr_gb300::rppi_build_table(f, e2lo.data(), e2hi.data(), tab.data());

  std::mt19937_64 rng(seed);
  std::uniform_real_distribution<double> U(0.0, 1.0);
  auto in_cyl = [&](const P3& c, double rmax, double zmax) {
    const double r = rmax * std::sqrt(U(rng)), t = 2 * M_PI * U(rng);
    return P3{c.x + r * std::cos(t), c.y + r * std::sin(t), c.z + (2 * U(rng) - 1) * zmax};
  };
  long checked = 0, certain = 0, mismatches = 0, counted = 0;
  auto check = [&](const P3& a, const P3& pj, const P3& pl) {
    const double A = rp_of(a, pj), Pj = pi_of(a, pj), B = rp_of(a, pl), Pl = pi_of(a, pl);
    if (!(Pj < sqr_pimax && A < sqr_rpmax && A > sqr_rpmin)) return;  // not list entries
    if (!(Pl < sqr_pimax && B < sqr_rpmax && B > sqr_rpmin)) return;
    ++checked;
    // The reference's decision for (anchor, j, l).
    const double P3v = pi_of(pj, pl), C = rp_of(pj, pl);
    long long ref = -1;
    if (P3v < sqr_pimax && C < sqr_rpmax && C > sqr_rpmin) ref = ref_index(A, B, C, Pj, Pl, P3v, sb, npi);
    // The classifier's inputs, as the kernel's list build forms them.
    const float xj = static_cast<float>(pj.x - a.x), yj = static_cast<float>(pj.y - a.y),
                zj = static_cast<float>(pj.z - a.z);
    const float xl = static_cast<float>(pl.x - a.x), yl = static_cast<float>(pl.y - a.y),
                zl = static_cast<float>(pl.z - a.z);
    const float rj = std::sqrt(static_cast<float>(A)), rl = std::sqrt(static_cast<float>(B));
    const unsigned mj = static_cast<unsigned>(exact_bin(A, sb)) |
                        (static_cast<unsigned>(std::floor(std::sqrt(static_cast<float>(Pj)))) << 16);
    const unsigned ml = static_cast<unsigned>(exact_bin(B, sb)) |
                        (static_cast<unsigned>(std::floor(std::sqrt(static_cast<float>(Pl)))) << 16);
    const long long got =
        ncorr_gb300::rppi_fast_index(xj, yj, zj, rj, mj, xl, yl, zl, rl, ml, f, tab.data());
    if (got == ncorr_gb300::kRppiUncertain) return;
    ++certain;
    if (got >= 0) ++counted;
    if (got != ref) {
      if (mismatches < 10)
        std::printf("mismatch: got %lld ref %lld  A %.17g B %.17g C %.17g Pj %.17g Pl %.17g P3 %.17g\n", got, ref, A,
                    B, C, Pj, Pl, P3v);
      ++mismatches;
    }
  };
  for (long it = 0; it < n_per_kind; ++it) {
    const P3 a{500.0 + 100.0 * U(rng), 500.0 + 100.0 * U(rng), 500.0 + 100.0 * U(rng)};
    // 1. random pair in the anchor's cylinder
    P3 pj = in_cyl(a, rpmax, pimax), pl = in_cyl(a, rpmax, pimax);
    check(a, pj, pl);
    // 2. third side's rp^2 on a bin edge: pl at distance edge e from pj in xy
    {
      const double e = edges[1 + static_cast<int>(U(rng) * (nb - 1))];
      const double t = 2 * M_PI * U(rng);
      pl = P3{pj.x + e * std::cos(t), pj.y + e * std::sin(t), pj.z + (2 * U(rng) - 1) * 5.0};
      check(a, pj, pl);
    }
    // 3. third side equal (to rounding) to the anchor side j: isosceles in xy
    {
      const double r = std::sqrt(rp_of(a, pj));
      const double t = 2 * M_PI * U(rng);
      pl = P3{pj.x + r * std::cos(t), pj.y + r * std::sin(t), a.z + (2 * U(rng) - 1) * 10.0};
      check(a, pj, pl);
      // anchor sides equal: pl on the circle of radius |a - pj| around a
      pl = P3{a.x + r * std::cos(t), a.y + r * std::sin(t), a.z + (2 * U(rng) - 1) * 10.0};
      check(a, pj, pl);
    }
    // 4. pi3 next to k^2: |dz3| = k up to a few ulps
    {
      const int k = 1 + static_cast<int>(U(rng) * (npi - 1));
      const double eps = (2 * U(rng) - 1) * 1e-6 * k;
      pl = in_cyl(a, rpmax, pimax);
      pl.z = pj.z + (U(rng) < 0.5 ? -1 : 1) * (k + eps);
      check(a, pj, pl);
    }
    // 5. nearly collinear in xy
    {
      const double s = U(rng);
      pl = P3{a.x + s * (pj.x - a.x) + 1e-6 * (2 * U(rng) - 1), a.y + s * (pj.y - a.y), pj.z + (2 * U(rng) - 1)};
      check(a, pj, pl);
      pl = P3{a.x + (1 + s) * (pj.x - a.x), a.y + (1 + s) * (pj.y - a.y) + 1e-7, pj.z};
      check(a, pj, pl);
    }
  }
  std::printf("checked %ld certain %ld counted %ld mismatches %ld\n", checked, certain, counted, mismatches);
  return mismatches ? 1 : 0;
}
