// Compiles against this repository's include/ exactly as a program written
// for the reference's headers would (the calls of the reference's
// source/main.cu:21-45 that need no GPU), then exercises them:
//   utils_roundtrip <dir>
// writes <dir>/cat.txt, reads it back, writes both result formats.
#include <cstdio>
#include <string>
#include <vector>

#include "cudaNcorr.hpp"
#include "survey.hpp"
#include "utils.hpp"

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  const std::string dir = argv[1];
  std::vector<double> bins = logspace(0.1, 20.0, 13);
  double3 box = {100.0, 100.0, 100.0};
  std::vector<double4> r = generateRandomCatalog(1000, box);
  for (const double4& p : r)
    if (!(p.x >= 0 && p.x < box.x && p.y >= 0 && p.y < box.y && p.z >= 0 && p.z < box.z && p.w == 1.0)) return 3;
  FILE* f = std::fopen((dir + "/cat.txt").c_str(), "w");
  for (const double4& p : r) std::fprintf(f, "%.17g %.17g %.17g %.17g\n", p.w, p.x, p.y, p.z);
  std::fclose(f);
  std::vector<double4> q = readCatalogTxt(dir + "/cat.txt", box, {1, 2, 3, 0});
  if (q.size() != r.size()) return 4;
  for (size_t i = 0; i < q.size(); ++i)
    if (q[i].x != r[i].x || q[i].y != r[i].y || q[i].z != r[i].z || q[i].w != r[i].w) return 5;
  std::vector<double3> tri = {{1.5, 2.5, 3.5}, {0.25, 1.0, 1.125}};
  std::vector<double2> pis = {{0.0, 1.0}, {2.0, 3.0}};
  std::vector<double> counts = {6.0, 1234567.0};
  writeToFileThreeD(dir + "/three_d.dat", tri, counts);
  writeToFileRppi(dir + "/rppi.dat", tri, pis, counts);
  bool threw = false;
  try {
    readCatalogTxt(dir + "/missing.txt", box, {0, 1, 2, 3});
  } catch (const std::runtime_error&) {
    threw = true;
  }
  if (!threw) return 6;
  std::printf("%zu %.6f\n", q.size(), bins.back());
  return 0;
}
