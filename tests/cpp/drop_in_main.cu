// A program written for the reference's public headers (the calls its
// example driver source/main.cu:20-45 and the survey example after it make),
// built with nvcc against this repository's include/ and run on the GPU:
//
//   drop_in_main <dir>
//
// reads <dir>/box.txt, <dir>/data.txt and <dir>/randoms.txt (columns
// x y z w), then
//   * box threeD: ncorr(box, 0, bins, false, {0,0,0}), calculateD1D2D3(p,p,p),
//     getTriBinsOut / getTriCountsOut -> <dir>/ddd_box.dat;
//   * survey threeD: prep_cat_survey(data, randoms, box, ori) with a
//     `survey` object, ncorr(box, 0, bins, true, ori), DDR ->
//     <dir>/ddr_survey.dat, and the shifted catalogues' box/ori ->
//     <dir>/survey_geometry.txt;
//   * box rppi: ncorr(box, 1, rp_bins, 8, false, {0,0,0}), calculateD1D2D3,
//     getTriBinsOut / getPiBinsOut / getTriCountsOut -> <dir>/ddd_rppi.dat.
// Every failure throws std::runtime_error, as the reference's calls do.
#include <cstdio>
#include <string>
#include <vector>
#include <vector_types.h>

#include "cudaNcorr.hpp"
#include "survey.hpp"
#include "utils.hpp"

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  const std::string dir = argv[1];
  try {
    // Box mode, threeD: linear edges built by the caller.
    std::vector<double> bins;
    for (int i = 0; i <= 10; ++i) bins.push_back(3.0 * i);
    double3 box = {200.0, 200.0, 200.0};
    std::vector<double4> p1 = readCatalogTxt(dir + "/box.txt", box, {0, 1, 2, 3});
    ncorr corr(box, 0, bins, false, {0.0, 0.0, 0.0});
    std::vector<double3> triBinsOut = corr.getTriBinsOut();
    std::vector<double> triCountsOut;
    corr.calculateD1D2D3(p1, p1, p1);
    triCountsOut = corr.getTriCountsOut();
    writeToFileThreeD(dir + "/ddd_box.dat", triBinsOut, triCountsOut);

    // Survey mode, threeD: joint shift of data and randoms, then DDR.
    double3 big = {1.0e6, 1.0e6, 1.0e6};
    std::vector<double4> dat = readCatalogTxt(dir + "/data.txt", big, {0, 1, 2, 3});
    std::vector<double4> ran = readCatalogTxt(dir + "/randoms.txt", big, {0, 1, 2, 3});
    cosmology fiducial{67.36, 0.313772, 0.686228};
    survey fid(fiducial);
    double3 sbox, ori;
    fid.prep_cat_survey(dat, ran, sbox, ori);
    std::vector<double> lbins = logspace(2.0, 30.0, 9);
    ncorr scorr(sbox, 0, lbins, true, ori);
    std::vector<double3> sBins = scorr.getTriBinsOut();
    scorr.calculateD1D2D3(dat, dat, ran);
    writeToFileThreeD(dir + "/ddr_survey.dat", sBins, scorr.getTriCountsOut());
    FILE* f = std::fopen((dir + "/survey_geometry.txt").c_str(), "w");
    if (!f) return 3;
    std::fprintf(f, "%.17g %.17g %.17g %.17g %.17g %.17g\n", sbox.x, sbox.y, sbox.z, ori.x, ori.y, ori.z);
    std::fclose(f);

    // Box mode, rppi: 6 rp bins, 8 unit pi bins.
    std::vector<double> rp = logspace(1.0, 12.0, 7);
    ncorr rcorr(box, 1, rp, 8, false, {0.0, 0.0, 0.0});
    rcorr.calculateD1D2D3(p1, p1, p1);
    std::vector<double3> rBins = rcorr.getTriBinsOut();
    std::vector<double2> piBins = rcorr.getPiBinsOut();
    writeToFileRppi(dir + "/ddd_rppi.dat", rBins, piBins, rcorr.getTriCountsOut());

    // An unsupported bin type throws, as the reference's constructor does.
    bool threw = false;
    try {
      ncorr bad(box, 2, bins, false, {0.0, 0.0, 0.0});
    } catch (const std::runtime_error&) {
      threw = true;
    }
    if (!threw) return 4;
    std::printf("%zu %zu %zu\n", triCountsOut.size(), sBins.size(), piBins.size());
  } catch (const std::exception& e) {
    std::fprintf(stderr, "error: %s\n", e.what());
    return 1;
  }
  return 0;
}
