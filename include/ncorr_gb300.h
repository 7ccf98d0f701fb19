/*
 * C ABI of the GB300 three-point correlation engine.
 *
 * This is the drop-in boundary for cudaNcorr's threeD counting path. Each
 * entry point replaces one member of the reference's C++ class `ncorr`
 * (include/cudaNcorr.hpp of cudaNcorr) or of its survey helpers
 * (include/survey.hpp, source/survey.cu); the cited lines are that project's.
 * include/cudaNcorr.hpp and include/survey.hpp in this repository rebuild the
 * reference's C++ classes on top of these calls, source-compatibly.
 *
 * Conventions
 *   - Catalogues are arrays of N x 4 doubles (x, y, z, w): the memory layout
 *     of std::vector<double4>. Inputs are only read.
 *   - Every call returns an ncorr_status; nothing throws across the ABI. The
 *     message of the last failure on the calling thread is ncorr_last_error().
 *   - A handle owns its CUDA stream and device buffers; distinct handles may be
 *     used from distinct threads concurrently (the reference keeps its
 *     parameters in __constant__ globals and is not re-entrant).
 *   - Results: triCountsAll_ is the full nb^3 histogram indexed
 *     idx3 + idx2*nb + idx1*nb*nb with idx1 <= idx2 <= idx3 (sorted bins of
 *     the sorted sides); triCountsOut_ is its compaction.
 */
#ifndef NCORR_GB300_H_
#define NCORR_GB300_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum ncorr_status {
  NCORR_OK = 0,
  NCORR_ERR_INVALID_ARGUMENT = 1, /* bad box, edges, sizes or null pointers */
  NCORR_ERR_NOT_IMPLEMENTED = 2,  /* rppi / smu bin types */
  NCORR_ERR_CUDA = 3,             /* a CUDA call failed; see ncorr_last_error() */
  NCORR_ERR_OUT_OF_GRID = 4,      /* a point outside the reference's cell grid, or non-finite */
  NCORR_ERR_CAPACITY = 5,         /* internal list capacity exceeded */
  NCORR_ERR_NO_DEVICE = 6         /* no usable CUDA device */
} ncorr_status;

/* Bin types of the reference (include/cudaNcorr.hpp:12). */
enum { NCORR_BIN_THREED = 0, NCORR_BIN_RPPI = 1, NCORR_BIN_SMU = 2 };

typedef struct ncorr_handle ncorr_handle;

/* Counters of the last calculation. */
typedef struct ncorr_stats {
  double ms_grid;          /* cell-list build (device time) */
  double ms_count;         /* triangle kernel (device time) */
  double ms_fold;          /* histogram fold (device time) */
  double ms_total;         /* host wall time of the whole call */
  uint64_t n_anchors;      /* anchors processed */
  uint64_t n_pair_evals;   /* candidate neighbours scanned (27-cell walk) */
  uint64_t n_pairs;        /* candidate triangles W (neighbour pairs visited) */
  uint64_t n_exact_pairs;  /* neighbours settled by the FP64 path */
  uint64_t n_exact_tris;   /* triangles settled by the FP64 path */
  uint64_t triangles;      /* sum of the full histogram (count mode) */
  uint64_t n_flagged_rows; /* neighbour rows re-examined for uncertain candidates */
  uint64_t n_queued;       /* candidates settled by the careful band or the FP64 path */
  int weighted;            /* 1: some weight != 1.0 (fixed-point weighted sums) */
  int symmetric;           /* orderings each visited triangle stands for: 1 (all (j,l)),
                              2 (p2 == p3: pairs j<l), 6 (p1 == p2 == p3 in a geometry
                              where all three vertices see each other identically) */
  int grid_ctas;           /* persistent CTAs of the triangle kernel */
  int list_capacity;       /* shared-memory neighbour-list capacity */
} ncorr_stats;

/* ncorr::ncorr(double3 box, int bin_type, std::vector<double>& bins,
 *              bool isSurvey, double3 ori)
 * include/cudaNcorr.hpp:14, source/cudaNcorr.cu:118-157.
 * edges: n_edges bin edges (strictly increasing, edges[0] >= 0). Cell edge is
 * r_max = edges[n_edges-1]; cells per axis ceil(box/r_max). bin_type other
 * than NCORR_BIN_THREED is rejected with NCORR_ERR_INVALID_ARGUMENT, as the
 * reference throws for it. */
int ncorr_create(const double box[3], int bin_type, const double* edges, int n_edges,
                 int is_survey, const double ori[3], ncorr_handle** out);

/* ncorr::ncorr(double3 box, int bin_type, std::vector<double>& bins,
 *              int numMinorBins, bool isSurvey, double3 ori)
 * include/cudaNcorr.hpp:15, source/cudaNcorr.cu:159-216. The rppi bin type is
 * not implemented by this engine: returns NCORR_ERR_NOT_IMPLEMENTED. */
int ncorr_create_rppi(const double box[3], int bin_type, const double* edges, int n_edges,
                      int num_minor_bins, int is_survey, const double ori[3], ncorr_handle** out);

/* Releases the handle and its device memory. Null is accepted. */
void ncorr_destroy(ncorr_handle* h);

/* ncorr::calculateD1D2D3(std::vector<double4>& p1, p2, p3)
 * include/cudaNcorr.hpp:19, source/cudaNcorr.cu:220-430.
 * Host arrays of n x 4 doubles. p1 are the anchors; p2 and p3 the second and
 * third vertices. Passing the same pointer (and size) for p2 and p3, or for
 * all three, tells the engine the catalogues are identical. Synchronous. */
int ncorr_calculate_d1d2d3(ncorr_handle* h, const double* p1, int64_t n1, const double* p2,
                           int64_t n2, const double* p3, int64_t n3);

/* Same computation on catalogues already resident in device memory (n x 4
 * doubles each, 16-byte aligned), ordered on `stream` (a cudaStream_t, or
 * null for the handle's own stream). Synchronises before returning, since
 * the results are read back to the handle. No reference counterpart. */
int ncorr_calculate_d1d2d3_device(ncorr_handle* h, const double* d_p1, int64_t n1,
                                  const double* d_p2, int64_t n2, const double* d_p3, int64_t n3,
                                  void* stream);

/* Number of entries of triCountsOut_ / triBinsOut_ (source/cudaNcorr.cu:145-154). */
int64_t ncorr_num_out(const ncorr_handle* h);

/* Number of bins per side. */
int ncorr_num_bins(const ncorr_handle* h);

/* ncorr::getTriBinsOut() (include/cudaNcorr.hpp:21, source/cudaNcorr.cu:106-108):
 * num_out x 3 bin mids into out (capacity cap doubles). */
int ncorr_get_tri_bins_out(const ncorr_handle* h, double* out, int64_t cap);

/* ncorr::getPiBinsOut() (include/cudaNcorr.hpp:23, source/cudaNcorr.cu:110-112):
 * always empty for the threeD bin type; *n receives 0. */
int ncorr_get_pi_bins_out(const ncorr_handle* h, double* out, int64_t cap, int64_t* n);

/* ncorr::getTriCountsOut() (include/cudaNcorr.hpp:25, source/cudaNcorr.cu:114-116):
 * num_out counts of the last calculation. */
int ncorr_get_tri_counts_out(const ncorr_handle* h, double* out, int64_t cap);

/* The full nb^3 histogram triCountsAll_ (private in the reference,
 * include/cudaNcorr.hpp:49), of which getTriCountsOut is a compaction. */
int ncorr_get_tri_counts_all(const ncorr_handle* h, double* out, int64_t cap);

/* Counters and timings of the last calculation. */
int ncorr_get_stats(const ncorr_handle* h, ncorr_stats* out);

/* Message of the last failure on this thread ("" if none). */
const char* ncorr_last_error(void);

/* survey::prep_cat_survey(std::vector<double4>& catalog, double3& box, double3& ori)
 * include/survey.hpp:22, source/survey.cu:94-104: box = max - min + 1.0,
 * ori = -min, catalogue shifted in place by -min. */
int survey_prep_cat(double* cat, int64_t n, double box[3], double ori[3]);

/* survey::prep_cat_survey(catalog1, catalog2, box, ori)
 * include/survey.hpp:23, source/survey.cu:106-128: joint bounding box of both
 * catalogues, both shifted in place. */
int survey_prep_cat2(double* cat1, int64_t n1, double* cat2, int64_t n2, double box[3],
                     double ori[3]);

/* survey::convert_coordinates (include/survey.hpp:20, source/survey.cu:39-57):
 * rows (RA deg, Dec deg, redshift z, w) -> (x, y, z, w) with comoving distance
 * d(z) = (c/100) * integral_0^z dz' / sqrt(OmegaM (1+z')^3 + OmegaLambda)
 * in Mpc/h (source/survey.cu:17-37; H0 is unused there and here).
 * cosmo = {H0, OmegaM, OmegaLambda}. in and out may alias. */
int survey_convert_coordinates(const double cosmo[3], const double* in, int64_t n, double* out);

/* logspace(start, end, n) (include/utils.hpp:9, source/utils.cu:16-27):
 * n log-spaced bin edges from start to end. */
int ncorr_logspace(double start, double end, int n, double* out);

/* Triangle count without any device allocation; no counterpart in the
 * reference. For callers that must not allocate device memory -- code given a
 * fixed device-memory budget up front, or running where a cudaMalloc or
 * cudaFree would synchronise the device and stall work queued by others. All
 * working memory is one 16 MiB array inside the library, held by every GPU
 * that loads it until the process exits; limits: at most 65536 points per
 * catalogue, 32768 cells, 31 bins per side, and neighbourhoods that fit the
 * kernel's on-chip lists (NCORR_ERR_CAPACITY otherwise). Inputs are device
 * catalogues (n x 4 doubles, 16-byte aligned); d_counts_all receives the
 * nb^3 doubles of triCountsAll_, as ncorr_get_tri_counts_all returns them.
 * The first call on each device looks up the array's device address, so make
 * it before any stream capture. Calls share the array: calls that overlap on
 * the GPU (other threads, other streams) race, so serialise them. Returns
 * after the work on `stream` (null: the legacy default stream) completes. */
int ncorr_count_noalloc(const double box[3], const double* edges, int n_edges, int is_survey,
                        const double* d_p1, int64_t n1, const double* d_p2, int64_t n2,
                        const double* d_p3, int64_t n3, double* d_counts_all, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* NCORR_GB300_H_ */
