/*
 * C ABI of the GB300 three-point correlation engine.
 *
 * This is the drop-in boundary for cudaNcorr's counting path (threeD and rppi
 * bin types). Each
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
  NCORR_ERR_NOT_IMPLEMENTED = 2,  /* a feature this engine lacks for the handle's bin type */
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
  uint64_t n_exact_tris;   /* triangles (rppi: pairs) settled by the FP64 path */
  uint64_t triangles;      /* sum of the full histogram (count mode) */
  uint64_t n_flagged_rows; /* threeD: (row, lane) flags of the pair loop re-examined for uncertain
                              candidates (each stands for up to four candidates) */
  uint64_t n_queued;       /* threeD: candidates settled by the careful band or the FP64 path;
                              rppi: pairs settled by the box-mode FP32 classifier */
  int weighted;            /* 1: some weight != 1.0 (fixed-point weighted sums) */
  int symmetric;           /* orderings each visited triangle stands for: 1 (all (j,l)),
                              2 (p2 == p3: pairs j<l), 6 (p1 == p2 == p3 in a geometry
                              where all three vertices see each other identically) */
  int grid_ctas;           /* persistent CTAs of the triangle kernel */
  int list_capacity;       /* per-warp neighbour-list capacity (entries, global memory) */
  double overflow;         /* rppi: count (or weight) of triangles whose reference index lies
                              past triCountsAll_ (pi bin numMinorBins from FP32 rounding);
                              the reference writes those out of bounds */
  double tail_idle;        /* threeD: share of the triangle kernel's CTA-time spent idle while
                              the last CTAs finished (0: all CTAs ended together) */
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
 * include/cudaNcorr.hpp:15, source/cudaNcorr.cu:159-216: the rppi bin type.
 * Sides are binned by rp (edges, as for threeD) and the two shortest by pi in
 * num_minor_bins unit bins [0,1), [1,2), ...; piMax = num_minor_bins. Box
 * cells are (rpMax, rpMax, piMax), line of sight z; survey cells are cubes of
 * sqrtf(rpMax^2 + piMax^2) (FP32, as the reference), line of sight the sum
 * of the three positions minus (ori.x, 0, 0) (the reference uploads only
 * ori.x). triCountsAll_ has nb^3 * num_minor_bins^2 entries indexed
 * idxPi2 + idxPi1*nPi + idx3*nPi^2 + idx2*nb*nPi^2 + idx1*nb^2*nPi^2.
 * bin_type other than NCORR_BIN_RPPI is rejected as the reference throws. */
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

/* numPiBins_ of an rppi handle (source/cudaNcorr.cu:178); 0 for threeD. */
int ncorr_num_pi_bins(const ncorr_handle* h);

/* ncorr::getTriBinsOut() (include/cudaNcorr.hpp:21, source/cudaNcorr.cu:106-108):
 * num_out x 3 bin mids into out (capacity cap doubles). */
int ncorr_get_tri_bins_out(const ncorr_handle* h, double* out, int64_t cap);

/* ncorr::getPiBinsOut() (include/cudaNcorr.hpp:23, source/cudaNcorr.cu:110-112):
 * rppi: num_out x 2 pi bins (l, m) into out (capacity cap doubles), *n = num_out;
 * threeD: empty, *n = 0. */
int ncorr_get_pi_bins_out(const ncorr_handle* h, double* out, int64_t cap, int64_t* n);

/* ncorr::getTriCountsOut() (include/cudaNcorr.hpp:25, source/cudaNcorr.cu:114-116):
 * num_out counts of the last calculation. */
int ncorr_get_tri_counts_out(const ncorr_handle* h, double* out, int64_t cap);

/* The full histogram triCountsAll_ (private in the reference,
 * include/cudaNcorr.hpp:49), of which getTriCountsOut is a compaction:
 * nb^3 entries (threeD) or nb^3 * numPiBins^2 (rppi). */
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

/* writeToFileThreeD(filename, triBins, counts) (include/utils.hpp:15-19,
 * source/utils.cu:161-181): one row "r1 r2 r3 count" per entry, each value
 * with 6 decimals. tri_bins: n x 3 (getTriBinsOut), counts: n. */
int ncorr_write_three_d(const char* filename, const double* tri_bins, const double* counts, int64_t n);

/* writeToFileRppi(filename, triBins, piBins, counts) (include/utils.hpp:21-26,
 * source/utils.cu:183-208): rows "r1 r2 r3 pi1 pi2 count". pi_bins: n x 2. */
int ncorr_write_rppi(const char* filename, const double* tri_bins, const double* pi_bins, const double* counts,
                     int64_t n);

/* readCatalogTxt(filename, box, pos_columns) (include/utils.hpp:36-40,
 * source/utils.cu:119-159): whitespace-separated text, one point per line;
 * pos_columns[0..3] name the columns of x, y, z and w. A coordinate outside
 * [0, box] fails with NCORR_ERR_OUT_OF_GRID and the line number, as the
 * reference throws; a line without one of the four columns fails too (the
 * reference leaves that point uninitialised). *n receives the number of
 * points; out (capacity cap points of 4 doubles) may be null to size it. */
int ncorr_read_catalog_txt(const char* filename, const double box[3], const int pos_columns[4], double* out,
                           int64_t cap, int64_t* n);

/* generateRandomCatalog(Np, box) (include/utils.hpp:11, source/utils.cu:41-52):
 * n points uniform in [0, box) per axis, weight 1. The reference seeds from
 * the clock and the thread number; here the stream depends only on `seed`. */
int ncorr_random_catalog(int64_t n, const double box[3], uint64_t seed, double* out);

/* Triangle count without any device allocation; no counterpart in the
 * reference. For callers that must not allocate device memory -- code given a
 * fixed device-memory budget up front, or running where a cudaMalloc or
 * cudaFree would synchronise the device and stall work queued by others. All
 * working memory is one 16 MiB array inside the library, held by every GPU
 * that loads it until the process exits; limits: at most 65536 points per
 * catalogue, 32768 cells, 31 bins per side, and neighbourhoods whose lists
 * fit the part of the array left after the catalogues' cell lists, for at
 * least one CTA of the triangle kernel (NCORR_ERR_CAPACITY otherwise; fewer
 * CTAs run when not all fit). Inputs are device
 * catalogues (n x 4 doubles, 16-byte aligned); d_counts_all receives the
 * nb^3 doubles of triCountsAll_, as ncorr_get_tri_counts_all returns them.
 * The first call on each device looks up the array's device address, so make
 * it before any stream capture; later calls outside a capture look it up
 * again (a device reset reloads the library's module and moves the array),
 * calls inside a capture reuse the last address found on that device, so do
 * not reset a device between that look-up and a captured call. Calls share
 * the array: calls that overlap on
 * the GPU (other threads, other streams) race, so serialise them. Returns
 * after the work on `stream` (null: the legacy default stream) completes. */
int ncorr_count_noalloc(const double box[3], const double* edges, int n_edges, int is_survey,
                        const double* d_p1, int64_t n1, const double* d_p2, int64_t n2,
                        const double* d_p3, int64_t n3, double* d_counts_all, void* stream);

/* ---- Work-queue scheduling. No counterpart in the reference, whose kernel
 * gives one thread to each anchor in input order (source/device.cu:259-315).
 * The schedule changes only the order in which CTAs take anchors; the counts
 * never depend on it. */
enum { NCORR_SCHED_DYNAMIC = 0, NCORR_SCHED_STATIC = 1, NCORR_SCHED_LEARNED = 2 };

/* The scheduler's work model: an MLP 28 -> 64 -> 64 -> 1 (ReLU) that maps a
 * cell's occupancies (log(1 + n) of its catalogue-1 count and of the 27
 * neighbour-slot counts) to log(1 + candidate pairs of its anchors). */
typedef struct ncorr_sched ncorr_sched;

/* Anchor order of later calls on h. DYNAMIC (default): cells in grid order,
 * CTAs take anchors from a shared counter. STATIC: cells in grid order, each
 * CTA one contiguous range. LEARNED: cells ordered by the work `model`
 * predicts, heaviest first, taken from a shared counter. `model` must stay
 * alive while h uses it. */
int ncorr_set_schedule(ncorr_handle* h, int mode, const ncorr_sched* model);

/* Tuning of later calls: rows per careful-flag group of the pair loop (8, 16
 * or 32; the uncertain candidates of a group are queued together) and copies
 * of each CTA histogram (1, 2 or 4, as many as fit in shared memory). The
 * results do not depend on them. */
int ncorr_set_tuning(ncorr_handle* h, int sub_j, int hist_copies);

/* When on, later calls record for each cell of the grid its 28 scheduler
 * features and the candidate pairs its catalogue-1 anchors took: the
 * training data of the work model. */
int ncorr_set_record_work(ncorr_handle* h, int on);
int64_t ncorr_num_cells(const ncorr_handle* h);
/* feats: n_cells x 28 floats; work: n_cells doubles (either may be null). */
int ncorr_get_cell_work(const ncorr_handle* h, float* feats, double* work, int64_t cap_cells);

/* Model life cycle; parameters are initialised from `seed` (He-uniform
 * weights, zero biases) on the current device. */
int ncorr_sched_create(uint64_t seed, ncorr_sched** out);
void ncorr_sched_destroy(ncorr_sched* s);
int ncorr_sched_num_params(void);
/* Parameter vector: W1 [28][64], b1 [64], W2 [64][64], b2 [64], w3 [64], b3. */
int ncorr_sched_get_params(const ncorr_sched* s, float* out, int64_t cap);
int ncorr_sched_set_params(ncorr_sched* s, const float* in, int64_t n);
/* Arithmetic of the model's forward pass, in prediction (ncorr_sched_predict
 * and the learned queue) and in training: NCORR_MLP_FP32 (default) or
 * NCORR_MLP_BF16, where weights, inputs and hidden activations are rounded to
 * bfloat16 and products are accumulated in FP32 (the master parameters, the
 * backward pass and Adam stay FP32). No counterpart in the reference, which
 * has no learned part. */
enum { NCORR_MLP_FP32 = 0, NCORR_MLP_BF16 = 1 };
int ncorr_sched_set_precision(ncorr_sched* s, int precision);

/* out[i] = model(feats[i]) for n host rows of 28 floats. */
int ncorr_sched_predict(ncorr_sched* s, const float* feats, int64_t n, float* out);
/* Gradient of the mean squared error (1/n) sum (model(x_i) - t_i)^2 over n
 * host samples, by the training kernels; *loss = sum of squared errors. */
int ncorr_sched_gradient(ncorr_sched* s, const float* feats, const float* target, int64_t n, float* grad,
                         float* loss);
/* Adam training on the GPU: `epochs` passes over the n samples in minibatches
 * of `batch` (a multiple of 64), shuffled from `seed`; *last_epoch_loss = mean
 * squared error over the last epoch. */
int ncorr_sched_train(ncorr_sched* s, const float* feats, const float* target, int64_t n, int epochs, int batch,
                      float lr, uint64_t seed, float* last_epoch_loss);

/* ---- Batches: many catalogue triples counted by one persistent launch of
 * the triangle kernel, captured with everything around it (copies, cell
 * lists, queue, exact pass, fold) in one CUDA graph. No counterpart in the
 * reference, where each triple is a separate calculateD1D2D3. All items share
 * h's box and bins; in every item either p2 == p3 or p2 != p3 (same array
 * and size), uniformly. Arrays (host, or device when on_device) are bound to
 * the batch: each ncorr_batch_run counts their current contents. */
typedef struct ncorr_batch ncorr_batch;

typedef struct ncorr_batch_stats {
  double ms_plan;       /* host wall time of ncorr_batch_create */
  double ms_autotune;   /* part of it spent timing tuning candidates */
  double ms_run;        /* device time of the last ncorr_batch_run graph */
  double ms_count;      /* device time of its triangle kernel */
  uint64_t n_work;      /* anchors in the queue (all items) */
  uint64_t n_pairs;     /* candidate triangles of the last run */
  uint64_t n_pair_evals; /* candidate neighbours scanned in the last run */
  uint64_t triangles;   /* sum over items of the folded counts (count mode) */
  int n_items;
  int n_catalogues;     /* distinct arrays gridded */
  int sub_j;            /* tuning in use */
  int hist_copies;
  int grid_ctas;
  int weighted;
  int graph_nodes;
} ncorr_batch_stats;

/* Plans the batch: grids and checks every catalogue once, sizes the lists,
 * builds the queue with h's schedule, times the tuning candidates on a
 * sample of the queue when `autotune` (else uses h's tuning), and captures
 * the graph. */
int ncorr_batch_create(ncorr_handle* h, int n_items, const double* const* p1, const int64_t* n1,
                       const double* const* p2, const int64_t* n2, const double* const* p3, const int64_t* n3,
                       int on_device, int autotune, ncorr_batch** out);
/* Replays the graph on `stream` (null: the batch's own) and waits for it. */
int ncorr_batch_run(ncorr_batch* b, void* stream);
/* triCountsAll_ of item `item` after the last run (nb^3 doubles). */
int ncorr_batch_get_counts_all(const ncorr_batch* b, int item, double* out, int64_t cap);
int ncorr_batch_get_stats(const ncorr_batch* b, ncorr_batch_stats* out);
void ncorr_batch_destroy(ncorr_batch* b);

#ifdef __cplusplus
}
#endif

#endif /* NCORR_GB300_H_ */
