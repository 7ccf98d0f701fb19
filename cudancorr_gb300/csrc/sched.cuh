// Learned scheduling of the triangle kernel's work queue.
//
// The triangle work of an anchor grows with the square of its neighbour
// count, so a few dense cells can hold most of a clustered catalogue's work.
// A small MLP predicts, for every cell, log(1 + candidate pairs of the
// anchors it holds) from 28 occupancies: the cell's own anchor count and the
// catalogue-2 (+3) counts of its 27 neighbour slots, each as log(1 + n).
// Cells are then queued heaviest first (items heaviest first in a batch), so
// the last positions the CTAs take are the light ones. The counts do not
// depend on the order; only the tail of the launch does.
#pragma once
#include "triangles.cuh"

namespace ncorr_gb300 {

constexpr int kMlpIn = 28;
constexpr int kMlpHidden = 64;
// Parameter vector: W1 [in][hidden], b1, W2 [hidden][hidden], b2, w3, b3.
constexpr int kMlpOffW1 = 0;
constexpr int kMlpOffB1 = kMlpOffW1 + kMlpIn * kMlpHidden;
constexpr int kMlpOffW2 = kMlpOffB1 + kMlpHidden;
constexpr int kMlpOffB2 = kMlpOffW2 + kMlpHidden * kMlpHidden;
constexpr int kMlpOffW3 = kMlpOffB2 + kMlpHidden;
constexpr int kMlpOffB3 = kMlpOffW3 + kMlpHidden;
constexpr int kMlpParams = kMlpOffB3 + 1;
constexpr int kMlpTile = 64;  // samples per CTA of the gradient kernel

// Buckets of the predicted log-work used to order cells (counting sort).
constexpr int kSchedBuckets = 256;
constexpr float kSchedPredMax = 40.0f;  // log(1 + work) mapped onto the buckets

// Features of every (item, cell): n_items * ncell rows of kMlpIn floats.
void launch_cell_features(const BatchItem* items, int n_items, const Geom& g, float* feats, cudaStream_t st);

// pred[i] = MLP(feats[i]); bf16: the BF16 forward pass (weights, inputs and
// activations rounded to bfloat16, FP32 accumulation).
void launch_mlp_predict(const float* params, const float* feats, int n, float* pred, cudaStream_t st,
                        bool bf16 = false);

// Mean-squared-error gradient over the n samples idx[0..n) (idx null: 0..n)
// of (feats, target): per-CTA partial sums, reduced in a fixed order by
// launch_mlp_reduce or launch_adam. Returns the number of CTAs used.
int launch_mlp_grad(const float* params, const float* feats, const float* target, const int* idx, int n,
                    float* partial, float* partial_loss, cudaStream_t st, bool bf16 = false);
size_t mlp_grad_smem_bytes();
void launch_mlp_reduce(const float* partial, const float* partial_loss, int nblk, float* grad, float* loss,
                       cudaStream_t st);
void launch_adam(float* params, const float* partial, int nblk, float* m, float* v, int step, float lr,
                 cudaStream_t st);

// Work queue in cell order, items in order: position w -> (item, anchor).
void launch_identity_queue(const int* item_off, int n_items, int* q_item, int* q_anchor, int n_work,
                           cudaStream_t st);

// Scratch of the learned order for n_items items of ncell cells.
struct OrderScratch {
  float* pred;          // n_items * ncell
  double* item_total;   // n_items
  int* item_rank;       // n_items
  int* ekey;            // n_items * ncell
  int* kcount;          // n_items * kSchedBuckets + 1
  int* kstart;          // n_items * kSchedBuckets + 1
  int* kcursor;         // n_items * kSchedBuckets + 1
  int* sorted;          // n_items * ncell
  int* acount;          // n_items * ncell + 1
  int* aoff;            // n_items * ncell + 1
  int* acursor;         // n_items * ncell + 1
};

// Queue in predicted-work order from pred (filled by launch_mlp_predict).
void launch_learned_queue(const BatchItem* items, int n_items, int ncell, const OrderScratch& s, int* q_item,
                          int* q_anchor, cudaStream_t st);

}  // namespace ncorr_gb300
