// Batched explicit-target ALS: parameter block shared by host and device.
#pragma once

#include <cuda_runtime.h>

namespace mlcp {

// All arrays are device pointers unless marked otherwise.
struct AlsParams {
  int nvec;          // vectors in the batch
  int ndof;          // modes D
  int nD;            // sum of basis sizes (reference layout row length)
  int nDp;           // sum of 4-padded basis sizes (FP32 copies)
  int npmax;         // max 4-padded basis size
  int nals;          // sweeps
  double pen_factor; // penalty = pen_factor * max(F weights) (1e-10 FP64 rule, 1e-5 FP32 rule)
  int rows_cta_max;  // max target terms owned by one CTA
  long long total_rows;     // sum of rG
  long long total_f_terms;  // sum of rF
  const int* nbas;   // [D]
  const int* off;    // [D+1] offsets in the reference layout
  const int* offp;   // [D+1] offsets of the 4-padded layout
  const int* rF;     // [nvec]
  const int* rG;     // [nvec]
  const long long* term_off;   // [nvec] first term (F) of each vector in base/coef
  const long long* g_row_off;  // [nvec] prefix sum of rG
  const long long* f_row_off;  // [nvec] prefix sum of rF
  const long long* gm_off;     // [nvec] start of each vector in gm
  const long long* sq_off;     // [nvec] prefix sum of rF*rF*D (Gram storage)
  double* base;      // reference-layout factors holding F (overwritten in place)
  double* coef;      // reference-layout weights holding F's weights
  const double* g_base;         // reference-layout factors holding the targets
  const double* g_coef;         // target weights (unused when shared_target)
  const long long* g_term_off;  // [nvec] first target term of each vector in g_base
  int shared_target;            // 1: every vector fits the same target terms (those
                                //    of vector 0) with its own weights from shared_w
  const double* shared_w;       // [nvec][rG] per-vector target weights (shared_target only)
  float* gm;         // FP32 mode-major target factors
  float* gc;         // FP32 target weights [total_rows]
  float* f32;        // FP32 copy of F [total_f_terms][nDp]
  double* gram;      // FP64 per-mode F Grams [total_f_terms * rF * D] (rF*rF*D per vector)
  double* suf;       // FP64 suffix products, same shape as gram
  int* status;       // [nvec] bit 0: non-positive Cholesky pivot
};

constexpr int kAlsThreads = 512;

// Shared memory of the cluster kernel for a CTA owning rows_cta target terms.
size_t als_smem_bytes(int rows_cta, int rF, int npmax);

// Host description of one batched reduction (see als_run in capi.cu).
struct AlsJob {
  int nvec = 0, ndof = 0, nals = 0;
  const int* nbas = nullptr;             // host [ndof]
  const int* rF = nullptr;               // host [nvec]
  const int* rG = nullptr;               // host [nvec]
  const long long* term_off = nullptr;   // host [nvec], F terms in d_base/d_coef
  double* d_base = nullptr;
  double* d_coef = nullptr;
  const double* g_base = nullptr;        // device; null: targets follow F in d_base
  const double* g_coef = nullptr;
  const long long* g_term_off = nullptr; // host [nvec]; null: term_off + rF
  const double* shared_w = nullptr;      // device [nvec][rG]: shared target of vector 0
  double pen_factor = 1.0e-10;           // reference FP64-build penalty rule
  int* d_status = nullptr;
};

// Enqueue the preparation kernel and the persistent cluster kernel
// (grid = nvec clusters of `cluster` CTAs).  Returns a Status.
// When t0/t1 are non-null they are recorded around the cluster kernel.
int als_launch(const AlsParams& p, int cluster, size_t smem, cudaStream_t st, cudaEvent_t t0 = nullptr,
               cudaEvent_t t1 = nullptr);

}  // namespace mlcp
