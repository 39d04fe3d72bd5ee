// Batched explicit-target ALS: parameter block shared by host and device.
#pragma once

#include <cuda_runtime.h>

#include "dword.cuh"

namespace mlcp {

// Row stride (floats) of mode d in the FP32 mode-major target copy: the basis
// size rounded up to a multiple of 4, plus 4 more when that count of float4
// is even, so consecutive rows start on different shared-memory bank groups
// (the copy is moved into shared memory unchanged by bulk copies).
__host__ __device__ inline int als_gstride(int n) {
  const int np = (n + 3) / 4 * 4;
  return ((np / 4) % 2 == 1) ? np : np + 4;
}

// Pipeline shape of the cluster kernel.
constexpr int kAlsThreads = 512;       // 16 warps per CTA
constexpr int kAlsWarps = kAlsThreads / 32;
constexpr int kAlsSolverWarps = 4;     // warps 0-3 run the double-word solves
constexpr int kAlsTileRows = 128;      // target terms per staged tile (4 per lane)

// Tensor-core form (AlsParams::tc): the per-mode dot products <G_j^d, F_i^d>
// of a tile are one tcgen05 MMA (M = 128 target terms, N = rF padded to 16,
// K = the basis size padded to 16) on BF16 three-way splits of both
// operands, accumulated in FP32 in tensor memory, and the running products
// live in tensor memory instead of shared memory.
constexpr int kAlsTcMaxRank = 32;      // largest rF of the tensor-core form
constexpr int kAlsTcCols = 512;        // tensor-memory columns taken per CTA
__host__ __device__ inline int als_tc_kp(int npmax) { return (npmax + 15) / 16 * 16; }
__host__ __device__ inline int als_tc_nf(int rF) { return (rF + 15) / 16 * 16; }
// Whether a CTA owning rows_cta target terms fits the tensor-core form:
// two MMA result buffers plus the running products of every tile (rF
// columns each) plus 16 columns of read slack within the allocation.
__host__ __device__ inline bool als_tc_fits(int rows_cta, int rF, int npmax) {
  if (rF < 1 || rF > kAlsTcMaxRank || npmax > 64) return false;
  const int ntiles = (rows_cta + kAlsTileRows - 1) / kAlsTileRows;
  return 2 * als_tc_nf(rF) + ntiles * rF + 16 <= kAlsTcCols;
}

// All arrays are device pointers unless marked otherwise.
struct AlsParams {
  int nvec;          // vectors in the batch
  int ndof;          // modes D (>= 2)
  int nD;            // sum of basis sizes (reference layout row length)
  int nDp;           // sum of 4-padded basis sizes (FP32 copies of F)
  int nDg;           // sum of als_gstride(basis sizes) (FP32 target copy)
  int npmax;         // max 4-padded basis size
  int rf_max;        // max rF over the batch (sizes the shared-memory carve)
  int gsmax;         // max als_gstride
  int nals;          // sweeps
  double pen_factor; // penalty = pen_factor * max(F weights) (1e-10 FP64 rule, 1e-5 FP32 rule)
  int cluster;       // CTAs per vector
  int stages;        // bulk-copy ring stages
  int tc;            // 1: the tensor-core form of the product passes (als_tc_fits must hold)
  int rows_cta_max;  // max target terms owned by one CTA
  long long total_rows;     // sum of rG
  long long total_f_terms;  // sum of rF
  const int* nbas;   // [D]
  const int* off;    // [D+1] offsets in the reference layout
  const int* offp;   // [D+1] offsets of the 4-padded layout (F copies)
  const int* offg;   // [D+1] offsets of the gstride layout (target copy)
  const int* rF;     // [nvec]
  const int* rG;     // [nvec]
  const long long* term_off;   // [nvec] first term (F) of each vector in base/coef
  const long long* g_row_off;  // [nvec] prefix sum of rG
  const long long* f_row_off;  // [nvec] prefix sum of rF
  const long long* gm_off;     // [nvec] start of each vector in gm (floats, multiple of 4)
  const long long* sq_off;     // [nvec] prefix sum of rF*rF*D
  double* base;      // reference-layout factors holding F (overwritten in place)
  double* coef;      // reference-layout weights holding F's weights
  const double* g_base;         // reference-layout factors holding the targets
  const double* g_coef;         // target weights (unused when shared_target)
  const long long* g_term_off;  // [nvec] first target term of each vector in g_base
  int shared_target;            // 1: every vector fits the same target terms (those
                                //    of vector 0) with its own weights from shared_w
  const double* shared_w;       // [nvec][rG] per-vector target weights (shared_target only)
  int g_host;                   // 1: g_base/g_coef are mapped host memory (read in term order)
  float* gm;         // FP32 mode-major target factors: mode d of term j at
                     //   gm + gm_off[v] + offg[d]*rG + j*gstride(n_d)
  float* gc;         // FP32 target weights [total_rows]
  float* f32;        // unit-normalised F factors, FP32 high parts [total_f_terms][nDp]
  float* f32lo;      // their FP32 low parts (double-word copy of the FP64 values)
  float* fcta;       // per-CTA working copy of the FP32 factors [total_f_terms*cluster][nDp]
  dw* gram;          // per-CTA double-word mode Grams [sq total * cluster]
  dw* suf;           // per-CTA double-word suffix products, same shape
  int* status;       // [nvec] bit 0: non-positive pivot; bit 1: pipeline wait timed out
};

// Shared memory of the cluster kernel.
size_t als_smem_bytes(int rows_cta, int rF, int npmax, int gsmax, int stages, int tc = 0);

// Launch shape chosen for a batch: cluster size, ring stages, engine, shared memory.
struct AlsShape {
  int cluster = 0, stages = 0, rows_cta = 0;
  int tc = 0;  // 1: tensor-core form
  size_t smem = 0;
};

// Product-pass engine: 0 automatic (the autotuner measures both forms; the
// rule without it takes the CUDA-core form), 1 CUDA cores only, 2 tensor
// cores wherever they fit.
int als_engine();
void set_als_engine(int e);
// Returns false (shape untouched) when no shape fits smem_limit.
bool als_choose_shape(int nvec, int rGmax, int rFmax, int npmax, int gsmax, int num_sms, size_t smem_limit,
                      AlsShape* out);

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
  bool g_host = false;                   // g_base/g_coef: mapped host memory
  const double* shared_w = nullptr;      // device [nvec][rG]: shared target of vector 0
  double pen_factor = 1.0e-10;           // reference FP64-build penalty rule
  int* d_status = nullptr;
};

// Enqueue the preparation kernel and the persistent cluster kernel
// (grid = nvec clusters of p.cluster CTAs).  Returns a Status.
// When t0/t1 are non-null they are recorded around the cluster kernel.
int als_launch(const AlsParams& p, size_t smem, cudaStream_t st, cudaEvent_t t0 = nullptr,
               cudaEvent_t t1 = nullptr);
// Failure-path self-test of the cluster kernel's bounded tile wait: a wait
// for a tile nobody issues must give up and report the abort status (2).
int als_wait_selftest(cudaStream_t st, int* flags_out);

}  // namespace mlcp
