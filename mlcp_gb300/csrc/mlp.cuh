// Learned ALS warm start: the MLP kernels' parameter blocks (mlp.cu).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace mlcp {

// C[M x N] = A[M x K] B[N x K]^T on tcgen05 tensor cores.  A, B: BF16,
// row-major with K contiguous (leading dimensions lda, ldb in elements,
// multiples of 8, base addresses 16-byte aligned).  M a multiple of 128, N
// of 16, K of 64.  Epilogue per element x = acc (+ bias[col]):
//   act 0: x;  act 1: max(x, 0);  act 2: x where mask[row][col] > 0, else 0
// and rows >= valid_m are written as 0.  Outputs (each optional): C FP32
// [M][ldc], Cb BF16 [M][ldcb], Ct BF16 transposed [N][ldct].
struct MlpGemm {
  const __nv_bfloat16* A;
  const __nv_bfloat16* B;
  int M, N, K;
  int lda, ldb;
  const float* bias;
  int act;
  const __nv_bfloat16* mask;
  int ldm;
  float* C;
  int ldc;
  __nv_bfloat16* Cb;
  int ldcb;
  __nv_bfloat16* Ct;
  int ldct;
  int valid_m;
  int* status;  // bit 1: an mbarrier wait timed out (result not valid); may be null
};

int mlp_gemm_launch(const MlpGemm& g, cudaStream_t st);
int mlp_loss_launch(const float* Y, const float* T, int m, int n, int ld, int rows_p, __nv_bfloat16* dY,
                    __nv_bfloat16* dYt, float* loss, cudaStream_t st);
int mlp_colsum_launch(const __nv_bfloat16* G, int rows, int n, int ld, float* db, cudaStream_t st);
int mlp_adam_launch(float* w, const float* g, float* m1, float* m2, int rows, int cols, float lr, float b1, float b2,
                    float eps, int step, __nv_bfloat16* wb, __nv_bfloat16* wt, cudaStream_t st);

// Feature rows, training targets and proposals of the warm start (one row
// per (vector, mode); every mode has the same basis size n).
struct WsBatch {
  int nvec, ndof, nD, n;     // n: the common basis size
  int ntop;                  // target terms per feature row (64)
  int rank;                  // rank of the proposal (F terms)
  int rgmax;                 // the selection bitmap's capacity in target terms (g_rank is clamped to it)
  const long long* g_off;    // [nvec] first target term of each vector in base/coef
  const int* g_rank;         // [nvec] target terms of each vector
  const long long* f_off;    // [nvec] first F term
  const double* base;        // reference layout, nD values per term
  const double* coef;
  double* f_base;            // proposal output (may alias base)
  double* f_coef;
};
// X[(v ndof + d)][k n + m] = G_{top k}^d(m) normalised (largest-magnitude entry
// positive), X[..][ntop n + k] = log10(|c_{top k}| / |c_{top 0}|) / 8, for the
// ntop largest-magnitude target weights of vector v; BF16, leading dim ldx.
// rgmax: the largest g_rank (sizes the selection bitmap).
int ws_features_launch(const WsBatch& b, __nv_bfloat16* X, int ldx, int rgmax, cudaStream_t st);
// T[(v ndof + d)][j n + m] = the mode-d factor of the reduction's term (rank
// terms at f_off) matched to the j-th largest-weight target term, unit, its
// sign aligned with that term's canonical factor; FP32, leading dim ldt.
int ws_targets_launch(const WsBatch& b, float* T, int ldt, int rgmax, cudaStream_t st);
// Proposal: F_i^d = Y[(v ndof + d)][i n + ..] normalised, F weights = the
// rank largest |target weights|; written at f_off into f_base / f_coef.
int ws_apply_launch(const WsBatch& b, const float* Y, int ldy, int rgmax, cudaStream_t st);

}  // namespace mlcp
