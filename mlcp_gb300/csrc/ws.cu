// Learned ALS warm start: the data kernels around the MLP (mlp.cu).
//
// One feature row per (vector, mode): the mode's factors of the vector's
// ntop largest-weight target terms, each scaled to unit norm with its
// largest-magnitude entry positive (a factor's sign and scale are
// arbitrary in CP format: the weight and the other modes absorb them),
// followed by the terms' log-weights.  The training target of the same row
// holds, in slot j, the mode's factor of the converged reduction's term that
// the j-th input term turned into (ws_targets_kernel).  A proposal turns the
// MLP's output slots back into unit factors, with the largest target weights
// as the starting weights (ALS overwrites the weights and the first mode's
// factors in its first step; the weights matter only through the penalty).
#include <cfloat>

#include "../../include/mlcp_gb300.h"
#include "common.cuh"
#include "context.cuh"
#include "mlp.cuh"

namespace mlcp {

namespace {

constexpr int kWsThreads = 256;

// Indices of the k largest |coef| among n entries (ties: lower index first),
// -1 past n; every thread returns with top[] filled.
__device__ void top_terms(const double* coef, int n, int k, unsigned* taken, int* top, float* rv, int* ri) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int w = tid; w < (n + 31) / 32; w += kWsThreads) taken[w] = 0u;
  __syncthreads();
  for (int q = 0; q < k; ++q) {
    float bv = -1.f;
    int bi = 0x7fffffff;
    for (int j = tid; j < n; j += kWsThreads) {
      if (taken[j >> 5] & (1u << (j & 31))) continue;
      const float a = (float)fabs(coef[j]);
      if (a > bv || (a == bv && j < bi)) {
        bv = a;
        bi = j;
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const float ov = __shfl_xor_sync(0xffffffffu, bv, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ov > bv || (ov == bv && oi < bi)) {
        bv = ov;
        bi = oi;
      }
    }
    if (lane == 0) {
      rv[warp] = bv;
      ri[warp] = bi;
    }
    __syncthreads();
    if (tid == 0) {
      float v = rv[0];
      int i = ri[0];
      for (int w = 1; w < kWsThreads / 32; ++w)
        if (rv[w] > v || (rv[w] == v && ri[w] < i)) {
          v = rv[w];
          i = ri[w];
        }
      const int pick = (v >= 0.f && i < n) ? i : -1;
      top[q] = pick;
      if (pick >= 0) taken[pick >> 5] |= 1u << (pick & 31);
    }
    __syncthreads();
  }
}

// Scale of a factor: 1/||g|| with the sign of its largest-magnitude entry
// (0 for a zero factor).
__device__ __forceinline__ double canon_scale(const double* g, int n) {
  double s2 = 0.0, big = 0.0;
  for (int m = 0; m < n; ++m) {
    s2 += g[m] * g[m];
    if (fabs(g[m]) > fabs(big)) big = g[m];
  }
  if (!(s2 > 0.0)) return 0.0;
  return (big < 0.0 ? -1.0 : 1.0) / sqrt(s2);
}

__global__ void __launch_bounds__(kWsThreads) ws_features_kernel(WsBatch b, __nv_bfloat16* X, int ldx) {
  extern __shared__ unsigned ws_smem[];
  __shared__ int top[64];
  __shared__ float rv[kWsThreads / 32];
  __shared__ int ri[kWsThreads / 32];
  const int v = blockIdx.x, n = b.n, D = b.ndof, K = b.ntop;
  const long long off = b.g_off[v];
  top_terms(b.coef + off, min(b.g_rank[v], b.rgmax), K, ws_smem, top, rv, ri);
  for (int item = threadIdx.x; item < D * K; item += kWsThreads) {
    const int d = item / K, k = item - d * K, j = top[k];
    __nv_bfloat16* row = X + (size_t)(v * D + d) * ldx;
    if (j < 0) {
      for (int m = 0; m < n; ++m) row[k * n + m] = __float2bfloat16_rn(0.f);
      row[K * n + k] = __float2bfloat16_rn(-1.f);
      continue;
    }
    const double* g = b.base + (size_t)(off + j) * b.nD + (size_t)d * n;
    const double s = canon_scale(g, n);
    for (int m = 0; m < n; ++m) row[k * n + m] = __float2bfloat16_rn((float)(g[m] * s));
    const double c0 = fabs(b.coef[off + top[0]]), ck = fabs(b.coef[off + j]);
    const double lw = (c0 > 0.0 && ck > 0.0) ? log10(ck / c0) / 8.0 : -1.0;
    row[K * n + k] = __float2bfloat16_rn((float)fmax(lw, -1.0));
  }
}

// Targets aligned with the inputs: output slot j (j < rank) stands for the
// j-th largest-weight target term, and its target is the reduction's term
// that term turned into -- the pairs (F term i, slot j) are matched greedily
// by the largest prod_d |<F_i^d, G_j^d>| / (|F_i^d| |G_j^d|), and each
// target factor takes the sign that makes its overlap with the slot's input
// factor (as canonicalised in the features) non-negative.  Ordering the
// reduction's terms by weight instead made the slots of nearly equal weights
// swap between samples, and the network learned their average.
__global__ void __launch_bounds__(kWsThreads) ws_targets_kernel(WsBatch b, float* T, int ldt) {
  extern __shared__ unsigned ws_smem[];
  __shared__ int top[64];
  __shared__ int slot_of[64];  // F term assigned to slot j
  __shared__ float ov[64 * 64];
  __shared__ float rv[kWsThreads / 32];
  __shared__ int ri[kWsThreads / 32];
  const int v = blockIdx.x, n = b.n, D = b.ndof, R = b.rank;
  const long long foff = b.f_off[v], goff = b.g_off[v];
  top_terms(b.coef + goff, min(b.g_rank[v], b.rgmax), R, ws_smem, top, rv, ri);
  for (int e = threadIdx.x; e < R * R; e += kWsThreads) {
    const int i = e / R, j = e - i * R;
    float o = 0.f;
    if (top[j] >= 0) {
      double prod = 1.0;
      for (int d = 0; d < D; ++d) {
        const double* f = b.base + (size_t)(foff + i) * b.nD + (size_t)d * n;
        const double* g = b.base + (size_t)(goff + top[j]) * b.nD + (size_t)d * n;
        double fg = 0.0, ff = 0.0, gg = 0.0;
        for (int m = 0; m < n; ++m) {
          fg += f[m] * g[m];
          ff += f[m] * f[m];
          gg += g[m] * g[m];
        }
        prod *= (ff > 0.0 && gg > 0.0) ? fabs(fg) / sqrt(ff * gg) : 0.0;
      }
      o = (float)prod;
    }
    ov[e] = o;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long used_i = 0ull, used_j = 0ull;
    for (int q = 0; q < R; ++q) slot_of[q] = q;
    for (int q = 0; q < R; ++q) {  // greedy: the best remaining (F term, slot) pair
      float best = -1.f;
      int bi = -1, bj = -1;
      for (int i = 0; i < R; ++i) {
        if (used_i >> i & 1ull) continue;
        for (int j = 0; j < R; ++j) {
          if (used_j >> j & 1ull) continue;
          if (ov[i * R + j] > best) {
            best = ov[i * R + j];
            bi = i;
            bj = j;
          }
        }
      }
      slot_of[bj] = bi;
      used_i |= 1ull << bi;
      used_j |= 1ull << bj;
    }
  }
  __syncthreads();
  for (int item = threadIdx.x; item < D * R; item += kWsThreads) {
    const int d = item / R, j = item - d * R;
    const double* f = b.base + (size_t)(foff + slot_of[j]) * b.nD + (size_t)d * n;
    double s2 = 0.0, dot = 0.0;
    if (top[j] >= 0) {
      const double* g = b.base + (size_t)(goff + top[j]) * b.nD + (size_t)d * n;
      const double gs = canon_scale(g, n);
      for (int m = 0; m < n; ++m) dot += f[m] * g[m] * gs;
    }
    for (int m = 0; m < n; ++m) s2 += f[m] * f[m];
    const double s = (s2 > 0.0) ? ((dot < 0.0) ? -1.0 : 1.0) / sqrt(s2) : 0.0;
    float* row = T + (size_t)(v * D + d) * ldt;
    for (int m = 0; m < n; ++m) row[j * n + m] = (float)(f[m] * s);
  }
}

__global__ void __launch_bounds__(kWsThreads) ws_apply_kernel(WsBatch b, const float* Y, int ldy) {
  extern __shared__ unsigned ws_smem[];
  __shared__ int top[64];
  __shared__ float rv[kWsThreads / 32];
  __shared__ int ri[kWsThreads / 32];
  const int v = blockIdx.x, n = b.n, D = b.ndof, R = b.rank;
  const long long goff = b.g_off[v], foff = b.f_off[v];
  top_terms(b.coef + goff, min(b.g_rank[v], b.rgmax), R, ws_smem, top, rv, ri);
  // weights first (f_coef may alias coef only at the F terms, which are not targets)
  for (int i = threadIdx.x; i < R; i += kWsThreads) b.f_coef[foff + i] = top[i] >= 0 ? fabs(b.coef[goff + top[i]]) : 0.0;
  for (int item = threadIdx.x; item < D * R; item += kWsThreads) {
    const int d = item / R, i = item - d * R;
    const float* y = Y + (size_t)(v * D + d) * ldy + (size_t)i * n;
    double s2 = 0.0;
    for (int m = 0; m < n; ++m) s2 += (double)y[m] * y[m];
    double* f = b.f_base + (size_t)(foff + i) * b.nD + (size_t)d * n;
    if (s2 > 0.0) {
      const double inv = 1.0 / sqrt(s2);
      for (int m = 0; m < n; ++m) f[m] = y[m] * inv;
    } else {
      for (int m = 0; m < n; ++m) f[m] = (m == i % n) ? 1.0 : 0.0;
    }
  }
}

size_t top_smem(const WsBatch& b, int rgmax) { return sizeof(unsigned) * (size_t)((rgmax + 31) / 32 + 1); }

}  // namespace

int ws_check(const WsBatch& b) {
  if (b.ntop < 1 || b.ntop > 64 || b.rank < 1 || b.rank > 64 || b.n < 1 || b.nD != b.ndof * b.n) {
    set_error("warm start: unsupported sizes (ntop=%d rank=%d n=%d ndof=%d nD=%d): modes of one basis size, "
              "ntop and rank at most 64", b.ntop, b.rank, b.n, b.ndof, b.nD);
    return kBadArgument;
  }
  return kOk;
}

int ws_features_launch(const WsBatch& b, __nv_bfloat16* X, int ldx, int rgmax, cudaStream_t st) {
  int rc = ws_check(b);
  if (rc) return rc;
  const size_t smem = top_smem(b, rgmax);
  if (smem > 48 * 1024 || rgmax < 1) {
    set_error("warm start: targets of %d terms outside the selection bitmap", rgmax);
    return kTooLarge;
  }
  WsBatch bb = b;
  bb.rgmax = rgmax;
  ws_features_kernel<<<b.nvec, kWsThreads, smem, st>>>(bb, X, ldx);
  MLCP_CUDA_TRY(cudaGetLastError());
  return kOk;
}

int ws_targets_launch(const WsBatch& b, float* T, int ldt, int rgmax, cudaStream_t st) {
  int rc = ws_check(b);
  if (rc) return rc;
  const size_t smem = top_smem(b, rgmax);
  if (smem > 24 * 1024 || rgmax < 1) {
    set_error("warm start: targets of %d terms outside the selection bitmap", rgmax);
    return kTooLarge;
  }
  WsBatch bb = b;
  bb.rgmax = rgmax;
  ws_targets_kernel<<<b.nvec, kWsThreads, smem, st>>>(bb, T, ldt);
  MLCP_CUDA_TRY(cudaGetLastError());
  return kOk;
}

int ws_apply_launch(const WsBatch& b, const float* Y, int ldy, int rgmax, cudaStream_t st) {
  int rc = ws_check(b);
  if (rc) return rc;
  const size_t smem = top_smem(b, rgmax);
  if (smem > 48 * 1024 || rgmax < 1) {
    set_error("warm start: targets of %d terms outside the selection bitmap", rgmax);
    return kTooLarge;
  }
  WsBatch bb = b;
  bb.rgmax = rgmax;
  ws_apply_kernel<<<b.nvec, kWsThreads, smem, st>>>(bb, Y, ldy);
  MLCP_CUDA_TRY(cudaGetLastError());
  return kOk;
}

}  // namespace mlcp

// ---------------------------------------------------------------------------
// extern "C" layer (device pointers; stream NULL: the library's stream)
// ---------------------------------------------------------------------------

namespace mlcp {
int finish_status(int status);
}

using namespace mlcp;

namespace {
cudaStream_t ws_stream(void* stream, int* rc) {
  if (stream) return static_cast<cudaStream_t>(stream);
  Context* ctx = get_context(rc);
  return ctx ? ctx->stream : nullptr;
}
}  // namespace

extern "C" int mlcp_mlp_gemm(const void* A, const void* B, int M, int N, int K, int lda, int ldb, const float* bias,
                             int act, const void* mask, int ldm, float* C, int ldc, void* Cb, int ldcb, void* Ct,
                             int ldct, int valid_m, int* d_status, void* stream) {
  int rc = kOk;
  cudaStream_t st = ws_stream(stream, &rc);
  if (rc) return finish_status(rc);
  if (!A || !B || (act == 2 && !mask) || act < 0 || act > 2) {
    set_error("mlcp_mlp_gemm: bad arguments");
    return finish_status(kBadArgument);
  }
  MlpGemm g;
  g.A = static_cast<const __nv_bfloat16*>(A); g.B = static_cast<const __nv_bfloat16*>(B);
  g.M = M; g.N = N; g.K = K; g.lda = lda; g.ldb = ldb; g.bias = bias; g.act = act;
  g.mask = static_cast<const __nv_bfloat16*>(mask); g.ldm = ldm; g.C = C; g.ldc = ldc;
  g.Cb = static_cast<__nv_bfloat16*>(Cb); g.ldcb = ldcb; g.Ct = static_cast<__nv_bfloat16*>(Ct); g.ldct = ldct;
  g.valid_m = valid_m; g.status = d_status;
  return finish_status(mlp_gemm_launch(g, st));
}

extern "C" int mlcp_mlp_loss(const float* Y, const float* T, int m, int n, int ld, int rows_p, void* dY, void* dYt,
                             float* loss, void* stream) {
  int rc = kOk;
  cudaStream_t st = ws_stream(stream, &rc);
  if (rc) return finish_status(rc);
  return finish_status(mlp_loss_launch(Y, T, m, n, ld, rows_p, static_cast<__nv_bfloat16*>(dY),
                                       static_cast<__nv_bfloat16*>(dYt), loss, st));
}

extern "C" int mlcp_mlp_colsum(const void* G, int rows, int n, int ld, float* db, void* stream) {
  int rc = kOk;
  cudaStream_t st = ws_stream(stream, &rc);
  if (rc) return finish_status(rc);
  return finish_status(mlp_colsum_launch(static_cast<const __nv_bfloat16*>(G), rows, n, ld, db, st));
}

extern "C" int mlcp_mlp_adam(float* w, const float* g, float* m1, float* m2, int rows, int cols, float lr, float b1,
                             float b2, float eps, int step, void* wb, void* wt, void* stream) {
  int rc = kOk;
  cudaStream_t st = ws_stream(stream, &rc);
  if (rc) return finish_status(rc);
  return finish_status(mlp_adam_launch(w, g, m1, m2, rows, cols, lr, b1, b2, eps, step,
                                       static_cast<__nv_bfloat16*>(wb), static_cast<__nv_bfloat16*>(wt), st));
}

namespace {
WsBatch make_ws(int nvec, int ndof, int n, int ntop, int rank, const long long* g_off, const int* g_rank,
                const long long* f_off, const double* base, const double* coef, double* f_base, double* f_coef) {
  WsBatch b;
  b.nvec = nvec; b.ndof = ndof; b.nD = ndof * n; b.n = n; b.ntop = ntop; b.rank = rank; b.rgmax = 0;
  b.g_off = g_off; b.g_rank = g_rank; b.f_off = f_off; b.base = base; b.coef = coef;
  b.f_base = f_base; b.f_coef = f_coef;
  return b;
}
}  // namespace

extern "C" int mlcp_ws_features(int nvec, int ndof, int n, int ntop, const long long* d_g_off, const int* d_g_rank,
                                int rgmax, const double* d_base, const double* d_coef, void* X, int ldx,
                                void* stream) {
  int rc = kOk;
  cudaStream_t st = ws_stream(stream, &rc);
  if (rc) return finish_status(rc);
  if (nvec < 1 || ldx < ntop * n + ntop) {
    set_error("mlcp_ws_features: nvec = %d, ldx = %d below ntop (n + 1) = %d", nvec, ldx, ntop * (n + 1));
    return finish_status(kBadArgument);
  }
  const WsBatch b = make_ws(nvec, ndof, n, ntop, 1, d_g_off, d_g_rank, nullptr, d_base, d_coef, nullptr, nullptr);
  return finish_status(ws_features_launch(b, static_cast<__nv_bfloat16*>(X), ldx, rgmax, st));
}

extern "C" int mlcp_ws_targets(int nvec, int ndof, int n, int rank, const long long* d_g_off, const int* d_g_rank,
                               int rgmax, const long long* d_f_off, const double* d_base, const double* d_coef, float* T,
                               int ldt, void* stream) {
  int rc = kOk;
  cudaStream_t st = ws_stream(stream, &rc);
  if (rc) return finish_status(rc);
  if (nvec < 1 || ldt < rank * n) {
    set_error("mlcp_ws_targets: nvec = %d, ldt = %d below rank n = %d", nvec, ldt, rank * n);
    return finish_status(kBadArgument);
  }
  const WsBatch b = make_ws(nvec, ndof, n, 1, rank, d_g_off, d_g_rank, d_f_off, d_base, d_coef, nullptr, nullptr);
  return finish_status(ws_targets_launch(b, T, ldt, rgmax, st));
}

extern "C" int mlcp_ws_apply(int nvec, int ndof, int n, int rank, const long long* d_g_off, const int* d_g_rank,
                             int rgmax, const long long* d_f_off, double* d_base, double* d_coef, const float* Y,
                             int ldy, void* stream) {
  int rc = kOk;
  cudaStream_t st = ws_stream(stream, &rc);
  if (rc) return finish_status(rc);
  if (nvec < 1 || ldy < rank * n) {
    set_error("mlcp_ws_apply: nvec = %d, ldy = %d below rank n = %d", nvec, ldy, rank * n);
    return finish_status(kBadArgument);
  }
  const WsBatch b = make_ws(nvec, ndof, n, 1, rank, d_g_off, d_g_rank, d_f_off, d_base, d_coef, d_base, d_coef);
  return finish_status(ws_apply_launch(b, Y, ldy, rgmax, st));
}
