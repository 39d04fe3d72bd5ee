// Learned ALS warm start: training and inference kernels of a small MLP
// (BF16 weights and activations, FP32 accumulation) that proposes the
// starting factors of an ALS rank reduction.  No counterpart in the
// reference, which starts its GPU ALS from a random CP vector
// (GPU_ALS_AA, src/GPUIterate.f90:191-210, GetRandomCPvec) or from a
// randomised interpolative decomposition on the CPU (reduc_RID,
// src/REDUCTIONML.f90:483-551).
//
// GEMM on the 5th-generation tensor cores: C[M x N] = A[M x K] B[N x K]^T
// with A and B BF16, K-major (row-major, K contiguous), one CTA of 4 warps
// per 128 x BN output tile (BN <= 256).  Per 64-wide K slice the operands
// are copied into shared memory in the canonical no-swizzle K-major layout
// (8-row x 16-byte core matrices: core (r/8, k/8) at ((r/8) 8 + k/8) 128
// bytes, so the core-matrix stride is 128 B along K and 1024 B along M/N),
// two stages deep; one elected thread issues four tcgen05.mma (kind::f16,
// M = 128, K = 16 each) into a TMEM accumulator and commits them to the
// stage's mbarrier, which the copies into that stage wait on (bounded
// waits: on expiry the kernel records status bit 1, stops issuing and
// still frees its tensor memory).  The epilogue reads the accumulator with
// tcgen05.ld (warp w: rows 32w..32w+31) and applies bias, ReLU or the ReLU
// derivative, writing FP32 and/or BF16 and a transposed BF16 copy (the
// operand layouts of the backward GEMMs).
#include <cuda_bf16.h>

#include <cstdint>

#include "common.cuh"
#include "mlp.cuh"

namespace mlcp {

namespace {

constexpr int kGemmThreads = 128;
constexpr int kBM = 128;
constexpr int kBK = 64;
constexpr int kMaxBN = 256;
constexpr int kStageA = kBM * kBK * 2;       // bytes
constexpr int kStageB = kMaxBN * kBK * 2;    // bytes
constexpr int kWaitLimit = 1 << 22;

__device__ __forceinline__ uint32_t saddr(const void* p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(saddr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait; false when the limit was reached.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  for (int it = 0; it < kWaitLimit; ++it)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(saddr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor, no swizzle, K-major canonical layout:
// start address, leading (K-direction) core-matrix offset 128 B, stride
// (M/N-direction) core-matrix offset 1024 B, descriptor version 1.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFFu);
  d |= (uint64_t)(128u >> 4) << 16;
  d |= (uint64_t)(1024u >> 4) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor of kind::f16: BF16 A and B, FP32 D, both K-major,
// M = 128, N = n.
__device__ __forceinline__ uint32_t idesc_bf16(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(kBM >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(saddr(bar))
               : "memory");
}

// 32 consecutive FP32 columns of this warp's 32 TMEM lanes (lane = row).
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int q = 0; q < 32; ++q) v[q] = __uint_as_float(r[q]);
}

// Copy rows [r0, r0 + rows) x K slice [k0, k0 + 64) of a K-major BF16 matrix
// into the core-matrix layout at dst (one 16-byte chunk per copy).
__device__ __forceinline__ void stage_tile(unsigned char* dst, const __nv_bfloat16* src, int ld, int r0, int rows,
                                           int k0) {
  for (int c = threadIdx.x; c < rows * 8; c += kGemmThreads) {
    const int r = c >> 3, kc = c & 7;
    unsigned char* d = dst + (((r >> 3) * 8 + kc) << 7) + ((r & 7) << 4);
    cp_async16(d, src + (size_t)(r0 + r) * ld + k0 + kc * 8);
  }
}

}  // namespace

__global__ void __launch_bounds__(kGemmThreads, 1) mlp_gemm_kernel(MlpGemm p) {
  extern __shared__ __align__(1024) unsigned char gsm[];
  unsigned char* sA = gsm;                        // [2][kStageA]
  unsigned char* sB = gsm + 2 * kStageA;          // [2][kStageB]
  __shared__ __align__(8) uint64_t bar[2];
  __shared__ uint32_t tmem_base;
  __shared__ int abort_flag;
  const int m0 = blockIdx.x * kBM, n0 = blockIdx.y * kMaxBN;
  const int bn = min(kMaxBN, p.N - n0);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(&tmem_base)),
                 "r"(kMaxBN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base;
  const uint32_t idesc = idesc_bf16(bn);
  const int KT = p.K / kBK;
  uint32_t phase[2] = {0u, 0u};
  for (int kt = 0; kt < KT; ++kt) {
    const int st = kt & 1;
    if (kt >= 2) {  // the MMAs of slice kt - 2 have finished reading this stage
      if (!abort_flag && !mbar_wait(&bar[st], phase[st])) atomicExch(&abort_flag, 1);
      phase[st] ^= 1u;
    }
    __syncthreads();
    if (abort_flag) break;
    stage_tile(sA + st * kStageA, p.A, p.lda, m0, kBM, kt * kBK);
    stage_tile(sB + st * kStageB, p.B, p.ldb, n0, bn, kt * kBK);
    cp_async_wait_all();
    fence_proxy_async();
    __syncthreads();
    if (threadIdx.x == 0) {
      tc_fence_after();
      const uint32_t a0 = saddr(sA + st * kStageA), b0 = saddr(sB + st * kStageB);
#pragma unroll
      for (int kk = 0; kk < kBK / 16; ++kk)
        mma_bf16(tmem, smem_desc(a0 + kk * 256), smem_desc(b0 + kk * 256), idesc, (kt > 0 || kk > 0) ? 1u : 0u);
      mma_commit(&bar[st]);
    }
  }
  // the last commit covers every MMA issued before it
  if (!abort_flag && KT > 0) {
    const int st = (KT - 1) & 1;
    if (!mbar_wait(&bar[st], phase[st])) atomicExch(&abort_flag, 1);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (!abort_flag) {
    const int row = m0 + warp * 32 + lane;
    const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
    for (int c0 = 0; c0 < bn; c0 += 32) {
      float v[32];
      tmem_ld32(trow + (uint32_t)c0, v);
#pragma unroll
      for (int q = 0; q < 32; ++q) {
        const int col = n0 + c0 + q;
        if (c0 + q >= bn) break;
        float x = v[q];
        if (p.bias) x += p.bias[col];
        if (p.act == 1) x = fmaxf(x, 0.f);
        if (p.act == 2) x = (__bfloat162float(p.mask[(size_t)row * p.ldm + col]) > 0.f) ? x : 0.f;
        if (row >= p.valid_m) x = 0.f;
        if (p.C) p.C[(size_t)row * p.ldc + col] = x;
        const __nv_bfloat16 xb = __float2bfloat16_rn(x);
        if (p.Cb) p.Cb[(size_t)row * p.ldcb + col] = xb;
        if (p.Ct) p.Ct[(size_t)col * p.ldct + row] = xb;
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kMaxBN) : "memory");
  if (threadIdx.x == 0 && abort_flag && p.status) atomicOr(p.status, 2);
}

size_t mlp_gemm_smem_bytes() { return 2 * (size_t)kStageA + 2 * (size_t)kStageB; }

int mlp_gemm_launch(const MlpGemm& g, cudaStream_t st) {
  if (g.M % kBM || g.K % kBK || g.N % 16 || g.N <= 0 || g.K <= 0 || g.lda % 8 || g.ldb % 8) {
    set_error("mlp gemm: unsupported shape M=%d N=%d K=%d (M multiple of 128, N of 16, K of 64)", g.M, g.N, g.K);
    return kBadArgument;
  }
  const size_t smem = mlp_gemm_smem_bytes();
  MLCP_CUDA_TRY(cudaFuncSetAttribute(mlp_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  dim3 grid(g.M / kBM, (g.N + kMaxBN - 1) / kMaxBN);
  mlp_gemm_kernel<<<grid, kGemmThreads, smem, st>>>(g);
  MLCP_CUDA_TRY(cudaGetLastError());
  return kOk;
}

// ---------------------------------------------------------------------------
// Loss, bias gradients, optimiser
// ---------------------------------------------------------------------------

// Mean squared error over the valid block (rows < m, cols < n) of Y against
// T (both [rows][ld] FP32); dY = 2 (Y - T) / (m n) as BF16 [rows][ld] and
// transposed [ld][rows_p]; loss accumulated into *loss.
__global__ void mlp_loss_kernel(const float* Y, const float* T, int m, int n, int ld, int rows_p,
                                __nv_bfloat16* dY, __nv_bfloat16* dYt, float* loss) {
  const long long total = (long long)rows_p * ld;
  const float scale = 2.f / ((float)m * (float)n);
  float part = 0.f;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(e / ld), c = (int)(e - (long long)r * ld);
    float g = 0.f;
    if (r < m && c < n) {
      const float d = Y[e] - T[e];
      part += d * d;
      g = scale * d;
    }
    const __nv_bfloat16 gb = __float2bfloat16_rn(g);
    dY[e] = gb;
    dYt[(size_t)c * rows_p + r] = gb;
  }
  for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, part / ((float)m * (float)n));
}

// db[c] = sum over rows of G[r][c] (BF16 [rows][ld]); one thread per column.
__global__ void mlp_colsum_kernel(const __nv_bfloat16* G, int rows, int n, int ld, float* db) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  float s = 0.f;
  for (int r = 0; r < rows; ++r) s += __bfloat162float(G[(size_t)r * ld + c]);
  db[c] = s;
}

// Adam step on FP32 master parameters [rows][cols]; writes the BF16 copy
// and, when wt is given, the transposed BF16 copy [cols][rows].
__global__ void mlp_adam_kernel(float* w, const float* g, float* m1, float* m2, int rows, int cols, float lr,
                                float b1, float b2, float eps, float c1, float c2, __nv_bfloat16* wb,
                                __nv_bfloat16* wt) {
  const long long total = (long long)rows * cols;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const float gv = g[e];
    const float a = b1 * m1[e] + (1.f - b1) * gv;
    const float b = b2 * m2[e] + (1.f - b2) * gv * gv;
    m1[e] = a;
    m2[e] = b;
    const float x = w[e] - lr * (a / c1) / (sqrtf(b / c2) + eps);
    w[e] = x;
    const __nv_bfloat16 xb = __float2bfloat16_rn(x);
    if (wb) wb[e] = xb;
    if (wt) {
      const int r = (int)(e / cols), c = (int)(e - (long long)r * cols);
      wt[(size_t)c * rows + r] = xb;
    }
  }
}

int mlp_loss_launch(const float* Y, const float* T, int m, int n, int ld, int rows_p, __nv_bfloat16* dY,
                    __nv_bfloat16* dYt, float* loss, cudaStream_t st) {
  const long long total = (long long)rows_p * ld;
  mlp_loss_kernel<<<(int)std::min<long long>((total + 255) / 256, 1024), 256, 0, st>>>(Y, T, m, n, ld, rows_p, dY,
                                                                                       dYt, loss);
  MLCP_CUDA_TRY(cudaGetLastError());
  return kOk;
}

int mlp_colsum_launch(const __nv_bfloat16* G, int rows, int n, int ld, float* db, cudaStream_t st) {
  mlp_colsum_kernel<<<(n + 127) / 128, 128, 0, st>>>(G, rows, n, ld, db);
  MLCP_CUDA_TRY(cudaGetLastError());
  return kOk;
}

int mlp_adam_launch(float* w, const float* g, float* m1, float* m2, int rows, int cols, float lr, float b1, float b2,
                    float eps, int step, __nv_bfloat16* wb, __nv_bfloat16* wt, cudaStream_t st) {
  const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
  const long long total = (long long)rows * cols;
  mlp_adam_kernel<<<(int)std::min<long long>((total + 255) / 256, 2048), 256, 0, st>>>(w, g, m1, m2, rows, cols, lr,
                                                                                       b1, b2, eps, c1, c2, wb, wt);
  MLCP_CUDA_TRY(cudaGetLastError());
  return kOk;
}

}  // namespace mlcp
