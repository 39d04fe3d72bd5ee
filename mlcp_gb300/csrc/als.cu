// Batched explicit-target ALS rank reduction on GB300.
//
// Computes, for every vector of a batch, the reference's ITERATE_ALS
// (src/als.cu:1021-1078, called through alscpp_ src/intertwining.cu:180):
//   for nals sweeps, for each mode k:
//     b(i,n)  = sum_j cG_j G_j^k(n) prod_{d!=k} <G_j^d, F_i^d>
//     BB(i,i') = prod_{d!=k} <F_i^d, F_i'^d> + pen delta(i,i'),  pen = 1e-10 max cF
//     X = BB^-1 b;  F_i^k = X(i,:) / ||X(i,:)||,  cF_i = ||X(i,:)||
//
// GB300 design: one persistent thread-block cluster per vector, 16 warps per
// CTA, each CTA owning a contiguous range of target terms j.
//  * State.  Each CTA keeps in shared memory, for its terms j and every F term
//    i, the running product P(j,i) = prod over all modes but one of
//    <G_j^d, F_i^d> (FP32).  Mode step t solves mode k = t mod D; kp and kn
//    are the modes before and after it.
//  * Phase B (critical path, all 16 warps): P(j,i) holds the product without
//    modes kp and k; multiply in <G_j^kp, Fnew_i^kp> with the factor solved in
//    the previous step, and accumulate b(i,n) += cG_j P(j,i) G_j^k(n).  The
//    partial b of the CTA goes to distributed shared memory.
//  * One cluster barrier.  Every CTA then gathers the partial right-hand sides
//    in the same order and runs the same R x R solve (warps 0-3), so each CTA
//    holds the identical new factor and nothing is broadcast back.
//  * Phase A (warps 4-15, concurrent with the solve): divide mode kn out of
//    P, <G_j^kn, F_i^kn> with the current factor, so that the next phase B
//    only has to multiply mode k back in.  Unsafe divisions (zero divisor,
//    product outside the normal FP32 range) are rebuilt from the factors.
//  * Target factors live in an FP32 mode-major copy, so the slice of one mode
//    for a CTA's terms is one contiguous run; tiles of 128 terms stream into a
//    ring of shared-memory stages with cp.async.bulk and mbarrier completion.
//  * The R x R normal equations, the F Gram products and the normalisation run
//    in double-word arithmetic (dword.cuh) on the FP32 pipes.  The normal
//    equations of the next step are formed when a solve ends; their FP32
//    inverse (the refinement's preconditioner) is computed in registers by a
//    warp that phase B leaves idle, when there is one.
// One launch covers all sweeps; the host is not involved between steps.

#include <cooperative_groups.h>
#include <cuda_bf16.h>
#include <cfloat>
#include <cstdint>

#include "common.cuh"
#include "als.cuh"
#include "dword.cuh"
#include "dwsolve.cuh"

namespace cg = cooperative_groups;

namespace mlcp {

// ---------------------------------------------------------------------------
// Preparation: FP32 mode-major target copy, FP32 weights, unit-normalised
// double-word copy of F.
// ---------------------------------------------------------------------------

// Vector owning row `row` of a prefix-sum table (binary search).
__device__ inline int owner(const long long* row_off, int nvec, long long row) {
  int lo = 0, hi = nvec - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (row_off[mid] <= row) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// One thread per (term, mode) element run; grid-stride.
// Target factors to the mode-major FP32 copy.  Block row y is one
// (vector, mode) pair, whose destination [rG][gs] is contiguous: consecutive
// threads write consecutive floats and read consecutive doubles of a factor.
// With a shared target only vector 0's terms are converted.
__global__ void __launch_bounds__(256) als_prep_target_kernel(AlsParams p) {
  const int nv = p.shared_target ? 1 : p.nvec;
  const long long x0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long xs = (long long)gridDim.x * blockDim.x;
  for (long long vd = blockIdx.y; vd < (long long)nv * p.ndof; vd += gridDim.y) {
    const int v = (int)(vd / p.ndof), d = (int)(vd - (long long)v * p.ndof);
    const int rG = p.rG[v], n = p.nbas[d], gs = als_gstride(n);
    const double* src = p.g_base + p.g_term_off[v] * (long long)p.nD + p.off[d];
    float* dst = p.gm + p.gm_off[v] + (long long)p.offg[d] * rG;
    // four entries per thread (gs is a multiple of 4): one 16-byte store
    const int g4 = gs / 4;
    const long long cnt = (long long)rG * g4;
    for (long long e = x0; e < cnt; e += xs) {
      const long long j = e / g4;
      const int q = 4 * (int)(e - j * g4);
      const double* s = src + j * p.nD + q;
      float4 o;
      o.x = (q < n) ? (float)s[0] : 0.f;
      o.y = (q + 1 < n) ? (float)s[1] : 0.f;
      o.z = (q + 2 < n) ? (float)s[2] : 0.f;
      o.w = (q + 3 < n) ? (float)s[3] : 0.f;
      reinterpret_cast<float4*>(dst)[e] = o;
    }
    if (d == 0 && !p.shared_target)
      for (long long j = x0; j < rG; j += xs) p.gc[p.g_row_off[v] + j] = (float)p.g_coef[p.g_term_off[v] + j];
  }
}

// The same conversion for targets in mapped host memory: entries are read in
// the caller's term-major order (consecutive threads, consecutive doubles of
// one vector's target terms), so the host link moves long contiguous runs;
// each goes to its mode's row of the mode-major copy, and the last entry of a
// mode's row also writes the row's zero padding.  Dynamic shared memory: the
// mode of every column, then the per-mode offsets.
__global__ void __launch_bounds__(256) als_prep_target_rows_kernel(AlsParams p) {
  extern __shared__ int prep_smem[];
  int* cmode = prep_smem;            // [nD]
  int* soff = cmode + p.nD;          // [D+1] reference-layout offsets
  int* soffg = soff + p.ndof + 1;    // [D+1] target-copy offsets
  for (int c = threadIdx.x; c <= p.ndof; c += blockDim.x) {
    soff[c] = p.off[c];
    soffg[c] = p.offg[c];
  }
  for (int c = threadIdx.x; c < p.nD; c += blockDim.x) {
    int d = 0;
    while (p.off[d + 1] <= c) ++d;
    cmode[c] = d;
  }
  __syncthreads();
  const int nv = p.shared_target ? 1 : p.nvec;
  const long long x0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long xs = (long long)gridDim.x * blockDim.x;
  for (int v = blockIdx.y; v < nv; v += gridDim.y) {
    const int rG = p.rG[v];
    const double* src = p.g_base + p.g_term_off[v] * (long long)p.nD;
    float* dst = p.gm + p.gm_off[v];
    const long long total = (long long)rG * p.nD;
    for (long long e = x0; e < total; e += xs) {
      const long long j = e / p.nD;
      const int c = (int)(e - j * p.nD), d = cmode[c], q = c - soff[d];
      const int n = soff[d + 1] - soff[d], gs = als_gstride(n);
      float* row = dst + (long long)soffg[d] * rG + j * gs;
      row[q] = (float)src[e];
      if (q == n - 1)
        for (int z = n; z < gs; ++z) row[z] = 0.f;
    }
    if (!p.shared_target)
      for (long long j = x0; j < rG; j += xs) p.gc[p.g_row_off[v] + j] = (float)p.g_coef[p.g_term_off[v] + j];
  }
}

// The target weights of a shared target, and F's factors.
__global__ void als_prep_kernel(AlsParams p) {
  const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long stride = (long long)gridDim.x * blockDim.x;
  if (p.shared_target)
    for (long long e = tid; e < p.total_rows; e += stride) p.gc[e] = (float)p.shared_w[e];
  // F: each factor scaled to unit 2-norm (a zero factor stays zero), split
  // into FP32 high and low parts.  Scaling F's factors only rescales the rows
  // and columns of the normal equations and the rows of b; the normalised
  // solution is unchanged, and the products stay inside the FP32 exponent
  // range for any factor norms the FP64 reference handles.
  for (long long e = tid; e < p.total_f_terms * p.ndof; e += stride) {
    const long long frow = e / p.ndof;
    const int d = (int)(e % p.ndof);
    const int v = owner(p.f_row_off, p.nvec, frow);
    const int i = (int)(frow - p.f_row_off[v]);
    const int n = p.nbas[d], np = round_up(n, 4);
    const double* src = p.base + (p.term_off[v] + i) * (long long)p.nD + p.off[d];
    double ss = 0.0;
    for (int q = 0; q < n; ++q) ss += src[q] * src[q];
    const double sc = (ss > 0.0) ? 1.0 / sqrt(ss) : 1.0;
    float* hi = p.f32 + frow * p.nDp + p.offp[d];
    float* lo = p.f32lo + frow * p.nDp + p.offp[d];
    for (int q = 0; q < np; ++q) {
      const double x = (q < n) ? src[q] * sc : 0.0;
      const float h = (float)x;
      hi[q] = h;
      lo[q] = (float)(x - (double)h);
    }
  }
}

// ---------------------------------------------------------------------------
// Bulk-copy ring primitives (cp.async.bulk + mbarrier, inline PTX)
// ---------------------------------------------------------------------------

namespace {

__device__ __forceinline__ uint32_t smem_addr(const void* ptr) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(ptr));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Global -> shared bulk copy completing on `bar` (addresses 16-byte aligned,
// size a multiple of 16).
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

// 8-byte asynchronous global -> shared copy, and the wait for this thread's copies.
__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

__device__ __forceinline__ void fence_async_shared() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void cluster_arrive() { asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory"); }
__device__ __forceinline__ void cluster_wait() { asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory"); }

// Iterations of mbarrier.try_wait (each suspends the thread for a bounded
// hardware interval) before a stage wait is declared failed.
constexpr int kWaitLimit = 1 << 20;

}  // namespace

// ---------------------------------------------------------------------------
// Shared-memory carve (host and device agree on it)
// ---------------------------------------------------------------------------

struct AlsSmem {
  int rFp, ldP, stage_floats, kp, nf;
  size_t bar, done, issued, fillno, flags, ring, P, cw, fa, fb, bred, bpart, BB, X, L, sk, dinv, u, nrm, misc, gi, b0, res,
      red, cb, fp, tcbar, tbase, total;
};

__host__ __device__ inline size_t carve(size_t* cursor, size_t bytes, size_t align) {
  const size_t o = (*cursor + align - 1) / align * align;
  *cursor = o + bytes;
  return o;
}

__host__ __device__ inline AlsSmem als_smem_layout(int rows_cta, int rF, int npmax, int gsmax, int stages,
                                                    int tc = 0) {
  AlsSmem s;
  s.rFp = round_up(rF, 4);
  s.ldP = round_up(rows_cta > 0 ? rows_cta : 1, 32);
  s.stage_floats = kAlsTileRows * 2 * gsmax;
  s.kp = als_tc_kp(npmax);
  s.nf = als_tc_nf(rF);
  size_t o = 0;
  s.bar = carve(&o, 8 * (size_t)stages, 16);
  s.done = carve(&o, 4 * (size_t)stages, 16);
  s.issued = carve(&o, 4 * (size_t)stages, 16);
  s.fillno = carve(&o, 4 * (size_t)stages, 16);
  s.flags = carve(&o, 4 * 8, 16);
  s.ring = carve(&o, sizeof(float) * (size_t)stages * s.stage_floats, 128);
  s.P = carve(&o, tc ? 0 : sizeof(float) * (size_t)s.rFp * s.ldP, 16);  // tensor memory in the tensor-core form
  s.cw = carve(&o, sizeof(float) * (size_t)s.ldP, 16);
  s.fa = carve(&o, sizeof(float) * (size_t)s.rFp * gsmax, 16);
  s.fb = carve(&o, sizeof(float) * (size_t)s.rFp * gsmax, 16);
  s.bred = carve(&o, sizeof(float) * kAlsWarps * 64, 16);
  s.bpart = carve(&o, sizeof(float) * 2 * (size_t)s.rFp * npmax, 16);
  s.BB = carve(&o, sizeof(dw) * (size_t)rF * rF, 16);
  s.X = carve(&o, sizeof(dw) * (size_t)rF * npmax, 16);
  s.L = carve(&o, sizeof(dw) * (size_t)rF * rF, 16);
  s.sk = carve(&o, sizeof(dw) * (size_t)rF * rF, 16);
  s.dinv = carve(&o, sizeof(dw) * (size_t)rF, 16);
  s.u = carve(&o, sizeof(dw) * (size_t)rF, 16);
  s.nrm = carve(&o, sizeof(dw) * (size_t)rF, 16);
  s.misc = carve(&o, sizeof(dw) * 4, 16);
  s.gi = carve(&o, sizeof(float) * 2 * (size_t)rF * rF, 16);
  s.b0 = carve(&o, sizeof(dw) * (size_t)rF * npmax, 16);
  s.res = carve(&o, sizeof(dw) * (size_t)rF * npmax, 16);
  s.red = carve(&o, sizeof(float) * 4, 16);
  // tensor-core form: two tiles' BF16 operand pieces (hi, mid, lo), the
  // factor's pieces, the MMA completion barriers, the tensor-memory base
  s.cb = carve(&o, tc ? (size_t)2 * 3 * kAlsTileRows * s.kp * 2 : 0, 128);
  s.fp = carve(&o, tc ? (size_t)3 * s.nf * s.kp * 2 : 0, 128);
  s.tcbar = carve(&o, 8 * 2, 16);
  s.tbase = carve(&o, 4, 16);
  s.total = o;
  return s;
}

namespace {

// Per-thread view of one CTA's part of the reduction.
struct Cta {
  int tid, warp, lane, rank, CL, v, D, rF, rFp, nIq, rG, row0, nrows, ntiles, ldP, gsmax, npmax, nDp, stages,
      stage_floats;
  uint64_t* bar;
  int* done;
  int* issued;
  unsigned* fillno;  // [stages] tile sequence number the stage was last armed with
  int* flags;  // [0] pipeline abort, [1] non-positive pivot seen, [2] FP32 inverse pivots positive
  float* ring;
  float* P;    // [rFp][ldP] running products (term index fastest)
  float* cw;   // [ldP] target weights of the CTA's terms
  float* fa;   // [rFp][gsmax] factor divided out in phase A / multiplied in the prologue
  float* fb;   // [rFp][gsmax] factor multiplied in by phase B (solved in the previous step)
  float* bred; // [warps][64] per-warp partial right-hand sides
  float* bpart;  // [2][rFp][npmax] CTA partial right-hand side (read by the cluster)
  dw *BB, *X, *L, *sk, *dinv, *u, *nrm, *misc;
  float* gi;   // [2][rF*rF] FP32 Gauss-Jordan buffers (the inverse ends in one)
  dw* b0;      // [rF][npmax] right-hand side (kept for the refinement residuals)
  dw* res;     // [rF][npmax] refinement residual
  float* red;  // [2][2] block maxima of the last refinement correction and of |X|
  const float* gm;  // this vector's FP32 target copy
  float* fcta;      // this CTA's FP32 factor copy [rF][nDp]
  dw* gram;         // this CTA's Grams [D][rF][rF]
  dw* suf;          // this CTA's suffix products [D][rF][rF]
  // tensor-core form
  int tc, kp, nf;         // engine; K and N of the MMA (basis and rF padded to 16)
  unsigned char* cb;      // [2][3][128 x kp] BF16 pieces of two target tiles (canonical K-major)
  unsigned char* fp;      // [3][nf x kp] BF16 pieces of the factor
  uint64_t* tcbar;        // [2] MMA completion of the two result buffers
  uint32_t tmem;          // tensor-memory base: results at columns [0, 2 nf), running products after
};

// Tile source: one or two mode slabs of the CTA's target terms.
struct TileSrc {
  const float* a;
  int gsa;
  const float* b;
  int gsb;
};

__device__ void issue_tile(const Cta& c, unsigned g, int T, const TileSrc& s) {
  const int st = (int)(g % (unsigned)c.stages);
  const int r0 = T * kAlsTileRows;
  const int rows = min(kAlsTileRows, c.nrows - r0);
  float* dst = c.ring + (size_t)st * c.stage_floats;
  const uint32_t ba = (uint32_t)(rows * s.gsa * 4);
  const uint32_t bb = s.b ? (uint32_t)(rows * s.gsb * 4) : 0u;
  c.issued[st] += 1;
  *(volatile unsigned*)&c.fillno[st] = g;
  fence_async_shared();
  mbar_expect_tx(&c.bar[st], ba + bb);
  bulk_load(dst, s.a + (long long)(c.row0 + r0) * s.gsa, ba, &c.bar[st]);
  if (s.b) bulk_load(dst + kAlsTileRows * s.gsa, s.b + (long long)(c.row0 + r0) * s.gsb, bb, &c.bar[st]);
}

// First tiles of a phase (one thread; the ring is idle).
__device__ void start_phase(const Cta& c, unsigned seq, const TileSrc& s) {
  for (int T = 0; T < c.ntiles && T < c.stages; ++T) issue_tile(c, seq + T, T, s);
}

// Wait until tile g has landed (every lane of the warp calls it).  The
// stage's phase parity alone cannot tell fill g from fill g - 2*stages, and a
// warp whose items skip tiles can reach fill g while the stage still holds
// an older one; so the stage must first be armed with g (fillno), after which
// every earlier fill of the stage has completed and the parity is unambiguous.
__device__ bool wait_tile(const Cta& c, unsigned g) {
  const int st = (int)(g % (unsigned)c.stages);
  const uint32_t par = (g / (unsigned)c.stages) & 1u;
  volatile int* abort_flag = c.flags;
  volatile unsigned* armed = c.fillno + st;
  // the whole warp decides together (callers are whole warps), so that the
  // warp stays converged for the shuffles of the consumers
  for (int it = 0; it < kWaitLimit; ++it) {
    const bool ready = *armed == g && mbar_try_wait(&c.bar[st], par);
    if (__all_sync(0xffffffffu, ready)) return true;
    if (__any_sync(0xffffffffu, *abort_flag != 0)) return false;
  }
  atomicExch(c.flags, 1);
  return false;
}

// The warp is done with tile g (index T in its phase); the last of the
// tile's `consumers` warps refills the stage with tile T + stages.
__device__ void release_tile(const Cta& c, unsigned g, int T, int consumers, const TileSrc& s) {
  __syncwarp();
  if (c.lane == 0) {
    const int st = (int)(g % (unsigned)c.stages);
    __threadfence_block();
    const int old = atomicAdd(&c.done[st], 1);
    if (old == consumers - 1) {
      c.done[st] = 0;
      if (T + c.stages < c.ntiles && !*(volatile int*)c.flags) issue_tile(c, g + c.stages, T + c.stages, s);
    }
  }
  __syncwarp();
}

// Quotient a / b from the approximate reciprocal plus one Newton correction.
__device__ __forceinline__ float div_nr(float a, float b) {
  const float r = f_rcp_approx(b);
  const float q = a * r;
  return fmaf(fmaf(-b, q, a), r, q);
}

// out[a][cc] = <G_row, F_{cc}> for the lane's four rows lane + 32a of a tile
// (row stride gs) and four factors f + cc*fld, over np padded entries.  Phase
// A, phase B and the prologue all use this routine, so a factor divided out
// of P is bit-identical to the one multiplied in earlier.
__device__ __forceinline__ void tile_dots(const float* tile, int gs, const float* f, int fld, int np, int lane,
                                          float (&out)[4][4]) {
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int cc = 0; cc < 4; ++cc) out[a][cc] = 0.f;
  for (int q = 0; q < np; q += 4) {
    float4 g[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) g[a] = *reinterpret_cast<const float4*>(tile + (lane + 32 * a) * gs + q);
#pragma unroll
    for (int cc = 0; cc < 4; ++cc) {
      const float4 x = *reinterpret_cast<const float4*>(f + cc * fld + q);
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        float s = out[a][cc];
        s = fmaf(g[a].x, x.x, s);
        s = fmaf(g[a].y, x.y, s);
        s = fmaf(g[a].z, x.z, s);
        s = fmaf(g[a].w, x.w, s);
        out[a][cc] = s;
      }
    }
  }
}

// prod over modes d not in {ex1, ex2} of <G_j^d, F_i^d>, straight from the
// FP32 copies in global memory (unsafe-division fallback; kept out of line to
// keep the hot loops small).  Called by a whole warp for one (j, i): one lane
// alone would leave its warp, and so phase A, waiting on D dependent
// global-memory dot products.
__device__ __noinline__ float rebuild_product(const Cta& c, const AlsParams& p, int j, int i, int ex1, int ex2) {
  // the whole warp, lane l taking modes l, l + 32, ...; the partial
  // products meet in a butterfly (multiplication commutes, so every lane
  // ends with the same value)
  float s = 1.f;
  for (int d = c.lane; d < c.D; d += 32) {
    if (d == ex1 || d == ex2) continue;
    const int n = p.nbas[d], gs = als_gstride(n);
    const float* g = c.gm + (long long)p.offg[d] * c.rG + (long long)(c.row0 + j) * gs;
    const float* f = c.fcta + (long long)i * c.nDp + p.offp[d];
    float t = 0.f;
    for (int q = 0; q < n; ++q) t = fmaf(g[q], f[q], t);
    s *= t;
  }
  for (int o = 16; o > 0; o >>= 1) s *= __shfl_xor_sync(0xffffffffu, s, o);
  return s;
}

// Stage the current FP32 factor of mode d from this CTA's copy into dst
// ([rFp][gsmax], zero rows beyond rF).  Threads [t0, t0 + nt) take part.
__device__ void load_factor(const Cta& c, const AlsParams& p, int d, float* dst, int t0, int nt) {
  const int np = round_up(p.nbas[d], 4);
  for (int e = c.tid - t0; e < c.rFp * np; e += nt) {
    const int i = e / np, q = e - i * np;
    dst[i * c.gsmax + q] = (i < c.rF) ? c.fcta[(long long)i * c.nDp + p.offp[d] + q] : 0.f;
  }
}

// Product pass over the tiles of mode d, items (tile, i-quad) dealt
// round-robin to warps [w0, w0 + nw):
//   divide = false: P(j,i) *= <G_j^d, F_i^d>            (prologue)
//   divide = true:  P(j,i) /= <G_j^d, F_i^d>, rebuilding prod_{d' not in
//                   {ex, d}} when the division is unsafe  (phase A)
// fa holds F^d.  One thread of the group must call start_phase first.
__device__ void product_pass(const Cta& c, const AlsParams& p, unsigned seq, int d, bool divide, int ex, int w0,
                             int nw) {
  const int n = p.nbas[d], np = round_up(n, 4), gs = als_gstride(n);
  const TileSrc src{c.gm + (long long)p.offg[d] * c.rG, gs, nullptr, 0};
  const int nitems = c.ntiles * c.nIq;
  for (int it = c.warp - w0; it < nitems; it += nw) {
    const int T = it / c.nIq, iq = it - T * c.nIq;
    const unsigned g = seq + (unsigned)T;
    if (wait_tile(c, g)) {
      const float* tile = c.ring + (size_t)(g % (unsigned)c.stages) * c.stage_floats;
      float po[4][4];
      tile_dots(tile, gs, c.fa + iq * 4 * c.gsmax, c.gsmax, np, c.lane, po);
      // every load before any store: a shared-memory store would order each
      // later load behind it (the compiler cannot prove they do not alias)
      float pv[4][4];
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        const int j = T * kAlsTileRows + c.lane + 32 * a;
#pragma unroll
        for (int cc = 0; cc < 4; ++cc) {
          const int i = iq * 4 + cc;
          pv[a][cc] = (j < c.nrows && i < c.rF) ? c.P[(size_t)i * c.ldP + j] : 0.f;
        }
      }
      // quotients without any call in the unrolled loop (a call would keep
      // the sixteen independent chains from overlapping); the rare unsafe
      // ones are marked and rebuilt afterwards
      unsigned rebuild = 0u;
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int cc = 0; cc < 4; ++cc) {
          if (!divide) {
            pv[a][cc] *= po[a][cc];
          } else {
            const float x = pv[a][cc];
            const float qv = div_nr(x, po[a][cc]);
            const bool ok = fabsf(x) >= FLT_MIN && fabsf(qv) <= FLT_MAX;  // also catches a zero divisor
            const int j = T * kAlsTileRows + c.lane + 32 * a, i = iq * 4 + cc;
            if (!ok && j < c.nrows && i < c.rF) rebuild |= 1u << (a * 4 + cc);
            pv[a][cc] = qv;
          }
        }
      // rebuilds, one entry at a time by the whole warp
      for (unsigned pending = __ballot_sync(0xffffffffu, rebuild != 0u); pending;
           pending = __ballot_sync(0xffffffffu, rebuild != 0u)) {
        const int L = __ffs(pending) - 1;
        const int bit = __ffs(__shfl_sync(0xffffffffu, rebuild, L)) - 1;
        const int a = bit >> 2, cc = bit & 3;
        const float qv = rebuild_product(c, p, T * kAlsTileRows + L + 32 * a, iq * 4 + cc, ex, d);
        if (c.lane == L) {
          rebuild &= rebuild - 1;
#pragma unroll
          for (int a2 = 0; a2 < 4; ++a2)
#pragma unroll
            for (int c2 = 0; c2 < 4; ++c2)
              if (a2 * 4 + c2 == bit) pv[a2][c2] = qv;
        }
      }
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        const int j = T * kAlsTileRows + c.lane + 32 * a;
        if (j >= c.nrows) continue;
#pragma unroll
        for (int cc = 0; cc < 4; ++cc) {
          const int i = iq * 4 + cc;
          if (i < c.rF) c.P[(size_t)i * c.ldP + j] = pv[a][cc];
        }
      }
    }
    release_tile(c, g, T, c.nIq, src);
  }
}

// Phase B, first right-hand-side columns [0, MW) (round 0): P(j,i) *= <G_j^kp,
// Fnew_i^kp>, then acc(i,m) += cG_j P(j,i) G_j^k(m) for the warp's i-quad.
template <int MW>
__device__ __forceinline__ void item_b0(const Cta& c, const float* tp, int gsp, int npp, const float* tk, int gsk,
                                        int T, int iq, float (&acc)[4][MW]) {
  float pn[4][4];
  tile_dots(tp, gsp, c.fb + iq * 4 * c.gsmax, c.gsmax, npp, c.lane, pn);
  // every load before any store (see product_pass), then the products, then
  // the stores; w ends as the weighted products cG_j P(j,i)
  float w[4][4], cwj[4];
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    const int j = T * kAlsTileRows + c.lane + 32 * a;
    const bool live = j < c.nrows;
    cwj[a] = live ? c.cw[j] : 0.f;
#pragma unroll
    for (int cc = 0; cc < 4; ++cc) w[a][cc] = live ? c.P[(size_t)(iq * 4 + cc) * c.ldP + j] : 0.f;
  }
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int cc = 0; cc < 4; ++cc) w[a][cc] *= pn[a][cc];
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    const int j = T * kAlsTileRows + c.lane + 32 * a;
    if (j < c.nrows)
#pragma unroll
      for (int cc = 0; cc < 4; ++cc) c.P[(size_t)(iq * 4 + cc) * c.ldP + j] = w[a][cc];
  }
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int cc = 0; cc < 4; ++cc) w[a][cc] *= cwj[a];
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    float4 g4[MW / 4];
#pragma unroll
    for (int m4 = 0; m4 < MW / 4; ++m4)
      g4[m4] = *reinterpret_cast<const float4*>(tk + (c.lane + 32 * a) * gsk + 4 * m4);
#pragma unroll
    for (int cc = 0; cc < 4; ++cc) {
      const float wv = w[a][cc];
#pragma unroll
      for (int m4 = 0; m4 < MW / 4; ++m4) {
        acc[cc][4 * m4 + 0] = fmaf(wv, g4[m4].x, acc[cc][4 * m4 + 0]);
        acc[cc][4 * m4 + 1] = fmaf(wv, g4[m4].y, acc[cc][4 * m4 + 1]);
        acc[cc][4 * m4 + 2] = fmaf(wv, g4[m4].z, acc[cc][4 * m4 + 2]);
        acc[cc][4 * m4 + 3] = fmaf(wv, g4[m4].w, acc[cc][4 * m4 + 3]);
      }
    }
  }
}

// Phase B, later right-hand-side columns [m0, m0 + MW): P is already updated.
template <int MW>
__device__ __forceinline__ void item_bm(const Cta& c, const float* tk, int gsk, int m0, int T, int iq,
                                        float (&acc)[4][MW]) {
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    const int j = T * kAlsTileRows + c.lane + 32 * a;
    const bool live = j < c.nrows;
    const float cwj = live ? c.cw[j] : 0.f;
    float w[4];
#pragma unroll
    for (int cc = 0; cc < 4; ++cc) w[cc] = live ? cwj * c.P[(size_t)(iq * 4 + cc) * c.ldP + j] : 0.f;
    float4 g4[MW / 4];
#pragma unroll
    for (int m4 = 0; m4 < MW / 4; ++m4)
      g4[m4] = *reinterpret_cast<const float4*>(tk + (c.lane + 32 * a) * gsk + m0 + 4 * m4);
#pragma unroll
    for (int cc = 0; cc < 4; ++cc)
#pragma unroll
      for (int m4 = 0; m4 < MW / 4; ++m4) {
        acc[cc][4 * m4 + 0] = fmaf(w[cc], g4[m4].x, acc[cc][4 * m4 + 0]);
        acc[cc][4 * m4 + 1] = fmaf(w[cc], g4[m4].y, acc[cc][4 * m4 + 1]);
        acc[cc][4 * m4 + 2] = fmaf(w[cc], g4[m4].z, acc[cc][4 * m4 + 2]);
        acc[cc][4 * m4 + 3] = fmaf(w[cc], g4[m4].w, acc[cc][4 * m4 + 3]);
      }
  }
}

// Whether the last warp has no i-quad in phase B (16 not a multiple of the
// i-quad count) and rF <= 32: it then inverts the step's normal equations in
// registers during the first round.
__device__ __forceinline__ bool phase_b_inverts(const Cta& c) {
  return !c.tc && c.rF <= 32 && (kAlsWarps / c.nIq) * c.nIq < kAlsWarps;
}

// Sums the 4 MW accumulators of each lane over the warp into out[cc MW + m]
// by recursive halving: at each level a lane sends the half of its values it
// gives up to its partner and adds the half it keeps, so 64 values (padded)
// cost 32 + 16 + 8 + 4 + 2 shuffles per lane instead of 5 per value.
template <int MW>
__device__ __forceinline__ void warp_sum_values(const float (&acc)[4][MW], int lane, float* out) {
  constexpr int NV = 4 * MW;
  constexpr int P2 = NV <= 16 ? 16 : (NV <= 32 ? 32 : 64);
  float v[P2];
#pragma unroll
  for (int q = 0; q < P2; ++q) v[q] = q < NV ? acc[q / MW][q % MW] : 0.f;
  int base = 0;
  int n = P2;
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) {
    const bool up = (lane & o) != 0;
    if (n > 1) {
      const int h = n / 2;
#pragma unroll
      for (int q = 0; q < P2 / 2; ++q) {
        if (q >= h) break;
        const float send = up ? v[q] : v[h + q];
        const float keep = up ? v[h + q] : v[q];
        v[q] = keep + __shfl_xor_sync(0xffffffffu, send, o);
      }
      if (up) base += h;
      n = h;
    } else {
      v[0] += __shfl_xor_sync(0xffffffffu, v[0], o);
    }
  }
  // this lane holds the totals of values base .. base + n - 1 (n = 1 or 2);
  // with fewer than 32 slots several lanes hold the same total
#pragma unroll
  for (int q = 0; q < 2; ++q)
    if (q < n && base + q < NV && (P2 >= 32 || (lane & 1) == 0)) out[base + q] = v[q];
}

// One round of phase B over all tiles (all 16 warps; warp -> i-quad iq =
// warp mod nIq, tiles T = warp / nIq (mod warps per i-quad)), ending with the
// CTA's partial right-hand side columns [16 round, 16 round + MW) in bout.
template <int MW>
__device__ void phase_b_round(const Cta& c, const AlsParams& p, unsigned seq, int round, int k, int kp, float* bout) {
  const int nk = p.nbas[k], gsk = als_gstride(nk);
  const int npp = round_up(p.nbas[kp], 4), gsp = als_gstride(p.nbas[kp]);
  const float* slab_k = c.gm + (long long)p.offg[k] * c.rG;
  const float* slab_p = c.gm + (long long)p.offg[kp] * c.rG;
  const TileSrc src = (round == 0) ? TileSrc{slab_p, gsp, slab_k, gsk} : TileSrc{slab_k, gsk, nullptr, 0};
  const int wpi = kAlsWarps / c.nIq;
  const bool active = c.warp < wpi * c.nIq;
  const int iq = c.warp % c.nIq, sub = c.warp / c.nIq;
  if (c.tid == 0) start_phase(c, seq, src);
  float acc[4][MW];
#pragma unroll
  for (int cc = 0; cc < 4; ++cc)
#pragma unroll
    for (int m = 0; m < MW; ++m) acc[cc][m] = 0.f;
  if (!active && round == 0 && c.warp == kAlsWarps - 1 && phase_b_inverts(c)) {
    // the idle warp inverts this step's normal equations (formed at the end
    // of the previous solve) for the solver warps
    const bool g = dwsolve::gj_inverse_warp(c.BB, c.rF, c.gi);
    if (c.lane == 0) c.flags[2] = g;
  }
  if (active) {
    for (int T = sub; T < c.ntiles; T += wpi) {
      const unsigned g = seq + (unsigned)T;
      if (wait_tile(c, g)) {
        const float* tile = c.ring + (size_t)(g % (unsigned)c.stages) * c.stage_floats;
        if (round == 0)
          item_b0<MW>(c, tile, gsp, npp, tile + kAlsTileRows * gsp, gsk, T, iq, acc);
        else
          item_bm<MW>(c, tile, gsk, 16 * round, T, iq, acc);
      }
      release_tile(c, g, T, c.nIq, src);
    }
    warp_sum_values<MW>(acc, c.lane, c.bred + c.warp * 64);
  }
  __syncthreads();
  // sum over the warps of each i-quad (fixed order)
  for (int e = c.tid; e < c.nIq * 4 * MW; e += kAlsThreads) {
    const int q4 = e / (4 * MW), r = e - q4 * 4 * MW, cc = r / MW, m = r - cc * MW;
    float s = 0.f;
    for (int sb = 0; sb < wpi; ++sb) s += c.bred[(q4 + sb * c.nIq) * 64 + cc * MW + m];
    bout[(q4 * 4 + cc) * c.npmax + 16 * round + m] = s;
  }
  __syncthreads();
}

// All rounds of phase B for mode k (previous mode kp); returns tiles used.
__device__ unsigned phase_b(const Cta& c, const AlsParams& p, unsigned seq, int k, int kp, float* bout) {
  const int npk = round_up(p.nbas[k], 4);
  unsigned used = 0;
  for (int round = 0; 16 * round < npk; ++round) {
    const int mw = min(16, npk - 16 * round);
    switch (mw) {
      case 4: phase_b_round<4>(c, p, seq + used, round, k, kp, bout); break;
      case 8: phase_b_round<8>(c, p, seq + used, round, k, kp, bout); break;
      case 12: phase_b_round<12>(c, p, seq + used, round, k, kp, bout); break;
      default: phase_b_round<16>(c, p, seq + used, round, k, kp, bout); break;
    }
    used += (unsigned)c.ntiles;
  }
  return used;
}

// ---------------------------------------------------------------------------
// Tensor-core form of the product passes (AlsParams::tc)
// ---------------------------------------------------------------------------
// For a tile of 128 target terms j and mode d the dot products
// D(j, i) = <G_j^d, F_i^d> of every F term i are one MMA on the 5th-generation
// tensor cores: A = the tile (128 x kp, K = the basis padded to 16), B = the
// factor (nf x kp), D in tensor memory (lane j, column i).  Both operands are
// split into three BF16 pieces, x = h + m + l (each the BF16 rounding of what
// the previous pieces leave, so the split is exact to 2^-27 of x), and six
// products mm + hl + lh + hm + mh + hh (smallest first) are accumulated in
// FP32: the dropped ml, lm, ll terms are below 2^-26 of the product, so the
// dots carry the accuracy of FP32 dots.  The same instructions on the same
// operands give bit-identical results, so a factor divided out of a running
// product is exactly the one multiplied in earlier, as in the CUDA-core form.
//
// The running products P(j, i) live in tensor memory (columns 2 nf + T rF + i
// for tile T), so a tile's update is tcgen05.ld of D and P, the product or
// quotient in registers, tcgen05.st of P: warp w reaches lanes 32 (w % 4) ..
// +31 (its rows of every tile) and the warps sharing a lane quarter split the
// F terms.  Tiles are pipelined two deep: while the warps update tile T from
// result buffer T % 2, the operand pieces of tile T + 1 are converted and its
// MMAs run into the other buffer.

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor, no swizzle, K-major canonical layout:
// 8-row x 16-byte core matrices, 128 B apart along K and sbo apart along
// M/N; descriptor version 1.
__device__ __forceinline__ uint64_t tc_desc(uint32_t addr, uint32_t sbo) {
  uint64_t d = (uint64_t)((addr >> 4) & 0x3FFFu);
  d |= (uint64_t)(128u >> 4) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor of kind::f16: BF16 A and B (K-major), FP32 D, M = 128, N = n.
__device__ __forceinline__ uint32_t tc_idesc(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                       uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void tc_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
               : "memory");
}

// LW consecutive FP32 columns of this warp's 32 lanes, waited for inside the
// same statement (so no use of the values can be scheduled before the wait).
template <int LW>
__device__ __forceinline__ void tm_ld(uint32_t taddr, float (&v)[LW]);

template <>
__device__ __forceinline__ void tm_ld<8>(uint32_t taddr, float (&v)[8]) {
  uint32_t r[8];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int q = 0; q < 8; ++q) v[q] = __uint_as_float(r[q]);
}

template <>
__device__ __forceinline__ void tm_ld<16>(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int q = 0; q < 16; ++q) v[q] = __uint_as_float(r[q]);
}

// One FP32 column of this warp's 32 lanes.
__device__ __forceinline__ void tm_st1(uint32_t taddr, float v) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x1.b32 [%0], {%1};" ::"r"(taddr), "r"(__float_as_uint(v)) : "memory");
}
__device__ __forceinline__ void tm_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// Tensor-memory address of column col in the lane quarter of this warp.
__device__ __forceinline__ uint32_t tm_addr(const Cta& c, int col) {
  return c.tmem + ((uint32_t)(32 * (c.warp & 3)) << 16) + (uint32_t)col;
}
__device__ __forceinline__ int tc_pcol(const Cta& c, int T) { return 2 * c.nf + T * c.rF; }
__device__ __forceinline__ unsigned char* tc_cbuf(const Cta& c, unsigned s) {
  return c.cb + (size_t)(s & 1u) * 3 * kAlsTileRows * c.kp * 2;
}

// BF16 three-way split of eight floats, packed per piece.
__device__ __forceinline__ void split3(const float (&x)[8], uint4& h, uint4& m, uint4& l) {
  uint32_t hw[4], mw[4], lw[4];
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    uint32_t ph = 0, pm = 0, pl = 0;
#pragma unroll
    for (int z = 0; z < 2; ++z) {
      const float v = x[2 * u + z];
      const __nv_bfloat16 bh = __float2bfloat16_rn(v);
      const float r1 = v - __bfloat162float(bh);
      const __nv_bfloat16 bm = __float2bfloat16_rn(r1);
      const float r2 = r1 - __bfloat162float(bm);
      const __nv_bfloat16 bl = __float2bfloat16_rn(r2);
      ph |= (uint32_t)__bfloat16_as_ushort(bh) << (16 * z);
      pm |= (uint32_t)__bfloat16_as_ushort(bm) << (16 * z);
      pl |= (uint32_t)__bfloat16_as_ushort(bl) << (16 * z);
    }
    hw[u] = ph;
    mw[u] = pm;
    lw[u] = pl;
  }
  h = make_uint4(hw[0], hw[1], hw[2], hw[3]);
  m = make_uint4(mw[0], mw[1], mw[2], mw[3]);
  l = make_uint4(lw[0], lw[1], lw[2], lw[3]);
}

// Rows [0, rows) of a matrix (row stride ld floats, n valid entries per
// row, entries [n, round_up(n, 4)) readable) as three BF16 pieces of a
// rows x kp operand in the canonical K-major layout: 16-byte chunk (r, kc)
// at ((r / 8) (kp / 8) + kc) 128 + (r % 8) 16 bytes; piece stride `piece`
// bytes.  Rows >= valid are written as zeros.  Threads t of nt.
__device__ __forceinline__ void tc_split_rows(const float* src, int ld, int n, int valid, int rows, int kp,
                                              unsigned char* dst, size_t piece, int t, int nt) {
  const int kc8 = kp / 8;
  for (int e = t; e < rows * kc8; e += nt) {
    const int r = e / kc8, kc = e - r * kc8, q0 = kc * 8;
    float x[8];
    float4 a = make_float4(0.f, 0.f, 0.f, 0.f), b = a;
    if (r < valid) {
      if (q0 < n) a = *reinterpret_cast<const float4*>(src + (size_t)r * ld + q0);
      if (q0 + 4 < n) b = *reinterpret_cast<const float4*>(src + (size_t)r * ld + q0 + 4);
    }
    x[0] = a.x; x[1] = a.y; x[2] = a.z; x[3] = a.w;
    x[4] = b.x; x[5] = b.y; x[6] = b.z; x[7] = b.w;
#pragma unroll
    for (int u = 0; u < 8; ++u)
      if (q0 + u >= n) x[u] = 0.f;
    uint4 h, m, l;
    split3(x, h, m, l);
    const size_t off = ((size_t)(r >> 3) * kc8 + kc) * 128 + (size_t)(r & 7) * 16;
    *reinterpret_cast<uint4*>(dst + off) = h;
    *reinterpret_cast<uint4*>(dst + piece + off) = m;
    *reinterpret_cast<uint4*>(dst + 2 * piece + off) = l;
  }
}

// The six MMAs of one tile (one thread): D[dcol..] = sum over K of A B^T.
__device__ __forceinline__ void tc_issue(const Cta& c, unsigned s) {
  tc_fence_after();
  const uint32_t a0 = smem_addr(tc_cbuf(c, s)), b0 = smem_addr(c.fp);
  const uint32_t pa = (uint32_t)kAlsTileRows * c.kp * 2, pb = (uint32_t)c.nf * c.kp * 2;
  const uint32_t sbo = (uint32_t)(c.kp / 8) * 128;
  const uint32_t idesc = tc_idesc(c.nf);
  const uint32_t dt = c.tmem + (uint32_t)((s & 1u) * c.nf);
  // pieces 0 = hi, 1 = mid, 2 = lo; (A, B) pairs smallest first
  const int ap[6] = {1, 0, 2, 0, 1, 0}, bq[6] = {1, 2, 0, 1, 0, 0};
  uint32_t acc = 0;
  for (int ks = 0; ks < c.kp / 16; ++ks)
#pragma unroll
    for (int u = 0; u < 6; ++u) {
      tc_mma(dt, tc_desc(a0 + ap[u] * pa + ks * 256, sbo), tc_desc(b0 + bq[u] * pb + ks * 256, sbo), idesc, acc);
      acc = 1;
    }
  tc_commit(&c.tcbar[s & 1u]);
}

// Bounded wait (whole warp) for the MMAs of tile sequence number s.
__device__ bool tc_wait(const Cta& c, unsigned s) {
  uint64_t* bar = &c.tcbar[s & 1u];
  const uint32_t par = (s >> 1) & 1u;
  for (int it = 0; it < kWaitLimit; ++it) {
    const bool ready = mbar_try_wait(bar, par);
    if (__all_sync(0xffffffffu, ready)) return true;
  }
  atomicExch(c.flags, 1);
  return false;
}

// Barrier of the warps taking part in a pass: all 16, or warps 4-15 (named
// barrier 2, the phase-A warps).
__device__ __forceinline__ void tc_part_sync(int nw) {
  if (nw == kAlsWarps) __syncthreads();
  else asm volatile("bar.sync 2, %0;" ::"r"(nw * 32) : "memory");
}

// One pipelined pass over the CTA's tiles of a slab (row stride gs, n
// entries): each tile's dot products with the factor whose pieces are in
// c.fp, one MMA batch per tile (sequence numbers tcseq, tcseq + 1, ...),
// then consume(T, ok) by the warps [w0, w0 + nw) (nw = 12 or 16).  The ring
// stage of a tile is released after its consumption.
// The ring stage of tile g (index T) is free: refill it with tile T + stages.
// One thread, after a barrier that follows every use of the stage.  The
// refill of tile T + 1 happens in the iteration before its conversion, so
// the tensor-core form needs at least three stages.
__device__ __forceinline__ void tc_release(const Cta& c, unsigned g, int T, const TileSrc& s) {
  if (T + c.stages < c.ntiles && !*(volatile int*)c.flags) issue_tile(c, g + c.stages, T + c.stages, s);
}

template <class Consume>
__device__ void tc_pass(const Cta& c, unsigned seq, unsigned tcseq, const TileSrc& src, int gs, int n, int w0,
                        int nw, Consume&& consume) {
  const int t = c.tid - 32 * w0, nt = 32 * nw;
  const size_t piece = (size_t)kAlsTileRows * c.kp * 2;
  auto convert = [&](int T) {
    const unsigned g = seq + (unsigned)T;
    const bool got = wait_tile(c, g);
    const float* tile = c.ring + (size_t)(g % (unsigned)c.stages) * c.stage_floats;
    const int rows = min(kAlsTileRows, c.nrows - T * kAlsTileRows);
    tc_split_rows(tile, gs, n, got ? rows : 0, kAlsTileRows, c.kp, tc_cbuf(c, tcseq + (unsigned)T), piece, t, nt);
  };
  // one barrier per tile: tile T + 1 is converted and its MMAs issued before
  // tile T is consumed, so they run while the warps wait for and use tile T.
  // Reuse is safe: MMA T + 1 writes the result buffer of tile T - 1, consumed
  // before this barrier, and convert T + 1 overwrites the operands of MMA
  // T - 1, which every thread waited for in the previous iteration.
  // The ring stage of tile T - 1 is released once, by the issuing thread,
  // after the barrier that follows every warp's use of it.
  if (c.ntiles > 0) convert(0);
  fence_async_shared();
  tc_part_sync(nw);
  if (t == 0 && c.ntiles > 0) tc_issue(c, tcseq);
  for (int T = 0; T < c.ntiles; ++T) {
    if (T + 1 < c.ntiles) {
      convert(T + 1);
      fence_async_shared();
      tc_fence_before();
      tc_part_sync(nw);
      if (t == 0) {
        tc_issue(c, tcseq + (unsigned)(T + 1));
        if (T > 0) tc_release(c, seq + (unsigned)(T - 1), T - 1, src);
      }
    }
    const bool ok = tc_wait(c, tcseq + (unsigned)T);
    tc_fence_after();
    consume(T, ok);
    tm_wait_st();
    tc_fence_before();
  }
  tc_part_sync(nw);
  if (t == 0 && c.ntiles > 0) {
    if (c.ntiles >= 2) tc_release(c, seq + (unsigned)(c.ntiles - 2), c.ntiles - 2, src);
    tc_release(c, seq + (unsigned)(c.ntiles - 1), c.ntiles - 1, src);
  }
}

// The F terms [i0, i0 + cnt) of this warp when nw warps share the rF terms
// four lane quarters at a time.
__device__ __forceinline__ void tc_cols(const Cta& c, int w0, int nw, int& i0, int& cnt, int& ci) {
  const int ng = nw >> 2, grp = (c.warp - w0) >> 2;
  ci = (c.rF + ng - 1) / ng;
  i0 = min(c.rF, grp * ci);
  cnt = min(c.rF, i0 + ci) - i0;
}

// Product pass of mode d (tensor-core form), warps [w0, w0 + nw):
//   kDivide = false: P(j,i) *= <G_j^d, F_i^d>            (prologue)
//   kDivide = true:  P(j,i) /= <G_j^d, F_i^d>, rebuilding prod_{d' not in
//                    {ex, d}} when the division is unsafe  (phase A)
// fa holds F^d.  One thread of the group must call start_phase first.
template <int LW, bool kDivide>
__device__ void tc_product_pass(const Cta& c, const AlsParams& p, unsigned seq, unsigned tcseq, int d, int ex,
                                int w0, int nw) {
  const int n = p.nbas[d], gs = als_gstride(n);
  const TileSrc src{c.gm + (long long)p.offg[d] * c.rG, gs, nullptr, 0};
  tc_split_rows(c.fa, c.gsmax, n, c.rF, c.nf, c.kp, c.fp, (size_t)c.nf * c.kp * 2, c.tid - 32 * w0, 32 * nw);
  int i0, cnt, ci;
  tc_cols(c, w0, nw, i0, cnt, ci);
  const int q = c.warp & 3;
  tc_pass(c, seq, tcseq, src, gs, n, w0, nw, [&](int T, bool ok) {
    if (cnt <= 0) return;
    const int j = T * kAlsTileRows + 32 * q + c.lane;
    const bool live = ok && j < c.nrows;
    float dv[LW], pv[LW];
    tm_ld<LW>(tm_addr(c, (int)((tcseq + (unsigned)T) & 1u) * c.nf + i0), dv);
    tm_ld<LW>(tm_addr(c, tc_pcol(c, T) + i0), pv);
    if (!kDivide) {
#pragma unroll
      for (int u = 0; u < LW; ++u)
        if (u < cnt) pv[u] *= dv[u];
    } else {
      unsigned rebuild = 0u;
#pragma unroll
      for (int u = 0; u < LW; ++u) {
        if (u >= cnt) continue;
        const float x = pv[u];
        const float qv = div_nr(x, dv[u]);
        const bool good = fabsf(x) >= FLT_MIN && fabsf(qv) <= FLT_MAX;  // also catches a zero divisor
        if (!good && live) rebuild |= 1u << u;
        pv[u] = qv;
      }
      for (unsigned pending = __ballot_sync(0xffffffffu, rebuild != 0u); pending;
           pending = __ballot_sync(0xffffffffu, rebuild != 0u)) {
        const int L = __ffs(pending) - 1;
        const int bit = __ffs(__shfl_sync(0xffffffffu, rebuild, L)) - 1;
        const float qv = rebuild_product(c, p, T * kAlsTileRows + 32 * q + L, i0 + bit, ex, d);
        if (c.lane == L) {
          rebuild &= rebuild - 1;
#pragma unroll
          for (int u = 0; u < LW; ++u)
            if (u == bit) pv[u] = qv;
        }
      }
    }
#pragma unroll
    for (int u = 0; u < LW; ++u)
      if (u < cnt) tm_st1(tm_addr(c, tc_pcol(c, T) + i0 + u), pv[u]);
  });
}

// Sums NV values of each lane over the warp into out[0 .. NV) by recursive
// halving (as warp_sum_values).
template <int NV>
__device__ __forceinline__ void warp_sum_flat(const float (&a)[NV], int lane, float* out) {
  constexpr int P2 = NV <= 16 ? 16 : (NV <= 32 ? 32 : 64);
  static_assert(NV <= 64, "at most 64 values per lane");
  float v[P2];
#pragma unroll
  for (int q = 0; q < P2; ++q) v[q] = q < NV ? a[q] : 0.f;
  int base = 0;
  int n = P2;
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) {
    const bool up = (lane & o) != 0;
    if (n > 1) {
      const int h = n / 2;
#pragma unroll
      for (int q = 0; q < P2 / 2; ++q) {
        if (q >= h) break;
        const float send = up ? v[q] : v[h + q];
        const float keep = up ? v[h + q] : v[q];
        v[q] = keep + __shfl_xor_sync(0xffffffffu, send, o);
      }
      if (up) base += h;
      n = h;
    } else {
      v[0] += __shfl_xor_sync(0xffffffffu, v[0], o);
    }
  }
#pragma unroll
  for (int q = 0; q < 2; ++q)
    if (q < n && base + q < NV && (P2 >= 32 || (lane & 1) == 0)) out[base + q] = v[q];
}

// One round of phase B (tensor-core form, all 16 warps) for right-hand-side
// columns [m0, m0 + MW): round 0 multiplies <G_j^kp, Fnew_i^kp> into P (one
// MMA batch per tile, factor pieces from fb); every round accumulates
// acc(i, m) += cG_j P(j,i) G_j^k(m0 + m) for the warp's F terms and lane
// rows, and ends with the CTA's partial right-hand side columns in bout.
template <int LW, int CI, int MW>
__device__ void tc_phase_b_round(const Cta& c, const AlsParams& p, unsigned seq, unsigned tcseq, int round, int m0,
                                 int k, int kp, float* bout) {
  const int gsk = als_gstride(p.nbas[k]);
  const int np_ = p.nbas[kp], gsp = als_gstride(np_);
  const float* slab_k = c.gm + (long long)p.offg[k] * c.rG;
  const float* slab_p = c.gm + (long long)p.offg[kp] * c.rG;
  const TileSrc src = (round == 0) ? TileSrc{slab_p, gsp, slab_k, gsk} : TileSrc{slab_k, gsk, nullptr, 0};
  const int koff = (round == 0) ? kAlsTileRows * gsp : 0;  // the k slab's place in a stage
  int i0, cnt, ci;
  tc_cols(c, 0, kAlsWarps, i0, cnt, ci);
  const int q = c.warp & 3, jj = 32 * q + c.lane;
  float acc[CI][MW];
#pragma unroll
  for (int u = 0; u < CI; ++u)
#pragma unroll
    for (int m = 0; m < MW; ++m) acc[u][m] = 0.f;
  auto accumulate = [&](int T, const float* stage, const float (&pv)[LW], bool live) {
    // rows beyond the CTA's terms hold arbitrary running products (0/0 after
    // a division): select them away, never multiply them by a zero weight
    const float cwj = live ? c.cw[T * kAlsTileRows + jj] : 0.f;
    float w[CI];
#pragma unroll
    for (int u = 0; u < CI; ++u) w[u] = (live && u < cnt) ? pv[u] * cwj : 0.f;
    const float* tk = stage + koff + jj * gsk + m0;
    float4 g4[MW / 4];
#pragma unroll
    for (int m4 = 0; m4 < MW / 4; ++m4) g4[m4] = *reinterpret_cast<const float4*>(tk + 4 * m4);
#pragma unroll
    for (int u = 0; u < CI; ++u)
#pragma unroll
      for (int m4 = 0; m4 < MW / 4; ++m4) {
        acc[u][4 * m4 + 0] = fmaf(w[u], g4[m4].x, acc[u][4 * m4 + 0]);
        acc[u][4 * m4 + 1] = fmaf(w[u], g4[m4].y, acc[u][4 * m4 + 1]);
        acc[u][4 * m4 + 2] = fmaf(w[u], g4[m4].z, acc[u][4 * m4 + 2]);
        acc[u][4 * m4 + 3] = fmaf(w[u], g4[m4].w, acc[u][4 * m4 + 3]);
      }
  };
  if (round == 0) {
    if (c.tid == 0) start_phase(c, seq, src);
    tc_split_rows(c.fb, c.gsmax, np_, c.rF, c.nf, c.kp, c.fp, (size_t)c.nf * c.kp * 2, c.tid, kAlsThreads);
    tc_pass(c, seq, tcseq, src, gsp, np_, 0, kAlsWarps, [&](int T, bool ok) {
      if (cnt <= 0) return;
      const unsigned g = seq + (unsigned)T;
      const float* stage = c.ring + (size_t)(g % (unsigned)c.stages) * c.stage_floats;
      const bool live = ok && T * kAlsTileRows + jj < c.nrows;
      float dv[LW], pv[LW];
      tm_ld<LW>(tm_addr(c, (int)((tcseq + (unsigned)T) & 1u) * c.nf + i0), dv);
      tm_ld<LW>(tm_addr(c, tc_pcol(c, T) + i0), pv);
#pragma unroll
      for (int u = 0; u < LW; ++u)
        if (u < cnt) pv[u] *= dv[u];
#pragma unroll
      for (int u = 0; u < LW; ++u)
        if (u < cnt) tm_st1(tm_addr(c, tc_pcol(c, T) + i0 + u), pv[u]);
      accumulate(T, stage, pv, live);
    });
  } else {
    __syncthreads();  // the ring is idle (every tile of the previous round released)
    if (c.tid == 0) start_phase(c, seq, src);
    for (int T = 0; T < c.ntiles; ++T) {
      const unsigned g = seq + (unsigned)T;
      const bool ok = wait_tile(c, g);
      if (cnt > 0) {
        const float* stage = c.ring + (size_t)(g % (unsigned)c.stages) * c.stage_floats;
        float pv[LW];
        tm_ld<LW>(tm_addr(c, tc_pcol(c, T) + i0), pv);
        accumulate(T, stage, pv, ok && T * kAlsTileRows + jj < c.nrows);
      }
      release_tile(c, g, T, kAlsWarps, src);
    }
  }
  {
    float flat[CI * MW];
#pragma unroll
    for (int u = 0; u < CI; ++u)
#pragma unroll
      for (int m = 0; m < MW; ++m) flat[u * MW + m] = acc[u][m];
    warp_sum_flat<CI * MW>(flat, c.lane, c.bred + c.warp * 64);
  }
  __syncthreads();
  // sum over the four lane quarters of each F term (fixed order)
  for (int e = c.tid; e < c.rF * MW; e += kAlsThreads) {
    const int i = e / MW, m = e - i * MW, grp = i / ci, u = i - grp * ci;
    float s = 0.f;
#pragma unroll
    for (int qq = 0; qq < 4; ++qq) s += c.bred[(qq + 4 * grp) * 64 + u * MW + m];
    bout[i * c.npmax + m0 + m] = s;
  }
  __syncthreads();
}

template <int LW, int CI, int RW>
__device__ unsigned tc_phase_b_rounds(const Cta& c, const AlsParams& p, unsigned seq, unsigned tcseq, int k, int kp,
                                      float* bout) {
  const int npk = round_up(p.nbas[k], 4);
  unsigned used = 0;
  for (int round = 0, m0 = 0; m0 < npk; ++round, m0 += RW) {
    const int mw = min(RW, npk - m0);
    if (mw >= RW) tc_phase_b_round<LW, CI, RW>(c, p, seq + used, tcseq, round, m0, k, kp, bout);
    else if (mw == 12) tc_phase_b_round<LW, CI, (RW > 12 ? 12 : RW)>(c, p, seq + used, tcseq, round, m0, k, kp, bout);
    else if (mw == 8) tc_phase_b_round<LW, CI, (RW > 8 ? 8 : RW)>(c, p, seq + used, tcseq, round, m0, k, kp, bout);
    else tc_phase_b_round<LW, CI, 4>(c, p, seq + used, tcseq, round, m0, k, kp, bout);
    used += (unsigned)c.ntiles;
  }
  return used;
}

// All rounds of phase B for mode k (tensor-core form); returns tiles used.
// Round widths keep CI x MW accumulators per lane within 64 registers.
__device__ unsigned tc_phase_b(const Cta& c, const AlsParams& p, unsigned seq, unsigned tcseq, int k, int kp,
                               float* bout) {
  const int cib = (c.rF + 3) / 4;
  if (cib <= 4) return tc_phase_b_rounds<8, 4, 16>(c, p, seq, tcseq, k, kp, bout);
  if (cib == 5) return tc_phase_b_rounds<8, 5, 12>(c, p, seq, tcseq, k, kp, bout);
  if (cib == 6) return tc_phase_b_rounds<8, 6, 8>(c, p, seq, tcseq, k, kp, bout);
  return tc_phase_b_rounds<8, 8, 8>(c, p, seq, tcseq, k, kp, bout);
}

// Running products of every tile set to 1 (tensor-core form, all warps).
__device__ void tc_init_products(const Cta& c) {
  int i0, cnt, ci;
  tc_cols(c, 0, kAlsWarps, i0, cnt, ci);
  for (int T = 0; T < c.ntiles; ++T)
    for (int u = 0; u < cnt; ++u) tm_st1(tm_addr(c, tc_pcol(c, T) + i0 + u), 1.f);
  tm_wait_st();
}

// The double-word solver team (threads 0-127, named barrier 1).
static_assert(kAlsSolverWarps == dwsolve::kSolverWarps, "solver team size");
using dwsolve::kSolverThreads;
using dwsolve::solver_sync;
using dwsolve::dw_ldlt;
using dwsolve::dw_ldlt_solve;
using dwsolve::gj_inverse;
using dwsolve::refine_solve;

// Suffix products for the next sweep: suf[d] = prod_{d' > d} gram[d']
// (elementwise), suf[D-1] = 1; and the prefix L reset to 1.  Threads t of
// nt (the solver warps, or the one warp that does this during phase B).
__device__ void dw_suffix(const Cta& c, int t, int nt) {
  const int rr = c.rF * c.rF;
  const dw* __restrict__ gram = c.gram;
  dw* __restrict__ suf = c.suf;
  for (int e = t; e < rr; e += nt) {
    dw a = dw_make(1.f);
    suf[(size_t)(c.D - 1) * rr + e] = a;
    // eight Gram entries loaded together per round (global memory)
    for (int d0 = c.D - 1; d0 >= 1; d0 -= 8) {
      dw gv[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) gv[u] = (d0 - u >= 1) ? gram[(size_t)(d0 - u) * rr + e] : dw_make(1.f);
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        if (d0 - u < 1) break;
        a = dw_mul(a, gv[u]);
        suf[(size_t)(d0 - u - 1) * rr + e] = a;
      }
    }
    c.L[e] = dw_make(1.f);
  }
}

// Gram matrix of the unit-normalised new factor of mode k (rows of X), stored
// for the suffix products of the next sweep and folded into the prefix L.
__device__ void dw_new_gram(const Cta& c, int k, int nk, int t, int nt) {
  const int rF = c.rF, rr = rF * rF;
  for (int e = t; e < rr; e += nt) {
    const int i = e % rF, i2 = e / rF;
    if (i > i2) continue;
    dw_acc acc = acc_zero();
    for (int q = 0; q < nk; ++q) acc_fma(acc, c.X[i + q * rF], c.X[i2 + q * rF]);
    const dw s = acc_value(acc);
    c.gram[(size_t)k * rr + i + i2 * rF] = s;
    c.gram[(size_t)k * rr + i2 + i * rF] = s;
    if (k < c.D - 1) {
      c.L[i + i2 * rF] = dw_mul(c.L[i + i2 * rF], s);
      if (i != i2) c.L[i2 + i * rF] = dw_mul(c.L[i2 + i * rF], s);
    }
  }
}

// The end of a solve: the caller's FP64 factor and weights (cluster rank 0,
// in the last sweep only: earlier values of a mode are overwritten unseen,
// and the conversions would hold the FP64 pipe on the critical path), the
// Gram of the new factor of mode k folded into the prefix L, the suffix
// products when a sweep ends, and the suffix of the next mode kn.  Threads t
// of nt; `warp_only` when they form one warp.
__device__ void post_solve(const Cta& c, const AlsParams& p, int k, int kn, int t, int nt, bool warp_only,
                           bool last_sweep) {
  const int rF = c.rF, nk = p.nbas[k], rr = rF * rF;
  if (c.rank == 0 && last_sweep) {
    double* fbase = p.base + p.term_off[c.v] * (long long)p.nD;
    for (int e = t; e < rF * nk; e += nt) {
      const int i = e / nk, q = e - i * nk;
      fbase[(long long)i * p.nD + p.off[k] + q] = dw_to_double(c.X[i + q * rF]);
    }
    for (int i = t; i < rF; i += nt) p.coef[p.term_off[c.v] + i] = dw_to_double(c.nrm[i]);
  }
  dw_new_gram(c, k, nk, t, nt);
  cp_async_wait_all();
  if (warp_only) __syncwarp(); else solver_sync();
  if (k == c.D - 1) {
    dw_suffix(c, t, nt);
    if (warp_only) __syncwarp(); else solver_sync();
    for (int e = t; e < rr; e += nt) c.sk[e] = c.suf[(size_t)kn * rr + e];
  }
  // the next step's normal equations (sk: the suffix of mode kn, copied at
  // the start of the solve unless the sweep just ended)
  const dw pen = c.misc[0];
  for (int e = t; e < rr; e += nt) {
    const dw sk = c.sk[e];
    dw b = dw_mul(c.L[e], sk);
    if (e % rF == e / rF) b = dw_add(b, pen);
    c.BB[e] = b;
  }
}

// The R x R solve of step t (mode k; kn is the next step's mode), run
// identically by every CTA of the cluster on the solver warps.
__device__ void solve_step(const Cta& c, const AlsParams& p, cg::cluster_group& cluster, int t, int k, int kn) {
  const int rF = c.rF, nk = p.nbas[k], npk = round_up(nk, 4);
  // the next mode's suffix products into sk, asynchronously (global memory;
  // unchanged unless this step ends a sweep)
  if (k < c.D - 1)
    for (int e = c.tid; e < rF * rF; e += kSolverThreads) cp_async8(c.sk + e, c.suf + (size_t)kn * rF * rF + e);
  // gather the partial right-hand sides of the cluster in rank order
  const size_t boff = (size_t)(t & 1) * c.rFp * c.npmax;
  // (mapa + ld.shared::cluster: explicit distributed-shared-memory loads,
  // all issued before the sums)
  for (int e = c.tid; e < rF * nk; e += kSolverThreads) {
    const int i = e % rF, n = e / rF;
    const uint32_t local = smem_addr(c.bpart + boff + i * c.npmax + n);
    float v[16];
#pragma unroll
    for (int r = 0; r < 16; ++r) {
      v[r] = 0.f;
      if (r < c.CL) {
        uint32_t remote;
        asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(remote) : "r"(local), "r"(r));
        asm volatile("ld.shared::cluster.f32 %0, [%1];" : "=f"(v[r]) : "r"(remote) : "memory");
      }
    }
    dw s = dw_make(0.f);
#pragma unroll
    for (int r = 0; r < 16; ++r)
      if (r < c.CL) s = dw_add_f(s, v[r]);
    c.b0[i + n * rF] = s;
  }
  // the normal equations BB (prefix of this sweep x suffix of the previous
  // one + penalty) were formed when the previous step ended
  solver_sync();
  // FP32 inverse + double-word refinement; the double-word LDL^T when the
  // FP32 inverse fails or the refinement does not settle (ill-conditioned BB)
  bool gj_ok;
  const float* inv = c.gi;
  if (phase_b_inverts(c)) {
    gj_ok = c.flags[2] != 0;  // inverted during phase B
  } else if (rF <= 32) {
    if (c.tid < 32) {
      const bool g = dwsolve::gj_inverse_warp(c.BB, rF, c.gi);
      if (c.tid == 0) c.flags[2] = g;
    }
    solver_sync();
    gj_ok = c.flags[2] != 0;
  } else {
    inv = gj_inverse(c.BB, rF, c.gi, &gj_ok);
  }
  int bad = 0;
  if (!(gj_ok && refine_solve(c.BB, rF, c.b0, c.X, nk, inv, c.res, c.red))) {
    for (int e = c.tid; e < rF * nk; e += kSolverThreads) c.X[e] = c.b0[e];
    bad = dw_ldlt(c.BB, rF, c.dinv, c.u);
    dw_ldlt_solve(c.BB, rF, c.dinv, c.X, nk);
  }
  dwsolve::dw_normalise_rows(c.X, rF, nk, c.nrm);
  solver_sync();
  // new factor: FP32 copy for phase B and for this CTA's rebuilds; the
  // caller's FP64 arrays from cluster rank 0
  for (int e = c.tid; e < c.rFp * npk; e += kSolverThreads) {
    const int i = e / npk, q = e - i * npk;
    const float x = (i < rF && q < nk) ? c.X[i + q * rF].hi : 0.f;
    c.fb[i * c.gsmax + q] = x;
    if (i < rF) c.fcta[(long long)i * c.nDp + p.offp[k] + q] = x;
  }
  post_solve(c, p, k, kn, c.tid, kSolverThreads, false, t >= (p.nals - 1) * c.D);
  if (c.tid == 0 && bad) c.flags[1] = 1;
}

// Warps that run phase A (the highest-numbered ones).  Phase A only has to
// finish within the solve; the solver's dependent chains compete with its
// warps for issue slots, so fewer of them can shorten the step.
constexpr int kDivideWarps = 12;
// Tensor-core form: phase A on warps 4-15 (three per lane quarter).
constexpr int kSolverWarpsAls = kAlsSolverWarps;
constexpr int kTcDivideWarps = kAlsWarps - kAlsSolverWarps;

// Barrier among the phase-A warps only (named barrier 2).
__device__ __forceinline__ void worker_sync() {
  asm volatile("bar.sync 2, %0;" ::"r"(kAlsThreads - kSolverThreads) : "memory");
}

}  // namespace

// ---------------------------------------------------------------------------
// Persistent cluster kernel
// ---------------------------------------------------------------------------

// kTc: the tensor-core form (its own instantiation, so that neither form's
// register allocation carries the other's).
template <bool kTc>
__global__ void __launch_bounds__(kAlsThreads, 1) als_cluster_kernel(AlsParams p) {
  cg::cluster_group cluster = cg::this_cluster();
  extern __shared__ __align__(128) unsigned char smem_raw[];

  Cta c;
  c.tid = threadIdx.x;
  c.warp = c.tid >> 5;
  c.lane = c.tid & 31;
  c.CL = p.cluster;
  c.rank = (int)cluster.block_rank();
  c.v = blockIdx.x / c.CL;
  c.D = p.ndof;
  c.rF = p.rF[c.v];
  c.rFp = round_up(c.rF, 4);
  c.nIq = c.rFp / 4;
  c.rG = p.rG[c.v];
  {
    const int rows_per = (c.rG + c.CL - 1) / c.CL;
    c.row0 = min(c.rG, c.rank * rows_per);
    c.nrows = min(c.rG, c.row0 + rows_per) - c.row0;
  }
  c.ntiles = (c.nrows + kAlsTileRows - 1) / kAlsTileRows;
  const AlsSmem lay = als_smem_layout(p.rows_cta_max, p.rf_max, p.npmax, p.gsmax, p.stages, p.tc);
  c.ldP = lay.ldP;
  c.gsmax = p.gsmax;
  c.npmax = p.npmax;
  c.nDp = p.nDp;
  c.stages = p.stages;
  c.stage_floats = lay.stage_floats;
  c.bar = reinterpret_cast<uint64_t*>(smem_raw + lay.bar);
  c.done = reinterpret_cast<int*>(smem_raw + lay.done);
  c.issued = reinterpret_cast<int*>(smem_raw + lay.issued);
  c.fillno = reinterpret_cast<unsigned*>(smem_raw + lay.fillno);
  c.flags = reinterpret_cast<int*>(smem_raw + lay.flags);
  c.ring = reinterpret_cast<float*>(smem_raw + lay.ring);
  c.P = reinterpret_cast<float*>(smem_raw + lay.P);
  c.cw = reinterpret_cast<float*>(smem_raw + lay.cw);
  c.fa = reinterpret_cast<float*>(smem_raw + lay.fa);
  c.fb = reinterpret_cast<float*>(smem_raw + lay.fb);
  c.bred = reinterpret_cast<float*>(smem_raw + lay.bred);
  c.bpart = reinterpret_cast<float*>(smem_raw + lay.bpart);
  c.BB = reinterpret_cast<dw*>(smem_raw + lay.BB);
  c.X = reinterpret_cast<dw*>(smem_raw + lay.X);
  c.L = reinterpret_cast<dw*>(smem_raw + lay.L);
  c.sk = reinterpret_cast<dw*>(smem_raw + lay.sk);
  c.dinv = reinterpret_cast<dw*>(smem_raw + lay.dinv);
  c.u = reinterpret_cast<dw*>(smem_raw + lay.u);
  c.nrm = reinterpret_cast<dw*>(smem_raw + lay.nrm);
  c.misc = reinterpret_cast<dw*>(smem_raw + lay.misc);
  c.gi = reinterpret_cast<float*>(smem_raw + lay.gi);
  c.b0 = reinterpret_cast<dw*>(smem_raw + lay.b0);
  c.res = reinterpret_cast<dw*>(smem_raw + lay.res);
  c.red = reinterpret_cast<float*>(smem_raw + lay.red);
  c.tc = kTc ? 1 : 0;
  c.kp = lay.kp;
  c.nf = lay.nf;
  c.cb = smem_raw + lay.cb;
  c.fp = smem_raw + lay.fp;
  c.tcbar = reinterpret_cast<uint64_t*>(smem_raw + lay.tcbar);
  uint32_t* tbase = reinterpret_cast<uint32_t*>(smem_raw + lay.tbase);
  c.tmem = 0;
  if (kTc && c.warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tbase)),
                 "r"(kAlsTcCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  c.gm = p.gm + p.gm_off[c.v];
  c.fcta = p.fcta + (p.f_row_off[c.v] * c.CL + (long long)c.rank * c.rF) * p.nDp;
  {
    const long long sq = p.sq_off[c.v] * c.CL + (long long)c.rank * c.rF * c.rF * c.D;
    c.gram = p.gram + sq;
    c.suf = p.suf + sq;
  }
  const int D = c.D, rF = c.rF, rr = rF * rF;

  // ---- prologue ----
  for (int e = c.tid; e < c.stages * c.stage_floats; e += kAlsThreads) c.ring[e] = 0.f;  // stale reads stay finite
  if (!kTc)
    for (int e = c.tid; e < lay.rFp * c.ldP; e += kAlsThreads) c.P[e] = (e / c.ldP < rF) ? 1.f : 0.f;
  for (int j = c.tid; j < c.ldP; j += kAlsThreads) c.cw[j] = (j < c.nrows) ? p.gc[p.g_row_off[c.v] + c.row0 + j] : 0.f;
  for (int e = c.tid; e < 2 * lay.rFp * c.npmax; e += kAlsThreads) c.bpart[e] = 0.f;
  if (c.tid < c.stages) {
    c.done[c.tid] = 0;
    c.issued[c.tid] = 0;
    c.fillno[c.tid] = 0xffffffffu;
  }
  if (c.tid < 8) c.flags[c.tid] = 0;
  if (c.tid == 0) {
    for (int s = 0; s < c.stages; ++s) mbar_init(&c.bar[s], 1);
    mbar_init(&c.tcbar[0], 1);
    mbar_init(&c.tcbar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  const float* f32v = p.f32 + p.f_row_off[c.v] * p.nDp;
  const float* f32lo_v = p.f32lo + p.f_row_off[c.v] * p.nDp;
  for (int e = c.tid; e < rF * p.nDp; e += kAlsThreads) c.fcta[e] = f32v[e];
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (kTc) {
    c.tmem = *tbase;
    tc_init_products(c);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
  }

  // running products without modes 0 and D-1 (the state phase B of step 0 expects)
  unsigned seq = 0;
  unsigned tcseq = 0;  // MMA batches issued so far (tensor-core form; the same count in every thread)
  for (int d = 1; d <= D - 2; ++d) {
    load_factor(c, p, d, c.fa, 0, kAlsThreads);
    __syncthreads();
    if (c.tid == 0) start_phase(c, seq, TileSrc{c.gm + (long long)p.offg[d] * c.rG, als_gstride(p.nbas[d]), nullptr, 0});
    if (kTc) {
      tc_product_pass<8, false>(c, p, seq, tcseq, d, -1, 0, kAlsWarps);
      tcseq += (unsigned)c.ntiles;
    } else {
      product_pass(c, p, seq, d, false, -1, 0, kAlsWarps);
    }
    seq += (unsigned)c.ntiles;
    __syncthreads();
  }
  // Grams of the starting factors (double-word), penalty
  for (int e = c.tid; e < D * rr; e += kAlsThreads) {
    const int d = e / rr, r = e - d * rr, i = r % rF, i2 = r / rF;
    if (i > i2) continue;
    const int n = p.nbas[d];
    const long long oa = (long long)i * p.nDp + p.offp[d], ob = (long long)i2 * p.nDp + p.offp[d];
    dw s = dw_make(0.f);
    for (int q = 0; q < n; ++q) s = dw_fma(dw_make(f32v[oa + q], f32lo_v[oa + q]), dw_make(f32v[ob + q], f32lo_v[ob + q]), s);
    c.gram[(size_t)d * rr + i + i2 * rF] = s;
    c.gram[(size_t)d * rr + i2 + i * rF] = s;
  }
  if (c.tid == 0) {
    const double* fc = p.coef + p.term_off[c.v];
    double mx = fc[0];
    for (int i = 1; i < rF; ++i) mx = fc[i] > mx ? fc[i] : mx;
    c.misc[0] = dw_from_double(mx * p.pen_factor);
  }
  __syncthreads();
  if (c.warp < kAlsSolverWarps) {
    dw_suffix(c, c.tid, kSolverThreads);
    solver_sync();
    const dw pen = c.misc[0];
    for (int e = c.tid; e < rr; e += kSolverThreads) {
      const dw sk = c.suf[e];
      c.sk[e] = sk;
      dw b = dw_mul(c.L[e], sk);
      if (e % rF == e / rF) b = dw_add(b, pen);
      c.BB[e] = b;
    }
  }
  load_factor(c, p, D - 1, c.fb, 0, kAlsThreads);
  __syncthreads();

  // ---- mode steps ----
  const int nsteps = p.nals * D;
  for (int t = 0; t < nsteps; ++t) {
    const int k = t % D, kp = (k + D - 1) % D, kn = (k + 1) % D;
    if (kTc) {
      seq += tc_phase_b(c, p, seq, tcseq, k, kp, c.bpart + (size_t)(t & 1) * c.rFp * c.npmax);
      tcseq += (unsigned)c.ntiles;
    } else {
      seq += phase_b(c, p, seq, k, kp, c.bpart + (size_t)(t & 1) * c.rFp * c.npmax);
    }
    cluster_arrive();
    if (c.warp < kAlsSolverWarps) {
      cluster_wait();
      solve_step(c, p, cluster, t, k, kn);
    } else {
      if (t + 1 < nsteps) {
        load_factor(c, p, kn, c.fa, kSolverThreads, kAlsThreads - kSolverThreads);
        worker_sync();
        if (c.tid == kSolverThreads)
          start_phase(c, seq, TileSrc{c.gm + (long long)p.offg[kn] * c.rG, als_gstride(p.nbas[kn]), nullptr, 0});
        if (kTc) {
          if ((rF + 2) / 3 <= 8) tc_product_pass<8, true>(c, p, seq, tcseq, kn, k, kSolverWarpsAls, kTcDivideWarps);
          else tc_product_pass<16, true>(c, p, seq, tcseq, kn, k, kSolverWarpsAls, kTcDivideWarps);
        } else if (c.warp >= kAlsWarps - kDivideWarps) {
          product_pass(c, p, seq, kn, true, k, kAlsWarps - kDivideWarps, kDivideWarps);
        }
      }
      cluster_wait();
    }
    if (t + 1 < nsteps) {
      seq += (unsigned)c.ntiles;
      if (kTc) tcseq += (unsigned)c.ntiles;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
  }
  // every CTA of the cluster has gathered before any shared memory goes away
  cluster_arrive();
  cluster_wait();
  if (c.tid == 0) {
    // bulk copies are all consumed by now; wait (bounded) on each stage's last fill anyway
    for (int s = 0; s < c.stages; ++s) {
      const int fills = c.issued[s];
      if (fills == 0) continue;
      for (int it = 0; it < kWaitLimit; ++it)
        if (mbar_try_wait(&c.bar[s], (uint32_t)((fills - 1) & 1))) break;
    }
    if (c.flags[0]) atomicOr(&p.status[c.v], 2);
    if (c.flags[1]) atomicOr(&p.status[c.v], 1);
  }
  if (kTc) {
    // every MMA batch was waited for by its consumers; free the tensor memory
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (c.warp == 0)
      asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(c.tmem), "r"(kAlsTcCols) : "memory");
  }
}

size_t als_smem_bytes(int rows_cta, int rF, int npmax, int gsmax, int stages, int tc) {
  return als_smem_layout(rows_cta, rF, npmax, gsmax, stages, tc).total;
}

bool als_choose_shape(int nvec, int rGmax, int rFmax, int npmax, int gsmax, int num_sms, size_t smem_limit,
                      AlsShape* out) {
  // Cluster size: the largest power of two (<= 16) whose clusters for the
  // whole batch still fit on the SMs at one CTA per SM; larger when the
  // running products of a CTA's term range need more shared memory.  Ring
  // depth: as many stages (2-6) as fit.
  // With the tensor-core engine forced (als_engine() == 2) the same walk
  // takes the tensor-core form wherever it fits.
  const bool want_tc = als_engine() == 2;
  int cl = 1;
  while (cl < 16 && cl * 2 * nvec <= num_sms) cl *= 2;
  for (;;) {
    const int rows = (rGmax + cl - 1) / cl;
    for (int tc = (want_tc && als_tc_fits(rows, rFmax, npmax)) ? 1 : 0; tc >= 0; --tc)
      for (int ns = 6; ns >= (tc ? 3 : 2); --ns) {
        const size_t b = als_smem_bytes(rows, rFmax, npmax, gsmax, ns, tc);
        if (b <= smem_limit) {
          out->cluster = cl;
          out->stages = ns;
          out->rows_cta = rows;
          out->tc = tc;
          out->smem = b;
          return true;
        }
      }
    if (cl >= 16) return false;
    cl *= 2;
  }
}

namespace {

// Failure-path self-test of the pipeline wait: one warp sets up a one-stage
// ring exactly as the cluster kernel does and waits for a tile that nobody
// issues.  wait_tile must give up after its iteration limit and raise the
// abort flag; out[0] receives the status bit the cluster kernel would report
// (2), out[1] whether the wait returned false.
__global__ void als_wait_selftest_kernel(int* out) {
  __shared__ __align__(8) uint64_t bar[1];
  __shared__ int done[1], issued[1], flags[8];
  __shared__ unsigned fillno[1];
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    done[0] = 0;
    issued[0] = 0;
    fillno[0] = 0xffffffffu;
  }
  if (threadIdx.x < 8) flags[threadIdx.x] = 0;
  __syncwarp();
  Cta c{};
  c.tid = threadIdx.x;
  c.lane = threadIdx.x & 31;
  c.stages = 1;
  c.bar = bar;
  c.done = done;
  c.issued = issued;
  c.fillno = fillno;
  c.flags = flags;
  const bool got = wait_tile(c, 0u);
  __syncwarp();
  if (threadIdx.x == 0) {
    out[0] = flags[0] ? 2 : 0;
    out[1] = got ? 0 : 1;
  }
}

}  // namespace

int als_wait_selftest(cudaStream_t st, int* flags_out) {
  int* d = nullptr;
  MLCP_CUDA_TRY(cudaMalloc(&d, 2 * sizeof(int)));
  als_wait_selftest_kernel<<<1, 32, 0, st>>>(d);
  cudaError_t e = cudaGetLastError();
  int h[2] = {0, 0};
  if (e == cudaSuccess) e = cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(d);
  if (e != cudaSuccess) {
    set_error("wait self-test failed: %s", cudaGetErrorString(e));
    return kCudaError;
  }
  if (!h[1]) {
    set_error("wait self-test: the wait for a tile that was never issued reported success");
    return kNumerical;
  }
  *flags_out = h[0];
  return kOk;
}

int als_launch(const AlsParams& p, size_t smem, cudaStream_t st, cudaEvent_t t0, cudaEvent_t t1) {
  int dev = 0, nsm = 0;
  MLCP_CUDA_TRY(cudaGetDevice(&dev));
  MLCP_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const long long nv = p.shared_target ? 1 : p.nvec;
  const size_t rows_smem = sizeof(int) * ((size_t)p.nD + 2 * (p.ndof + 1));
  if (p.g_host && rows_smem <= 48 * 1024) {
    als_prep_target_rows_kernel<<<dim3(32, (unsigned)std::min<long long>(nv, 65535)), 256, rows_smem, st>>>(p);
  } else {
    const long long nvd = nv * p.ndof;
    als_prep_target_kernel<<<dim3(16, (unsigned)std::min<long long>(nvd, 65535)), 256, 0, st>>>(p);
  }
  MLCP_CUDA_TRY(cudaGetLastError());
  const long long work = std::max<long long>(p.shared_target ? p.total_rows : 0, p.total_f_terms * p.ndof);
  long long blocks = (work + 255) / 256;
  if (blocks > (long long)nsm * 8) blocks = (long long)nsm * 8;
  if (blocks < 1) blocks = 1;
  als_prep_kernel<<<(int)blocks, 256, 0, st>>>(p);
  MLCP_CUDA_TRY(cudaGetLastError());
  if (t0) MLCP_CUDA_TRY(cudaEventRecord(t0, st));
  auto fn = p.tc ? als_cluster_kernel<true> : als_cluster_kernel<false>;
  MLCP_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  if (p.cluster > 8) MLCP_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(p.nvec * p.cluster);
  cfg.blockDim = dim3(kAlsThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = p.cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  MLCP_CUDA_TRY(cudaLaunchKernelEx(&cfg, fn, p));
  if (t1) MLCP_CUDA_TRY(cudaEventRecord(t1, st));
  return kOk;
}

}  // namespace mlcp
