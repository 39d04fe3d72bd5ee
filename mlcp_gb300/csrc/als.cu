// Batched explicit-target ALS rank reduction on GB300.
//
// Computes, for every vector of a batch, the reference's ITERATE_ALS
// (src/als.cu:1021-1078, called through alscpp_ src/intertwining.cu:180):
//   for nals sweeps, for each mode k:
//     b(i,n)  = sum_j cG_j G_j^k(n) prod_{d!=k} <G_j^d, F_i^d>
//     BB(i,i') = prod_{d!=k} <F_i^d, F_i'^d> + pen delta(i,i'),  pen = 1e-10 max cF
//     X = BB^-1 b;  F_i^k = X(i,:) / ||X(i,:)||,  cF_i = ||X(i,:)||
//
// GB300 design (one persistent thread-block cluster per vector):
//  * The target G is converted once to an FP32 mode-major copy, so the slice
//    of mode k for a range of terms is one contiguous run of memory.
//  * Each CTA of the cluster owns a contiguous range of target terms j and
//    keeps, per term and per F term i, the running product
//    PS(j,i) = prod_d <G_j^d, F_i^d> in shared memory.  A mode step divides
//    the old mode-k factor out and, after the solve, multiplies the new one in,
//    so each mode step streams only the mode-k slice of G (the reference
//    rebuilds the full product over all modes at every step).  Entries whose
//    division is unsafe (zero divisor, subnormal product) are rebuilt from
//    the factors directly.
//  * The products and contractions run in FP32 with FP32 accumulation; the
//    per-step R x R normal equations, their regularisation, the F Gram
//    products and the normalisation run in FP64 on the cluster's rank-0 CTA.
//  * Partial right-hand sides are reduced through distributed shared memory
//    and the new factor is broadcast back the same way; one cluster barrier
//    pair per mode step, no host round trip, one launch for all sweeps.

#include <cooperative_groups.h>
#include <cfloat>

#include "common.cuh"
#include "als.cuh"

namespace cg = cooperative_groups;

namespace mlcp {

// ---------------------------------------------------------------------------
// Preparation: FP32 mode-major target, FP32 copy of F, FP32 target weights.
// ---------------------------------------------------------------------------

// One thread per (vector, target term, mode) element run; grid-stride.
__global__ void als_prep_kernel(AlsParams p) {
  const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long stride = (long long)gridDim.x * blockDim.x;
  // target factors: one element run per (target term, mode); with a shared
  // target only vector 0's terms are converted (gm_off is 0 for every vector)
  const long long grows = p.shared_target ? (long long)p.rG[0] : p.total_rows;
  for (long long e = tid; e < grows * p.ndof; e += stride) {
    const long long row = e / p.ndof;
    const int d = (int)(e % p.ndof);
    // locate vector: binary search over row offsets
    int lo = 0, hi = p.nvec - 1;
    while (lo < hi) {
      int mid = (lo + hi + 1) >> 1;
      if (p.g_row_off[mid] <= row) lo = mid; else hi = mid - 1;
    }
    const int v = p.shared_target ? 0 : lo;
    const int j = (int)(row - p.g_row_off[v]);
    const int rG = p.rG[v];
    const int n = p.nbas[d], np = round_up(n, 4);
    const double* src = p.g_base + (p.g_term_off[v] + j) * (long long)p.nD + p.off[d];
    float* dst = p.gm + p.gm_off[v] + (long long)p.offp[d] * rG + (long long)j * np;
    for (int i = 0; i < np; ++i) dst[i] = (i < n) ? (float)src[i] : 0.f;
    if (d == 0 && !p.shared_target) p.gc[p.g_row_off[v] + j] = (float)p.g_coef[p.g_term_off[v] + j];
  }
  if (p.shared_target)
    for (long long e = tid; e < p.total_rows; e += stride) p.gc[e] = (float)p.shared_w[e];
  // FP32 copy of F
  for (long long e = tid; e < p.total_f_terms * p.ndof; e += stride) {
    const long long frow = e / p.ndof;
    const int d = (int)(e % p.ndof);
    int lo = 0, hi = p.nvec - 1;
    while (lo < hi) {
      int mid = (lo + hi + 1) >> 1;
      if (p.f_row_off[mid] <= frow) lo = mid; else hi = mid - 1;
    }
    const int v = lo;
    const int i = (int)(frow - p.f_row_off[v]);
    const int n = p.nbas[d], np = round_up(n, 4);
    const double* src = p.base + (p.term_off[v] + i) * (long long)p.nD + p.off[d];
    float* dst = p.f32 + (p.f_row_off[v] + i) * (long long)p.nDp + p.offp[d];
    for (int q = 0; q < np; ++q) dst[q] = (q < n) ? (float)src[q] : 0.f;
  }
}

// ---------------------------------------------------------------------------
// Persistent cluster kernel
// ---------------------------------------------------------------------------

namespace {

constexpr int kThreads = kAlsThreads;
constexpr int kTileRows = 256;  // target terms staged per tile (multiple of 4)
constexpr int kWtStride = kTileRows + 1;  // odd stride: per-term weight rows on distinct banks

struct Smem {
  float* ps;      // [rFp][rows_cta] running products (term index fastest: conflict-free)
  float* fold;    // [rFp][npmax] FP32 old factor of the mode being solved
  float* fnew;    // [rFp][npmax] FP32 new factor of the mode just solved
  float* wt;      // [rFp][kWtStride] weights c_j * PS(j,i) of the tile
  float* gt;      // [kTileRows][gstride] target factors of mode k for the tile
  float* gp;      // [kTileRows][gstride] target factors of the previous mode for the tile
  float* bpart;   // [rFp][npmax] partial right-hand side of this CTA
  float* red;     // [kThreads][16] reduction scratch
  double* BB;     // [rF][rF]
  double* X;      // [rF][npmax] column-major rF x n (ld rF)
  double* L;      // [rF][rF] prefix of F Gram products
  double* misc;   // [4]
  double* dinv;   // [rF] reciprocal pivots of the LDL^T factor
  double* u;      // [rF] LDL^T scratch column
  int* flags;     // [4]
};

// Row stride of staged tiles: an odd number of float4 per row keeps the
// float4 accesses of consecutive rows on distinct shared-memory banks.
__host__ __device__ inline int tile_stride(int npmax) { return ((npmax / 4) % 2 == 1) ? npmax : npmax + 4; }

// Quotient a / b from the approximate reciprocal plus one Newton correction
// (within an ulp or two of the rounded quotient).
__device__ __forceinline__ float div_nr(float a, float b) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(b));
  float q = a * r;
  return fmaf(fmaf(-b, q, a), r, q);
}

// <g, f> over NP padded entries; g in registers, f in shared memory.
template <int NP>
__device__ __forceinline__ float dot_reg(const float (&g)[NP], const float* f, int np) {
  float s = 0.f;
#pragma unroll
  for (int q = 0; q < NP; q += 4) {
    if (q < np) {
      float4 y = *reinterpret_cast<const float4*>(f + q);
      s = fmaf(g[q], y.x, s);
      s = fmaf(g[q + 1], y.y, s);
      s = fmaf(g[q + 2], y.z, s);
      s = fmaf(g[q + 3], y.w, s);
    }
  }
  return s;
}

template <int NP>
__device__ __forceinline__ void load_row(float (&g)[NP], const float* src, int np) {
#pragma unroll
  for (int q = 0; q < NP; q += 4) {
    float4 x = (q < np) ? *reinterpret_cast<const float4*>(src + q) : make_float4(0.f, 0.f, 0.f, 0.f);
    g[q] = x.x; g[q + 1] = x.y; g[q + 2] = x.z; g[q + 3] = x.w;
  }
}

// Plain dot product of two padded FP32 runs in global memory (rebuild path).
__device__ inline float dot_global(const float* a, const float* b, int np) {
  float s = 0.f;
  for (int q = 0; q < np; ++q) s = fmaf(a[q], b[q], s);
  return s;
}

}  // namespace

template <int NP>
__global__ void __launch_bounds__(kThreads, 1) als_cluster_kernel(AlsParams p) {
  cg::cluster_group cluster = cg::this_cluster();
  const int CL = (int)cluster.num_blocks();
  const int rank = (int)cluster.block_rank();
  const int v = blockIdx.x / CL;
  if (v >= p.nvec) return;  // whole cluster exits together (same v)

  const int tid = threadIdx.x;
  const int D = p.ndof;
  const int rF = p.rF[v], rG = p.rG[v];
  const int rFp = round_up(rF, 4);
  const int npmax = p.npmax;
  const int rows_per = (rG + CL - 1) / CL;
  const int row0 = min(rG, rank * rows_per);
  const int row1 = min(rG, row0 + rows_per);
  const int nrows = row1 - row0;

  extern __shared__ __align__(16) unsigned char smem_raw[];
  Smem s;
  {
    unsigned char* ptr = smem_raw;
    auto take = [&](size_t bytes) { unsigned char* r = ptr; ptr += round_up((int)bytes, 16); return r; };
    s.ps = (float*)take(sizeof(float) * (size_t)p.rows_cta_max * rFp);
    s.fold = (float*)take(sizeof(float) * rFp * npmax);
    s.fnew = (float*)take(sizeof(float) * rFp * npmax);
    s.wt = (float*)take(sizeof(float) * kWtStride * rFp);
    s.gt = (float*)take(sizeof(float) * kTileRows * tile_stride(npmax));
    s.gp = (float*)take(sizeof(float) * kTileRows * tile_stride(npmax));
    s.bpart = (float*)take(sizeof(float) * rFp * npmax);
    s.red = (float*)take(sizeof(float) * kThreads * 16);
    s.BB = (double*)take(sizeof(double) * rF * rF);
    s.X = (double*)take(sizeof(double) * rF * npmax);
    s.L = (double*)take(sizeof(double) * rF * rF);
    s.misc = (double*)take(sizeof(double) * 4);
    s.dinv = (double*)take(sizeof(double) * rF);
    s.u = (double*)take(sizeof(double) * rF);
    s.flags = (int*)take(sizeof(int) * 4);
  }

  const float* gm = p.gm + p.gm_off[v];
  const float* gc = p.gc + p.g_row_off[v];
  float* f32 = p.f32 + p.f_row_off[v] * p.nDp;
  double* fbase = p.base + p.term_off[v] * (long long)p.nD;
  double* fcoef = p.coef + p.term_off[v];
  double* gram = p.gram + p.sq_off[v];   // [D][rF][rF]
  double* suf = p.suf + p.sq_off[v];     // [D][rF][rF]

  // ---- prologue: running products over all modes, F Grams, penalty ----
  const int psld = p.rows_cta_max;
  for (int e = tid; e < rFp * psld; e += kThreads) s.ps[e] = 1.f;
  __syncthreads();
  for (int d = 0; d < D; ++d) {
    const int np = round_up(p.nbas[d], 4);
    for (int e = tid; e < rFp * np; e += kThreads) {
      const int i = e / np, q = e % np;
      s.fold[i * npmax + q] = (i < rF) ? f32[(long long)i * p.nDp + p.offp[d] + q] : 0.f;
    }
    __syncthreads();
    const float* gmd = gm + (long long)p.offp[d] * rG;
    for (int r = tid; r < nrows; r += kThreads) {
      float g[NP];
      load_row<NP>(g, gmd + (long long)(row0 + r) * np, np);
      for (int i = 0; i < rF; ++i) s.ps[i * psld + r] *= dot_reg<NP>(g, s.fold + i * npmax, np);
    }
    __syncthreads();
  }
  // F Grams (FP64): CTA rank handles modes d = rank, rank+CL, ...
  for (int d = rank; d < D; d += CL) {
    const int n = p.nbas[d];
    for (int e = tid; e < rF * rF; e += kThreads) {
      const int i = e % rF, i2 = e / rF;
      const double* a = fbase + (long long)i * p.nD + p.off[d];
      const double* b = fbase + (long long)i2 * p.nD + p.off[d];
      double t = 0.0;
      for (int q = 0; q < n; ++q) t += a[q] * b[q];
      gram[(long long)d * rF * rF + e] = t;
    }
  }
  if (rank == 0 && tid == 0) {
    double pen = fcoef[0];
    for (int i = 1; i < rF; ++i) pen = fcoef[i] > pen ? fcoef[i] : pen;
    s.misc[0] = pen * p.pen_factor;
  }
  __threadfence();
  cluster.sync();

  const int nib = rFp / 4;  // i-blocks of the right-hand-side register tiles
  const int nsteps = p.nals * D;

  for (int t = 0; t < nsteps; ++t) {
    const int k = t % D;
    const int kprev = (t > 0) ? (t - 1) % D : -1;
    const int nk = p.nbas[k], npk = round_up(nk, 4);
    const int npp = (kprev >= 0) ? round_up(p.nbas[kprev], 4) : 0;
    const int nnb = npk / 4;                 // n-blocks
    const int nblk = nib * nnb;              // register blocks (<= kThreads, host-checked)
    const int ngroups = kThreads / nblk;     // row groups
    const int my_blk = tid % nblk, my_grp = tid / nblk;
    const bool acc_active = my_grp < ngroups;
    const int ib = my_blk / nnb, nb = my_blk % nnb;
    float acc[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) acc[q] = 0.f;

    // old factor of mode k (FP32)
    for (int e = tid; e < rFp * npk; e += kThreads) {
      const int i = e / npk, q = e % npk;
      s.fold[i * npmax + q] = (i < rF) ? f32[(long long)i * p.nDp + p.offp[k] + q] : 0.f;
    }
    __syncthreads();

    const float* gmk = gm + (long long)p.offp[k] * rG;
    const float* gmp = (kprev >= 0) ? gm + (long long)p.offp[kprev] * rG : nullptr;

    const int gsd = tile_stride(npmax);
    constexpr int kRowSlots = kTileRows / 4;  // register block = rows {rb, rb+64, rb+128, rb+192}
    for (int tile0 = 0; tile0 < nrows; tile0 += kTileRows) {
      const int tr = min(kTileRows, nrows - tile0);
      // -- stage the tile's factors of modes k and kprev (coalesced float4) --
      for (int e = tid; e < kTileRows * (npk / 4); e += kThreads) {
        const int r = e / (npk / 4), q = (e % (npk / 4)) * 4;
        float4 x = make_float4(0.f, 0.f, 0.f, 0.f);
        if (r < tr) x = *reinterpret_cast<const float4*>(gmk + (long long)(row0 + tile0 + r) * npk + q);
        *reinterpret_cast<float4*>(s.gt + r * gsd + q) = x;
      }
      if (kprev >= 0) {
        for (int e = tid; e < kTileRows * (npp / 4); e += kThreads) {
          const int r = e / (npp / 4), q = (e % (npp / 4)) * 4;
          float4 x = make_float4(0.f, 0.f, 0.f, 0.f);
          if (r < tr) x = *reinterpret_cast<const float4*>(gmp + (long long)(row0 + tile0 + r) * npp + q);
          *reinterpret_cast<float4*>(s.gp + r * gsd + q) = x;
        }
      }
      __syncthreads();
      // -- running products: fold in the new factor of kprev, divide out mode k.
      //    Register blocks of 4 terms x 4 F terms; consecutive threads take
      //    consecutive terms, so shared-memory accesses are conflict-free and
      //    the F reads of a warp are broadcasts. --
      for (int blk = tid; blk < kRowSlots * nib; blk += kThreads) {
        const int rb = blk % kRowSlots, ibk = blk / kRowSlots;
        float po[16], pn[16];
#pragma unroll
        for (int q = 0; q < 16; ++q) { po[q] = 0.f; pn[q] = 1.f; }
        for (int q = 0; q < npk; q += 4) {
          float4 g[4], f[4];
#pragma unroll
          for (int a = 0; a < 4; ++a) g[a] = *reinterpret_cast<const float4*>(s.gt + (rb + a * kRowSlots) * gsd + q);
#pragma unroll
          for (int c = 0; c < 4; ++c) f[c] = *reinterpret_cast<const float4*>(s.fold + (ibk * 4 + c) * npmax + q);
#pragma unroll
          for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int c = 0; c < 4; ++c) {
              float v = po[a * 4 + c];
              v = fmaf(g[a].x, f[c].x, v);
              v = fmaf(g[a].y, f[c].y, v);
              v = fmaf(g[a].z, f[c].z, v);
              v = fmaf(g[a].w, f[c].w, v);
              po[a * 4 + c] = v;
            }
        }
        if (kprev >= 0) {
#pragma unroll
          for (int q = 0; q < 16; ++q) pn[q] = 0.f;
          for (int q = 0; q < npp; q += 4) {
            float4 g[4], f[4];
#pragma unroll
            for (int a = 0; a < 4; ++a) g[a] = *reinterpret_cast<const float4*>(s.gp + (rb + a * kRowSlots) * gsd + q);
#pragma unroll
            for (int c = 0; c < 4; ++c) f[c] = *reinterpret_cast<const float4*>(s.fnew + (ibk * 4 + c) * npmax + q);
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
              for (int c = 0; c < 4; ++c) {
                float v = pn[a * 4 + c];
                v = fmaf(g[a].x, f[c].x, v);
                v = fmaf(g[a].y, f[c].y, v);
                v = fmaf(g[a].z, f[c].z, v);
                v = fmaf(g[a].w, f[c].w, v);
                pn[a * 4 + c] = v;
              }
          }
        }
        // elementwise update; the rare unsafe divisions are rebuilt after the
        // loop so that the common path stays branch-light
        unsigned rebuild = 0u;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
          const int rt = rb + a * kRowSlots;  // row within the tile
          const bool live = rt < tr;
          const float cj = live ? gc[row0 + tile0 + rt] : 0.f;
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            const int i = ibk * 4 + c;
            float psk = 0.f;
            if (live && i < rF) {
              const float tot = s.ps[i * psld + tile0 + rt] * pn[a * 4 + c];
              const float d = po[a * 4 + c];
              if (d != 0.f && fabsf(tot) >= FLT_MIN && fabsf(tot) <= FLT_MAX) {
                psk = div_nr(tot, d);
                s.ps[i * psld + tile0 + rt] = psk;  // holds prod_{d != k} until mode k is solved
              } else {
                rebuild |= 1u << (a * 4 + c);
              }
            }
            s.wt[i * kWtStride + rt] = cj * psk;
          }
        }
        while (rebuild) {
          // unsafe division: rebuild prod_{d' != k} <G_j^d', F_i^d'> directly
          const int bit = __ffs(rebuild) - 1;
          rebuild &= rebuild - 1;
          const int a = bit / 4, c = bit % 4;
          const int rt = rb + a * kRowSlots, i = ibk * 4 + c;
          const int j = row0 + tile0 + rt;
          float psk = 1.f;
          for (int dd = 0; dd < D; ++dd) {
            if (dd == k) continue;
            const int npd = round_up(p.nbas[dd], 4);
            psk *= dot_global(gm + (long long)p.offp[dd] * rG + (long long)j * npd,
                              f32 + (long long)i * p.nDp + p.offp[dd], npd);
          }
          s.ps[i * psld + tile0 + rt] = psk;
          s.wt[i * kWtStride + rt] = gc[j] * psk;
        }
      }
      __syncthreads();
      // -- right-hand-side accumulation: acc(ib*4+a, nb*4+c) += w(r,i) g(r,n) --
      if (acc_active) {
        for (int rr = my_grp; rr < tr; rr += ngroups) {
          const float w0 = s.wt[(ib * 4 + 0) * kWtStride + rr];
          const float w1 = s.wt[(ib * 4 + 1) * kWtStride + rr];
          const float w2 = s.wt[(ib * 4 + 2) * kWtStride + rr];
          const float w3 = s.wt[(ib * 4 + 3) * kWtStride + rr];
          const float4 g = *reinterpret_cast<const float4*>(s.gt + rr * gsd + nb * 4);
          acc[0] = fmaf(w0, g.x, acc[0]);  acc[1] = fmaf(w0, g.y, acc[1]);
          acc[2] = fmaf(w0, g.z, acc[2]);  acc[3] = fmaf(w0, g.w, acc[3]);
          acc[4] = fmaf(w1, g.x, acc[4]);  acc[5] = fmaf(w1, g.y, acc[5]);
          acc[6] = fmaf(w1, g.z, acc[6]);  acc[7] = fmaf(w1, g.w, acc[7]);
          acc[8] = fmaf(w2, g.x, acc[8]);  acc[9] = fmaf(w2, g.y, acc[9]);
          acc[10] = fmaf(w2, g.z, acc[10]); acc[11] = fmaf(w2, g.w, acc[11]);
          acc[12] = fmaf(w3, g.x, acc[12]); acc[13] = fmaf(w3, g.y, acc[13]);
          acc[14] = fmaf(w3, g.z, acc[14]); acc[15] = fmaf(w3, g.w, acc[15]);
        }
      }
      __syncthreads();
    }
    // -- reduce the row groups into this CTA's partial right-hand side --
    if (acc_active) {
#pragma unroll
      for (int q = 0; q < 16; ++q) s.red[(my_grp * nblk + my_blk) * 16 + q] = acc[q];
    }
    __syncthreads();
    for (int e = tid; e < nblk * 16; e += kThreads) {
      const int blk = e / 16, q = e % 16;
      float sum = 0.f;
      for (int gI = 0; gI < ngroups; ++gI) sum += s.red[(gI * nblk + blk) * 16 + q];
      const int i = (blk / nnb) * 4 + q / 4, n = (blk % nnb) * 4 + q % 4;
      s.bpart[i * npmax + n] = sum;
    }
    cluster.sync();

    // -- rank 0: FP64 normal equations for mode k --
    if (rank == 0) {
      for (int e = tid; e < rF * nk; e += kThreads) {
        const int i = e % rF, n = e / rF;
        double sum = 0.0;
        for (int c = 0; c < CL; ++c) {
          const float* bp = cluster.map_shared_rank(s.bpart, c);
          sum += (double)bp[i * npmax + n];
        }
        s.X[i + n * rF] = sum;
      }
      if (k == 0) {
        // sweep start: suffix products of the current Grams, empty prefix
        for (int e = tid; e < rF * rF; e += kThreads) {
          double a = 1.0;
          suf[(long long)(D - 1) * rF * rF + e] = 1.0;
          for (int d = D - 1; d >= 1; --d) {
            a *= gram[(long long)d * rF * rF + e];
            suf[(long long)(d - 1) * rF * rF + e] = a;
          }
          s.L[e] = 1.0;
        }
      }
      __syncthreads();
      const double pen = s.misc[0];
      for (int e = tid; e < rF * rF; e += kThreads) {
        const int i = e % rF, i2 = e / rF;
        double bb = s.L[e] * suf[(long long)k * rF * rF + e];
        if (i == i2) bb += pen;
        s.BB[e] = bb;
      }
      __syncthreads();
      block_ldlt(s.BB, rF, rF, s.dinv, s.u, &s.flags[0]);
      block_ldlt_solve(s.BB, rF, rF, s.dinv, s.X, nk, rF);
      // normalise each term's new factor (max-scaled 2-norm), write F
      for (int i = tid; i < rF; i += kThreads) {
        double nrm, inv;
        scaled_norm(s.X + i, nk, rF, &nrm, &inv);
        for (int n = 0; n < nk; ++n) s.X[i + n * rF] *= inv;
        fcoef[i] = nrm;
      }
      __syncthreads();
      for (int e = tid; e < rFp * npk; e += kThreads) {
        const int i = e / npk, q = e % npk;
        const double x = (i < rF && q < nk) ? s.X[i + q * rF] : 0.0;
        const float xf = (float)x;
        if (i < rF) {
          if (q < nk) fbase[(long long)i * p.nD + p.off[k] + q] = x;
          f32[(long long)i * p.nDp + p.offp[k] + q] = xf;
        }
        for (int c = 0; c < CL; ++c) cluster.map_shared_rank(s.fnew, c)[i * npmax + q] = xf;
      }
      // new Gram of mode k and prefix update
      for (int e = tid; e < rF * rF; e += kThreads) {
        const int i = e % rF, i2 = e / rF;
        double t2 = 0.0;
        for (int n = 0; n < nk; ++n) t2 += s.X[i + n * rF] * s.X[i2 + n * rF];
        gram[(long long)k * rF * rF + e] = t2;
        s.L[e] *= t2;
      }
      if (tid == 0 && s.flags[0] != 0) atomicOr(&p.status[v], 1);
      __threadfence();
    }
    cluster.sync();
  }
}

size_t als_smem_bytes(int rows_cta, int rF, int npmax) {
  // mirrors the carve order at the top of als_cluster_kernel
  const int rFp = round_up(rF, 4);
  size_t b = 0;
  auto take = [&](size_t bytes) { b += (size_t)round_up((int)bytes, 16); };
  take(sizeof(float) * (size_t)rows_cta * rFp);
  take(sizeof(float) * rFp * npmax);
  take(sizeof(float) * rFp * npmax);
  take(sizeof(float) * kWtStride * rFp);
  take(sizeof(float) * kTileRows * tile_stride(npmax));
  take(sizeof(float) * kTileRows * tile_stride(npmax));
  take(sizeof(float) * rFp * npmax);
  take(sizeof(float) * kThreads * 16);
  take(sizeof(double) * rF * rF);
  take(sizeof(double) * rF * npmax);
  take(sizeof(double) * rF * rF);
  take(sizeof(double) * 4);
  take(sizeof(double) * rF);
  take(sizeof(double) * rF);
  take(sizeof(int) * 4);
  return b;
}

namespace {

template <int NP>
int launch_cluster(const AlsParams& prm, int cluster, size_t smem, cudaStream_t st) {
  auto fn = als_cluster_kernel<NP>;
  MLCP_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  if (cluster > 8) MLCP_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(prm.nvec * cluster);
  cfg.blockDim = dim3(kThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  MLCP_CUDA_TRY(cudaLaunchKernelEx(&cfg, fn, prm));
  return kOk;
}

}  // namespace

int als_launch(const AlsParams& p, int cluster, size_t smem, cudaStream_t st, cudaEvent_t t0, cudaEvent_t t1) {
  int dev = 0, nsm = 0;
  MLCP_CUDA_TRY(cudaGetDevice(&dev));
  MLCP_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const long long work = (p.total_rows > p.total_f_terms ? p.total_rows : p.total_f_terms) * p.ndof;
  long long blocks = (work + 255) / 256;
  if (blocks > (long long)nsm * 8) blocks = (long long)nsm * 8;
  if (blocks < 1) blocks = 1;
  als_prep_kernel<<<(int)blocks, 256, 0, st>>>(p);
  MLCP_CUDA_TRY(cudaGetLastError());
  if (t0) MLCP_CUDA_TRY(cudaEventRecord(t0, st));
  int rc;
  if (p.npmax <= 16) rc = launch_cluster<16>(p, cluster, smem, st);
  else if (p.npmax <= 32) rc = launch_cluster<32>(p, cluster, smem, st);
  else rc = launch_cluster<64>(p, cluster, smem, st);
  if (rc == kOk && t1) MLCP_CUDA_TRY(cudaEventRecord(t1, st));
  return rc;
}

}  // namespace mlcp
