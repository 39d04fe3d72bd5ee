// Rayleigh quotients of the vectors of a block under the operator list:
// reference GetQHQdiag (src/BlockUtils.f90:385-408) with RayleighQuotient2
// (:658-688), the `update = F` path that the reference runs on the CPU after
// intertwinecpp_ (src/Solver.f90:499-504).
//
// The reference applies every Hamiltonian term to every rank-1 term of v and
// accumulates <v, w> (O(R T (sum n^2 + R nD)) per vector).  Here one CTA per
// vector computes, for every distinct operator u of every mode d (slot 0 is
// the identity), the Gram
//   M_d,u(i, j) = <v_i^d, h_u v_j^d>
// once, after which
//   <v|H|v> = sum_t alpha_t sum_ij c_i c_j prod_d M_d,op(t,d)(i, j)
//   <v|v>   = sum_ij c_i c_j prod_d M_d,0(i, j).
// Everything is FP64, as in the reference: the work per vector is small and
// the result is an eigenvalue estimate compared at the 1e-7 relative level.
#include <algorithm>

#include "common.cuh"
#include "intertwine.cuh"

namespace mlcp {

namespace {

constexpr int kRqThreads = 256;

// Sum over the block in a fixed order; thread 0 gets the result.
__device__ double block_sum64(double v, double* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < kRqThreads / 32; ++w) s += red[w];
  return s;
}

// Mode of the global operator slot g (uoff[d] <= g < uoff[d+1]).
__device__ __forceinline__ int slot_mode(const OpTable& t, int g) {
  int d = 0;
  while (d + 1 < t.D && t.uoff[d + 1] <= g) ++d;
  return d;
}

__global__ void __launch_bounds__(kRqThreads) rq_kernel(RqParams p) {
  const OpTable& t = p.ops;
  const int v = p.v0 + blockIdx.x;
  const int R = t.R, D = t.D, nD = p.nD, npm = t.npmax, RR = R * R, U = t.utot;
  const double* vb = p.base + (size_t)v * R * nD;
  const double* vc = p.coef + (size_t)v * R;
  double* M = p.work + (size_t)blockIdx.x * p.work_stride;  // [U][R][R]
  double* Y = M + (size_t)U * RR;                                 // [U][npm][R]
  __shared__ double red[kRqThreads / 32];

  // Y_u(a, j) = sum_b h_u(a, b) v_j^d(b) for the non-identity operators
  for (int e = threadIdx.x; e < U * npm * R; e += kRqThreads) {
    const int g = e / (npm * R), rem = e - g * npm * R, a = rem / R, j = rem - a * R;
    const int d = slot_mode(t, g), n = t.nbas[d];
    if (a >= n || t.ident[g]) continue;
    const double* h = t.hmat64 + (size_t)g * npm * npm + (size_t)a * npm;
    const double* x = vb + (size_t)j * nD + t.off[d];
    double acc = 0.0;
    for (int b = 0; b < n; ++b) acc = fma(h[b], x[b], acc);
    Y[(size_t)g * npm * R + a * R + j] = acc;
  }
  __syncthreads();
  // M_u(i, j) = sum_a v_i^d(a) Y_u(a, j); the identity gives the mode Gram
  for (int e = threadIdx.x; e < U * RR; e += kRqThreads) {
    const int g = e / RR, ij = e - g * RR, i = ij / R, j = ij - i * R;
    const int d = slot_mode(t, g), n = t.nbas[d];
    const double* xi = vb + (size_t)i * nD + t.off[d];
    double acc = 0.0;
    if (t.ident[g]) {
      const double* xj = vb + (size_t)j * nD + t.off[d];
      for (int a = 0; a < n; ++a) acc = fma(xi[a], xj[a], acc);
    } else {
      const double* y = Y + (size_t)g * npm * R + j;
      for (int a = 0; a < n; ++a) acc = fma(xi[a], y[a * R], acc);
    }
    M[(size_t)g * RR + ij] = acc;
  }
  __syncthreads();
  // the term sums and the norm
  const int T = t.T;
  double num = 0.0, den = 0.0;
  for (int e = threadIdx.x; e < (T + 1) * RR; e += kRqThreads) {
    const int tt = e / RR, ij = e - tt * RR, i = ij / R, j = ij - i * R;
    double prod = vc[i] * vc[j];
    if (tt < T) {
      for (int d = 0; d < D; ++d) prod *= M[(size_t)(t.uoff[d] + t.uid[(size_t)tt * D + d]) * RR + ij];
      num = fma(t.alpha[tt], prod, num);
    } else {
      for (int d = 0; d < D; ++d) prod *= M[(size_t)t.uoff[d] * RR + ij];
      den += prod;
    }
  }
  num = block_sum64(num, red);
  den = block_sum64(den, red);
  if (threadIdx.x == 0) p.out[v] = num / den;
}

constexpr int kPairChunk = 128;  // (r, s) entries per pass of a pair CTA

// y[v][g][s][a] = (h_g x_s^d)(a), d the mode of slot g (identity slots copy
// the factor; entries a >= n_d are zero).
__global__ void __launch_bounds__(256) rq_apply_kernel(OpTable t, int nvec, int nD, const double* base, double* y) {
  const int R = t.R, npm = t.npmax;
  const long long total = (long long)nvec * t.utot * R * npm;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int a = (int)(e % npm);
    const long long q = e / npm;
    const int r = (int)(q % R);
    const long long q2 = q / R;
    const int g = (int)(q2 % t.utot), v = (int)(q2 / t.utot);
    const int d = slot_mode(t, g), n = t.nbas[d];
    double acc = 0.0;
    if (a < n) {
      const double* x = base + ((size_t)v * R + r) * nD + t.off[d];
      if (t.ident[g]) {
        acc = x[a];
      } else {
        const double* h = t.hmat64 + (size_t)g * npm * npm + (size_t)a * npm;
        for (int b = 0; b < n; ++b) acc = fma(h[b], x[b], acc);
      }
    }
    y[e] = acc;
  }
}

// One CTA per pair i >= j of the block:
//   A(i, j) = <Q_j|H|Q_i> = sum_t alpha_t sum_rs c_j,r c_i,s prod_d M_d,op(t,d)(r, s)
//   S(i, j) = <Q_j|Q_i>   = sum_rs c_j,r c_i,s prod_d M_d,0(r, s)
// with M_g(r, s) = <q_j,r^d, h_g q_i,s^d> from the applied factors y.  Each
// thread takes one (r, s) per pass and keeps its M values in a shared-memory
// column ([utot][kPairChunk]); FP64, fixed-order block sums.
__global__ void __launch_bounds__(kPairChunk) rq_pair_kernel(RqPairParams p) {
  const OpTable& t = p.ops;
  extern __shared__ double msm[];  // [utot][kPairChunk]
  __shared__ double red[2][kPairChunk / 32];
  const int e = blockIdx.x;
  int i = (int)((sqrt(8.0 * e + 1.0) - 1.0) / 2.0);
  while ((i + 1) * (i + 2) / 2 <= e) ++i;
  while (i * (i + 1) / 2 > e) --i;
  const int j = e - i * (i + 1) / 2;
  const int R = t.R, RR = R * R, D = t.D, U = t.utot, npm = t.npmax, tid = threadIdx.x;
  const double* qj = p.base + (size_t)j * R * p.nD;
  const double* cj = p.coef + (size_t)j * R;
  const double* ci = p.coef + (size_t)i * R;
  const double* yi = p.y + (size_t)i * U * R * npm;
  double* col = msm + tid;
  double accA = 0.0, accS = 0.0;
  for (int rs0 = 0; rs0 < RR; rs0 += kPairChunk) {
    const int rs = rs0 + tid;
    if (rs < RR) {
      const int r = rs / R, sv = rs - r * R;
      for (int g = 0; g < U; ++g) {
        const int d = slot_mode(t, g), n = t.nbas[d];
        const double* x = qj + (size_t)r * p.nD + t.off[d];
        const double* yv = yi + ((size_t)g * R + sv) * npm;
        double m = 0.0;
        for (int a = 0; a < n; ++a) m = fma(x[a], yv[a], m);
        col[(size_t)g * kPairChunk] = m;
      }
      const double cc = cj[r] * ci[sv];
      double ps = cc;
      for (int d = 0; d < D; ++d) ps *= col[(size_t)t.uoff[d] * kPairChunk];
      accS += ps;
      double pa = 0.0;
      for (int tt = 0; tt < t.T; ++tt) {
        double prod = t.alpha[tt];
        for (int d = 0; d < D; ++d) prod *= col[(size_t)(t.uoff[d] + t.uid[(size_t)tt * D + d]) * kPairChunk];
        pa += prod;
      }
      accA = fma(cc, pa, accA);
    }
  }
  const int lane = tid & 31, warp = tid >> 5;
  for (int o = 16; o > 0; o >>= 1) {
    accA += __shfl_xor_sync(0xffffffffu, accA, o);
    accS += __shfl_xor_sync(0xffffffffu, accS, o);
  }
  if (lane == 0) {
    red[0][warp] = accA;
    red[1][warp] = accS;
  }
  __syncthreads();
  if (tid == 0) {
    double a = 0.0, sv = 0.0;
    for (int w = 0; w < kPairChunk / 32; ++w) {
      a += red[0][w];
      sv += red[1][w];
    }
    p.A[i + (size_t)j * p.nvec] = a;
    p.S[i + (size_t)j * p.nvec] = sv;
  }
}

}  // namespace

int rq_apply_launch(const OpTable& t, int nvec, int nD, const double* base, double* y, cudaStream_t st) {
  const long long total = (long long)nvec * t.utot * t.R * t.npmax;
  const int blocks = (int)std::min<long long>((total + 255) / 256, 4096LL);
  rq_apply_kernel<<<blocks, 256, 0, st>>>(t, nvec, nD, base, y);
  MLCP_CUDA_TRY(cudaGetLastError());
  return kOk;
}

size_t rq_pair_smem(const OpTable& t) { return sizeof(double) * (size_t)t.utot * kPairChunk; }

int rq_pair_launch(const RqPairParams& p, int smem_optin, cudaStream_t st) {
  const size_t smem = rq_pair_smem(p.ops);
  if (smem + 1024 > (size_t)smem_optin) {
    set_error("the block's H matrix: %d distinct operators exceed the shared memory of one pair", p.ops.utot);
    return kTooLarge;
  }
  MLCP_CUDA_TRY(cudaFuncSetAttribute(rq_pair_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const long long npairs = (long long)p.nvec * (p.nvec + 1) / 2;
  rq_pair_kernel<<<(unsigned)npairs, kPairChunk, smem, st>>>(p);
  MLCP_CUDA_TRY(cudaGetLastError());
  return kOk;
}

size_t rq_work_doubles(const OpTable& t) {
  return (size_t)t.utot * t.R * t.R + (size_t)t.utot * t.npmax * t.R;
}

int rq_launch(const RqParams& p, cudaStream_t st) {
  const int nv = p.nvec - p.v0;
  if (nv <= 0) return kOk;
  RqParams q = p;
  q.work_stride = (long long)rq_work_doubles(p.ops);
  rq_kernel<<<nv, kRqThreads, 0, st>>>(q);
  MLCP_CUDA_TRY(cudaGetLastError());
  return kOk;
}

}  // namespace mlcp
