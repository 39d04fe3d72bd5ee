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

}  // namespace

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
