// Operator update for the next tree layer: reference UpdateOperMat
// (src/Updater.f90:110-151), which for a primitive operator X of mode m forms
//   QXQ(i,j) = <Q_j, X_m Q_i>,  j >= i,
// by applying X to mode m of every term of Q_i (PRODXV, dspmv) and taking a
// full CP inner product with every Q_j, then stores QXQ packed (upper
// triangle by columns, SymPackMat2Vec) as the operator's new matrix.
//
// Here all operators of one mode go in one call:
//   opermat_apply_kernel: Y_x,i,r = X_x q_i,r^m for every operator, vector
//     and term (packed upper-triangular X, as dspmv 'U');
//   opermat_pair_kernel, one CTA per pair i <= j:
//     S(r,s) = c_i,r c_j,s prod_{d != m} <q_i,r^d, q_j,s^d>      (once)
//     QXQ_x(i,j) = sum_rs S(r,s) <Y_x,i,r, q_j,s^m>             (per operator)
//   with fixed-order block reductions.  FP64, as the reference.
#include <algorithm>
#include <cstdio>
#include <mutex>
#include <vector>

#include "../../include/mlcp_gb300.h"
#include "common.cuh"
#include "context.cuh"

namespace mlcp {

int finish_status(int status);

namespace {

constexpr int kPairThreads = 128;
constexpr int kMaxX = 16;  // operators per pass of the pair kernel

struct OpMatParams {
  int m, R, D, nD, B, n, o, nx;
  const int* nbas;      // device [D]
  const double* base;   // block, reference layout
  const double* coef;
  const double* xmats;  // [nx][n(n+1)/2]
  double* Y;            // [nx][B][R][n]
  double* out;          // [nx][B(B+1)/2]
};

__global__ void opermat_apply_kernel(OpMatParams p) {
  const long long total = (long long)p.nx * p.B * p.R * p.n;
  const size_t np = (size_t)p.n * (p.n + 1) / 2;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int a = (int)(e % p.n);
    const long long xir = e / p.n;  // (x, i, r)
    const int r = (int)(xir % p.R);
    const long long xi = xir / p.R;
    const int i = (int)(xi % p.B), x = (int)(xi / p.B);
    const double* X = p.xmats + (size_t)x * np;
    const double* q = p.base + ((size_t)i * p.R + r) * p.nD + p.o;
    double acc = 0.0;
    for (int b = 0; b < p.n; ++b) {
      const int ir = a < b ? a : b, ic = a < b ? b : a;
      acc = fma(X[ir + (size_t)ic * (ic + 1) / 2], q[b], acc);
    }
    p.Y[(((size_t)x * p.B + i) * p.R + r) * p.n + a] = acc;
  }
}

__global__ void __launch_bounds__(kPairThreads) opermat_pair_kernel(OpMatParams p, int x0, int nxp) {
  // pair e -> (i, j), i <= j, e = i + j (j + 1) / 2
  const int e = blockIdx.x;
  int j = (int)((sqrt(8.0 * e + 1.0) - 1.0) / 2.0);
  while ((j + 1) * (j + 2) / 2 <= e) ++j;
  while (j * (j + 1) / 2 > e) --j;
  const int i = e - j * (j + 1) / 2;
  const int R = p.R, nD = p.nD, n = p.n;
  const double* qi = p.base + (size_t)i * R * nD;
  const double* qj = p.base + (size_t)j * R * nD;
  double acc[kMaxX];
#pragma unroll
  for (int x = 0; x < kMaxX; ++x) acc[x] = 0.0;
  for (int rs = threadIdx.x; rs < R * R; rs += blockDim.x) {
    const int r = rs / R, s = rs % R;
    double S = p.coef[(size_t)i * R + r] * p.coef[(size_t)j * R + s];
    int o = 0;
    for (int d = 0; d < p.D; ++d) {
      const int nd = p.nbas[d];
      if (d != p.m) {
        double t = 0.0;
        for (int q = 0; q < nd; ++q) t = fma(qi[(size_t)r * nD + o + q], qj[(size_t)s * nD + o + q], t);
        S *= t;
      }
      o += nd;
    }
    const double* yj = qj + (size_t)s * nD + p.o;
#pragma unroll
    for (int x = 0; x < kMaxX; ++x) {
      if (x >= nxp) break;
      const double* y = p.Y + (((size_t)(x0 + x) * p.B + i) * R + r) * n;
      double t = 0.0;
      for (int a = 0; a < n; ++a) t = fma(y[a], yj[a], t);
      acc[x] = fma(S, t, acc[x]);
    }
  }
  __shared__ double red[kPairThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int x = 0; x < nxp; ++x) {
    double v = acc[x];
    for (int w = 16; w > 0; w >>= 1) v += __shfl_xor_sync(0xffffffffu, v, w);
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
      double tot = 0.0;
      for (int w = 0; w < kPairThreads / 32; ++w) tot += red[w];
      p.out[(size_t)(x0 + x) * p.B * (p.B + 1) / 2 + e] = tot;
    }
  }
}

int update_opermat(Context* ctx, int imode, const double* base, const double* coef, const int* nbas, int rk, int ndof,
                   int nbloc, int nx, const double* xmats, double* qxq) {
  if (ndof < 1 || imode < 1 || imode > ndof || rk < 1 || nbloc < 1 || nx < 1) {
    set_error("updateopermatcpp_: bad sizes (imode=%d ndof=%d rk=%d nbloc=%d nx=%d)", imode, ndof, rk, nbloc, nx);
    return kBadArgument;
  }
  std::vector<int> off(ndof + 1, 0);
  for (int d = 0; d < ndof; ++d) {
    if (nbas[d] < 1) {
      set_error("updateopermatcpp_: nbas[%d] = %d", d, nbas[d]);
      return kBadArgument;
    }
    off[d + 1] = off[d] + nbas[d];
  }
  OpMatParams p;
  p.m = imode - 1;
  p.R = rk;
  p.D = ndof;
  p.nD = off[ndof];
  p.B = nbloc;
  p.n = nbas[p.m];
  p.o = off[p.m];
  p.nx = nx;
  const size_t nvals = (size_t)nbloc * rk * p.nD, np = (size_t)p.n * (p.n + 1) / 2,
               nq = (size_t)nbloc * (nbloc + 1) / 2;
  size_t bytes = 0;
  auto take = [&](size_t b) { size_t o = align256(bytes); bytes = o + b; return o; };
  const size_t o_base = take(sizeof(double) * nvals), o_coef = take(sizeof(double) * (size_t)nbloc * rk),
               o_x = take(sizeof(double) * nx * np), o_nb = take(sizeof(int) * ndof),
               o_y = take(sizeof(double) * (size_t)nx * nbloc * rk * p.n), o_out = take(sizeof(double) * nx * nq);
  cudaStream_t st = ctx->stream;
  if (bytes > ctx->cyc_bytes) {
    if (ctx->cyc) {
      MLCP_CUDA_TRY(cudaStreamSynchronize(st));
      MLCP_CUDA_TRY(cudaFree(ctx->cyc));
      ctx->cyc = nullptr;
      ctx->cyc_bytes = 0;
    }
    MLCP_CUDA_TRY(cudaMalloc(&ctx->cyc, bytes));
    ctx->cyc_bytes = bytes;
  }
  char* b = static_cast<char*>(ctx->cyc);
  p.base = reinterpret_cast<const double*>(b + o_base);
  p.coef = reinterpret_cast<const double*>(b + o_coef);
  p.xmats = reinterpret_cast<const double*>(b + o_x);
  p.nbas = reinterpret_cast<const int*>(b + o_nb);
  p.Y = reinterpret_cast<double*>(b + o_y);
  p.out = reinterpret_cast<double*>(b + o_out);
  MLCP_CUDA_TRY(cudaMemcpyAsync(b + o_base, base, sizeof(double) * nvals, cudaMemcpyHostToDevice, st));
  MLCP_CUDA_TRY(cudaMemcpyAsync(b + o_coef, coef, sizeof(double) * nbloc * rk, cudaMemcpyHostToDevice, st));
  MLCP_CUDA_TRY(cudaMemcpyAsync(b + o_x, xmats, sizeof(double) * nx * np, cudaMemcpyHostToDevice, st));
  MLCP_CUDA_TRY(cudaMemcpyAsync(b + o_nb, nbas, sizeof(int) * ndof, cudaMemcpyHostToDevice, st));
  const long long items = (long long)nx * nbloc * rk * p.n;
  const int blocks = (int)std::min<long long>((items + 255) / 256, (long long)ctx->num_sms * 8);
  opermat_apply_kernel<<<blocks, 256, 0, st>>>(p);
  MLCP_CUDA_TRY(cudaGetLastError());
  for (int x0 = 0; x0 < nx; x0 += kMaxX) {
    opermat_pair_kernel<<<(unsigned)nq, kPairThreads, 0, st>>>(p, x0, std::min(kMaxX, nx - x0));
    MLCP_CUDA_TRY(cudaGetLastError());
  }
  MLCP_CUDA_TRY(cudaMemcpyAsync(qxq, p.out, sizeof(double) * nx * nq, cudaMemcpyDeviceToHost, st));
  MLCP_CUDA_TRY(cudaStreamSynchronize(st));
  return kOk;
}

}  // namespace

}  // namespace mlcp

extern "C" void updateopermatcpp_(const int& imode, double* base, double* coef, int* nbas, const int& rk,
                                  const int& ndof, const int& nbloc, const int& nx, double* xmats, double* qxq) {
  int rc = mlcp::kOk;
  mlcp::Context* ctx = mlcp::get_context(&rc);
  if (ctx) {
    std::lock_guard<std::mutex> lk(ctx->mu);
    rc = mlcp::update_opermat(ctx, imode, base, coef, nbas, rk, ndof, nbloc, nx, xmats, qxq);
  }
  mlcp::finish_status(rc);
  if (rc != mlcp::kOk) fprintf(stderr, "updateopermatcpp_: %s\n", mlcp::last_error());
}
