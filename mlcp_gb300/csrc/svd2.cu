// Two-mode reduction by SVD: reference reduc_SVDa / reduc_SVDb
// (src/REDUCTIONML.f90:296-392) with CP2DtoMat (src/SepdRepn.f90:518-558),
// SolveWithSVD (LAPACK DGESVD, src/LinAlg.f90:432-466) and RebuildfromSVD
// (src/REDUCTIONML.f90:394-439).  For a two-mode CP vector G the reference
// multiplies out A = sum_k c_k a_k b_k^T (nr x nc), takes its SVD
// A = U S V^T, keeps ncomp = the leading singular values >= redtol * s_1
// (at least one), truncates to nrk = min(nr, nc, rF, ncomp) and returns
// F with coef = s_i, mode 1 = U(:, i), mode 2 = V(:, i).  Its 'a' and 'b'
// variants differ only in how the SVD is reached (dense A vs. QR of the
// factors), so both are this one routine; results agree up to rounding and
// the signs of singular-vector pairs.
//
// GB300 mapping:
//   svd2_form_kernel   many CTAs per vector: the matrix M (A, or A^T when
//                      nr < nc, so that M is m x n with m >= n) in FP64, in
//                      column order into global scratch;
//   svd2_jacobi_kernel one CTA per vector: one-sided Jacobi (Hestenes) on
//                      the n columns of M in shared memory (global memory
//                      when it does not fit), with the parallel
//                      round-robin ordering -- n/2 disjoint column pairs per
//                      round, one warp per pair -- until a sweep makes no
//                      rotation; then column norms = singular values, a
//                      stable descending sort, the reference's truncation,
//                      the rebuild and (optionally) NORMCOEF, in FP64.
// The sweeps run in double-word arithmetic (about 48 bits, dword.cuh) on M
// scaled by a power of two: an FP64 instruction holds this part's FP64 pipe
// for 64 cycles per warp, which made FP64 sweeps slower than one CPU core,
// while double-word operations issue on the FP32 pipes.  One-sided Jacobi
// computes every singular value to high relative accuracy (Demmel and
// Veselic, SIAM J. Matrix Anal. Appl. 13 (1992) 1204-1245); with 48-bit
// arithmetic the results agree with LAPACK's FP64 SVD to about 1e-13 of s_1,
// far inside the reference's rank cut of 1e-12 s_1.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <mutex>
#include <vector>

#include "../../include/mlcp_gb300.h"
#include "common.cuh"
#include "context.cuh"
#include "dword.cuh"
#include "intertwine.cuh"

namespace mlcp {

int finish_status(int status);

namespace {

constexpr int kSvdThreads = 1024;
constexpr int kSvdWarps = kSvdThreads / 32;
constexpr int kPairLanes = 16;                  // lanes per column pair in the sweeps
constexpr int kGroupsPerWarp = 32 / kPairLanes;
constexpr int kMaxN = 256;       // min(nr, nc)
constexpr int kMaxM = 4096;      // max(nr, nc)
constexpr int kMaxSweeps = 40;
constexpr float kTinySq = 7.8886091e-31f;        // (2^-50)^2
constexpr long long kApplyMaxBlocks = 2048;     // grid-stride cap of the apply kernel

struct Shape {
  int m, n, n2;  // M is m x n (m >= n); n2 = n rounded up to even
  bool tr;       // M = A^T (nr < nc)
};

__host__ __device__ inline Shape shape_of(int nr, int nc) {
  Shape s;
  s.tr = nr < nc;
  s.m = s.tr ? nc : nr;
  s.n = s.tr ? nr : nc;
  s.n2 = (s.n + 1) & ~1;
  return s;
}

// Scratch of one vector: M (n2 x m) and, for the global-memory variant, V.
__host__ __device__ inline size_t work_doubles(const Shape& s) {
  return (size_t)s.n2 * s.m + (size_t)s.n2 * s.n2;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// M(i, j) of vector blockIdx.y, i < m (row factor), j < n (column factor),
// stored at work[v][j * m + i].
__global__ void __launch_bounds__(256) svd2_form_kernel(Svd2Params p) {
  const Shape s = shape_of(p.nr, p.nc);
  const int v = blockIdx.y;
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long long)s.m * s.n) return;
  const int j = (int)(e / s.m), i = (int)(e - (long long)j * s.m);
  // row factor: mode 2 when transposed, else mode 1; column factor the other
  const int ia = s.tr ? j : i, ib = s.tr ? i : j;  // index into mode 1 / mode 2
  double acc = 0.0;
  if (!p.hv) {
    const int nD = p.nr + p.nc;
    const double* b = p.in_base + (p.shared_base ? (size_t)0 : (size_t)v * p.K * nD);
    const double* c = p.in_coef + (size_t)v * p.K;
    for (int k = 0; k < p.K; ++k) acc = fma(c[k] * b[(size_t)k * nD + ia], b[(size_t)k * nD + p.nr + ib], acc);
  } else {
    const OpTable& t = p.ops;
    const int R = t.R, npm = t.npmax;
    const double* y = p.y + (size_t)v * t.utot * R * npm;
    const double* c = p.v_coef + (size_t)v * R;
    const int u0 = t.uoff[0], u1 = t.uoff[1];
    for (int tt = 0; tt < t.T; ++tt) {
      const double* ya = y + (size_t)(u0 + t.uid[2 * tt]) * R * npm + ia;
      const double* yb = y + (size_t)(u1 + t.uid[2 * tt + 1]) * R * npm + ib;
      double st = 0.0;
      for (int r = 0; r < R; ++r) st = fma(c[r] * ya[(size_t)r * npm], yb[(size_t)r * npm], st);
      acc = fma(t.alpha[tt], st, acc);
    }
    // the shift terms of PRODHV (ishift = 1): - shift_v * v
    const double* ya = y + (size_t)u0 * R * npm + ia;
    const double* yb = y + (size_t)u1 * R * npm + ib;
    double st = 0.0;
    for (int r = 0; r < R; ++r) st = fma(c[r] * ya[(size_t)r * npm], yb[(size_t)r * npm], st);
    acc = fma(-p.shift[v], st, acc);
  }
  p.work[(size_t)v * work_doubles(s) + e] = acc;
}

// Jacobi rotation that makes columns x and y orthogonal, from their Gram
// entries (Rutishauser's formulas: t the smaller root of
// t^2 + 2 zeta t - 1 = 0, zeta = (beta - alpha) / (2 gamma)).  t is taken in
// FP32 (beta - alpha formed in double-word first, so near-equal norms do not
// cancel); c = 1 / sqrt(1 + t^2) and s = c t are then double-word, so that
// c^2 + s^2 = 1 to double-word accuracy whatever t's own rounding.  A t off
// by 1e-7 relative still cuts gamma by seven digits; the sweeps repeat.
__device__ __forceinline__ void jacobi_rotation(dw al, dw be, dw ga, dw* c, dw* s) {
  const float zeta = __fdiv_rn(dw_sub(be, al).hi, __fmul_rn(2.f, ga.hi));
  const float az = fabsf(zeta);
  float t;
  if (az > 1.0e15f)
    t = __fdiv_rn(0.5f, zeta);
  else
    t = __fdiv_rn(zeta >= 0.f ? 1.f : -1.f, __fadd_rn(az, __fsqrt_rn(__fmaf_rn(zeta, zeta, 1.f))));
  // c = (1 + t^2)^-1/2 by two Newton steps in double-word from the FP32
  // seed (2^-22 -> 2^-44 -> double-word rounding): a one-step c would make
  // c^2 + s^2 - 1 about 1e-13 and scale the columns at every rotation
  const dw u = dw_add_f(two_prod(t, t), 1.f);
  dw r{f_rsqrt_approx(u.hi), 0.f};
#pragma unroll
  for (int it = 0; it < 2; ++it) {
    const dw e = dw_add_f(dw_neg(dw_mul(u, dw_mul(r, r))), 1.f);
    r = dw_add(r, dw_mul(r, dw_mul_f(e, 0.5f)));
  }
  *c = r;
  *s = dw_mul_f(r, t);
}

// all lanes end with the same double-word sum (dw_add_sloppy is symmetric
// in its arguments: its two-sums are exact)
__device__ __forceinline__ dw warp_sum_dw(dw v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const dw w{__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
    v = dw_add_sloppy(v, w);
  }
  return v;
}

// The same over the kPairLanes lanes of a pair group (xor offsets below the
// group width stay inside the group).
__device__ __forceinline__ dw group_sum_dw(dw v) {
#pragma unroll
  for (int o = kPairLanes / 2; o > 0; o >>= 1) {
    const dw w{__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
    v = dw_add_sloppy(v, w);
  }
  return v;
}

// x <- c x - s y, y <- s x + c y over n entries (strided by the pair group)
__device__ __forceinline__ void rotate_cols(dw* x, dw* y, int n, dw c, dw s, int lane) {
  for (int i = lane; i < n; i += kPairLanes) {
    const dw xi = x[i], yi = y[i];
    x[i] = dw_add_sloppy(dw_mul(c, xi), dw_neg(dw_mul(s, yi)));
    y[i] = dw_add_sloppy(dw_mul(s, xi), dw_mul(c, yi));
  }
}

template <bool kShared>
__global__ void __launch_bounds__(kSvdThreads) svd2_jacobi_kernel(Svd2Params p) {
  extern __shared__ __align__(16) double smem[];
  __shared__ double sig[kMaxN], vnorm[kMaxN], mnorm[kMaxN];
  __shared__ int ord[kMaxN];
  __shared__ double red[kSvdWarps];
  __shared__ int flag, nkeep;
  const Shape sh = shape_of(p.nr, p.nc);
  const int m = sh.m, n = sh.n, n2 = sh.n2;
  const int v = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  double* gw = p.work + (size_t)v * work_doubles(sh);
  // the sweeps run on double-word copies of M and V, in place of the FP64
  // values (same 8 bytes per entry)
  dw* M = reinterpret_cast<dw*>(kShared ? smem : gw);
  dw* V = M + (size_t)n2 * m;
  // scale M by a power of two so that its largest entry lies in [0.5, 1):
  // the FP32 exponent range then covers every square the sweeps form
  double amax = 0.0;
  for (int e = tid; e < n * m; e += kSvdThreads) amax = fmax(amax, fabs(gw[e]));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) amax = fmax(amax, __shfl_xor_sync(0xffffffffu, amax, o));
  if (lane == 0) red[warp] = amax;
  __syncthreads();
  if (tid == 0) {
    double a = 0.0;
    for (int w = 0; w < kSvdWarps; ++w) a = fmax(a, red[w]);
    int ex = 0;
    if (a > 0.0) frexp(a, &ex);
    sig[0] = ldexp(1.0, -ex);
  }
  __syncthreads();
  const double scale = sig[0];
  __syncthreads();
  for (int e = tid; e < n2 * m; e += kSvdThreads) {
    const double x = e < n * m ? gw[e] * scale : 0.0;
    M[e] = dw_from_double(x);
  }
  for (int e = tid; e < n2 * n2; e += kSvdThreads) V[e] = dw{(e % n2 == e / n2) ? 1.f : 0.f, 0.f};
  __syncthreads();
  // Columns whose norm falls below skip = 0.01 redtol / sqrt(n) of the
  // largest starting column norm take no further rotations: together they
  // span singular values below 0.01 redtol s_1 (s_1 is at least the largest
  // column norm), which the rank cut drops, and leaving them unorthogonalised
  // moves the kept singular values by less than that.  A low-rank input
  // (the usual H v) would otherwise spend most sweeps rotating rounding noise.
  float cmax = 0.f;
  for (int j = warp; j < n; j += kSvdWarps) {
    const dw* x = M + (size_t)j * m;
    float a = 0.f;
    for (int i = lane; i < m; i += 32) a = fmaf(x[i].hi, x[i].hi, a);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    cmax = fmaxf(cmax, a);
  }
  if (lane == 0) red[warp] = (double)cmax;
  __syncthreads();
  float tiny = kTinySq;
  {
    double mx = 0.0;
    for (int w = 0; w < kSvdWarps; ++w) mx = fmax(mx, red[w]);
    const double rel = 0.01 * p.redtol / sqrt((double)n);
    tiny = fmaxf(tiny, (float)(rel * rel * mx));
  }
  __syncthreads();

  // rotate while |x.y| > sqrt(m) 2^-46 |x| |y|: about the orthogonality that
  // double-word columns can hold, reached in the same number of sweeps as a
  // looser bound
  const float tol = sqrtf((float)m) * 1.4210855e-14f;
  bool converged = false;
  for (int sweep = 0; sweep < kMaxSweeps; ++sweep) {
    if (tid == 0) flag = 0;
    __syncthreads();
    for (int k = 0; k < n2 - 1; ++k) {
      // a group of kPairLanes lanes per column pair, two pairs per warp
      // instruction; every lane of a warp runs the same number of slots so
      // that the group shuffles stay converged
      for (int q0 = warp * kGroupsPerWarp; q0 < n2 / 2; q0 += kSvdWarps * kGroupsPerWarp) {
        const int q = q0 + lane / kPairLanes, gl = lane % kPairLanes;
        const bool live = q < n2 / 2;
        int a = 0, b = 0;
        if (q == 0) {
          a = n2 - 1;
          b = k;
        } else if (live) {
          a = (k + q) % (n2 - 1);
          b = (k - q + n2 - 1) % (n2 - 1);
        }
        dw* x = M + (size_t)a * m;
        dw* y = M + (size_t)b * m;
        dw_acc aa = acc_zero(), ab = acc_zero(), ag = acc_zero();
        for (int i = gl; live && i < m; i += kPairLanes) {
          const dw xi = x[i], yi = y[i];
          acc_fma(aa, xi, xi);
          acc_fma(ab, yi, yi);
          acc_fma(ag, xi, yi);
        }
        const dw al = group_sum_dw(acc_value(aa)), be = group_sum_dw(acc_value(ab)),
                 ga = group_sum_dw(acc_value(ag));
        // columns below the skip norm (or 2^-50 of the largest entry) stay
        // as they are: they cannot move a singular value above the rank cut
        if (live && al.hi > tiny && be.hi > tiny && fabsf(ga.hi) > tol * __fsqrt_rn(al.hi) * __fsqrt_rn(be.hi)) {
          dw c, s;
          jacobi_rotation(al, be, ga, &c, &s);
          rotate_cols(x, y, m, c, s, gl);
          rotate_cols(V + (size_t)a * n2, V + (size_t)b * n2, n2, c, s, gl);
          if (gl == 0) flag = 1;
        }
      }
      __syncthreads();
    }
    const int f = flag;
    __syncthreads();
    if (!f) {
      converged = true;
      break;
    }
  }

  // singular values: M = M0 V holds for the computed V, whose columns carry
  // the same rounding-level norm drift as M's, so s_j = |M_j| / |V_j|
  // (unscaled); the rebuild divides M_j by |M_j| and V_j by |V_j|
  for (int j = warp; j < n; j += kSvdWarps) {
    const dw* x = M + (size_t)j * m;
    const dw* y = V + (size_t)j * n2;
    dw_acc a = acc_zero(), b = acc_zero();
    for (int i = lane; i < m; i += 32) acc_fma(a, x[i], x[i]);
    for (int i = lane; i < n2; i += 32) acc_fma(b, y[i], y[i]);
    const dw ta = warp_sum_dw(acc_value(a)), tb = warp_sum_dw(acc_value(b));
    if (lane == 0) {
      const double mn = sqrt(dw_to_double(ta)), vn = sqrt(dw_to_double(tb));
      sig[j] = mn / vn / scale;
      vnorm[j] = vn;
      mnorm[j] = mn;
    }
  }
  __syncthreads();
  // stable descending order
  for (int j = tid; j < n; j += kSvdThreads) {
    const double sj = sig[j];
    int pos = 0;
    for (int k = 0; k < n; ++k) pos += (sig[k] > sj) || (sig[k] == sj && k < j);
    ord[pos] = j;
  }
  __syncthreads();
  if (tid == 0) {
    const double cut = p.redtol * sig[ord[0]];
    int ncomp = 1;
    for (int i = 1; i < n; ++i) {
      if (fabs(sig[ord[i]]) < cut) break;
      ncomp = i + 1;
    }
    nkeep = min(min(p.nr, p.nc), min(p.rout, ncomp));
    if (p.out_rank) p.out_rank[v] = nkeep;
    if (!converged && p.status) atomicOr(&p.status[v], 4);
  }
  __syncthreads();
  const int nrk = nkeep, nD = p.nr + p.nc;
  double* ob = p.out_base + (size_t)v * p.rout * nD;
  double* oc = p.out_coef + (size_t)v * p.rout;
  // rebuild: term k = (s_j, U(:, j), V(:, j)) for j = ord[k]
  for (int k = warp; k < p.rout; k += kSvdWarps) {
    double* o = ob + (size_t)k * nD;
    double* ou = o + (sh.tr ? p.nr : 0);  // the factor of length m
    double* ov = o + (sh.tr ? 0 : p.nr);  // the factor of length n
    if (k >= nrk) {
      for (int i = lane; i < nD; i += 32) o[i] = 0.0;
      if (lane == 0) oc[k] = 0.0;
      continue;
    }
    const int j = ord[k];
    const double s = sig[j];
    const dw* x = M + (size_t)j * m;
    if (s > 0.0) {
      const double inv = 1.0 / mnorm[j];
      for (int i = lane; i < m; i += 32) ou[i] = dw_to_double(x[i]) * inv;
    } else {  // all of A is zero: unit vectors, weight zero
      for (int i = lane; i < m; i += 32) ou[i] = (i == k % m) ? 1.0 : 0.0;
    }
    const dw* vc = V + (size_t)j * n2;
    const double vinv = 1.0 / vnorm[j];
    for (int i = lane; i < n; i += 32) ov[i] = dw_to_double(vc[i]) * vinv;
    if (lane == 0) oc[k] = s;
  }
  if (!p.normalize) return;
  __syncthreads();
  // NORMCOEF (src/MODVECVECML.f90:295-352): unit factors with their norms
  // moved into the weights, then the weights divided by the vector's norm
  for (int k = warp; k < nrk; k += kSvdWarps) {
    double* o = ob + (size_t)k * nD;
    double n1 = 0.0, n2s = 0.0;
    for (int i = lane; i < p.nr; i += 32) n1 = fma(o[i], o[i], n1);
    for (int i = lane; i < p.nc; i += 32) n2s = fma(o[p.nr + i], o[p.nr + i], n2s);
    n1 = sqrt(warp_sum(n1));
    n2s = sqrt(warp_sum(n2s));
    for (int i = lane; i < p.nr; i += 32) o[i] /= n1;
    for (int i = lane; i < p.nc; i += 32) o[p.nr + i] /= n2s;
    if (lane == 0) oc[k] *= n1 * n2s;
  }
  __syncthreads();
  double part = 0.0;
  for (int e = tid; e < nrk * nrk; e += kSvdThreads) {
    const int a = e / nrk, b = e - a * nrk;
    const double* fa = ob + (size_t)a * nD;
    const double* fb = ob + (size_t)b * nD;
    double d1 = 0.0, d2 = 0.0;
    for (int i = 0; i < p.nr; ++i) d1 = fma(fa[i], fb[i], d1);
    for (int i = 0; i < p.nc; ++i) d2 = fma(fa[p.nr + i], fb[p.nr + i], d2);
    part = fma(oc[a] * oc[b], d1 * d2, part);
  }
  part = warp_sum(part);
  if (lane == 0) red[warp] = part;
  __syncthreads();
  if (tid == 0) {
    double tot = 0.0;
    for (int w = 0; w < kSvdWarps; ++w) tot += red[w];
    sig[0] = 1.0 / sqrt(fabs(tot));
  }
  __syncthreads();
  const double sc = sig[0];
  for (int k = tid; k < nrk; k += kSvdThreads) oc[k] *= sc;
}

// y[v][g][r][a] = (h_g x_r^d)(a) for the operator slots g of the two-mode
// table (d = the slot's mode); identity slots copy the factor.
__global__ void __launch_bounds__(256) svd2_apply_kernel(OpTable t, int nvec, int nD, const double* base, double* y) {
  const int R = t.R, npm = t.npmax;
  const long long total = (long long)nvec * t.utot * R * npm;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int a = (int)(e % npm);
    const long long q = e / npm;
    const int r = (int)(q % R);
    const long long q2 = q / R;
    const int g = (int)(q2 % t.utot), v = (int)(q2 / t.utot);
    const int d = g >= t.uoff[1] ? 1 : 0, n = t.nbas[d];
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

}  // namespace

size_t svd2_work_doubles(int nr, int nc) { return work_doubles(shape_of(nr, nc)); }

int svd2_apply_launch(const OpTable& t, int nvec, int nD, const double* base, double* y, cudaStream_t st) {
  const long long total = (long long)nvec * t.utot * t.R * t.npmax;
  const int blocks = (int)std::min<long long>((total + 255) / 256, kApplyMaxBlocks);
  svd2_apply_kernel<<<blocks, 256, 0, st>>>(t, nvec, nD, base, y);
  MLCP_CUDA_TRY(cudaGetLastError());
  return kOk;
}

int svd2_launch(const Svd2Params& p, int smem_optin, cudaStream_t st) {
  const Shape s = shape_of(p.nr, p.nc);
  if (p.nvec < 1) return kOk;
  if (s.n > kMaxN || s.m > kMaxM || p.nvec > 65535) {
    set_error("two-mode SVD: basis sizes %d x %d exceed %d x %d or %d vectors exceed 65535", p.nr, p.nc, kMaxM,
              kMaxN, p.nvec);
    return kTooLarge;
  }
  const long long elems = (long long)s.m * s.n;
  dim3 fg((unsigned)((elems + 255) / 256), (unsigned)p.nvec);
  svd2_form_kernel<<<fg, 256, 0, st>>>(p);
  MLCP_CUDA_TRY(cudaGetLastError());
  const size_t smem = sizeof(double) * work_doubles(s);
  // static shared arrays of the kernel, with room for their alignment
  const size_t stat = sizeof(double) * (3 * kMaxN + kSvdWarps) + sizeof(int) * (kMaxN + 2) + 64;
  if (smem + stat <= (size_t)smem_optin) {
    static std::once_flag once;
    static cudaError_t attr_err = cudaSuccess;
    std::call_once(once, [&] {
      attr_err = cudaFuncSetAttribute(svd2_jacobi_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)(smem_optin - stat));
    });
    MLCP_CUDA_TRY(attr_err);
    svd2_jacobi_kernel<true><<<p.nvec, kSvdThreads, smem, st>>>(p);
  } else {
    svd2_jacobi_kernel<false><<<p.nvec, kSvdThreads, 0, st>>>(p);
  }
  MLCP_CUDA_TRY(cudaGetLastError());
  return kOk;
}

namespace {

// Batched reduc_SVD on host buffers: nvec vectors of rG terms each, reduced
// to at most rF terms.
int reduc_svd(Context* ctx, const double* base, const double* coef, const int* nbas, int rG, int nvec, int rF,
              double redtol, double* obase, double* ocoef, int* orank) {
  if (rG < 1 || nvec < 1 || rF < 1 || nbas[0] < 1 || nbas[1] < 1 || !(redtol >= 0.0)) {
    set_error("reducsvdcpp_: bad sizes (nbas=%d,%d rG=%d nvec=%d rF=%d redtol=%g)", nbas[0], nbas[1], rG, nvec, rF,
              redtol);
    return kBadArgument;
  }
  const int nr = nbas[0], nc = nbas[1], nD = nr + nc;
  const Shape s = shape_of(nr, nc);
  if (s.n > kMaxN || s.m > kMaxM || nvec > 65535) {
    set_error("reducsvdcpp_: basis sizes %d x %d exceed %d x %d or %d vectors exceed 65535", nr, nc, kMaxM, kMaxN,
              nvec);
    return kTooLarge;
  }
  size_t bytes = 0;
  auto take = [&](size_t b) { size_t o = align256(bytes); bytes = o + b; return o; };
  const size_t o_in = take(sizeof(double) * (size_t)nvec * rG * nD), o_ic = take(sizeof(double) * (size_t)nvec * rG),
               o_ob = take(sizeof(double) * (size_t)nvec * rF * nD), o_oc = take(sizeof(double) * (size_t)nvec * rF),
               o_rk = take(sizeof(int) * (size_t)nvec), o_st = take(sizeof(int) * (size_t)nvec),
               o_w = take(sizeof(double) * (size_t)nvec * work_doubles(s));
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
  Svd2Params p{};
  p.nvec = nvec;
  p.nr = nr;
  p.nc = nc;
  p.rout = rF;
  p.redtol = redtol;
  p.normalize = 0;
  p.K = rG;
  p.in_base = reinterpret_cast<const double*>(b + o_in);
  p.in_coef = reinterpret_cast<const double*>(b + o_ic);
  p.hv = 0;
  p.out_base = reinterpret_cast<double*>(b + o_ob);
  p.out_coef = reinterpret_cast<double*>(b + o_oc);
  p.out_rank = reinterpret_cast<int*>(b + o_rk);
  p.status = reinterpret_cast<int*>(b + o_st);
  p.work = reinterpret_cast<double*>(b + o_w);
  MLCP_CUDA_TRY(cudaMemcpyAsync(b + o_in, base, sizeof(double) * (size_t)nvec * rG * nD, cudaMemcpyHostToDevice, st));
  MLCP_CUDA_TRY(cudaMemcpyAsync(b + o_ic, coef, sizeof(double) * (size_t)nvec * rG, cudaMemcpyHostToDevice, st));
  MLCP_CUDA_TRY(cudaMemsetAsync(p.status, 0, sizeof(int) * nvec, st));
  int rc = svd2_launch(p, ctx->smem_optin, st);
  if (rc) return rc;
  std::vector<int> status(nvec);
  MLCP_CUDA_TRY(cudaMemcpyAsync(obase, p.out_base, sizeof(double) * (size_t)nvec * rF * nD, cudaMemcpyDeviceToHost, st));
  MLCP_CUDA_TRY(cudaMemcpyAsync(ocoef, p.out_coef, sizeof(double) * (size_t)nvec * rF, cudaMemcpyDeviceToHost, st));
  MLCP_CUDA_TRY(cudaMemcpyAsync(orank, p.out_rank, sizeof(int) * nvec, cudaMemcpyDeviceToHost, st));
  MLCP_CUDA_TRY(cudaMemcpyAsync(status.data(), p.status, sizeof(int) * nvec, cudaMemcpyDeviceToHost, st));
  MLCP_CUDA_TRY(cudaStreamSynchronize(st));
  for (int v = 0; v < nvec; ++v)
    if (status[v]) {
      set_error("reducsvdcpp_: the Jacobi sweeps of vector %d did not converge", v);
      return kNumerical;
    }
  return kOk;
}

}  // namespace

}  // namespace mlcp

extern "C" void reducsvdcpp_(double* base, double* coef, int* nbas, const int& rG, const int& nvec, const int& rF,
                             const double& redtol, double* obase, double* ocoef, int* orank) {
  int rc = mlcp::kOk;
  mlcp::Context* ctx = mlcp::get_context(&rc);
  if (ctx) {
    std::lock_guard<std::mutex> lk(ctx->mu);
    rc = mlcp::reduc_svd(ctx, base, coef, nbas, rG, nvec, rF, redtol, obase, ocoef, orank);
  }
  mlcp::finish_status(rc);
  if (rc != mlcp::kOk) fprintf(stderr, "reducsvdcpp_: %s\n", mlcp::last_error());
}
