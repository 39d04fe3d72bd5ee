// Block Rayleigh-Ritz step of the intertwined cycle (reference
// GenEigvalProblem, src/intertw_mvp.cu:589-654, and solve_geneigval,
// src/linalg.cu:22-69, cusolverDnDsygvd with itype 1, jobz V, lower).
//
//  * gep_inner_kernel: A(i,j) = <Q_j, (HQ)_i>, S(i,j) = <Q_j, Q_i> for j <= i,
//    full CP inner products in FP64 (one CTA per pair).
//  * gep_solve_kernel (one CTA): S = L L^T, C = L^-1 A L^-T in FP64;
//    eigenvectors of C by parallel cyclic Jacobi (round-robin ordering,
//    disjoint rotations per round), first in FP32 in shared memory, then
//    refined in FP64: the FP32 vectors V are orthonormalised (two
//    Newton-Schulz steps), C' = V^T C V is formed and FP64 Jacobi sweeps
//    diagonalise it (quadratic convergence from the FP32 start: two or three
//    sweeps), the rotations accumulating into V.  Eigenvalues are the
//    diagonal of C'.  The FP64 stage matters: the vector updates combine
//    the block with the eigenvectors, and for nearly degenerate states (the
//    benchmark block has relative gaps of 4e-5) FP32 eigenvectors are off
//    by ~1e-7 / gap, which moved the updated vectors by 1e-5 against the
//    reference's FP64 sygvd.  X = L^-T V with unit columns.  Eigenpairs are
//    returned in ascending order, each eigenvector with its largest-magnitude
//    entry positive.
#include <cfloat>

#include "common.cuh"
#include "intertwine.cuh"

namespace mlcp {

namespace {
constexpr int kPairThreads = 128;
constexpr int kSolveThreads = 1024;
}

__global__ void __launch_bounds__(kPairThreads) gep_inner_kernel(GepParams p) {
  // pair index -> (i, j), j <= i
  const int e = blockIdx.x;
  int i = (int)((sqrt(8.0 * e + 1.0) - 1.0) / 2.0);
  while ((i + 1) * (i + 2) / 2 <= e) ++i;
  while (i * (i + 1) / 2 > e) --i;
  const int j = e - i * (i + 1) / 2;
  const int R = p.R, D = p.D, nD = p.nD;
  const double* qj = p.q_base + (size_t)j * R * nD;
  const double* qjc = p.q_coef + (size_t)j * R;
  const double* qi = p.q_base + (size_t)i * R * nD;
  const double* qic = p.q_coef + (size_t)i * R;
  const double* hi = p.hq_base + (size_t)i * R * nD;
  const double* hic = p.hq_coef + (size_t)i * R;
  double accA = 0.0, accS = 0.0;
  for (int rs = threadIdx.x; rs < R * R; rs += blockDim.x) {
    const int r = rs / R, s = rs % R;
    double pa = qjc[r] * hic[s], ps = qjc[r] * qic[s];
    int o = 0;
    for (int d = 0; d < D; ++d) {
      const int n = p.nbas[d];
      double ta = 0.0, ts = 0.0;
      for (int q = 0; q < n; ++q) {
        const double x = qj[(size_t)r * nD + o + q];
        ta += x * hi[(size_t)s * nD + o + q];
        ts += x * qi[(size_t)s * nD + o + q];
      }
      pa *= ta;
      ps *= ts;
      o += n;
    }
    accA += pa;
    accS += ps;
  }
  __shared__ double ra[kPairThreads], rs_[kPairThreads];
  ra[threadIdx.x] = accA;
  rs_[threadIdx.x] = accS;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      ra[threadIdx.x] += ra[threadIdx.x + w];
      rs_[threadIdx.x] += rs_[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    p.A[i + (size_t)j * p.nbloc] = ra[0];
    p.S[i + (size_t)j * p.nbloc] = rs_[0];
  }
}

// Rotation (c, s) zeroing the (p,q) entry of a symmetric 2x2 block.
__device__ inline void jacobi_rotation(float app, float aqq, float apq, float* c, float* s) {
  if (apq == 0.f) {
    *c = 1.f;
    *s = 0.f;
    return;
  }
  const float theta = (aqq - app) / (2.f * apq);
  const float t = copysignf(1.f, theta) / (fabsf(theta) + sqrtf(theta * theta + 1.f));
  *c = rsqrtf(t * t + 1.f);
  *s = t * *c;
}

__global__ void __launch_bounds__(kSolveThreads) gep_solve_kernel(GepParams p) {
  const int B = p.nbloc;
  const int Bp = (B + 1) / 2 * 2;  // even size for the round-robin schedule (padding index is inert)
  const int tid = threadIdx.x, nt = blockDim.x;
  double* L = p.work;                        // [B][B] Cholesky factor (lower)
  double* C = L + (size_t)B * B;             // [B][B]
  double* Wm = C + (size_t)B * B;            // [B][B]
  double* lam = Wm + (size_t)B * B;          // [B]
  double* invd = lam + B;                    // [B]
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float* Cf = reinterpret_cast<float*>(smem_raw);  // [Bp][Bp]
  float* Vf = Cf + (size_t)Bp * Bp;                // [Bp][Bp]
  float* rc = Vf + (size_t)Bp * Bp;                // [Bp/2] cosines
  float* rs = rc + Bp / 2;                         // [Bp/2] sines
  int* pq = reinterpret_cast<int*>(rs + Bp / 2);   // [Bp] pair members
  __shared__ double red[32];
  __shared__ int info;

  // ---- S = L L^T (lower triangle of S) ----
  for (int e = tid; e < B * B; e += nt) {
    const int r = e % B, c = e / B;
    L[e] = (r >= c) ? p.S[e] : 0.0;
  }
  if (tid == 0) info = 0;
  __syncthreads();
  for (int j = 0; j < B; ++j) {
    if (tid == 0) {
      double d = L[j + (size_t)j * B];
      if (!(d > 0.0)) { info = j + 1; d = fabs(d) + 1e-300; }
      const double l = sqrt(d);
      L[j + (size_t)j * B] = l;
      invd[j] = 1.0 / l;
    }
    __syncthreads();
    const double inv = invd[j];
    for (int i = j + 1 + tid; i < B; i += nt) L[i + (size_t)j * B] *= inv;
    __syncthreads();
    const int m = B - j - 1;
    for (int e = tid; e < m * m; e += nt) {
      const int c = j + 1 + e / m, i = j + 1 + e % m;
      if (i >= c) L[i + (size_t)c * B] -= L[i + (size_t)j * B] * L[c + (size_t)j * B];
    }
    __syncthreads();
  }
  // ---- C = L^-1 A L^-T (A symmetric from its lower triangle) ----
  for (int e = tid; e < B * B; e += nt) {
    const int r = e % B, c = e / B;
    C[e] = (r >= c) ? p.A[e] : p.A[c + (size_t)r * B];
  }
  __syncthreads();
  for (int j = 0; j < B; ++j) {  // C <- L^-1 C (rows)
    for (int c = tid; c < B; c += nt) C[j + (size_t)c * B] *= invd[j];
    __syncthreads();
    for (int e = tid; e < (B - j - 1) * B; e += nt) {
      const int i = j + 1 + e % (B - j - 1), c = e / (B - j - 1);
      C[i + (size_t)c * B] -= L[i + (size_t)j * B] * C[j + (size_t)c * B];
    }
    __syncthreads();
  }
  for (int j = 0; j < B; ++j) {  // C <- C L^-T (columns)
    for (int r = tid; r < B; r += nt) C[r + (size_t)j * B] *= invd[j];
    __syncthreads();
    for (int e = tid; e < (B - j - 1) * B; e += nt) {
      const int c = j + 1 + e / B, r = e % B;
      C[r + (size_t)c * B] -= C[r + (size_t)j * B] * L[c + (size_t)j * B];
    }
    __syncthreads();
  }
  // ---- FP32 cyclic Jacobi (round-robin) ----
  for (int e = tid; e < Bp * Bp; e += nt) {
    const int r = e % Bp, c = e / Bp;
    const bool in = r < B && c < B;
    Cf[e] = in ? (float)(0.5 * (C[r + (size_t)c * B] + C[c + (size_t)r * B])) : 0.f;
    Vf[e] = (r == c) ? 1.f : 0.f;
  }
  __syncthreads();
  const int npairs = Bp / 2;
  for (int sweep = 0; sweep < 30; ++sweep) {
    // convergence: off-diagonal mass relative to the diagonal
    double off = 0.0, dia = 0.0;
    for (int e = tid; e < Bp * Bp; e += nt) {
      const double v = Cf[e];
      if (e % Bp == e / Bp) dia += v * v; else off += v * v;
    }
    for (int o = 16; o > 0; o >>= 1) {
      off += __shfl_xor_sync(0xffffffffu, off, o);
      dia += __shfl_xor_sync(0xffffffffu, dia, o);
    }
    __syncthreads();
    if (tid % 32 == 0) red[tid / 32] = off;
    __syncthreads();
    double offt = 0.0;
    for (int w = 0; w < nt / 32; ++w) offt += red[w];
    __syncthreads();
    if (tid % 32 == 0) red[tid / 32] = dia;
    __syncthreads();
    double diat = 0.0;
    for (int w = 0; w < nt / 32; ++w) diat += red[w];
    __syncthreads();
    if (offt <= 1e-12 * diat || offt == 0.0) break;
    for (int round = 0; round < Bp - 1; ++round) {
      // pair k: (Bp-1, round) for k = 0, else ((round+k) mod (Bp-1), (round-k) mod (Bp-1))
      for (int k = tid; k < npairs; k += nt) {
        int a, b;
        if (k == 0) {
          a = Bp - 1;
          b = round;
        } else {
          a = (round + k) % (Bp - 1);
          b = (round - k + (Bp - 1)) % (Bp - 1);
        }
        if (a > b) { const int t = a; a = b; b = t; }
        pq[2 * k] = a;
        pq[2 * k + 1] = b;
        jacobi_rotation(Cf[a + (size_t)a * Bp], Cf[b + (size_t)b * Bp], Cf[a + (size_t)b * Bp], &rc[k], &rs[k]);
      }
      __syncthreads();
      // rows: C <- J^T C
      for (int e = tid; e < npairs * Bp; e += nt) {
        const int k = e / Bp, col = e % Bp;
        const int a = pq[2 * k], b = pq[2 * k + 1];
        const float c = rc[k], s = rs[k];
        const float xa = Cf[a + (size_t)col * Bp], xb = Cf[b + (size_t)col * Bp];
        Cf[a + (size_t)col * Bp] = c * xa - s * xb;
        Cf[b + (size_t)col * Bp] = s * xa + c * xb;
      }
      __syncthreads();
      // columns: C <- C J, V <- V J
      for (int e = tid; e < npairs * Bp; e += nt) {
        const int k = e / Bp, row = e % Bp;
        const int a = pq[2 * k], b = pq[2 * k + 1];
        const float c = rc[k], s = rs[k];
        const float xa = Cf[row + (size_t)a * Bp], xb = Cf[row + (size_t)b * Bp];
        Cf[row + (size_t)a * Bp] = c * xa - s * xb;
        Cf[row + (size_t)b * Bp] = s * xa + c * xb;
        const float va = Vf[row + (size_t)a * Bp], vb = Vf[row + (size_t)b * Bp];
        Vf[row + (size_t)a * Bp] = c * va - s * vb;
        Vf[row + (size_t)b * Bp] = s * va + c * vb;
      }
      __syncthreads();
    }
  }
  // ---- FP64 refinement of the eigenvectors ----
  double* V = invd + B;              // [B][B] FP64 eigenvectors (columns)
  double* C2 = V + (size_t)B * B;    // [B][B] V^T C V, diagonalised in place
  for (int e = tid; e < B * B; e += nt) {
    const int r = e % B, c = e / B;
    V[e] = (double)Vf[r + (size_t)c * Bp];
  }
  __syncthreads();
  for (int ns = 0; ns < 2; ++ns) {  // V <- V (3 I - V^T V) / 2
    for (int e = tid; e < B * B; e += nt) {  // Wm = V^T V
      const int r = e % B, c = e / B;
      double acc = 0.0;
      for (int k = 0; k < B; ++k) acc += V[k + (size_t)r * B] * V[k + (size_t)c * B];
      Wm[e] = acc;
    }
    __syncthreads();
    for (int e = tid; e < B * B; e += nt) {  // C2 = V (1.5 I - 0.5 Wm)
      const int r = e % B, c = e / B;
      double acc = 1.5 * V[r + (size_t)c * B];
      for (int k = 0; k < B; ++k) acc -= 0.5 * V[r + (size_t)k * B] * Wm[k + (size_t)c * B];
      C2[e] = acc;
    }
    __syncthreads();
    for (int e = tid; e < B * B; e += nt) V[e] = C2[e];
    __syncthreads();
  }
  for (int e = tid; e < B * B; e += nt) {  // Wm = C V
    const int r = e % B, c = e / B;
    double acc = 0.0;
    for (int k = 0; k < B; ++k) acc += C[r + (size_t)k * B] * V[k + (size_t)c * B];
    Wm[e] = acc;
  }
  __syncthreads();
  for (int e = tid; e < B * B; e += nt) {  // C2 = V^T C V, symmetrised
    const int r = e % B, c = e / B;
    double a1 = 0.0, a2 = 0.0;
    for (int k = 0; k < B; ++k) {
      a1 += V[k + (size_t)r * B] * Wm[k + (size_t)c * B];
      a2 += V[k + (size_t)c * B] * Wm[k + (size_t)r * B];
    }
    C2[e] = 0.5 * (a1 + a2);
  }
  __syncthreads();
  const int npB = B / 2;  // pairs of the odd index padding are skipped below
  for (int sweep = 0; sweep < 12; ++sweep) {
    double off = 0.0, dia = 0.0;
    for (int e = tid; e < B * B; e += nt) {
      const double v = C2[e];
      if (e % B == e / B) dia += v * v; else off += v * v;
    }
    for (int o = 16; o > 0; o >>= 1) {
      off += __shfl_xor_sync(0xffffffffu, off, o);
      dia += __shfl_xor_sync(0xffffffffu, dia, o);
    }
    __syncthreads();
    if (tid % 32 == 0) red[tid / 32] = off;
    __syncthreads();
    double offt = 0.0;
    for (int w = 0; w < nt / 32; ++w) offt += red[w];
    __syncthreads();
    if (tid % 32 == 0) red[tid / 32] = dia;
    __syncthreads();
    double diat = 0.0;
    for (int w = 0; w < nt / 32; ++w) diat += red[w];
    __syncthreads();
    if (offt <= 1e-30 * diat || offt == 0.0) break;
    (void)npB;
    for (int round = 0; round < Bp - 1; ++round) {
      double* rcd = Wm;           // [Bp/2] cosines (Wm is free until the back substitution)
      double* rsd = Wm + Bp / 2;  // [Bp/2] sines
      for (int k = tid; k < npairs; k += nt) {
        int a, b;
        if (k == 0) {
          a = Bp - 1;
          b = round;
        } else {
          a = (round + k) % (Bp - 1);
          b = (round - k + (Bp - 1)) % (Bp - 1);
        }
        if (a > b) { const int t = a; a = b; b = t; }
        pq[2 * k] = a;
        pq[2 * k + 1] = b;
        double c = 1.0, sn = 0.0;
        if (b < B) {  // index Bp - 1 = B is padding when B is odd
          const double app = C2[a + (size_t)a * B], aqq = C2[b + (size_t)b * B], apq = C2[a + (size_t)b * B];
          if (apq != 0.0) {
            const double theta = (aqq - app) / (2.0 * apq);
            const double t = copysign(1.0, theta) / (fabs(theta) + sqrt(theta * theta + 1.0));
            c = 1.0 / sqrt(t * t + 1.0);
            sn = t * c;
          }
        }
        rcd[k] = c;
        rsd[k] = sn;
      }
      __syncthreads();
      for (int e = tid; e < npairs * B; e += nt) {  // rows: C2 <- J^T C2
        const int k = e / B, col = e % B;
        const int a = pq[2 * k], b = pq[2 * k + 1];
        if (b >= B) continue;
        const double c = rcd[k], sn = rsd[k];
        const double xa = C2[a + (size_t)col * B], xb = C2[b + (size_t)col * B];
        C2[a + (size_t)col * B] = c * xa - sn * xb;
        C2[b + (size_t)col * B] = sn * xa + c * xb;
      }
      __syncthreads();
      for (int e = tid; e < npairs * B; e += nt) {  // columns: C2 <- C2 J, V <- V J
        const int k = e / B, row = e % B;
        const int a = pq[2 * k], b = pq[2 * k + 1];
        if (b >= B) continue;
        const double c = rcd[k], sn = rsd[k];
        const double xa = C2[row + (size_t)a * B], xb = C2[row + (size_t)b * B];
        C2[row + (size_t)a * B] = c * xa - sn * xb;
        C2[row + (size_t)b * B] = sn * xa + c * xb;
        const double va = V[row + (size_t)a * B], vb = V[row + (size_t)b * B];
        V[row + (size_t)a * B] = c * va - sn * vb;
        V[row + (size_t)b * B] = sn * va + c * vb;
      }
      __syncthreads();
    }
  }
  for (int c = tid; c < B; c += nt) {
    double den = 0.0;
    for (int k = 0; k < B; ++k) den += V[k + (size_t)c * B] * V[k + (size_t)c * B];
    lam[c] = C2[c + (size_t)c * B];
    invd[c] = 1.0 / sqrt(den);  // reuse: column scale
  }
  __syncthreads();
  // X = L^-T V (back substitution per column, columns in parallel through rows)
  for (int e = tid; e < B * B; e += nt) {
    const int r = e % B, c = e / B;
    Wm[e] = V[r + (size_t)c * B] * invd[c];
  }
  __syncthreads();
  for (int jr = B - 1; jr >= 0; --jr) {
    for (int c = tid; c < B; c += nt) Wm[jr + (size_t)c * B] /= L[jr + (size_t)jr * B];
    __syncthreads();
    for (int e = tid; e < jr * B; e += nt) {
      const int i = e % jr, c = e / jr;
      Wm[i + (size_t)c * B] -= L[jr + (size_t)i * B] * Wm[jr + (size_t)c * B];
    }
    __syncthreads();
  }
  // ---- ascending order, sign convention, output ----
  if (tid == 0) {
    for (int k = 0; k < B; ++k) pq[k] = k;
    for (int a = 0; a < B; ++a) {  // selection sort (B <= a few hundred)
      int m = a;
      for (int b = a + 1; b < B; ++b)
        if (lam[pq[b]] < lam[pq[m]]) m = b;
      const int t = pq[a]; pq[a] = pq[m]; pq[m] = t;
    }
  }
  __syncthreads();
  for (int c = tid; c < B; c += nt) {
    const int src = pq[c];
    int imax = 0;
    double amax = -1.0;
    for (int r = 0; r < B; ++r) {
      const double a = fabs(Wm[r + (size_t)src * B]);
      if (a > amax) { amax = a; imax = r; }
    }
    const double sg = (Wm[imax + (size_t)src * B] < 0.0) ? -1.0 : 1.0;
    for (int r = 0; r < B; ++r) p.U[r + (size_t)c * B] = sg * Wm[r + (size_t)src * B];
    p.eigv[c] = lam[src];
  }
  if (tid == 0 && info) atomicOr(p.status, 2);
}

size_t gep_work_doubles(int nbloc) { return (size_t)5 * nbloc * nbloc + 2 * nbloc; }

int gep_launch(const GepParams& p, cudaStream_t st) {
  const int B = p.nbloc;
  const int npairs = B * (B + 1) / 2;
  gep_inner_kernel<<<npairs, kPairThreads, 0, st>>>(p);
  MLCP_CUDA_TRY(cudaGetLastError());
  return gep_solve_launch(p, st);
}

int gep_solve_launch(const GepParams& p, cudaStream_t st) {
  const int B = p.nbloc;
  const int Bp = (B + 1) / 2 * 2;
  const size_t smem = sizeof(float) * ((size_t)2 * Bp * Bp + Bp) + sizeof(int) * Bp + 64;
  MLCP_CUDA_TRY(cudaFuncSetAttribute(gep_solve_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  gep_solve_kernel<<<1, kSolveThreads, smem, st>>>(p);
  MLCP_CUDA_TRY(cudaGetLastError());
  return kOk;
}

// ---------------------------------------------------------------------------
// Weight normalisation: coef /= sqrt(|<F,F>|) for each rank-R vector.
// ---------------------------------------------------------------------------

__global__ void normalize_coefs_kernel(int R, int D, int nD, const int* nbas, const double* base, double* coef) {
  const int v = blockIdx.x;
  const double* b = base + (size_t)v * R * nD;
  double* c = coef + (size_t)v * R;
  double acc = 0.0;
  for (int e = threadIdx.x; e < R * R; e += blockDim.x) {
    const int i = e % R, k = e / R;
    double prod = c[i] * c[k];
    int o = 0;
    for (int d = 0; d < D; ++d) {
      double t = 0.0;
      for (int q = 0; q < nbas[d]; ++q) t += b[(size_t)i * nD + o + q] * b[(size_t)k * nD + o + q];
      prod *= t;
      o += nbas[d];
    }
    acc += prod;
  }
  __shared__ double red[256];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  const double q = sqrt(fabs(red[0]));
  __syncthreads();
  for (int i = threadIdx.x; i < R; i += blockDim.x) c[i] /= q;
}

int normalize_coefs_launch(int nvec, int R, int D, int nD, const int* nbas, const double* base, double* coef,
                           cudaStream_t st) {
  normalize_coefs_kernel<<<nvec, 256, 0, st>>>(R, D, nD, nbas, base, coef);
  MLCP_CUDA_TRY(cudaGetLastError());
  return kOk;
}

}  // namespace mlcp
