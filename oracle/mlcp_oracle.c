/*
 * CPU oracle for the MLCP GPU power-iteration hot path (TEST INFRASTRUCTURE).
 *
 * Only tests/, the smoke entry and bench.py's CPU-baseline leg call this code,
 * as the checker.  It restates the reference's CUDA algorithm in FP64 C, the
 * Fortran host's CPU ALS reduction (reduc_ALS) and the Fortran host's CPU
 * power solver (solver pals: ALS_POW3, ALS_ORTHO_2, PRODHV_ALS2,
 * ALS_SUMLCVEC_2); each function names the reference file:line it follows.
 * The reference has no golden data for this path; the restatement of the
 * CUDA algorithm is pinned against the reference's own FP64 CUDA library,
 * built from its sources and run on the GPU (ALS to 1e-12, one power cycle
 * to 1e-8 relative), and the Fortran twins agree with it stage by stage to
 * rounding where the two algorithms coincide.
 *
 * Built with -ffp-contract=off so that x86 and Arm hosts give identical bits.
 */
#include "mlcp_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------ */
/* CP-vector views                                                      */
/* ------------------------------------------------------------------ */

typedef struct {
  int nrk;           /* number of terms */
  int ndof;          /* number of modes */
  int nD;            /* sum of basis sizes */
  const int *nbas;   /* basis size per mode */
  const int *off;    /* mode offsets, off[ndof] == nD */
  double *coef;      /* nrk weights */
  double *base;      /* nrk * nD factors */
} cpv;

/* Reference src/cpvector.cu:291 (PointCPvecRtermsonGPU): a window of R terms. */
static cpv cp_window(const cpv *v, int iR, int R) {
  cpv w = *v;
  w.nrk = R;
  w.coef = v->coef + iR;
  w.base = v->base + (size_t)iR * v->nD;
  return w;
}

static int *make_offsets(const int *nbas, int ndof) {
  int *off = (int *)malloc(sizeof(int) * (ndof + 1));
  off[0] = 0;
  for (int d = 0; d < ndof; ++d) off[d + 1] = off[d] + nbas[d];
  return off;
}

/* ------------------------------------------------------------------ */
/* Inner-product building blocks (reference src/modvecvec.cu)          */
/* ------------------------------------------------------------------ */

/* constpstot (src/modvecvec.cu:724): PS(i1,i2) = [cv][cw] prod_{d != idof}
 * <v_i1^d, w_i2^d>, column-major with leading dimension v->nrk. */
static void pstot(const cpv *v, const cpv *w, double *PS, int idof, int multv, int multw) {
  for (int i2 = 0; i2 < w->nrk; ++i2) {
    for (int i1 = 0; i1 < v->nrk; ++i1) {
      const double *a = v->base + (size_t)i1 * v->nD;
      const double *b = w->base + (size_t)i2 * w->nD;
      double normND = 1.0;
      if (multv) normND *= v->coef[i1];
      if (multw) normND *= w->coef[i2];
      int s = 0;
      for (int d = 0; d < v->ndof; ++d) {
        int n = v->nbas[d];
        if (d != idof) {
          double norm1D = 0.0;
          for (int k = 0; k < n; ++k) norm1D += a[s + k] * b[s + k];
          normND *= norm1D;
        }
        s += n;
      }
      PS[i1 + (size_t)i2 * v->nrk] = normND;
    }
  }
}

/* constpsk with reset (src/modvecvec.cu:360): PS(i1,i2) = <v_i1^k, w_i2^k>. */
static void psk(const cpv *v, const cpv *w, double *PS, int k) {
  int n = v->nbas[k], o = v->off[k];
  for (int i2 = 0; i2 < w->nrk; ++i2)
    for (int i1 = 0; i1 < v->nrk; ++i1) {
      const double *a = v->base + (size_t)i1 * v->nD + o;
      const double *b = w->base + (size_t)i2 * w->nD + o;
      double t = 0.0;
      for (int j = 0; j < n; ++j) t += a[j] * b[j];
      PS[i1 + (size_t)i2 * v->nrk] = t;
    }
}

/* Sum of all entries in row-then-array order: sumoverrow (src/modvecvec.cu:1154)
 * followed by sumarray (:1193). */
static double sum_all(const double *M, int nr, int nc) {
  double total = 0.0;
  for (int r = 0; r < nr; ++r) {
    double row = 0.0;
    for (int c = 0; c < nc; ++c) row += M[r + (size_t)c * nr];
    total += row;
  }
  return total;
}

/* constbjk (src/als.cu:332 and :361): bjk(i1,i2) += fac * sum_j w.coef[j]
 * w_j^k(i2) PS(j,i1); bjk is column-major rk x n_k, PS has leading dim w->nrk. */
static void bjk_accumulate(const cpv *w, const double *PS, double *bjk, int rkv, int k, const double *fac) {
  int n = w->nbas[k], o = w->off[k];
  for (int i2 = 0; i2 < n; ++i2)
    for (int i1 = 0; i1 < rkv; ++i1) {
      double t = 0.0;
      if (!fac) t = bjk[i1 + (size_t)i2 * rkv];
      for (int j = 0; j < w->nrk; ++j)
        t += w->coef[j] * w->base[(size_t)j * w->nD + o + i2] * PS[j + (size_t)i1 * w->nrk];
      if (fac) t = fac[0] * t + bjk[i1 + (size_t)i2 * rkv];
      bjk[i1 + (size_t)i2 * rkv] = t;
    }
}

/* normonebase (src/modvecvec.cu:225): max-scaled 2-norm of mode idof of each
 * term; the factor is divided by it and the weight replaced by it. */
static void normonebase(cpv *v, int idof) {
  int n = v->nbas[idof], o = v->off[idof];
  for (int r = 0; r < v->nrk; ++r) {
    double *x = v->base + (size_t)r * v->nD + o;
    double largest = 0.0;
    for (int k = 0; k < n; ++k) largest = (largest > fabs(x[k])) ? largest : fabs(x[k]);
    double norm1D = 0.0;
    for (int k = 0; k < n; ++k) {
      double t = x[k] / largest;
      norm1D += t * t;
    }
    norm1D = largest * sqrt(fabs(norm1D));
    for (int k = 0; k < n; ++k) x[k] /= norm1D;
    v->coef[r] = norm1D;
  }
}

/* Coefficient renormalisation used after sweeps: constpstot(F,F,-1,T,T),
 * sumoverrow, sumarray, normalizecoef (src/intertw_mvp.cu:491-494). */
static void normalize_coefs(cpv *F, double *BB) {
  pstot(F, F, BB, -1, 1, 1);
  double s = sum_all(BB, F->nrk, F->nrk);
  double q = sqrt(fabs(s));
  for (int r = 0; r < F->nrk; ++r) F->coef[r] /= q;
}

/* setpenalty (src/als.cu:248): the largest weight times 1e-10 in the FP64
 * build or 1e-5 in the FP32 build.  The factor is selectable per stage of the
 * cycle (orc_set_cycle_penalties); every stage defaults to the FP64 rule. */
static double g_pen_als = 1.0e-10, g_pen_mvp = 1.0e-10, g_pen_gs = 1.0e-10, g_pen_upd = 1.0e-10;
void orc_set_penalty_factor(double f) { g_pen_als = g_pen_mvp = g_pen_gs = g_pen_upd = f; }
void orc_set_cycle_penalties(double mvp, double gs, double upd) {
  g_pen_mvp = mvp;
  g_pen_gs = gs;
  g_pen_upd = upd;
}
static double penalty_f(const double *coef, int n, double factor) {
  double p = coef[0];
  for (int i = 1; i < n; ++i) p = (coef[i] > p) ? coef[i] : p;
  return p * factor;
}

/* ------------------------------------------------------------------ */
/* Dense solves                                                        */
/* ------------------------------------------------------------------ */

/* solve_linsys (src/linalg.cu:73): LU with partial pivoting of the n x n
 * column-major A (dgetrf), then forward/back substitution for nrhs columns
 * of B (dgetrs, no transpose).  A and B are overwritten. */
static void lu_solve(double *A, double *B, int n, int nrhs, int *ipiv) {
  for (int j = 0; j < n; ++j) {
    int p = j;
    double amax = fabs(A[j + (size_t)j * n]);
    for (int i = j + 1; i < n; ++i) {
      double a = fabs(A[i + (size_t)j * n]);
      if (a > amax) { amax = a; p = i; }
    }
    ipiv[j] = p;
    if (p != j)
      for (int c = 0; c < n; ++c) {
        double t = A[j + (size_t)c * n]; A[j + (size_t)c * n] = A[p + (size_t)c * n]; A[p + (size_t)c * n] = t;
      }
    double piv = A[j + (size_t)j * n];
    if (piv != 0.0)
      for (int i = j + 1; i < n; ++i) A[i + (size_t)j * n] /= piv;
    for (int c = j + 1; c < n; ++c) {
      double u = A[j + (size_t)c * n];
      for (int i = j + 1; i < n; ++i) A[i + (size_t)c * n] -= A[i + (size_t)j * n] * u;
    }
  }
  for (int c = 0; c < nrhs; ++c) {
    double *b = B + (size_t)c * n;
    for (int j = 0; j < n; ++j)
      if (ipiv[j] != j) { double t = b[j]; b[j] = b[ipiv[j]]; b[ipiv[j]] = t; }
    for (int j = 0; j < n; ++j)
      for (int i = j + 1; i < n; ++i) b[i] -= A[i + (size_t)j * n] * b[j];
    for (int j = n - 1; j >= 0; --j) {
      b[j] /= A[j + (size_t)j * n];
      for (int i = 0; i < j; ++i) b[i] -= A[i + (size_t)j * n] * b[j];
    }
  }
}

/* Cyclic Jacobi eigen-decomposition of the symmetric n x n column-major C
 * (overwritten); eigenvalues to w, eigenvectors (columns) to V. */
static void jacobi_eig(double *C, int n, double *w, double *V) {
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) V[i + (size_t)j * n] = (i == j) ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0, diag = 0.0;
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        double c = C[i + (size_t)j * n];
        if (i != j) off += c * c; else diag += c * c;
      }
    if (off <= 1e-30 * diag || off == 0.0) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        double apq = C[p + (size_t)q * n];
        if (apq == 0.0) continue;
        double app = C[p + (size_t)p * n], aqq = C[q + (size_t)q * n];
        double theta = (aqq - app) / (2.0 * apq);
        double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; ++k) { /* columns p,q */
          double ckp = C[k + (size_t)p * n], ckq = C[k + (size_t)q * n];
          C[k + (size_t)p * n] = c * ckp - s * ckq;
          C[k + (size_t)q * n] = s * ckp + c * ckq;
        }
        for (int k = 0; k < n; ++k) { /* rows p,q */
          double cpk = C[p + (size_t)k * n], cqk = C[q + (size_t)k * n];
          C[p + (size_t)k * n] = c * cpk - s * cqk;
          C[q + (size_t)k * n] = s * cpk + c * cqk;
        }
        for (int k = 0; k < n; ++k) {
          double vkp = V[k + (size_t)p * n], vkq = V[k + (size_t)q * n];
          V[k + (size_t)p * n] = c * vkp - s * vkq;
          V[k + (size_t)q * n] = s * vkp + c * vkq;
        }
      }
  }
  for (int i = 0; i < n; ++i) w[i] = C[i + (size_t)i * n];
}

/* solve_geneigval (src/linalg.cu:22, cusolverDnDsygvd itype=1, jobz=V,
 * uplo=L): B = L L^T, C = L^-1 A L^-T, C = Y diag(w) Y^T, X = L^-T Y. */
int orc_sygv(int n, const double *A, const double *B, double *w, double *X) {
  double *L = (double *)calloc((size_t)n * n, sizeof(double));
  double *C = (double *)calloc((size_t)n * n, sizeof(double));
  double *Y = (double *)calloc((size_t)n * n, sizeof(double));
  double *wt = (double *)malloc(sizeof(double) * n);
  int info = 0;
  for (int j = 0; j < n; ++j) { /* Cholesky of the lower triangle of B */
    double s = B[j + (size_t)j * n];
    for (int k = 0; k < j; ++k) s -= L[j + (size_t)k * n] * L[j + (size_t)k * n];
    if (!(s > 0.0)) { info = j + 1; s = fabs(s) + 1e-300; }
    double ljj = sqrt(s);
    L[j + (size_t)j * n] = ljj;
    for (int i = j + 1; i < n; ++i) {
      double t = B[i + (size_t)j * n];
      for (int k = 0; k < j; ++k) t -= L[i + (size_t)k * n] * L[j + (size_t)k * n];
      L[i + (size_t)j * n] = t / ljj;
    }
  }
  /* symmetric A from its lower triangle */
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) C[i + (size_t)j * n] = (i >= j) ? A[i + (size_t)j * n] : A[j + (size_t)i * n];
  /* C <- L^-1 C (forward substitution on each column) */
  for (int c = 0; c < n; ++c)
    for (int i = 0; i < n; ++i) {
      double t = C[i + (size_t)c * n];
      for (int k = 0; k < i; ++k) t -= L[i + (size_t)k * n] * C[k + (size_t)c * n];
      C[i + (size_t)c * n] = t / L[i + (size_t)i * n];
    }
  /* C <- C L^-T (forward substitution on each row) */
  for (int r = 0; r < n; ++r)
    for (int j = 0; j < n; ++j) {
      double t = C[r + (size_t)j * n];
      for (int k = 0; k < j; ++k) t -= C[r + (size_t)k * n] * L[j + (size_t)k * n];
      C[r + (size_t)j * n] = t / L[j + (size_t)j * n];
    }
  for (int j = 0; j < n; ++j) /* symmetrise rounding */
    for (int i = j + 1; i < n; ++i) {
      double a = 0.5 * (C[i + (size_t)j * n] + C[j + (size_t)i * n]);
      C[i + (size_t)j * n] = a; C[j + (size_t)i * n] = a;
    }
  jacobi_eig(C, n, wt, Y);
  /* X = L^-T Y (back substitution on each column) */
  double *Xt = (double *)malloc(sizeof(double) * (size_t)n * n);
  for (int c = 0; c < n; ++c)
    for (int i = n - 1; i >= 0; --i) {
      double t = Y[i + (size_t)c * n];
      for (int k = i + 1; k < n; ++k) t -= L[k + (size_t)i * n] * Xt[k + (size_t)c * n];
      Xt[i + (size_t)c * n] = t / L[i + (size_t)i * n];
    }
  /* ascending order (stable selection), then sign normalisation */
  int *idx = (int *)malloc(sizeof(int) * n);
  for (int i = 0; i < n; ++i) idx[i] = i;
  for (int i = 0; i < n; ++i) {
    int m = i;
    for (int j = i + 1; j < n; ++j)
      if (wt[idx[j]] < wt[idx[m]]) m = j;
    int t = idx[i]; idx[i] = idx[m]; idx[m] = t;
  }
  for (int c = 0; c < n; ++c) {
    int src = idx[c];
    w[c] = wt[src];
    int imax = 0;
    double amax = -1.0;
    for (int i = 0; i < n; ++i) {
      double a = fabs(Xt[i + (size_t)src * n]);
      if (a > amax) { amax = a; imax = i; }
    }
    double sg = (Xt[imax + (size_t)src * n] < 0.0) ? -1.0 : 1.0;
    for (int i = 0; i < n; ++i) X[i + (size_t)c * n] = sg * Xt[i + (size_t)src * n];
  }
  free(idx); free(Xt); free(L); free(C); free(Y); free(wt);
  return info;
}

/* ------------------------------------------------------------------ */
/* Explicit-G ALS (reference src/als.cu:976-1078)                      */
/* ------------------------------------------------------------------ */

typedef struct {
  int rk, nmax;
  double *BB, *BBk, *bjk, *tmp;
  int *ipiv;
} work_t;

static void work_init(work_t *w, int rk, int nmax, int nblocmax) {
  w->rk = rk; w->nmax = nmax;
  int m = rk > nblocmax ? rk : nblocmax;
  w->BB = (double *)malloc(sizeof(double) * (size_t)rk * rk);
  w->BBk = (double *)malloc(sizeof(double) * (size_t)rk * rk);
  w->bjk = (double *)malloc(sizeof(double) * (size_t)rk * nmax);
  w->tmp = (double *)malloc(sizeof(double) * (size_t)m);
  w->ipiv = (int *)malloc(sizeof(int) * rk);
}
static void work_free(work_t *w) { free(w->BB); free(w->BBk); free(w->bjk); free(w->tmp); free(w->ipiv); }

/* Test knob (no counterpart in the reference): when set, each ALS
 * right-hand side is rounded to FP32 before the solve, to measure how far an
 * FP64 ALS trajectory moves under FP32-level noise in b. */
static int g_rhs_fp32 = 0;
void orc_set_rhs_fp32(int on) { g_rhs_fp32 = on; }

static void add_penalty(double *BB, int rk, double pen) {
  for (int i = 0; i < rk; ++i) BB[i + (size_t)i * rk] += pen;
}

/* replacevwithsolns (src/als.cu:310): F^idof(r,:) = X(r,:). */
static void replace_with_solution(cpv *F, const double *X, int idof) {
  int n = F->nbas[idof], o = F->off[idof];
  for (int r = 0; r < F->nrk; ++r)
    for (int i = 0; i < n; ++i) F->base[(size_t)r * F->nD + o + i] = X[r + (size_t)i * F->nrk];
}

/* ITERATE_ALS (src/als.cu:1021) with als_build_linear_system (:976). */
static void iterate_als(cpv *Q, int rk, int nbloc, int nals, work_t *W) {
  if (nals == 0) return;
  cpv F = cp_window(Q, 0, rk);
  double pen = penalty_f(F.coef, rk, g_pen_als);
  for (int it = 0; it < nals; ++it)
    for (int j = 0; j < Q->ndof; ++j) {
      int n = Q->nbas[j];
      memset(W->bjk, 0, sizeof(double) * (size_t)rk * n);
      for (int k = 1; k < nbloc; ++k) {
        cpv G = cp_window(Q, k * rk, rk);
        pstot(&G, &F, W->BB, j, 0, 0);
        bjk_accumulate(&G, W->BB, W->bjk, rk, j, NULL);
      }
      pstot(&F, &F, W->BB, j, 0, 0);
      add_penalty(W->BB, rk, pen);
      if (g_rhs_fp32)
        for (int e = 0; e < rk * n; ++e) W->bjk[e] = (double)(float)W->bjk[e];
      lu_solve(W->BB, W->bjk, rk, n, W->ipiv);
      replace_with_solution(&F, W->bjk, j);
      normonebase(&F, j);
    }
}

static int max_nbas(const int *nbas, int ndof) {
  int m = 0;
  for (int d = 0; d < ndof; ++d) m = nbas[d] > m ? nbas[d] : m;
  return m;
}

void orc_alscpp(double *coef, double *base, const int *nbas, int ndof, int rF, int rG, int nals) {
  int *off = make_offsets(nbas, ndof);
  cpv Q = {rF + rG, ndof, off[ndof], nbas, off, coef, base};
  work_t W;
  work_init(&W, rF, max_nbas(nbas, ndof), 1);
  iterate_als(&Q, rF, (rF + rG) / rF, nals, &W);
  work_free(&W);
  free(off);
}

void orc_als_batched(int nvec, double *const *coef, double *const *base, const int *nbas, int ndof,
                     const int *rF, const int *rG, int nals, int nthreads) {
#ifdef _OPENMP
  if (nthreads < 1) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
#endif
  for (int v = 0; v < nvec; ++v) orc_alscpp(coef[v], base[v], nbas, ndof, rF[v], rG[v], nals);
  (void)nthreads;
}

/* ------------------------------------------------------------------ */
/* The Fortran host's CPU ALS reduction (src/REDUCTIONML.f90:593-731)   */
/* ------------------------------------------------------------------ */

/* PRODND (src/MODVECVECML.f90:432-461): prod over modes d != kskip of
 * <a^d, b^d>, modes in increasing order, each dot summed in basis order.
 * kskip < 0 includes every mode. */
static double prodnd(const double *a, const double *b, const int *nbas, int ndof, int kskip) {
  double prod = 1.0;
  int gi = 0;
  for (int d = 0; d < ndof; ++d) {
    if (d != kskip) {
      double s = 0.0;
      for (int j = 0; j < nbas[d]; ++j) s += a[gi + j] * b[gi + j];
      prod *= s;
    }
    gi += nbas[d];
  }
  return prod;
}

/* UpdateBB / UpdatePS (src/MODVECVECML.f90:622-708): multiply (divide = 0)
 * or divide (divide = 1) the running products by the mode-k dots. */
static void update_bb(const double *fb, int rF, int nD, int gi, int n, double *BB, int divide) {
  for (int i = 0; i < rF; ++i)
    for (int j = i; j < rF; ++j) {
      double p = 0.0;
      for (int r = 0; r < n; ++r) p += fb[(size_t)i * nD + gi + r] * fb[(size_t)j * nD + gi + r];
      if (divide) p = 1.0 / p;
      BB[i + (size_t)j * rF] *= p;
    }
  for (int i = 1; i < rF; ++i)
    for (int j = 0; j < i; ++j) BB[i + (size_t)j * rF] = BB[j + (size_t)i * rF];
}

static void update_ps(const double *fb, int rF, const double *gb, int rG, int nD, int gi, int n, double *PS,
                      int divide) {
  for (int i = 0; i < rG; ++i)
    for (int j = 0; j < rF; ++j) {
      double p = 0.0;
      for (int r = 0; r < n; ++r) p += gb[(size_t)i * nD + gi + r] * fb[(size_t)j * nD + gi + r];
      if (divide) p = 1.0 / p;
      PS[i + (size_t)j * rG] *= p;
    }
}

/* CONSTBBTOT / CONSTPSTOT (src/MODVECVECML.f90:465-528), skipping mode kskip. */
static void const_bb(const double *fb, int rF, const int *nbas, int ndof, int nD, int kskip, double *BB) {
  for (int i = 0; i < rF; ++i)
    for (int j = i; j < rF; ++j)
      BB[i + (size_t)j * rF] = prodnd(fb + (size_t)j * nD, fb + (size_t)i * nD, nbas, ndof, kskip);
  for (int i = 1; i < rF; ++i)
    for (int j = 0; j < i; ++j) BB[i + (size_t)j * rF] = BB[j + (size_t)i * rF];
}

static void const_ps(const double *fb, int rF, const double *gb, int rG, const int *nbas, int ndof, int nD,
                     int kskip, double *PS) {
  for (int i = 0; i < rG; ++i)
    for (int j = 0; j < rF; ++j)
      PS[i + (size_t)j * rG] = prodnd(fb + (size_t)j * nD, gb + (size_t)i * nD, nbas, ndof, kskip);
}

/* reduc_ALS: F (rF terms, updated in place) fitted to G (rG terms) by nitn
 * ALS sweeps over the modes.  Penalty 1e-15 max c_G on the diagonal.  With
 * more than three modes BB and PS are kept by division and multiplication
 * of one mode's dots; otherwise rebuilt at every mode step.  LU solve
 * (dgetrf/dgetrs), then each row of the solution normalised into its
 * weight.  Returns 0, or 1 when a weight came out NaN (the reference then
 * restarts from GetRandomCPvec's random vector, whose generator is not
 * restated; the caller sees the flag instead). */
int orc_reduc_als(const double *gcoef, const double *gbase, int rG, double *fcoef, double *fbase, int rF,
                  const int *nbas, int ndof, int nitn) {
  if (nitn <= 0) return 0;
  int nD = 0, nmax = 0;
  for (int d = 0; d < ndof; ++d) {
    nD += nbas[d];
    nmax = nbas[d] > nmax ? nbas[d] : nmax;
  }
  const int update = ndof > 3;
  double *BB = (double *)malloc(sizeof(double) * rF * rF);
  double *BBmem = (double *)malloc(sizeof(double) * rF * rF);
  double *PS = (double *)malloc(sizeof(double) * (size_t)rG * rF);
  double *bjk = (double *)malloc(sizeof(double) * (size_t)rF * nmax);
  int *ipiv = (int *)malloc(sizeof(int) * rF);
  double gmax = gcoef[0];
  for (int j = 1; j < rG; ++j) gmax = gcoef[j] > gmax ? gcoef[j] : gmax;
  const double valpen = gmax * 1.0e-15;
  int bad = 0;
  if (update) {
    const_bb(fbase, rF, nbas, ndof, nD, 0, BBmem);
    const_ps(fbase, rF, gbase, rG, nbas, ndof, nD, 0, PS);
  }
  int kp = -1;
  for (int itn = 0; itn < nitn && !bad; ++itn) {
    int gst = 0;
    for (int k = 0; k < ndof; ++k) {
      const int n = nbas[k];
      if (update) {
        if (kp >= 0) {
          update_bb(fbase, rF, nD, gst, n, BBmem, 1);
          update_ps(fbase, rF, gbase, rG, nD, gst, n, PS, 1);
        }
        memcpy(BB, BBmem, sizeof(double) * rF * rF);
      } else {
        const_bb(fbase, rF, nbas, ndof, nD, k, BB);
        const_ps(fbase, rF, gbase, rG, nbas, ndof, nD, k, PS);
      }
      for (int i = 0; i < rF; ++i) BB[i + (size_t)i * rF] += valpen;
      /* b_j_k(l', nr), bjk column-major [rF][n] (Beylkin eq. 3.4) */
      for (int e = 0; e < rF * n; ++e) bjk[e] = 0.0;
      for (int ir = 0; ir < n; ++ir)
        for (int j = 0; j < rG; ++j) {
          const double gtmp = gcoef[j] * gbase[(size_t)j * nD + gst + ir];
          for (int i = 0; i < rF; ++i) bjk[i + (size_t)ir * rF] += gtmp * PS[j + (size_t)i * rG];
        }
      lu_solve(BB, bjk, rF, n, ipiv);
      for (int i = 0; i < rF; ++i) {
        double s = 0.0;
        for (int ir = 0; ir < n; ++ir) s += bjk[i + (size_t)ir * rF] * bjk[i + (size_t)ir * rF];
        const double rnorm = sqrt(fabs(s));
        fcoef[i] = rnorm;
        for (int ir = 0; ir < n; ++ir) fbase[(size_t)i * nD + gst + ir] = bjk[i + (size_t)ir * rF] / rnorm;
      }
      for (int i = 0; i < rF; ++i)
        if (fcoef[i] != fcoef[i]) bad = 1;
      if (bad) break;
      if (update && (itn < nitn - 1 || k < ndof - 1)) {
        update_bb(fbase, rF, nD, gst, n, BBmem, 0);
        update_ps(fbase, rF, gbase, rG, nD, gst, n, PS, 0);
      }
      gst += n;
      kp = k;
    }
  }
  free(BB);
  free(BBmem);
  free(PS);
  free(bjk);
  free(ipiv);
  return bad;
}

/* reduc_ALS over a batch of independent reductions, OpenMP over vectors (as
 * the Fortran host runs its per-vector reductions). */
int orc_reduc_als_batched(int nvec, const double *const *gcoef, const double *const *gbase, const int *rG,
                          double *const *fcoef, double *const *fbase, const int *rF, const int *nbas, int ndof,
                          int nitn, int nthreads) {
  int bad = 0;
#ifdef _OPENMP
  if (nthreads < 1) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads) reduction(+ : bad)
#endif
  for (int v = 0; v < nvec; ++v)
    bad += orc_reduc_als(gcoef[v], gbase[v], rG[v], fcoef[v], fbase[v], rF[v], nbas, ndof, nitn);
  (void)nthreads;
  return bad;
}

/* ------------------------------------------------------------------ */
/* Hamiltonian term application (reference src/intertw_mvp.cu:39)       */
/* ------------------------------------------------------------------ */

typedef struct {
  int T, ndof;
  const int *opid, *mptr;
  const double *coef, *mat;
} hoplist;

/* mvp_kernel (src/intertw_mvp.cu:39): G^d_r = alpha_d h_{t,d} v^d_r with the
 * packed upper-triangular operator h[ir + ic(ic+1)/2], alpha_0 = Hcoef[t]. */
static void apply_term(const hoplist *H, int t, const cpv *v, cpv *G) {
  for (int d = 0; d < v->ndof; ++d) {
    int n = v->nbas[d], o = v->off[d];
    int hsft = H->mptr[H->opid[t * v->ndof + d] - 1] - 1;
    double alpha = (d == 0) ? H->coef[t] : 1.0;
    for (int r = 0; r < v->nrk; ++r) {
      const double *x = v->base + (size_t)r * v->nD + o;
      double *y = G->base + (size_t)r * v->nD + o;
      for (int ib = 0; ib < n; ++ib) {
        double t2 = 0.0;
        for (int i = 0; i < n; ++i) {
          int ir = i < ib ? i : ib, ic = i < ib ? ib : i;
          t2 += x[i] * H->mat[hsft + ir + ic * (ic + 1) / 2];
        }
        y[ib] = t2 * alpha;
      }
    }
  }
}

/* mvp_build_linear_system (src/intertw_mvp.cu:380). */
static void mvp_build(const hoplist *H, const cpv *Fo, cpv *F, cpv *G, work_t *W, int idof, int ishift,
                      double Eshift, int recalcB) {
  int rk = F->nrk, n = F->nbas[idof], o = F->off[idof];
  memset(W->bjk, 0, sizeof(double) * (size_t)rk * n);
  memcpy(G->coef, Fo->coef, sizeof(double) * rk);
  for (int t = 0; t < H->T; ++t) {
    apply_term(H, t, Fo, G);
    pstot(G, F, W->BB, idof, 0, 0);
    bjk_accumulate(G, W->BB, W->bjk, rk, idof, NULL);
  }
  memcpy(G->base, Fo->base, sizeof(double) * (size_t)rk * F->nD);
  pstot(G, F, W->BB, idof, 0, 0);
  if (ishift != 0) {
    for (int r = 0; r < rk; ++r)
      for (int i = 0; i < n; ++i) G->base[(size_t)r * F->nD + o + i] *= -Eshift;
    bjk_accumulate(G, W->BB, W->bjk, rk, idof, NULL);
    if (ishift < 0)
      for (int i = 0; i < rk * n; ++i) W->bjk[i] *= -1.0;
  }
  if (recalcB) {
    memcpy(G->base, F->base, sizeof(double) * (size_t)rk * F->nD);
    pstot(G, F, W->BB, idof, 0, 0);
  }
}

/* POW_ALS (src/intertw_mvp.cu:452): F <- ALS fit of (H - E)F, mode by mode. */
static void pow_als(const hoplist *H, cpv *F, cpv *G, work_t *W, int npow, int ishift, double Eshift) {
  if (npow == 0) return;
  double pen = penalty_f(F->coef, F->nrk, g_pen_mvp);
  for (int it = 0; it < npow; ++it) {
    for (int j = 0; j < F->ndof; ++j) {
      int n = F->nbas[j];
      mvp_build(H, F, F, G, W, j, ishift, Eshift, 0);
      add_penalty(W->BB, F->nrk, pen);
      lu_solve(W->BB, W->bjk, F->nrk, n, W->ipiv);
      replace_with_solution(F, W->bjk, j);
      normonebase(F, j);
    }
    normalize_coefs(F, W->BB);
  }
}

/* PRODHV_ALS (src/intertw_mvp.cu:501): F <- ALS fit of H Fo, starting at Fo. */
static void prodhv_als(const hoplist *H, const cpv *Fo, cpv *F, cpv *G, work_t *W, int nals) {
  if (nals == 0) return;
  memcpy(F->coef, Fo->coef, sizeof(double) * F->nrk);
  memcpy(F->base, Fo->base, sizeof(double) * (size_t)F->nrk * F->nD);
  double pen = penalty_f(Fo->coef, F->nrk, g_pen_mvp);
  for (int it = 0; it < nals; ++it)
    for (int j = 0; j < F->ndof; ++j) {
      int n = F->nbas[j];
      mvp_build(H, Fo, F, G, W, j, 0, 0.0, 1);
      add_penalty(W->BB, F->nrk, pen);
      lu_solve(W->BB, W->bjk, F->nrk, n, W->ipiv);
      replace_with_solution(F, W->bjk, j);
      normonebase(F, j);
    }
}

static cpv cp_alloc(int rk, const int *nbas, const int *off, int ndof) {
  cpv v = {rk, ndof, off[ndof], nbas, off, NULL, NULL};
  v.coef = (double *)calloc(rk, sizeof(double));
  v.base = (double *)calloc((size_t)rk * off[ndof], sizeof(double));
  return v;
}
static void cp_free(cpv *v) { free(v->coef); free(v->base); }

/* MatrixVectorProducts (src/intertw_mvp.cu:553): POW_ALS on every vector. */
void orc_pow_als_block(double *base, double *coef, const int *nbas, int rk, int ndof, int nbloc,
                       const int *opid, const int *mptr, const double *Hcoef, const double *mat,
                       int T, int npow, int ishift, double Eshift, int nthreads) {
  int *off = make_offsets(nbas, ndof);
  cpv Q = {rk * nbloc, ndof, off[ndof], nbas, off, coef, base};
  hoplist H = {T, ndof, opid, mptr, Hcoef, mat};
  int nmax = max_nbas(nbas, ndof);
#ifdef _OPENMP
  if (nthreads < 1) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
#endif
  for (int i = 0; i < nbloc; ++i) {
    work_t W;
    work_init(&W, rk, nmax, nbloc);
    cpv F = cp_window(&Q, i * rk, rk);
    cpv G = cp_alloc(rk, nbas, off, ndof);
    pow_als(&H, &F, &G, &W, npow, ishift, Eshift);
    cp_free(&G);
    work_free(&W);
  }
  (void)nthreads;
  free(off);
}

/* ------------------------------------------------------------------ */
/* Gram-Schmidt and vector updates (reference src/intertw_lcv.cu)       */
/* ------------------------------------------------------------------ */

/* lcv_build_linear_system (src/intertw_lcv.cu:77). gcoef[k] is the weight
 * of vector k; with gs != 0 the weights of k < iv are recomputed as
 * -<Q_k, F> (gramsumoverrow + sumarray, :51 and :117). */
static void lcv_build(const cpv *Q, cpv *F, work_t *W, double *gcoef, int idof, int iv, int gs) {
  int rk = F->nrk, n = F->nbas[idof];
  memset(W->bjk, 0, sizeof(double) * (size_t)rk * n);
  for (int k = 0; k < iv; ++k) {
    cpv G = cp_window(Q, k * rk, rk);
    pstot(&G, F, W->BB, idof, 0, 0);
    if (gs) {
      psk(&G, F, W->BBk, idof);
      double total = 0.0;
      for (int row = 0; row < rk; ++row) {
        double u = 0.0;
        for (int col = 0; col < rk; ++col)
          u -= F->coef[col] * W->BB[row + (size_t)col * rk] * W->BBk[row + (size_t)col * rk];
        u *= G.coef[row];
        total += u;
      }
      gcoef[k] = total;
    }
    bjk_accumulate(&G, W->BB, W->bjk, rk, idof, &gcoef[k]);
  }
  pstot(F, F, W->BB, idof, 0, 0);
  if (gs) bjk_accumulate(F, W->BB, W->bjk, rk, idof, &gcoef[iv]);
}

/* GramSchmidt (src/intertw_lcv.cu:131). */
void orc_gram_schmidt(double *base, double *coef, const int *nbas, int rk, int ndof, int nbloc, int nals) {
  if (nals == 0) return;
  int *off = make_offsets(nbas, ndof);
  cpv Q = {rk * nbloc, ndof, off[ndof], nbas, off, coef, base};
  work_t W;
  work_init(&W, rk, max_nbas(nbas, ndof), nbloc);
  double *gcoef = (double *)malloc(sizeof(double) * nbloc);
  for (int i = 0; i < nbloc; ++i) gcoef[i] = 1.0;
  cpv F = cp_window(&Q, 0, rk);
  normalize_coefs(&F, W.BB);
  for (int iv = 1; iv < nbloc; ++iv) {
    F = cp_window(&Q, iv * rk, rk);
    double pen = penalty_f(F.coef, rk, g_pen_gs);
    for (int it = 0; it < nals; ++it)
      for (int j = 0; j < ndof; ++j) {
        int n = nbas[j];
        lcv_build(&Q, &F, &W, gcoef, j, iv, 1);
        add_penalty(W.BB, rk, pen);
        lu_solve(W.BB, W.bjk, rk, n, W.ipiv);
        replace_with_solution(&F, W.bjk, j);
        normonebase(&F, j);
        normalize_coefs(&F, W.BB);
      }
  }
  free(gcoef);
  work_free(&W);
  free(off);
}

/* GenEigvalProblem (src/intertw_mvp.cu:589): QHQ(i,j) = <Q_j, H Q_i> with H Q_i
 * from PRODHV_ALS, S(i,j) = <Q_j, Q_i>, j <= i; then the generalised problem. */
void orc_gen_eig(const double *base, const double *coef, const int *nbas, int rk, int ndof, int nbloc,
                 const int *opid, const int *mptr, const double *Hcoef, const double *mat, int T,
                 int nals, double *eigv, double *U, int nthreads) {
  int *off = make_offsets(nbas, ndof);
  cpv Q = {rk * nbloc, ndof, off[ndof], nbas, off, (double *)coef, (double *)base};
  hoplist H = {T, ndof, opid, mptr, Hcoef, mat};
  int nmax = max_nbas(nbas, ndof);
  double *QHQ = (double *)calloc((size_t)nbloc * nbloc, sizeof(double));
  double *S = (double *)calloc((size_t)nbloc * nbloc, sizeof(double));
#ifdef _OPENMP
  if (nthreads < 1) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
#endif
  for (int i = 0; i < nbloc; ++i) {
    work_t W;
    work_init(&W, rk, nmax, nbloc);
    cpv Fo = cp_window(&Q, i * rk, rk);
    cpv F = cp_alloc(rk, nbas, off, ndof);
    cpv G = cp_alloc(rk, nbas, off, ndof);
    prodhv_als(&H, &Fo, &F, &G, &W, nals);
    if (nals == 0) { /* PRODHV_ALS returns early: F keeps its prior (zero) contents */ }
    for (int j = 0; j <= i; ++j) {
      cpv Gj = cp_window(&Q, j * rk, rk);
      pstot(&Gj, &F, W.BB, -1, 1, 1);
      QHQ[i + (size_t)j * nbloc] = sum_all(W.BB, rk, rk);
      pstot(&Gj, &Fo, W.BB, -1, 1, 1);
      S[i + (size_t)j * nbloc] = sum_all(W.BB, rk, rk);
    }
    cp_free(&F); cp_free(&G);
    work_free(&W);
  }
  (void)nthreads;
  orc_sygv(nbloc, QHQ, S, eigv, U);
  free(QHQ); free(S); free(off);
}

/* VectorUpdates (src/intertw_lcv.cu:270) with UPDATES_ALS (:209): the new
 * vector i is the ALS fit of sum_l U(l,i) Q_l, starting from Q_i. */
void orc_vector_updates(double *base, double *coef, const int *nbas, int rk, int ndof, int nbloc,
                        const double *U, int nals, int nthreads) {
  int *off = make_offsets(nbas, ndof);
  int nD = off[ndof];
  cpv Q = {rk * nbloc, ndof, nD, nbas, off, coef, base};
  int nmax = max_nbas(nbas, ndof);
  double *newbase = (double *)malloc(sizeof(double) * (size_t)rk * nbloc * nD);
  double *newcoef = (double *)malloc(sizeof(double) * (size_t)rk * nbloc);
  memcpy(newbase, base, sizeof(double) * (size_t)rk * nbloc * nD);
  memcpy(newcoef, coef, sizeof(double) * (size_t)rk * nbloc);
#ifdef _OPENMP
  if (nthreads < 1) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
#endif
  for (int i = 0; i < nbloc; ++i) {
    if (nals == 0) continue;
    work_t W;
    work_init(&W, rk, nmax, nbloc);
    cpv F = {rk, ndof, nD, nbas, off, newcoef + (size_t)i * rk, newbase + (size_t)i * rk * nD};
    double pen = penalty_f(F.coef, rk, g_pen_upd);
    double *gcoef = (double *)malloc(sizeof(double) * nbloc);
    memcpy(gcoef, U + (size_t)i * nbloc, sizeof(double) * nbloc);
    for (int it = 0; it < nals; ++it)
      for (int j = 0; j < ndof; ++j) {
        int n = nbas[j];
        lcv_build(&Q, &F, &W, gcoef, j, nbloc, 0);
        add_penalty(W.BB, rk, pen);
        lu_solve(W.BB, W.bjk, rk, n, W.ipiv);
        replace_with_solution(&F, W.bjk, j);
        normonebase(&F, j);
      }
    normalize_coefs(&F, W.BB);
    free(gcoef);
    work_free(&W);
  }
  (void)nthreads;
  memcpy(base, newbase, sizeof(double) * (size_t)rk * nbloc * nD);
  memcpy(coef, newcoef, sizeof(double) * (size_t)rk * nbloc);
  free(newbase); free(newcoef); free(off);
}

/* intertwinecpp_ (src/intertwining.cu:98): MVP -> GS -> (GEP -> updates). */
void orc_intertwine(double *base, double *coef, const int *nbas, int rk, int ndof, int nbloc,
                    const int *opid, const int *mptr, const double *Hcoef, const double *mat,
                    int TxD, int nops, int msize, double *eigv, int npow, int ncpu, int nals,
                    int update, int ishift, double Eshift) {
  (void)nops; (void)msize;
  int T = TxD / ndof;
  orc_pow_als_block(base, coef, nbas, rk, ndof, nbloc, opid, mptr, Hcoef, mat, T, npow, ishift, Eshift, ncpu);
  orc_gram_schmidt(base, coef, nbas, rk, ndof, nbloc, nals);
  if (update) {
    double *U = (double *)malloc(sizeof(double) * (size_t)nbloc * nbloc);
    orc_gen_eig(base, coef, nbas, rk, ndof, nbloc, opid, mptr, Hcoef, mat, T, nals, eigv, U, ncpu);
    orc_vector_updates(base, coef, nbas, rk, ndof, nbloc, U, nals, ncpu);
    free(U);
  }
}

/* RayleighQuotient2 (reference src/BlockUtils.f90:658-688): <v|H|v> / <v|v>
 * with H applied exactly.  As the reference does, each Hamiltonian term t is
 * applied to one rank-1 term i of v at a time (PRODHVR1: w^d = alpha_d
 * h_{t,d} v_i^d, alpha_0 = Hcoef[t], the packed upper-triangular operators
 * of apply_term) and the product is accumulated against v (PRODVV). */
double orc_rayleigh_quotient(const double *base, const double *coef, const int *nbas, int rk, int ndof,
                             const int *opid, const int *mptr, const double *Hcoef, const double *mat, int T) {
  int *off = make_offsets(nbas, ndof);
  const int nD = off[ndof];
  double *w = (double *)malloc(sizeof(double) * (size_t)nD);
  double num = 0.0;
  for (int i = 0; i < rk; ++i) {
    const double *vi = base + (size_t)i * nD;
    for (int t = 0; t < T; ++t) {
      for (int d = 0; d < ndof; ++d) {
        const int n = nbas[d], o = off[d];
        const int hsft = mptr[opid[t * ndof + d] - 1] - 1;
        const double alpha = (d == 0) ? Hcoef[t] : 1.0;
        for (int ib = 0; ib < n; ++ib) {
          double acc = 0.0;
          for (int a = 0; a < n; ++a) {
            const int ir = a < ib ? a : ib, ic = a < ib ? ib : a;
            acc += vi[o + a] * mat[hsft + ir + ic * (ic + 1) / 2];
          }
          w[o + ib] = acc * alpha;
        }
      }
      /* PRODVV(v, w): sum_j c_j c_i prod_d <v_j^d, w^d> */
      double s = 0.0;
      for (int j = 0; j < rk; ++j) {
        const double *vj = base + (size_t)j * nD;
        double prod = coef[j] * coef[i];
        for (int d = 0; d < ndof; ++d) {
          double dot = 0.0;
          for (int a = 0; a < nbas[d]; ++a) dot += vj[off[d] + a] * w[off[d] + a];
          prod *= dot;
        }
        s += prod;
      }
      num += s;
    }
  }
  /* PRODVV(v): sum_ij c_i c_j prod_d <v_i^d, v_j^d> */
  double den = 0.0;
  for (int i = 0; i < rk; ++i)
    for (int j = 0; j < rk; ++j) {
      double prod = coef[i] * coef[j];
      for (int d = 0; d < ndof; ++d) {
        double dot = 0.0;
        for (int a = 0; a < nbas[d]; ++a)
          dot += base[(size_t)i * nD + off[d] + a] * base[(size_t)j * nD + off[d] + a];
        prod *= dot;
      }
      den += prod;
    }
  free(w);
  free(off);
  return num / den;
}

/* GetQHQdiag (reference src/BlockUtils.f90:385-408): qhqd[i] =
 * RayleighQuotient2(Q_i, H) for i = nconv .. nbloc-1; entries below nconv are
 * left as they are. */
void orc_qhq_diag(const double *base, const double *coef, const int *nbas, int rk, int ndof, int nbloc, int nconv,
                  const int *opid, const int *mptr, const double *Hcoef, const double *mat, int T, double *qhqd,
                  int nthreads) {
  int nD = 0;
  for (int d = 0; d < ndof; ++d) nD += nbas[d];
#ifdef _OPENMP
  if (nthreads < 1) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
#endif
  for (int i = nconv < 0 ? 0 : nconv; i < nbloc; ++i)
    qhqd[i] = orc_rayleigh_quotient(base + (size_t)i * rk * nD, coef + (size_t)i * rk, nbas, rk, ndof, opid, mptr,
                                    Hcoef, mat, T);
  (void)nthreads;
}

/* GetSpectralRange (reference src/Solver.f90:563-654), the branch for more
 * than two modes, from the two starting vectors in base/coef: bounds from
 * their Rayleigh quotients, then ncyc rounds of npow power steps of
 * (H - btmp_j) -- btmp_0 the midpoint of the bounds, btmp_1 = 0 -- each
 * round ending with new bounds; finally the range padded by 0.1 % of its
 * width on each side.  The power step is the POW_ALS restatement above
 * (src/intertw_mvp.cu:452; its CPU twin ALS_POW3, src/ALSPow.f90:569-660). */
void orc_spectral_range(double *base, double *coef, const int *nbas, int rk, int ndof, int npow, int ncyc,
                        const int *opid, const int *mptr, const double *Hcoef, const double *mat, int T,
                        double *bounds) {
  int nD = 0;
  for (int d = 0; d < ndof; ++d) nD += nbas[d];
  double b[2], btmp[2];
  for (int j = 0; j < 2; ++j)
    b[j] = orc_rayleigh_quotient(base + (size_t)j * rk * nD, coef + (size_t)j * rk, nbas, rk, ndof, opid, mptr,
                                 Hcoef, mat, T);
  btmp[0] = 0.5 * (b[0] + b[1]);
  btmp[1] = 0.0;
  for (int i = 0; i < ncyc; ++i) {
    for (int j = 0; j < 2; ++j) {
      double *vb = base + (size_t)j * rk * nD, *vc = coef + (size_t)j * rk;
      orc_pow_als_block(vb, vc, nbas, rk, ndof, 1, opid, mptr, Hcoef, mat, T, npow, 1, btmp[j], 1);
      b[j] = orc_rayleigh_quotient(vb, vc, nbas, rk, ndof, opid, mptr, Hcoef, mat, T);
    }
    btmp[0] = 0.5 * (b[0] + b[1]);
  }
  const double pad = 0.001 * (b[1] - b[0]);
  bounds[0] = b[0] - pad;
  bounds[1] = b[1] + pad;
}

/* UpdateOperMat (reference src/Updater.f90:110-151) for nx operators of
 * mode imode (1-based) given packed upper-triangular (as dspmv 'U', column
 * by column) back to back: for each i, XQ = X applied to mode imode of every
 * term of Q_i (PRODXV, :155-189), then QXQ(i,j) = <Q_j, XQ> (PRODVV) for
 * j >= i, packed upper-triangular (SymPackMat2Vec, src/Utils.f90:559-595)
 * into qxq[x][i + j(j+1)/2]. */
void orc_update_opermat(int imode, const double *base, const double *coef, const int *nbas, int rk, int ndof,
                        int nbloc, int nx, const double *xmats, double *qxq) {
  int *off = make_offsets(nbas, ndof);
  const int nD = off[ndof], m = imode - 1, n = nbas[m], o = off[m];
  const size_t np = (size_t)n * (n + 1) / 2, nq = (size_t)nbloc * (nbloc + 1) / 2;
  double *xq = (double *)malloc(sizeof(double) * (size_t)rk * nD);
  for (int x = 0; x < nx; ++x) {
    const double *X = xmats + (size_t)x * np;
    for (int i = 0; i < nbloc; ++i) {
      const double *qi = base + (size_t)i * rk * nD;
      memcpy(xq, qi, sizeof(double) * (size_t)rk * nD);
      for (int r = 0; r < rk; ++r)
        for (int a = 0; a < n; ++a) {
          double acc = 0.0;
          for (int b = 0; b < n; ++b) {
            const int ir = a < b ? a : b, ic = a < b ? b : a;
            acc += X[ir + ic * (ic + 1) / 2] * qi[(size_t)r * nD + o + b];
          }
          xq[(size_t)r * nD + o + a] = acc;
        }
      for (int j = i; j < nbloc; ++j)
        qxq[(size_t)x * nq + i + (size_t)j * (j + 1) / 2] =
            orc_cp_dot(base + (size_t)j * rk * nD, coef + (size_t)j * rk, rk, xq, coef + (size_t)i * rk, rk, nbas,
                       ndof);
    }
  }
  free(xq);
  free(off);
}

double orc_cp_dot(const double *vb, const double *vc, int rv, const double *wb, const double *wc, int rw,
                  const int *nbas, int ndof) {
  int *off = make_offsets(nbas, ndof);
  cpv v = {rv, ndof, off[ndof], nbas, off, (double *)vc, (double *)vb};
  cpv w = {rw, ndof, off[ndof], nbas, off, (double *)wc, (double *)wb};
  double total = 0.0;
  double *col = (double *)malloc(sizeof(double) * rv);
  for (int j = 0; j < rw; ++j) {
    cpv wj = cp_window(&w, j, 1);
    pstot(&v, &wj, col, -1, 1, 1);
    for (int i = 0; i < rv; ++i) total += col[i];
  }
  free(col);
  free(off);
  return total;
}

/* ------------------------------------------------------------------ */
/* The Fortran host's CPU power cycle (solver pals, src/Solver.f90:508-538) */
/* ------------------------------------------------------------------ */
/*
 * Iterate's CPU branch for the ALS power solver (styp = -1) runs, per cycle:
 * ALS_POW_alg on vectors nconv.. (OpenMP over vectors), ALS_ORTHO_alg, and
 * with update = T Diagonalize(intw = T): GetQHQ3 (PRODHV_ALS_alg, then
 * PRODVV), GetOverlaps, SolveGenEigval (DSYGV 'U'), UpdateVecs2
 * (ALS_SUMLCVEC_alg).  The routines restated here are the ones that run at
 * lowmem = 4, the value of the reference's sample input: ALS_POW3,
 * ALS_ORTHO_2, PRODHV_ALS2 and ALS_SUMLCVEC_2 (the dispatchers fall back to
 * the _2 forms for lowmem 4, src/ALSUtils.f90:112-121, :141-150,
 * src/ALSPow.f90:131-140).  Unlike the reference's GPU path, vectors of a
 * block may have different ranks (the `ranks` table of ALS_ORTHO_2): the
 * terms of vector v are terms toff[v] .. toff[v] + ranks[v] - 1 of the block.
 * Every penalty is 1e-10 times the largest weight of the vector being fitted,
 * as these routines hard-code it.
 */

typedef struct {
  double *BB, *BBmem, *PS, *bjk, *T, *psk;
  int *ipiv;
} pals_ws;

static pals_ws pals_ws_alloc(int rF, int rG, int nmax) {
  pals_ws w;
  w.BB = (double *)malloc(sizeof(double) * rF * rF);
  w.BBmem = (double *)malloc(sizeof(double) * rF * rF);
  w.PS = (double *)malloc(sizeof(double) * (size_t)rG * rF);
  w.psk = (double *)malloc(sizeof(double) * (size_t)rG * rF);
  w.bjk = (double *)malloc(sizeof(double) * (size_t)rF * nmax);
  w.T = (double *)malloc(sizeof(double) * nmax);
  w.ipiv = (int *)malloc(sizeof(int) * rF);
  return w;
}

static void pals_ws_free(pals_ws *w) {
  free(w->BB); free(w->BBmem); free(w->PS); free(w->psk); free(w->bjk); free(w->T); free(w->ipiv);
}

static double dot_n(const double *a, const double *b, int n) {
  double s = 0.0;
  for (int j = 0; j < n; ++j) s += a[j] * b[j];
  return s;
}

static double maxval(const double *c, int n) {
  double m = c[0];
  for (int i = 1; i < n; ++i) m = c[i] > m ? c[i] : m;
  return m;
}

/* HVBaseProd (src/MODHVECML.f90:170-209): y = fac h_{t,d} x, fac = opcoef(t)
 * on the first mode and 1 elsewhere, h packed upper-triangular (dspmv 'U');
 * the identity is stored as an explicit operator in the hoplist. */
static void hv_base_prod(const hoplist *H, int t, int d, const double *x, double *y, int n) {
  const double *h = H->mat + H->mptr[H->opid[t * H->ndof + d] - 1] - 1;
  const double fac = (d == 0) ? H->coef[t] : 1.0;
  for (int ib = 0; ib < n; ++ib) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) {
      const int ir = i < ib ? i : ib, ic = i < ib ? ib : i;
      s += h[ir + ic * (ic + 1) / 2] * x[i];
    }
    y[ib] = fac * s;
  }
}

/* PRODVV_AA (src/MODVECVECML.f90:356-392): <F,F> from the upper triangle
 * doubled plus the diagonal. */
static double prodvv_aa(const double *coef, const double *base, int r, const int *nbas, int ndof, int nD) {
  double s = 0.0;
  for (int i = 0; i < r - 1; ++i)
    for (int j = i + 1; j < r; ++j)
      s += coef[i] * coef[j] * prodnd(base + (size_t)i * nD, base + (size_t)j * nD, nbas, ndof, -1);
  s = 2 * s;
  for (int i = 0; i < r; ++i)
    s += coef[i] * coef[i] * prodnd(base + (size_t)i * nD, base + (size_t)i * nD, nbas, ndof, -1);
  return s;
}

/* PRODVV_AB (src/MODVECVECML.f90:394-430): <F,G>. */
static double prodvv_ab(const double *fc, const double *fb, int rF, const double *gc, const double *gb, int rG,
                        const int *nbas, int ndof, int nD) {
  double s = 0.0;
  for (int i = 0; i < rF; ++i)
    for (int j = 0; j < rG; ++j)
      s += fc[i] * gc[j] * prodnd(fb + (size_t)i * nD, gb + (size_t)j * nD, nbas, ndof, -1);
  return s;
}

/* NORMBASE + NORMCOEF (src/MODVECVECML.f90:295-352): every factor scaled to
 * unit 2-norm with the norms moved into the weight, then the weights scaled
 * so that <F,F> = 1. */
static void normcoef(double *coef, double *base, int r, const int *nbas, const int *off, int ndof) {
  const int nD = off[ndof];
  for (int i = 0; i < r; ++i) {
    double nd = 1.0;
    for (int d = 0; d < ndof; ++d) {
      double *x = base + (size_t)i * nD + off[d];
      const double n1 = sqrt(dot_n(x, x, nbas[d]));
      for (int j = 0; j < nbas[d]; ++j) x[j] = x[j] / n1;
      nd = nd * n1;
    }
    coef[i] = coef[i] * nd;
  }
  const double s = 1 / sqrt(fabs(prodvv_aa(coef, base, r, nbas, ndof, nD)));
  for (int i = 0; i < r; ++i) coef[i] = coef[i] * s;
}

/* "Construct improved F" (e.g. src/ALSPow.f90:622-627): weight i = the
 * 2-norm of row i of the solution, mode factor = the row over it.  Returns 1
 * when a weight is NaN (the reference aborts there). */
static int rows_to_mode(double *coef, double *base, int rF, int nD, int gst, const double *bjk, int n) {
  int bad = 0;
  for (int i = 0; i < rF; ++i) {
    double s = 0.0;
    for (int ir = 0; ir < n; ++ir) s += bjk[i + (size_t)ir * rF] * bjk[i + (size_t)ir * rF];
    const double rnorm = sqrt(fabs(s));
    coef[i] = rnorm;
    for (int ir = 0; ir < n; ++ir) base[(size_t)i * nD + gst + ir] = bjk[i + (size_t)ir * rF] / rnorm;
  }
  for (int i = 0; i < rF; ++i)
    if (coef[i] != coef[i]) bad = 1;
  return bad;
}

/* BuildbjkDirectX (src/ALSPow.f90:1154-1310): for mode k,
 *   BB(i,l)  = prod_{m != k} <F_l^m, Fo_i^m>   (recalcB: <F_l^m, F_i^m>),
 *   bjk(l,:) = sum_t sum_i co_i [prod_{m != k} <F_l^m, h_{t,m} Fo_i^m>] h_{t,k} Fo_i^k
 *              - E sum_i co_i BB(i,l) Fo_i^k            (ishift != 0),
 * negated at k = 0 when ishift < 0.  The other modes are visited in the
 * order k+1, ..., D-1, 0, ..., k-1; T holds one applied factor. */
static void buildbjk_direct(const hoplist *H, const double *focoef, const double *fobase, const double *fbase, int rF,
                            const int *nbas, const int *off, int ndof, int k, int ishift, double Eshift, double *BB,
                            double *bjk, double *T, int recalcB) {
  const int nD = off[ndof], n = nbas[k];
  for (int e = 0; e < rF * n; ++e) bjk[e] = 0.0;
  for (int t = 0; t < H->T; ++t)
    for (int i = 0; i < rF; ++i) {
      for (int l = 0; l < rF; ++l) BB[i + (size_t)l * rF] = 1.0;
      for (int m = 1; m < ndof; ++m) {
        const int mm = (k + m) % ndof;
        hv_base_prod(H, t, mm, fobase + (size_t)i * nD + off[mm], T, nbas[mm]);
        for (int l = 0; l < rF; ++l)
          BB[i + (size_t)l * rF] *= dot_n(fbase + (size_t)l * nD + off[mm], T, nbas[mm]);
      }
      hv_base_prod(H, t, k, fobase + (size_t)i * nD + off[k], T, n);
      for (int l = 0; l < rF; ++l) {
        const double tmp = focoef[i] * BB[i + (size_t)l * rF];
        for (int j = 0; j < n; ++j) bjk[l + (size_t)j * rF] += tmp * T[j];
      }
    }
  for (int i = 0; i < rF; ++i) {
    for (int l = 0; l < rF; ++l) BB[i + (size_t)l * rF] = 1.0;
    const double tmp = -Eshift * focoef[i];
    for (int m = 1; m < ndof; ++m) {
      const int mm = (k + m) % ndof;
      const double *x = fobase + (size_t)i * nD + off[mm];
      for (int l = 0; l < rF; ++l) BB[i + (size_t)l * rF] *= dot_n(fbase + (size_t)l * nD + off[mm], x, nbas[mm]);
    }
    if (ishift != 0) {
      const double *x = fobase + (size_t)i * nD + off[k];
      for (int l = 0; l < rF; ++l) {
        const double tmp2 = tmp * BB[i + (size_t)l * rF];
        for (int j = 0; j < n; ++j) bjk[l + (size_t)j * rF] += tmp2 * x[j];
      }
    }
  }
  if (k == 0 && ishift < 0)
    for (int e = 0; e < rF * n; ++e) bjk[e] = -bjk[e];
  if (recalcB) {  /* upper triangle, then mirrored */
    for (int i = 0; i < rF; ++i) {
      for (int l = i; l < rF; ++l) BB[i + (size_t)l * rF] = 1.0;
      for (int m = 1; m < ndof; ++m) {
        const int mm = (k + m) % ndof;
        const double *x = fbase + (size_t)i * nD + off[mm];
        for (int l = i; l < rF; ++l) BB[i + (size_t)l * rF] *= dot_n(fbase + (size_t)l * nD + off[mm], x, nbas[mm]);
      }
    }
    for (int i = 1; i < rF; ++i)
      for (int l = 0; l < i; ++l) BB[i + (size_t)l * rF] = BB[l + (size_t)i * rF];
  }
}

/* ALS_POW3 (src/ALSPow.f90:569-660): nitn in-place sweeps of F <- ALS fit of
 * (H - E)F; each mode step builds BB and bjk from F itself
 * (BuildbjkDirectX(F, F, ...)), adds 1e-10 max c (taken once), solves by LU
 * and moves the row norms into the weights; after the last mode the weights
 * are scaled to <F,F> = 1.  Returns 1 on a NaN weight. */
static int pals_pow3(const hoplist *H, double *coef, double *base, int rF, const int *nbas, const int *off, int ndof,
                     int nitn, int ishift, double Eshift, pals_ws *w) {
  if (nitn == 0) return 0;
  const int nD = off[ndof];
  const double valpen = maxval(coef, rF) * 1.0e-10;
  for (int itn = 0; itn < nitn; ++itn)
    for (int k = 0; k < ndof; ++k) {
      const int n = nbas[k];
      buildbjk_direct(H, coef, base, base, rF, nbas, off, ndof, k, ishift, Eshift, w->BB, w->bjk, w->T, 0);
      for (int i = 0; i < rF; ++i) w->BB[i + (size_t)i * rF] += valpen;
      lu_solve(w->BB, w->bjk, rF, n, w->ipiv);
      if (rows_to_mode(coef, base, rF, nD, off[k], w->bjk, n)) return 1;
      if (k == ndof - 1) {
        const double s = 1 / sqrt(fabs(prodvv_aa(coef, base, rF, nbas, ndof, nD)));
        for (int i = 0; i < rF; ++i) coef[i] = coef[i] * s;
      }
    }
  return 0;
}

/* UpdateXPS (src/ALSPow.f90:937-1032), divide = 0, and the PS half of
 * DowndateXPS (:1034-1150), divide = 1: row ik = t rF + i of the
 * rG x rF matrix PS (rG = T rF, plus rF rows for the shift) is multiplied
 * or divided by <F_l^k, h_{t,k} Fo_i^k>; the shift rows by <F_l^k, Fo_i^k>,
 * negated on mode 0.  With divide set, bjk(l,:) += co_i PS(ik,l) h Fo_i^k
 * (and + E co_i PS(ik,l) (+-Fo_i^k) for the shift rows).  On mode 0 with
 * ishift < 0 PS (and bjk) change sign. */
static void xps_step(const hoplist *H, const double *focoef, const double *fobase, const double *fbase, int rF,
                     const int *nbas, const int *off, int ndof, int k, int ishift, double Eshift, double *PS,
                     double *bjk, double *T, int divide) {
  const int nD = off[ndof], n = nbas[k];
  const int rG = rF * H->T + (ishift != 0 ? rF : 0);
  if (divide)
    for (int e = 0; e < rF * n; ++e) bjk[e] = 0.0;
  int ik = 0;
  for (int t = 0; t < H->T; ++t)
    for (int i = 0; i < rF; ++i, ++ik) {
      hv_base_prod(H, t, k, fobase + (size_t)i * nD + off[k], T, n);
      for (int l = 0; l < rF; ++l) {
        const double prod = dot_n(fbase + (size_t)l * nD + off[k], T, n);
        if (!divide) {
          PS[ik + (size_t)l * rG] = PS[ik + (size_t)l * rG] * prod;
        } else {
          PS[ik + (size_t)l * rG] = PS[ik + (size_t)l * rG] / prod;
          const double tmp = focoef[i] * PS[ik + (size_t)l * rG];
          for (int j = 0; j < n; ++j) bjk[l + (size_t)j * rF] += tmp * T[j];
        }
      }
    }
  if (ishift != 0) {
    for (int i = 0; i < rF; ++i, ++ik) {
      const double tmp = Eshift * focoef[i];
      for (int j = 0; j < n; ++j) T[j] = fobase[(size_t)i * nD + off[k] + j];
      if (k == 0)
        for (int j = 0; j < n; ++j) T[j] = -T[j];
      for (int l = 0; l < rF; ++l) {
        const double prod = dot_n(fbase + (size_t)l * nD + off[k], T, n);
        if (!divide) {
          PS[ik + (size_t)l * rG] = PS[ik + (size_t)l * rG] * prod;
        } else {
          PS[ik + (size_t)l * rG] = PS[ik + (size_t)l * rG] / prod;
          const double tmp2 = tmp * PS[ik + (size_t)l * rG];
          for (int j = 0; j < n; ++j) bjk[l + (size_t)j * rF] += tmp2 * T[j];
        }
      }
    }
    if (k == 0 && ishift < 0) {
      for (size_t e = 0; e < (size_t)rG * rF; ++e) PS[e] = -PS[e];
      if (divide)
        for (int e = 0; e < rF * n; ++e) bjk[e] = -bjk[e];
    }
  }
}

/* PRODHV_ALS2 (src/ALSPow.f90:664-780): F <- ALS fit of (H - E)Fo, starting
 * from F = Fo, by nitn sweeps.  BB = <F,F> without mode 0 at the start
 * (CONSTBBTOT), then kept by UpdateBB division / multiplication; PS starts
 * at 1 and takes every mode by UpdateXPS; each mode step divides its mode
 * out of PS while building bjk (DowndateXPS), adds 1e-10 max c_Fo, solves by
 * LU and moves the row norms into the weights, then multiplies the new mode
 * back into BB and PS (except after the very last step).  No final
 * normalisation.  Returns 1 on a NaN weight. */
static int pals_prodhv2(const hoplist *H, const double *focoef, const double *fobase, double *coef, double *base,
                        int rF, const int *nbas, const int *off, int ndof, int ishift, double Eshift, int nitn,
                        pals_ws *w) {
  if (nitn == 0) return 0;
  const int nD = off[ndof];
  const int rG = rF * H->T + (ishift != 0 ? rF : 0);
  memcpy(coef, focoef, sizeof(double) * rF);
  memcpy(base, fobase, sizeof(double) * (size_t)rF * nD);
  const double valpen = maxval(coef, rF) * 1.0e-10;
  const_bb(base, rF, nbas, ndof, nD, 0, w->BBmem);
  for (size_t e = 0; e < (size_t)rG * rF; ++e) w->PS[e] = 1.0;
  for (int k = 0; k < ndof; ++k)
    xps_step(H, focoef, fobase, base, rF, nbas, off, ndof, k, ishift, Eshift, w->PS, NULL, w->T, 0);
  int kp = -1;
  for (int itn = 0; itn < nitn; ++itn)
    for (int k = 0; k < ndof; ++k) {
      const int n = nbas[k];
      if (kp >= 0) update_bb(base, rF, nD, off[k], n, w->BBmem, 1);
      memcpy(w->BB, w->BBmem, sizeof(double) * rF * rF);
      for (int i = 0; i < rF; ++i) w->BB[i + (size_t)i * rF] += valpen;
      xps_step(H, focoef, fobase, base, rF, nbas, off, ndof, k, ishift, Eshift, w->PS, w->bjk, w->T, 1);
      lu_solve(w->BB, w->bjk, rF, n, w->ipiv);
      if (rows_to_mode(coef, base, rF, nD, off[k], w->bjk, n)) return 1;
      if (itn < nitn - 1 || k < ndof - 1) {
        update_bb(base, rF, nD, off[k], n, w->BBmem, 0);
        xps_step(H, focoef, fobase, base, rF, nbas, off, ndof, k, ishift, Eshift, w->PS, NULL, w->T, 0);
      }
      kp = k;
    }
  return 0;
}

/* CONSTPSk (src/MODVECVECML.f90:532-569) for one block of PS: P(j,i) =
 * <G_j^k, F_i^k>, leading dimension ld. */
static void const_psk(const double *fb, int rF, const double *gb, int rT, int nD, int gi, int n, double *P, int ld) {
  for (int j = 0; j < rT; ++j)
    for (int i = 0; i < rF; ++i) P[j + (size_t)i * ld] = dot_n(gb + (size_t)j * nD + gi, fb + (size_t)i * nD + gi, n);
}

/* ALS_ORTHO_2 (src/ALSUtils.f90:156-377): ALS-guided Gram-Schmidt.  Q_0 is
 * normalised (NORMCOEF).  Each later Q_v is refitted, nitn sweeps, to
 *   Q_v + sum_{l<v} coefs_l Q_l,   coefs_l = -<Q_l, Q_v> (from the full PS,
 * recomputed at every mode step);
 * PS (rows: the terms of Q_0..Q_v, columns: the terms of Q_v) starts as the
 * full products (CONSTPSTOT), and each mode step divides mode k out of it,
 * takes BB from the Q_v rows plus 1e-10 max c_v (taken once per vector),
 * builds bjk from the coefs-weighted terms, solves by LU, moves the row
 * norms into the weights, multiplies the new mode k back into PS and scales
 * the weights of Q_v to unit norm with the Q_v block of PS.  The loops over
 * l and over the entries of bjk are OpenMP-parallel, as in the reference.
 * Returns 1 on a NaN weight. */
static int pals_ortho2(double *coef, double *base, const int *ranks, const int *toff, int nbloc, const int *nbas,
                       const int *off, int ndof, int nitn, int nthreads) {
  if (nitn == 0) return 0;
  const int nD = off[ndof];
  int nmax = 0, rmax = 0;
  for (int d = 0; d < ndof; ++d) nmax = nbas[d] > nmax ? nbas[d] : nmax;
  for (int v = 0; v < nbloc; ++v) rmax = ranks[v] > rmax ? ranks[v] : rmax;
  const int rtot = toff[nbloc - 1] + ranks[nbloc - 1];
  double *coefs = (double *)malloc(sizeof(double) * nbloc);
  double *PS = (double *)malloc(sizeof(double) * (size_t)rtot * rmax);
  double *P2 = (double *)malloc(sizeof(double) * (size_t)rtot * rmax);
  double *BB = (double *)malloc(sizeof(double) * rmax * rmax);
  double *bjk = (double *)malloc(sizeof(double) * (size_t)rmax * nmax);
  int *ipiv = (int *)malloc(sizeof(int) * rmax);
  int bad = 0;
#ifdef _OPENMP
  if (nthreads < 1) nthreads = omp_get_max_threads();
#endif
  (void)nthreads;
  normcoef(coef, base, ranks[0], nbas, off, ndof);
  for (int iv = 1; iv < nbloc && !bad; ++iv) {
    double *fc = coef + toff[iv], *fb = base + (size_t)toff[iv] * nD;
    const int rF = ranks[iv], rG = toff[iv] + rF, s = toff[iv];
    const double valpen = maxval(fc, rF) * 1.0e-10;
    coefs[iv] = 1.0;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
    for (int l = 0; l <= iv; ++l) {
      const double *gb = base + (size_t)toff[l] * nD;
      for (int j = 0; j < ranks[l]; ++j)
        for (int i = 0; i < rF; ++i)
          PS[toff[l] + j + (size_t)i * rG] = prodnd(fb + (size_t)i * nD, gb + (size_t)j * nD, nbas, ndof, -1);
    }
    for (int itn = 0; itn < nitn && !bad; ++itn)
      for (int k = 0; k < ndof; ++k) {
        const int n = nbas[k], gst = off[k];
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
        for (int l = 0; l < iv; ++l) {
          double c = 0.0;
          for (int i = 0; i < rF; ++i)
            for (int j = 0; j < ranks[l]; ++j) c = c - PS[toff[l] + j + (size_t)i * rG] * fc[i] * coef[toff[l] + j];
          coefs[l] = c;
        }
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
        for (int l = 0; l <= iv; ++l) {
          const_psk(fb, rF, base + (size_t)toff[l] * nD, ranks[l], nD, gst, n, P2 + toff[l], rG);
          for (int j = 0; j < ranks[l]; ++j)
            for (int i = 0; i < rF; ++i)
              PS[toff[l] + j + (size_t)i * rG] = PS[toff[l] + j + (size_t)i * rG] / P2[toff[l] + j + (size_t)i * rG];
        }
        for (int i = 0; i < rF; ++i)
          for (int j = 0; j < rF; ++j) BB[j + (size_t)i * rF] = PS[s + j + (size_t)i * rG];
        for (int i = 0; i < rF; ++i) BB[i + (size_t)i * rF] += valpen;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
        for (int m = 0; m < n * rF; ++m) {
          const int i = m / n, ir = m % n;
          double b = 0.0;
          for (int l = 0; l <= iv; ++l)
            for (int j = 0; j < ranks[l]; ++j)
              b = b + coefs[l] * coef[toff[l] + j] * base[(size_t)(toff[l] + j) * nD + gst + ir] *
                          PS[toff[l] + j + (size_t)i * rG];
          bjk[i + (size_t)ir * rF] = b;
        }
        lu_solve(BB, bjk, rF, n, ipiv);
        if (rows_to_mode(fc, fb, rF, nD, gst, bjk, n)) { bad = 1; break; }
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
        for (int l = 0; l <= iv; ++l) {
          const_psk(fb, rF, base + (size_t)toff[l] * nD, ranks[l], nD, gst, n, P2 + toff[l], rG);
          for (int j = 0; j < ranks[l]; ++j)
            for (int i = 0; i < rF; ++i)
              PS[toff[l] + j + (size_t)i * rG] = PS[toff[l] + j + (size_t)i * rG] * P2[toff[l] + j + (size_t)i * rG];
        }
        double rn = 0.0;
        for (int i = 0; i < rF; ++i) {
          rn = rn + PS[s + i + (size_t)i * rG] * fc[i] * fc[i];
          for (int j = 0; j < i; ++j) rn = rn + 2 * PS[s + j + (size_t)i * rG] * fc[i] * fc[j];
        }
        rn = 1 / sqrt(fabs(rn));
        for (int i = 0; i < rF; ++i) fc[i] = rn * fc[i];
      }
  }
  free(coefs); free(PS); free(P2); free(BB); free(bjk); free(ipiv);
  return bad;
}

/* ALS_SUMLCVEC_2 (src/ALSUtils.f90:731-891): F (rF terms, starting guess in
 * place) <- ALS fit of sum_l w_l Q_l by nitn sweeps.  PS (rows: the terms of
 * every Q_l, columns: the terms of F) and BB = <F,F> start as the full
 * products and are kept by dividing mode k out before its step and
 * multiplying the new mode k back after it (PS not after the very last
 * step); penalty 1e-10 max c_F (taken once); at the end the weights are
 * scaled to unit norm with BB.  Returns 1 on a NaN weight. */
static int pals_sumlcvec2(double *fcoef, double *fbase, int rF, const double *qcoef, const double *qbase,
                          const int *ranks, const int *toff, int nbloc, const double *w, const int *nbas,
                          const int *off, int ndof, int nitn, pals_ws *ws) {
  if (nitn == 0) return 0;
  const int nD = off[ndof], rG = toff[nbloc - 1] + ranks[nbloc - 1];
  double *PS = ws->PS, *P2 = ws->psk, *BBmem = ws->BBmem, *BB = ws->BB, *bjk = ws->bjk;
  const double valpen = maxval(fcoef, rF) * 1.0e-10;
  for (int l = 0; l < nbloc; ++l)
    for (int j = 0; j < ranks[l]; ++j)
      for (int i = 0; i < rF; ++i)
        PS[toff[l] + j + (size_t)i * rG] =
            prodnd(fbase + (size_t)i * nD, qbase + (size_t)(toff[l] + j) * nD, nbas, ndof, -1);
  const_bb(fbase, rF, nbas, ndof, nD, -1, BBmem);
  for (int itn = 0; itn < nitn; ++itn)
    for (int k = 0; k < ndof; ++k) {
      const int n = nbas[k], gst = off[k];
      for (int l = 0; l < nbloc; ++l) {
        const_psk(fbase, rF, qbase + (size_t)toff[l] * nD, ranks[l], nD, gst, n, P2 + toff[l], rG);
        for (int j = 0; j < ranks[l]; ++j)
          for (int i = 0; i < rF; ++i)
            PS[toff[l] + j + (size_t)i * rG] = PS[toff[l] + j + (size_t)i * rG] / P2[toff[l] + j + (size_t)i * rG];
      }
      update_bb(fbase, rF, nD, gst, n, BBmem, 1);
      memcpy(BB, BBmem, sizeof(double) * rF * rF);
      for (int i = 0; i < rF; ++i) BB[i + (size_t)i * rF] += valpen;
      for (int e = 0; e < rF * n; ++e) bjk[e] = 0.0;
      for (int ir = 0; ir < n; ++ir)
        for (int l = 0; l < nbloc; ++l)
          for (int j = 0; j < ranks[l]; ++j) {
            const double gtmp = w[l] * qcoef[toff[l] + j] * qbase[(size_t)(toff[l] + j) * nD + gst + ir];
            for (int i = 0; i < rF; ++i) bjk[i + (size_t)ir * rF] += gtmp * PS[toff[l] + j + (size_t)i * rG];
          }
      lu_solve(BB, bjk, rF, n, ws->ipiv);
      if (rows_to_mode(fcoef, fbase, rF, nD, gst, bjk, n)) return 1;
      if (itn < nitn - 1 || k < ndof - 1)
        for (int l = 0; l < nbloc; ++l) {
          const_psk(fbase, rF, qbase + (size_t)toff[l] * nD, ranks[l], nD, gst, n, P2 + toff[l], rG);
          for (int j = 0; j < ranks[l]; ++j)
            for (int i = 0; i < rF; ++i)
              PS[toff[l] + j + (size_t)i * rG] = PS[toff[l] + j + (size_t)i * rG] * P2[toff[l] + j + (size_t)i * rG];
        }
      update_bb(fbase, rF, nD, gst, n, BBmem, 0);
    }
  double rn = 0.0;
  for (int i = 0; i < rF; ++i) {
    rn = rn + BBmem[i + (size_t)i * rF] * (fcoef[i] * fcoef[i]);
    for (int j = 0; j < i; ++j) rn = rn + 2 * BBmem[i + (size_t)j * rF] * fcoef[i] * fcoef[j];
  }
  rn = 1 / sqrt(fabs(rn));
  for (int i = 0; i < rF; ++i) fcoef[i] = rn * fcoef[i];
  return 0;
}

/* PRODHV_ALS3 (src/ALSPow.f90:784-865): the least-memory form of
 * PRODHV_ALS2.  Every mode step rebuilds BB = <F,F> and bjk from Fo and H
 * directly (BuildbjkDirectX with recalcB), then adds 1e-10 max c_Fo, solves
 * by LU and moves the row norms into the weights.  Returns 1 on a NaN. */
static int pals_prodhv3(const hoplist *H, const double *focoef, const double *fobase, double *coef, double *base,
                        int rF, const int *nbas, const int *off, int ndof, int ishift, double Eshift, int nitn,
                        pals_ws *w) {
  if (nitn == 0) return 0;
  const int nD = off[ndof];
  memcpy(coef, focoef, sizeof(double) * rF);
  memcpy(base, fobase, sizeof(double) * (size_t)rF * nD);
  const double valpen = maxval(coef, rF) * 1.0e-10;
  for (int itn = 0; itn < nitn; ++itn)
    for (int k = 0; k < ndof; ++k) {
      const int n = nbas[k];
      buildbjk_direct(H, focoef, fobase, base, rF, nbas, off, ndof, k, ishift, Eshift, w->BB, w->bjk, w->T, 1);
      for (int i = 0; i < rF; ++i) w->BB[i + (size_t)i * rF] += valpen;
      lu_solve(w->BB, w->bjk, rF, n, w->ipiv);
      if (rows_to_mode(coef, base, rF, nD, off[k], w->bjk, n)) return 1;
    }
  return 0;
}

/* ALS_ORTHO_3 (src/ALSUtils.f90:381-528): ALS_ORTHO_2 without the stored
 * PS.  At every mode step k of vector v, for each l <= v the block
 * P_l(j,i) = prod_{m != k} <Q_l,j^m, Q_v,i^m> is rebuilt (CONSTPSTOT_OMP),
 * with l < v also the mode-k block (CONSTPSk_OMP) for the coefficient
 * coefs_l = -<Q_l, Q_v>; bjk accumulates l by l.  BB is the Q_v block plus
 * 1e-10 max c_v (taken once per vector); after the solve the Q_v block is
 * multiplied by the new mode-k Gram (UpdateBB) and the weights scaled to
 * unit norm with it.  The blocks are built OpenMP-parallel over l, then
 * summed in the reference's order.  Returns 1 on a NaN weight. */
static int pals_ortho3(double *coef, double *base, const int *ranks, const int *toff, int nbloc, const int *nbas,
                       const int *off, int ndof, int nitn, int nthreads) {
  if (nitn == 0) return 0;
  const int nD = off[ndof];
  int nmax = 0, rmax = 0;
  for (int d = 0; d < ndof; ++d) nmax = nbas[d] > nmax ? nbas[d] : nmax;
  for (int v = 0; v < nbloc; ++v) rmax = ranks[v] > rmax ? ranks[v] : rmax;
  const int rtot = toff[nbloc - 1] + ranks[nbloc - 1];
  double *coefs = (double *)malloc(sizeof(double) * nbloc);
  double *P = (double *)malloc(sizeof(double) * (size_t)rtot * rmax);   /* block l at rows toff[l].. */
  double *Pk = (double *)malloc(sizeof(double) * (size_t)rtot * rmax);
  double *BB = (double *)malloc(sizeof(double) * rmax * rmax);
  double *BBmem = (double *)malloc(sizeof(double) * rmax * rmax);
  double *bjk = (double *)malloc(sizeof(double) * (size_t)rmax * nmax);
  int *ipiv = (int *)malloc(sizeof(int) * rmax);
  int bad = 0;
#ifdef _OPENMP
  if (nthreads < 1) nthreads = omp_get_max_threads();
#endif
  (void)nthreads;
  normcoef(coef, base, ranks[0], nbas, off, ndof);
  for (int iv = 1; iv < nbloc && !bad; ++iv) {
    double *fc = coef + toff[iv], *fb = base + (size_t)toff[iv] * nD;
    const int rF = ranks[iv], rG = toff[iv] + rF, s = toff[iv];
    const double valpen = maxval(fc, rF) * 1.0e-10;
    for (int itn = 0; itn < nitn && !bad; ++itn)
      for (int k = 0; k < ndof; ++k) {
        const int n = nbas[k], gik = off[k];
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
        for (int l = 0; l <= iv; ++l) {
          const double *gb = base + (size_t)toff[l] * nD;
          for (int j = 0; j < ranks[l]; ++j)
            for (int i = 0; i < rF; ++i)
              P[toff[l] + j + (size_t)i * rG] = prodnd(fb + (size_t)i * nD, gb + (size_t)j * nD, nbas, ndof, k);
          if (l < iv) const_psk(fb, rF, gb, ranks[l], nD, gik, n, Pk + toff[l], rG);
        }
        for (int e = 0; e < rF * n; ++e) bjk[e] = 0.0;
        for (int l = 0; l <= iv; ++l) {
          double c = 1.0;
          if (l < iv) {
            c = 0.0;
            for (int j = 0; j < ranks[l]; ++j)
              for (int i = 0; i < rF; ++i)
                c = c - P[toff[l] + j + (size_t)i * rG] * Pk[toff[l] + j + (size_t)i * rG] * coef[toff[l] + j] * fc[i];
          }
          coefs[l] = c;
          for (int j = 0; j < ranks[l]; ++j) {
            const double gtmp = coefs[l] * coef[toff[l] + j];
            const double *q = base + (size_t)(toff[l] + j) * nD + gik;
            for (int i = 0; i < rF; ++i) {
              const double g2 = gtmp * P[toff[l] + j + (size_t)i * rG];
              for (int ir = 0; ir < n; ++ir) bjk[i + (size_t)ir * rF] += g2 * q[ir];
            }
          }
        }
        for (int i = 0; i < rF; ++i)
          for (int j = 0; j < rF; ++j) BBmem[j + (size_t)i * rF] = P[s + j + (size_t)i * rG];
        memcpy(BB, BBmem, sizeof(double) * rF * rF);
        for (int i = 0; i < rF; ++i) BB[i + (size_t)i * rF] += valpen;
        lu_solve(BB, bjk, rF, n, ipiv);
        if (rows_to_mode(fc, fb, rF, nD, gik, bjk, n)) { bad = 1; break; }
        update_bb(fb, rF, nD, gik, n, BBmem, 0);
        double rn = 0.0;
        for (int i = 0; i < rF; ++i) {
          rn = rn + BBmem[i + (size_t)i * rF] * (fc[i] * fc[i]);
          for (int j = 0; j < i; ++j) rn = rn + 2 * BBmem[j + (size_t)i * rF] * fc[i] * fc[j];
        }
        rn = 1 / sqrt(fabs(rn));
        for (int i = 0; i < rF; ++i) fc[i] = rn * fc[i];
      }
  }
  free(coefs); free(P); free(Pk); free(BB); free(BBmem); free(bjk); free(ipiv);
  return bad;
}

/* ALS_SUMLCVEC_3 (src/ALSUtils.f90:895-1045): ALS_SUMLCVEC_2 without the
 * stored PS.  bjk is built term by term of every Q_l: the products over the
 * modes other than k (visited k+1, ..., D-1, 0, ..., k-1) of <F_i, Q_l,j>,
 * times w_l c_l,j Q_l,j^k; BB = <F,F> is kept by UpdateBB as in the _2 form,
 * and the weights are scaled to unit norm at the end.  Returns 1 on a NaN. */
static int pals_sumlcvec3(double *fcoef, double *fbase, int rF, const double *qcoef, const double *qbase,
                          const int *ranks, const int *toff, int nbloc, const double *w, const int *nbas,
                          const int *off, int ndof, int nitn, pals_ws *ws) {
  if (nitn == 0) return 0;
  const int nD = off[ndof];
  double *BBmem = ws->BBmem, *BB = ws->BB, *bjk = ws->bjk, *PSr = ws->psk;
  const double valpen = maxval(fcoef, rF) * 1.0e-10;
  const_bb(fbase, rF, nbas, ndof, nD, -1, BBmem);
  for (int itn = 0; itn < nitn; ++itn)
    for (int k = 0; k < ndof; ++k) {
      const int n = nbas[k], gik = off[k];
      for (int e = 0; e < rF * n; ++e) bjk[e] = 0.0;
      for (int l = 0; l < nbloc; ++l)
        for (int j = 0; j < ranks[l]; ++j) {
          const double *q = qbase + (size_t)(toff[l] + j) * nD;
          for (int i = 0; i < rF; ++i) PSr[i] = 1.0;
          for (int m = 1; m < ndof; ++m) {
            const int mm = (k + m) % ndof;
            for (int i = 0; i < rF; ++i) PSr[i] = PSr[i] * dot_n(fbase + (size_t)i * nD + off[mm], q + off[mm], nbas[mm]);
          }
          const double gtmp = w[l] * qcoef[toff[l] + j];
          for (int i = 0; i < rF; ++i) {
            const double g2 = gtmp * PSr[i];
            for (int ir = 0; ir < n; ++ir) bjk[i + (size_t)ir * rF] += g2 * q[gik + ir];
          }
        }
      update_bb(fbase, rF, nD, gik, n, BBmem, 1);
      memcpy(BB, BBmem, sizeof(double) * rF * rF);
      for (int i = 0; i < rF; ++i) BB[i + (size_t)i * rF] += valpen;
      lu_solve(BB, bjk, rF, n, ws->ipiv);
      if (rows_to_mode(fcoef, fbase, rF, nD, gik, bjk, n)) return 1;
      update_bb(fbase, rF, nD, gik, n, BBmem, 0);
    }
  double rn = 0.0;
  for (int i = 0; i < rF; ++i) {
    rn = rn + BBmem[i + (size_t)i * rF] * (fcoef[i] * fcoef[i]);
    for (int j = 0; j < i; ++j) rn = rn + 2 * BBmem[i + (size_t)j * rF] * fcoef[i] * fcoef[j];
  }
  rn = 1 / sqrt(fabs(rn));
  for (int i = 0; i < rF; ++i) fcoef[i] = rn * fcoef[i];
  return 0;
}

static int *rank_offsets(const int *ranks, int nbloc) {
  int *toff = (int *)malloc(sizeof(int) * (nbloc + 1));
  toff[0] = 0;
  for (int v = 0; v < nbloc; ++v) toff[v + 1] = toff[v] + ranks[v];
  return toff;
}

int orc_pals_pow3(double *base, double *coef, const int *nbas, int ndof, int nbloc, const int *ranks, int nconv,
                  const int *opid, const int *mptr, const double *Hcoef, const double *mat, int T, int npow,
                  int ishift, double Eshift, int nthreads) {
  int *off = make_offsets(nbas, ndof), *toff = rank_offsets(ranks, nbloc);
  const int nD = off[ndof], nmax = max_nbas(nbas, ndof);
  hoplist H = {T, ndof, opid, mptr, Hcoef, mat};
  int bad = 0;
#ifdef _OPENMP
  if (nthreads < 1) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads) reduction(+ : bad)
#endif
  for (int v = nconv < 0 ? 0 : nconv; v < nbloc; ++v) {
    pals_ws w = pals_ws_alloc(ranks[v], 1, nmax);
    bad += pals_pow3(&H, coef + toff[v], base + (size_t)toff[v] * nD, ranks[v], nbas, off, ndof, npow, ishift,
                     Eshift, &w);
    pals_ws_free(&w);
  }
  (void)nthreads;
  free(off); free(toff);
  return bad;
}

int orc_pals_ortho2(double *base, double *coef, const int *nbas, int ndof, int nbloc, const int *ranks, int nitn,
                    int nthreads) {
  int *off = make_offsets(nbas, ndof), *toff = rank_offsets(ranks, nbloc);
  const int bad = pals_ortho2(coef, base, ranks, toff, nbloc, nbas, off, ndof, nitn, nthreads);
  free(off); free(toff);
  return bad;
}

int orc_pals_ortho3(double *base, double *coef, const int *nbas, int ndof, int nbloc, const int *ranks, int nitn,
                    int nthreads) {
  int *off = make_offsets(nbas, ndof), *toff = rank_offsets(ranks, nbloc);
  const int bad = pals_ortho3(coef, base, ranks, toff, nbloc, nbas, off, ndof, nitn, nthreads);
  free(off); free(toff);
  return bad;
}

static int prodhv_any(const double *fobase, const double *focoef, double *base, double *coef, const int *nbas,
                      int ndof, int rF, const int *opid, const int *mptr, const double *Hcoef, const double *mat,
                      int T, int ishift, double Eshift, int nitn, int lowmem) {
  int *off = make_offsets(nbas, ndof);
  hoplist H = {T, ndof, opid, mptr, Hcoef, mat};
  pals_ws w = pals_ws_alloc(rF, rF * T + rF, max_nbas(nbas, ndof));
  const int bad = lowmem == 3
                      ? pals_prodhv3(&H, focoef, fobase, coef, base, rF, nbas, off, ndof, ishift, Eshift, nitn, &w)
                      : pals_prodhv2(&H, focoef, fobase, coef, base, rF, nbas, off, ndof, ishift, Eshift, nitn, &w);
  pals_ws_free(&w);
  free(off);
  return bad;
}

int orc_pals_prodhv2(const double *fobase, const double *focoef, double *base, double *coef, const int *nbas,
                     int ndof, int rF, const int *opid, const int *mptr, const double *Hcoef, const double *mat,
                     int T, int ishift, double Eshift, int nitn) {
  return prodhv_any(fobase, focoef, base, coef, nbas, ndof, rF, opid, mptr, Hcoef, mat, T, ishift, Eshift, nitn, 4);
}

int orc_pals_prodhv3(const double *fobase, const double *focoef, double *base, double *coef, const int *nbas,
                     int ndof, int rF, const int *opid, const int *mptr, const double *Hcoef, const double *mat,
                     int T, int ishift, double Eshift, int nitn) {
  return prodhv_any(fobase, focoef, base, coef, nbas, ndof, rF, opid, mptr, Hcoef, mat, T, ishift, Eshift, nitn, 3);
}

static int update_vecs2(double *base, double *coef, const int *nbas, int ndof, int nbloc, const int *ranks,
                        const double *U, int nitn, int nthreads, int lowmem) {
  int *off = make_offsets(nbas, ndof), *toff = rank_offsets(ranks, nbloc);
  const int nD = off[ndof], nmax = max_nbas(nbas, ndof), rtot = toff[nbloc];
  double *qb = (double *)malloc(sizeof(double) * (size_t)rtot * nD);
  double *qc = (double *)malloc(sizeof(double) * rtot);
  memcpy(qb, base, sizeof(double) * (size_t)rtot * nD);
  memcpy(qc, coef, sizeof(double) * rtot);
  int bad = 0;
#ifdef _OPENMP
  if (nthreads < 1) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads) reduction(+ : bad)
#endif
  for (int v = 0; v < nbloc; ++v) {
    pals_ws w = pals_ws_alloc(ranks[v], rtot, nmax);
    bad += lowmem == 3 ? pals_sumlcvec3(coef + toff[v], base + (size_t)toff[v] * nD, ranks[v], qc, qb, ranks, toff,
                                        nbloc, U + (size_t)v * nbloc, nbas, off, ndof, nitn, &w)
                       : pals_sumlcvec2(coef + toff[v], base + (size_t)toff[v] * nD, ranks[v], qc, qb, ranks, toff,
                                        nbloc, U + (size_t)v * nbloc, nbas, off, ndof, nitn, &w);
    pals_ws_free(&w);
  }
  (void)nthreads;
  free(qb); free(qc); free(off); free(toff);
  return bad;
}

int orc_pals_sumlcvec2(double *base, double *coef, const int *nbas, int ndof, int nbloc, const int *ranks,
                       const double *U, int nitn, int nthreads) {
  return update_vecs2(base, coef, nbas, ndof, nbloc, ranks, U, nitn, nthreads, 4);
}

int orc_pals_sumlcvec3(double *base, double *coef, const int *nbas, int ndof, int nbloc, const int *ranks,
                       const double *U, int nitn, int nthreads) {
  return update_vecs2(base, coef, nbas, ndof, nbloc, ranks, U, nitn, nthreads, 3);
}

/* Diagonalize with intertwining (src/BlockUtils.f90:184-225): GetQHQ3
 * (:309-345: H Q_i by PRODHV_ALS2 with nitn sweeps and no shift, then
 * QHQ(i,j) = <Q_j, H Q_i> for j >= i, OpenMP over i), GetOverlaps (:347-381:
 * S(i,j) = <Q_j, Q_i>, j >= i), SolveGenEigval (src/LinAlg.f90:380-428,
 * DSYGV itype 1 on the upper triangles), then UpdateVecs2 (:479-516):
 * vector i <- ALS_SUMLCVEC_2 fit of sum_l U(l,i) Q_l starting from Q_i.
 * eigv receives the eigenvalues (ascending); U (column-major, column i =
 * eigenvector i, largest-magnitude entry positive) when not NULL.
 * Requires nitn >= 1 (PRODHV_ALS2 returns an undefined H Q_i otherwise).
 * Returns the number of NaN events, or -1 on a failed eigensolve. */
int orc_pals_diagonalize(double *base, double *coef, const int *nbas, int ndof, int nbloc, const int *ranks,
                         const int *opid, const int *mptr, const double *Hcoef, const double *mat, int T, int nitn,
                         int lowmem, double *eigv, double *Uout, int nthreads) {
  if (nitn < 1) return -1;
  int *off = make_offsets(nbas, ndof), *toff = rank_offsets(ranks, nbloc);
  const int nD = off[ndof], nmax = max_nbas(nbas, ndof);
  hoplist H = {T, ndof, opid, mptr, Hcoef, mat};
  double *QHQ = (double *)calloc((size_t)nbloc * nbloc, sizeof(double));
  double *S = (double *)calloc((size_t)nbloc * nbloc, sizeof(double));
  double *U = (double *)malloc(sizeof(double) * (size_t)nbloc * nbloc);
  int bad = 0;
#ifdef _OPENMP
  if (nthreads < 1) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads) reduction(+ : bad)
#endif
  for (int i = 0; i < nbloc; ++i) {
    const int rF = ranks[i];
    pals_ws w = pals_ws_alloc(rF, rF * T, nmax);
    double *hc = (double *)malloc(sizeof(double) * rF);
    double *hb = (double *)malloc(sizeof(double) * (size_t)rF * nD);
    bad += lowmem == 3
               ? pals_prodhv3(&H, coef + toff[i], base + (size_t)toff[i] * nD, hc, hb, rF, nbas, off, ndof, 0, 0.0,
                              nitn, &w)
               : pals_prodhv2(&H, coef + toff[i], base + (size_t)toff[i] * nD, hc, hb, rF, nbas, off, ndof, 0, 0.0,
                              nitn, &w);
    for (int j = i; j < nbloc; ++j)
      QHQ[i + (size_t)j * nbloc] =
          prodvv_ab(coef + toff[j], base + (size_t)toff[j] * nD, ranks[j], hc, hb, rF, nbas, ndof, nD);
    free(hc); free(hb);
    pals_ws_free(&w);
  }
  const int nij = nbloc * (nbloc + 1) / 2;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads)
#endif
  for (int ij = 0; ij < nij; ++ij) {
    int i = 0, rem = ij;
    while (rem >= nbloc - i) { rem -= nbloc - i; ++i; }
    const int j = i + rem;
    S[i + (size_t)j * nbloc] = prodvv_ab(coef + toff[j], base + (size_t)toff[j] * nD, ranks[j], coef + toff[i],
                                         base + (size_t)toff[i] * nD, ranks[i], nbas, ndof, nD);
  }
  (void)nthreads;
  /* DSYGV 'U' reads the upper triangles; the eigensolver here reads lower. */
  for (int j = 0; j < nbloc; ++j)
    for (int i = j + 1; i < nbloc; ++i) {
      QHQ[i + (size_t)j * nbloc] = QHQ[j + (size_t)i * nbloc];
      S[i + (size_t)j * nbloc] = S[j + (size_t)i * nbloc];
    }
  if (orc_sygv(nbloc, QHQ, S, eigv, U) != 0) {
    bad = -1;
  } else {
    if (Uout) memcpy(Uout, U, sizeof(double) * (size_t)nbloc * nbloc);
    bad += update_vecs2(base, coef, nbas, ndof, nbloc, ranks, U, nitn, nthreads, lowmem);
  }
  free(QHQ); free(S); free(U); free(off); free(toff);
  return bad;
}

/* One cycle of Iterate's CPU branch for solver pals (src/Solver.f90:508-538)
 * at lowmem = 4: ALS_POW3 (npow sweeps of H - Eshift, ishift) on vectors
 * nconv..nbloc-1, OpenMP over vectors; ALS_ORTHO_2 (nals sweeps); with
 * update, Diagonalize with intertwining (nals sweeps), which fills eigv.
 * Without update the reference goes on to GetQHQdiag and SortVecs, which
 * the caller applies.  Returns the number of NaN events (the reference
 * aborts on one), or -1 on a failed eigensolve. */
int orc_pals_cycle(double *base, double *coef, const int *nbas, int ndof, int nbloc, const int *ranks, int nconv,
                   const int *opid, const int *mptr, const double *Hcoef, const double *mat, int T, int npow,
                   int nals, int lowmem, int update, int ishift, double Eshift, double *eigv, int nthreads) {
  if (lowmem < 0 || lowmem > 4) return -2;
  int bad = orc_pals_pow(base, coef, nbas, ndof, nbloc, ranks, nconv, opid, mptr, Hcoef, mat, T, npow, ishift, Eshift,
                         lowmem, nthreads);
  if (bad) return bad;
  bad = lowmem == 3 ? orc_pals_ortho3(base, coef, nbas, ndof, nbloc, ranks, nals, nthreads)
                    : orc_pals_ortho2(base, coef, nbas, ndof, nbloc, ranks, nals, nthreads);
  if (bad) return bad;
  if (update)
    bad = orc_pals_diagonalize(base, coef, nbas, ndof, nbloc, ranks, opid, mptr, Hcoef, mat, T, nals, lowmem, eigv,
                               NULL, nthreads);
  return bad;
}

/* ------------------------------------------------------------------ */
/* The Fortran host's plain power solver (solver powr): PowrRecurse,    */
/* GRAMORTHO / pGRAMORTHO, with reduc = reduc_ALS                       */
/* ------------------------------------------------------------------ */

/* PRODHV (src/MODHVECML.f90:50-110): the explicit product (H - E)F of
 * rF (T + [ishift != 0]) terms, term t rF + i = c_i (x) h_{t,m} F_i^m with
 * opcoef(t) in the first mode's factor (HVBaseProd); the shift terms are
 * |E| c_i (x) F_i^m with the sign of -E (ishift > 0) in the first mode's
 * factor (VecScalarMult, VecSignChange, src/MODVECVECML.f90:66-100); with
 * ishift < 0 the H terms change sign instead. */
static void prodhv_explicit(const hoplist *H, const double *fc, const double *fb, int rF, const int *nbas,
                            const int *off, int ndof, int ishift, double E, double *gc, double *gb) {
  const int nD = off[ndof], rFH = rF * H->T, n0 = nbas[0];
  int ik = 0;
  for (int t = 0; t < H->T; ++t)
    for (int i = 0; i < rF; ++i, ++ik) {
      gc[ik] = fc[i];
      for (int d = 0; d < ndof; ++d)
        hv_base_prod(H, t, d, fb + (size_t)i * nD + off[d], gb + (size_t)ik * nD + off[d], nbas[d]);
    }
  if (ishift == 0) return;
  for (int i = 0; i < rF; ++i, ++ik) {
    gc[ik] = fabs(E) * fc[i];
    memcpy(gb + (size_t)ik * nD, fb + (size_t)i * nD, sizeof(double) * nD);
    if (E < 0.0)
      for (int q = 0; q < n0; ++q) gb[(size_t)ik * nD + q] = -gb[(size_t)ik * nD + q];
  }
  const int s0 = ishift > 0 ? rFH : 0, s1 = ishift > 0 ? rFH + rF : rFH;
  for (int r = s0; r < s1; ++r)
    for (int q = 0; q < n0; ++q) gb[(size_t)r * nD + q] = -gb[(size_t)r * nD + q];
}

void orc_prodhv(const double *base, const double *coef, const int *nbas, int ndof, int rF, const int *opid,
                const int *mptr, const double *Hcoef, const double *mat, int T, int ishift, double Eshift,
                double *gbase, double *gcoef) {
  int *off = make_offsets(nbas, ndof);
  hoplist H = {T, ndof, opid, mptr, Hcoef, mat};
  prodhv_explicit(&H, coef, base, rF, nbas, off, ndof, ishift, Eshift, gcoef, gbase);
  free(off);
}

/* PowrRecurse (src/BlockPower.f90:49-73) for more than two modes (redND =
 * ALS): npow times, w = PRODHV(v, ishift 1, E), v <- reduc_ALS of w from v
 * (nloop sweeps; reduc_AB keeps v as the starting guess, its rank being the
 * target rank), NORMCOEF(v).  Returns 1 on a NaN weight. */
int orc_powr_recurse(double *base, double *coef, const int *nbas, int ndof, int rF, const int *opid, const int *mptr,
                     const double *Hcoef, const double *mat, int T, int npow, double Eshift, int nloop) {
  int *off = make_offsets(nbas, ndof);
  const int nD = off[ndof], rG = rF * (T + 1);
  hoplist H = {T, ndof, opid, mptr, Hcoef, mat};
  double *gc = (double *)malloc(sizeof(double) * rG);
  double *gb = (double *)malloc(sizeof(double) * (size_t)rG * nD);
  int bad = 0;
  for (int i = 0; i < npow && !bad; ++i) {
    prodhv_explicit(&H, coef, base, rF, nbas, off, ndof, 1, Eshift, gc, gb);
    bad = orc_reduc_als(gc, gb, rG, coef, base, rF, nbas, ndof, nloop);
    if (!bad) normcoef(coef, base, rF, nbas, off, ndof);
  }
  free(gc); free(gb); free(off);
  return bad;
}

/* GRAMORTHO (src/BlockUtils.f90:22-68, k = 0) and pGRAMORTHO (:72-123,
 * vectors 0..k-1 already orthonormal): for each later vector i, NORMCOEF(Q_i),
 * w_l = -<Q_i, Q_l> (l < i; OpenMP over l), v = Q_i + sum_l w_l Q_l built
 * explicitly (SUMLCVEC: |w_l| in the weights, the sign in the first mode's
 * factor), Q_i <- reduc_ALS of v from Q_i (nloop sweeps), NORMCOEF(Q_i).
 * GRAMORTHO first normalises Q_0.  Returns the number of NaN events. */
int orc_gramortho(double *base, double *coef, const int *nbas, int ndof, int nbloc, const int *ranks, int k,
                  int nloop, int nthreads) {
  int *off = make_offsets(nbas, ndof), *toff = rank_offsets(ranks, nbloc);
  const int nD = off[ndof], n0 = nbas[0], rtot = toff[nbloc];
  double *w = (double *)malloc(sizeof(double) * nbloc);
  double *vc = (double *)malloc(sizeof(double) * rtot);
  double *vb = (double *)malloc(sizeof(double) * (size_t)rtot * nD);
  int bad = 0;
#ifdef _OPENMP
  if (nthreads < 1) nthreads = omp_get_max_threads();
#endif
  (void)nthreads;
  if (k <= 0) {
    normcoef(coef, base, ranks[0], nbas, off, ndof);
    k = 1;
  }
  for (int i = k; i < nbloc && !bad; ++i) {
    double *qc = coef + toff[i], *qb = base + (size_t)toff[i] * nD;
    normcoef(qc, qb, ranks[i], nbas, off, ndof);
    w[i] = 1.0;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
    for (int l = 0; l < i; ++l)
      w[l] = -prodvv_ab(qc, qb, ranks[i], coef + toff[l], base + (size_t)toff[l] * nD, ranks[l], nbas, ndof, nD);
    const int rv = toff[i] + ranks[i];
    for (int l = 0; l <= i; ++l)
      for (int j = 0; j < ranks[l]; ++j) {
        const int r = toff[l] + j;
        vc[r] = fabs(w[l]) * coef[r];
        memcpy(vb + (size_t)r * nD, base + (size_t)r * nD, sizeof(double) * nD);
        if (w[l] < 0.0)
          for (int q = 0; q < n0; ++q) vb[(size_t)r * nD + q] = -vb[(size_t)r * nD + q];
      }
    if (rv > ranks[i]) bad += orc_reduc_als(vc, vb, rv, qc, qb, ranks[i], nbas, ndof, nloop);
    if (!bad) normcoef(qc, qb, ranks[i], nbas, off, ndof);
  }
  free(w); free(vc); free(vb); free(off); free(toff);
  return bad;
}

/* ------------------------------------------------------------------ */
/* ALS_POW0 / ALS_POW1 / ALS_POW2: the power step at lowmem 0, 1, 2     */
/* ------------------------------------------------------------------ */

/* PRODHV1 (src/ALSPow.f90:869-935): the mode-k factors and the weights of
 * the explicit G = (H - E)F rewritten from the current F (term t rF + i:
 * c_i, h_{t,k} F_i^k; shift rows: |E| c_i, F_i^k).  VecScalarMult changes
 * the sign of the shift rows' first-mode factors when E < 0, at every call;
 * at k = 0 the shift rows (ishift > 0) or the H rows (ishift < 0) change
 * sign in the first mode, as PRODHV does. */
static void prodhv1(const hoplist *H, const double *fc, const double *fb, int rF, const int *nbas, const int *off,
                    int ndof, int k, int ishift, double E, double *gc, double *gb) {
  const int nD = off[ndof], rFH = rF * H->T, n = nbas[k], n0 = nbas[0];
  int ik = 0;
  for (int t = 0; t < H->T; ++t)
    for (int i = 0; i < rF; ++i, ++ik) {
      gc[ik] = fc[i];
      hv_base_prod(H, t, k, fb + (size_t)i * nD + off[k], gb + (size_t)ik * nD + off[k], n);
    }
  if (ishift == 0) return;
  for (int i = 0; i < rF; ++i) {
    memcpy(gb + (size_t)(rFH + i) * nD + off[k], fb + (size_t)i * nD + off[k], sizeof(double) * n);
    gc[rFH + i] = fabs(E) * fc[i];
    if (E < 0.0)
      for (int q = 0; q < n0; ++q) gb[(size_t)(rFH + i) * nD + q] = -gb[(size_t)(rFH + i) * nD + q];
  }
  if (k == 0) {
    const int s0 = ishift > 0 ? rFH : 0, s1 = ishift > 0 ? rFH + rF : rFH;
    for (int r = s0; r < s1; ++r)
      for (int q = 0; q < n0; ++q) gb[(size_t)r * nD + q] = -gb[(size_t)r * nD + q];
  }
}

/* bjk(i, ir) = sum_j c_G,j G_j^k(ir) PS(j, i), rows ir, then terms j. */
static void bjk_from_ps(const double *gc, const double *gb, int rG, int nD, int gst, int n, const double *PS, int rF,
                        double *bjk) {
  for (int e = 0; e < rF * n; ++e) bjk[e] = 0.0;
  for (int ir = 0; ir < n; ++ir)
    for (int j = 0; j < rG; ++j) {
      const double gtmp = gc[j] * gb[(size_t)j * nD + gst + ir];
      for (int i = 0; i < rF; ++i) bjk[i + (size_t)ir * rF] += gtmp * PS[j + (size_t)i * rG];
    }
}

/* ALS_POW0 (src/ALSPow.f90:146-290): the explicit G = PRODHV(F) and one
 * Gram (F, F) and one overlap (G, F) per mode; each mode step multiplies the
 * other modes' matrices (modes k+1, k+2, ... cyclically), adds 1e-15 max c_G
 * (the weights of the first G), solves, normalises the weights after the last
 * mode, then rewrites G's mode k from the new F (PRODHV1) and that mode's
 * two matrices (not after the very last step).  Returns 1 on a NaN. */
static int pals_pow0(const hoplist *H, double *coef, double *base, int rF, const int *nbas, const int *off, int ndof,
                     int nitn, int ishift, double Eshift) {
  if (nitn == 0) return 0;
  const int nD = off[ndof], rG = rF * H->T + (ishift != 0 ? rF : 0), nmax = max_nbas(nbas, ndof);
  double *gc = (double *)malloc(sizeof(double) * rG);
  double *gb = (double *)malloc(sizeof(double) * (size_t)rG * nD);
  double *BB = (double *)malloc(sizeof(double) * (size_t)rF * rF * ndof);
  double *PS = (double *)malloc(sizeof(double) * (size_t)rG * rF * ndof);
  double *bjk = (double *)malloc(sizeof(double) * (size_t)rF * nmax);
  int *ipiv = (int *)malloc(sizeof(int) * rF);
  const size_t sb = (size_t)rF * rF, sp = (size_t)rG * rF;
  prodhv_explicit(H, coef, base, rF, nbas, off, ndof, ishift, Eshift, gc, gb);
  const double valpen = maxval(gc, rG) * 1.0e-15;
  for (int d = 1; d < ndof; ++d) {
    for (size_t e = 0; e < sb; ++e) BB[d * sb + e] = 1.0;
    update_bb(base, rF, nD, off[d], nbas[d], BB + d * sb, 0);
    for (size_t e = 0; e < sp; ++e) PS[d * sp + e] = 1.0;
    update_ps(base, rF, gb, rG, nD, off[d], nbas[d], PS + d * sp, 0);
  }
  int bad = 0;
  for (int itn = 0; itn < nitn && !bad; ++itn)
    for (int k = 0; k < ndof; ++k) {
      const int n = nbas[k];
      double *Bk = BB + k * sb, *Pk = PS + k * sp;
      const int k1 = (k + 1) % ndof;
      memcpy(Bk, BB + k1 * sb, sizeof(double) * sb);
      memcpy(Pk, PS + k1 * sp, sizeof(double) * sp);
      for (int l = 2; l < ndof; ++l) {
        const int kp = (k + l) % ndof;
        for (size_t e = 0; e < sb; ++e) Bk[e] = Bk[e] * BB[kp * sb + e];
        for (size_t e = 0; e < sp; ++e) Pk[e] = Pk[e] * PS[kp * sp + e];
      }
      for (int i = 0; i < rF; ++i) Bk[i + (size_t)i * rF] += valpen;
      bjk_from_ps(gc, gb, rG, nD, off[k], n, Pk, rF, bjk);
      lu_solve(Bk, bjk, rF, n, ipiv);
      if (rows_to_mode(coef, base, rF, nD, off[k], bjk, n)) { bad = 1; break; }
      if (k == ndof - 1) {
        const double s = 1 / sqrt(fabs(prodvv_aa(coef, base, rF, nbas, ndof, nD)));
        for (int i = 0; i < rF; ++i) coef[i] = coef[i] * s;
      }
      if (itn < nitn - 1 || k < ndof - 1) {
        prodhv1(H, coef, base, rF, nbas, off, ndof, k, ishift, Eshift, gc, gb);
        for (size_t e = 0; e < sb; ++e) Bk[e] = 1.0;
        update_bb(base, rF, nD, off[k], n, Bk, 0);
        for (size_t e = 0; e < sp; ++e) Pk[e] = 1.0;
        update_ps(base, rF, gb, rG, nD, off[k], n, Pk, 0);
      }
    }
  free(gc); free(gb); free(BB); free(PS); free(bjk); free(ipiv);
  return bad;
}

/* ALS_POW1 (src/ALSPow.f90:294-440): the explicit G = PRODHV(F); with more
 * than three modes BB and PS are kept by dividing mode k out before its step
 * and multiplying the new one back after it, otherwise rebuilt at every step;
 * penalty 1e-15 max c_G (the first G); after each step G's mode k is
 * rewritten from the new F (PRODHV1).  Returns 1 on a NaN. */
static int pals_pow1(const hoplist *H, double *coef, double *base, int rF, const int *nbas, const int *off, int ndof,
                     int nitn, int ishift, double Eshift) {
  if (nitn == 0) return 0;
  const int nD = off[ndof], rG = rF * H->T + (ishift != 0 ? rF : 0), nmax = max_nbas(nbas, ndof);
  const int update = ndof > 3;
  double *gc = (double *)malloc(sizeof(double) * rG);
  double *gb = (double *)malloc(sizeof(double) * (size_t)rG * nD);
  double *BB = (double *)malloc(sizeof(double) * rF * rF);
  double *BBmem = (double *)malloc(sizeof(double) * rF * rF);
  double *PS = (double *)malloc(sizeof(double) * (size_t)rG * rF);
  double *bjk = (double *)malloc(sizeof(double) * (size_t)rF * nmax);
  int *ipiv = (int *)malloc(sizeof(int) * rF);
  prodhv_explicit(H, coef, base, rF, nbas, off, ndof, ishift, Eshift, gc, gb);
  const double valpen = maxval(gc, rG) * 1.0e-15;
  if (update) {
    const_bb(base, rF, nbas, ndof, nD, 0, BBmem);
    const_ps(base, rF, gb, rG, nbas, ndof, nD, 0, PS);
  }
  int kp = -1, bad = 0;
  for (int itn = 0; itn < nitn && !bad; ++itn)
    for (int k = 0; k < ndof; ++k) {
      const int n = nbas[k];
      if (update) {
        if (kp >= 0) {
          update_bb(base, rF, nD, off[k], n, BBmem, 1);
          update_ps(base, rF, gb, rG, nD, off[k], n, PS, 1);
        }
        memcpy(BB, BBmem, sizeof(double) * rF * rF);
      } else {
        const_bb(base, rF, nbas, ndof, nD, k, BB);
        const_ps(base, rF, gb, rG, nbas, ndof, nD, k, PS);
      }
      for (int i = 0; i < rF; ++i) BB[i + (size_t)i * rF] += valpen;
      bjk_from_ps(gc, gb, rG, nD, off[k], n, PS, rF, bjk);
      lu_solve(BB, bjk, rF, n, ipiv);
      bad = rows_to_mode(coef, base, rF, nD, off[k], bjk, n);
      if (k == ndof - 1) {
        const double s = 1 / sqrt(fabs(prodvv_aa(coef, base, rF, nbas, ndof, nD)));
        for (int i = 0; i < rF; ++i) coef[i] = coef[i] * s;
      }
      prodhv1(H, coef, base, rF, nbas, off, ndof, k, ishift, Eshift, gc, gb);
      if (bad) break;
      if (update && (itn < nitn - 1 || k < ndof - 1)) {
        update_bb(base, rF, nD, off[k], n, BBmem, 0);
        update_ps(base, rF, gb, rG, nD, off[k], n, PS, 0);
      }
      kp = k;
    }
  free(gc); free(gb); free(BB); free(BBmem); free(PS); free(bjk); free(ipiv);
  return bad;
}

/* ALS_POW2 (src/ALSPow.f90:444-565): PRODHV_ALS2's update and downdate of
 * BB and PS (UpdateXPS / DowndateXPS with Fold = F), in place, penalty
 * 1e-10 max c_F, the weights normalised after the last mode.  Returns 1 on
 * a NaN. */
static int pals_pow2(const hoplist *H, double *coef, double *base, int rF, const int *nbas, const int *off, int ndof,
                     int nitn, int ishift, double Eshift, pals_ws *w) {
  if (nitn == 0) return 0;
  const int nD = off[ndof];
  const int rG = rF * H->T + (ishift != 0 ? rF : 0);
  const double valpen = maxval(coef, rF) * 1.0e-10;
  const_bb(base, rF, nbas, ndof, nD, 0, w->BBmem);
  for (size_t e = 0; e < (size_t)rG * rF; ++e) w->PS[e] = 1.0;
  for (int k = 0; k < ndof; ++k)
    xps_step(H, coef, base, base, rF, nbas, off, ndof, k, ishift, Eshift, w->PS, NULL, w->T, 0);
  int kp = -1;
  for (int itn = 0; itn < nitn; ++itn)
    for (int k = 0; k < ndof; ++k) {
      const int n = nbas[k];
      if (kp >= 0) update_bb(base, rF, nD, off[k], n, w->BBmem, 1);
      memcpy(w->BB, w->BBmem, sizeof(double) * rF * rF);
      for (int i = 0; i < rF; ++i) w->BB[i + (size_t)i * rF] += valpen;
      xps_step(H, coef, base, base, rF, nbas, off, ndof, k, ishift, Eshift, w->PS, w->bjk, w->T, 1);
      lu_solve(w->BB, w->bjk, rF, n, w->ipiv);
      if (rows_to_mode(coef, base, rF, nD, off[k], w->bjk, n)) return 1;
      if (k == ndof - 1) {
        const double s = 1 / sqrt(fabs(prodvv_aa(coef, base, rF, nbas, ndof, nD)));
        for (int i = 0; i < rF; ++i) coef[i] = coef[i] * s;
      }
      if (itn < nitn - 1 || k < ndof - 1) {
        update_bb(base, rF, nD, off[k], n, w->BBmem, 0);
        xps_step(H, coef, base, base, rF, nbas, off, ndof, k, ishift, Eshift, w->PS, NULL, w->T, 0);
      }
      kp = k;
    }
  return 0;
}

/* ALS_POW_alg (src/ALSPow.f90:83-112) on vectors nconv..nbloc-1, OpenMP over
 * vectors: lowmem 0 ALS_POW0, 1 ALS_POW1, 2 ALS_POW2, 3 and 4 ALS_POW3. */
int orc_pals_pow(double *base, double *coef, const int *nbas, int ndof, int nbloc, const int *ranks, int nconv,
                 const int *opid, const int *mptr, const double *Hcoef, const double *mat, int T, int npow, int ishift,
                 double Eshift, int lowmem, int nthreads) {
  if (lowmem < 0 || lowmem > 4) return -2;
  if (lowmem >= 3)
    return orc_pals_pow3(base, coef, nbas, ndof, nbloc, ranks, nconv, opid, mptr, Hcoef, mat, T, npow, ishift,
                         Eshift, nthreads);
  int *off = make_offsets(nbas, ndof), *toff = rank_offsets(ranks, nbloc);
  const int nD = off[ndof], nmax = max_nbas(nbas, ndof);
  hoplist H = {T, ndof, opid, mptr, Hcoef, mat};
  int bad = 0;
#ifdef _OPENMP
  if (nthreads < 1) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads) reduction(+ : bad)
#endif
  for (int v = nconv < 0 ? 0 : nconv; v < nbloc; ++v) {
    double *c = coef + toff[v], *b = base + (size_t)toff[v] * nD;
    const int r = ranks[v];
    if (lowmem == 0) {
      bad += pals_pow0(&H, c, b, r, nbas, off, ndof, npow, ishift, Eshift);
    } else if (lowmem == 1) {
      bad += pals_pow1(&H, c, b, r, nbas, off, ndof, npow, ishift, Eshift);
    } else {
      pals_ws w = pals_ws_alloc(r, r * T + r, nmax);
      bad += pals_pow2(&H, c, b, r, nbas, off, ndof, npow, ishift, Eshift, &w);
      pals_ws_free(&w);
    }
  }
  (void)nthreads;
  free(off); free(toff);
  return bad;
}
