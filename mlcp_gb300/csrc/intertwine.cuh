// Intertwined power cycle (reference src/intertwining.cu:98, intertw_mvp.cu,
// intertw_lcv.cu): parameter blocks shared by host and device.
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "dword.cuh"

namespace mlcp {

// Operator list prepared once per distinct HopList (cached on the device).
// Per mode d the distinct operators used by any term get local indices
// u = 0..nops_mode[d]-1; u = 0 is always the identity.
struct OpTable {
  int D, T, R;              // modes, terms, vector rank
  int nDp;                  // sum of 4-padded basis sizes
  int npmax;                // max padded basis size
  int umax;                 // max operators in one mode
  int utot;                 // total operators over modes
  const int* nbas;          // [D]
  const int* off;           // [D+1] reference layout offsets
  const int* offp;          // [D+1] padded offsets
  const int* uoff;          // [D+1] first global operator slot of each mode
  const int* uid;           // [T*D] local operator index of term t at mode d
  const unsigned char* ident;  // [utot] 1 if the operator is the identity
  const dw* hdw;            // [utot][npmax][npmax] dense operators in double-word (power sweeps)
  const double* hmat64;     // [utot][npmax][npmax] the same in FP64 (Rayleigh quotients)
  const double* alpha;      // [T] term coefficients
  const int* order;         // [D][T] terms grouped by their operator at mode j
  const int* gstart;        // [D][umax+1] group starts in order[j]
};

// Ragged ranks (an extension; the reference requires equal ranks in a block,
// src/GPUIterate.f90:152-158): a vector of rank r <= R is stored with R terms,
// those beyond r at zero weight.  The fitting kernels keep it a rank-r fit:
// rows and columns >= r of its normal equations are the identity, the same
// rows of its right-hand side the first unit vector (so the solve leaves them
// decoupled and finite), and their weights are set back to zero after every
// solve, so they contribute nothing to any product, overlap or norm.

// Per-vector sweep of ALS-fitted operator applications.
struct OpAlsParams {
  OpTable ops;
  int nvec;
  int nD;
  int mode;           // 0: POW_ALS (F fits (H - E)F in place), 1: PRODHV_ALS (F fits H Fo)
  int nsweeps;
  int ishift;
  double eshift;
  const double* eshift_v;  // per-vector shifts (device) overriding eshift, or null
  double pen_factor;      // penalty = pen_factor * max(Fo weights) (1e-10: the reference's FP64 rule)
  const double* fo_base;  // Fo vectors (reference layout, rank R each, vector v at v*R terms)
  const double* fo_coef;
  double* f_base;         // F output (may alias fo for POW)
  double* f_coef;
  dw* mscr;               // [nvec][utot][R][R] operator Grams M = Fo^T h F
  dw* wscr;               // [nvec][umax][R][R] grouped term products W
  dw* zscr;               // [nvec][umax][R][npmax] h Fo_j
  double* g64;            // [nvec][D][R][R] FP64 Grams of F
  int* status;            // [nvec]
  const int* rank_v;      // [nvec] ranks <= R (terms beyond carry zero weight), or null: all R
  int tabulate;           // set by opals_launch: term/operator tables copied to shared memory
};

int opals_launch(const OpAlsParams& p, cudaStream_t st);
// Smallest shared-memory footprint of the kernel (no resident operators, no tables).
size_t opals_smem_bytes(const OpTable& t);

// ALS-guided Gram-Schmidt over a block (reference src/intertw_lcv.cu:131).
struct GsParams {
  int D, R, nbloc, nD, nDp, npmax, nals;
  const int* nbas;
  const int* off;
  const int* offp;
  double* base;   // block, in place
  double* coef;
  double* work;   // per-CTA scratch for the arrays that do not fit in shared memory (gs_work_doubles)
  int* status;
  const int* rank_v;  // [nbloc] ranks <= R (terms beyond carry zero weight), or null: all R
  int cl;             // CTAs per cluster asked for (0: the 16-CTA rule; see gs_tuned_cluster)
  // set by gs_launch
  int nkmax;             // earlier vectors owned by one CTA, at most
  int gmask;             // array groups placed in global scratch
  long long work_stride; // scratch entries of one CTA
  int ngrp;              // clusters sharing the block (1: one cluster, no grid-wide step)
  dw* xpart;             // [2][ngrp][R * npmax] cluster partial right-hand sides (ngrp > 1)
  unsigned* xctr;        // [0] arrivals of the cluster leaders, [1] abort word; zeroed before the launch (ngrp > 1)
};
int gs_launch(const GsParams& p, cudaStream_t st);
// The measured cluster size for p's block shape (cached per process, device
// and shape; the first call times one sweep per candidate size on a scratch
// copy of the block, scratch_base/scratch_coef of the block's size).  *cl
// receives 0 (the rule) when the search is off or the size is fixed.
int gs_tuned_cluster(const GsParams& p, int device, double* scratch_base, double* scratch_coef, cudaStream_t st,
                     int* cl);
// Appends one line per tuned block shape to out.
void gs_tune_report(std::string& out);
// Doubles of GsParams::work needed for a block of nbloc vectors (npm: the
// largest 4-padded basis size).
size_t gs_work_doubles(int nbloc, int R, int nD, int D, int npm);

// Vector updates (reference VectorUpdates / UPDATES_ALS, src/intertw_lcv.cu:
// 209-304): vector i of the new block is the nals-sweep ALS fit, started from
// Q_i, of sum_k U(k,i) Q_k, weights then divided by its norm; double-word.
struct UpdParams {
  int D, R, B, nD, npmax, nals;
  int tile;               // block terms per shared-memory tile (set by upd_launch)
  int cl;                 // CTAs per output vector (a cluster; set by upd_launch)
  int resident;           // 1: the block overlaps of a CTA's terms in shared memory (set by upd_launch)
  const int* nbas;        // [D] (device)
  const int* off;         // [D+1] reference-layout offsets (device)
  const double* q;        // old block (reference layout)
  const double* qc;
  const double* U;        // [B][B] column-major: U(k, i) = U[k + i B]
  double* qn;             // new block
  double* qnc;
  dw* qdw;                // upd_qdw_dw(B, R, nD): the old block's factors, double-word, mode-major
  dw* work;               // upd_work_dw(B, R, D): per-vector overlaps, Grams, target weights
  double pen_factor;      // penalty = pen_factor * max(weights of Q_i)
  int* status;            // [B] bit 0: non-positive pivot
  const int* rank_v;      // [B] ranks <= R (terms beyond carry zero weight), or null: all R
};
int upd_launch(UpdParams p, int smem_optin, cudaStream_t st);
size_t upd_work_dw(int B, int R, int D);
size_t upd_qdw_dw(int B, int R, int nD);

// Block Rayleigh-Ritz inner products: QHQ(i,j) = <Q_j, HQ_i>, S(i,j) = <Q_j, Q_i>, j <= i.
struct GepParams {
  int D, R, nbloc, nD;
  const int* nbas;
  const double* q_base;
  const double* q_coef;
  const double* hq_base;
  const double* hq_coef;
  double* A;  // [nbloc][nbloc] column-major (lower triangle filled)
  double* S;
  double* eigv;   // [nbloc]
  double* U;      // [nbloc][nbloc] eigenvectors (column-major)
  double* work;   // scratch, see gep_work_doubles
  int* status;
};
int gep_launch(const GepParams& p, cudaStream_t st);
size_t gep_work_doubles(int nbloc);

// Rayleigh quotients <Q_v|H|Q_v>/<Q_v|Q_v> of vectors v0..nvec-1 of a block
// (reference GetQHQdiag / RayleighQuotient2), H applied exactly, FP64.
struct RqParams {
  OpTable ops;
  int v0, nvec, nD;
  const double* base;  // block, reference layout
  const double* coef;
  double* work;        // rq_work_doubles(ops) per vector v0..nvec-1
  double* out;         // [nvec] (entries v0.. written)
  long long work_stride;  // set by rq_launch
};
int rq_launch(const RqParams& p, cudaStream_t st);
size_t rq_work_doubles(const OpTable& t);

// The block's H and overlap matrices with H applied exactly (reference GetQHQ
// and GetOverlaps, src/BlockUtils.f90:229-264, :347-381): A(i, j) =
// <Q_j|H|Q_i>, S(i, j) = <Q_j|Q_i> for i >= j, column-major [nvec][nvec], in
// FP64.  y: the operators applied to every factor (rq_apply_launch).
struct RqPairParams {
  OpTable ops;
  int nvec, nD;
  const double* base;
  const double* coef;
  const double* y;  // [nvec][utot][R][npmax]
  double* A;
  double* S;
};
int rq_apply_launch(const OpTable& t, int nvec, int nD, const double* base, double* y, cudaStream_t st);
int rq_pair_launch(const RqPairParams& p, int smem_optin, cudaStream_t st);

// The generalised eigensolver of the Rayleigh-Ritz step alone, on A and S
// already formed (lower triangles).
int gep_solve_launch(const GepParams& p, cudaStream_t st);

// Two-mode reduction by SVD (reference reduc_SVDa/b, src/REDUCTIONML.f90:
// 296-392): per vector, the nr x nc matrix A of a CP sum is formed, its SVD
// computed, and the leading singular triplets written back as CP terms.
// The input is either K plain CP terms per vector (hv = 0) or the terms of
// (H - shift_v) v for a rank-R two-mode vector v (hv = 1: PRODHV with
// ishift = 1, K = (T + 1) R, operator applications from svd2_apply_launch).
struct Svd2Params {
  int nvec, nr, nc;
  int rout;           // output terms per vector (the reduction rank)
  double redtol;      // singular values below redtol * s_1 are dropped
  int normalize;      // 1: NORMCOEF the result (unit factors, unit norm)
  int K;              // input terms per vector
  const double* in_base;  // hv = 0: [nvec][K][nr + nc], or [K][nr + nc] for every vector (shared_base)
  const double* in_coef;  // hv = 0: [nvec][K]
  int shared_base;        // hv = 0: every vector combines the same K terms with its own weights
  int hv;
  OpTable ops;            // hv = 1: the operator list (D = 2)
  const double* y;        // hv = 1: [nvec][utot][R][npmax] operators applied to v's factors
  const double* v_coef;   // hv = 1: [nvec][R]
  const double* shift;    // hv = 1: [nvec] energy shifts (device)
  double* out_base;       // [nvec][rout][nr + nc]
  double* out_coef;       // [nvec][rout]
  int* out_rank;          // [nvec] terms kept (rest zero), or null
  int* status;            // [nvec] bit 2: the Jacobi sweeps did not converge
  double* work;           // svd2_work_doubles(nr, nc) per vector
};
int svd2_launch(const Svd2Params& p, int smem_optin, cudaStream_t st);
size_t svd2_work_doubles(int nr, int nc);
// y[v][g][r][:] = h_g x_r^d(g) for every operator slot g of a two-mode
// table and term r of vector v (the identity copies).
int svd2_apply_launch(const OpTable& t, int nvec, int nD, const double* base, double* y, cudaStream_t st);

// Divide the weights of each rank-R vector by its norm (FP64).
int normalize_coefs_launch(int nvec, int R, int D, int nD, const int* nbas, const double* base, double* coef,
                           cudaStream_t st);

}  // namespace mlcp
