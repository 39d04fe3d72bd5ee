/*
 * mlcp_gb300 — GB300-native replacement for MLCP's GPU power-iteration path.
 *
 * C ABI.  The first three entry points carry exactly the signatures of the
 * reference's extern "C" layer (src/intertwining.cu:31, :98, :180), which
 * MLCP's Fortran host binds through an implicit interface (gfortran name
 * mangling: lower case plus a trailing underscore; every argument passed by
 * reference, src/GPUIterate.f90:78, :162, :273).  prec_typ is double, as in
 * the shipped build (Makefile:17, src/global.h:9-13).  Fortran LOGICAL
 * arguments are read as one byte (`const bool &`), as the reference does.
 *
 * Unlike the reference, no entry point calls exit() or cudaDeviceReset():
 * errors are recorded and can be read with mlcp_gb300_last_error(); the CUDA
 * context, a device workspace and the uploaded operator list persist across
 * calls.
 *
 * CP-vector layout for all calls (src/cpvector.cu:407-414): term r, mode d,
 * index i at base[r*nD + off_d + i], off_d = sum_{e<d} nbas[e]; coef[r] per
 * term.  Operator lists follow src/hoplist.h:2-7 (1-based opid and mptr,
 * packed upper-triangular symmetric matrices).
 */
#ifndef MLCP_GB300_H
#define MLCP_GB300_H

#include <stddef.h>

#if defined(__GNUC__)
#define MLCP_API __attribute__((visibility("default")))
#else
#define MLCP_API
#endif

#ifdef __cplusplus
#define MLCP_REF(T) const T&
#define MLCP_INOUT(T) T&
extern "C" {
#else
#include <stdbool.h>
#define MLCP_REF(T) const T*
#define MLCP_INOUT(T) T*
#endif

/* Replaces src/intertwining.cu:31 (intwdevicemem_): prints the device memory
 * this implementation needs for one power cycle of the given shape. */
MLCP_API void intwdevicemem_(MLCP_REF(int) rk, MLCP_REF(int) ndof, MLCP_REF(int) nbloc, MLCP_REF(int) TxD,
                    MLCP_REF(int) nops, MLCP_REF(int) msize, MLCP_REF(int) ncpu, MLCP_REF(bool) update,
                    const int *nbas);

/* Replaces src/intertwining.cu:98 (intertwinecpp_): one intertwined power
 * cycle on a block of nbloc vectors of rank rk — npow ALS-fitted applications
 * of (H - Eshift) (sign flipped when ishift < 0; no shift when ishift == 0),
 * ALS-guided Gram-Schmidt, and, when update is true, the block Rayleigh-Ritz
 * problem (eigenvalues to eigv, ascending) followed by ALS-fitted vector
 * updates.  base/coef/eigv are overwritten in place.  ncpu is accepted and
 * ignored: the whole block is processed by batched kernels. */
MLCP_API void intertwinecpp_(double *base, double *coef, int *nbas, MLCP_REF(int) rk, MLCP_REF(int) ndof,
                    MLCP_REF(int) nbloc, int *opid, int *mptr, double *Hcoef, double *mat, MLCP_REF(int) TxD,
                    MLCP_REF(int) nops, MLCP_REF(int) msize, double *eigv, MLCP_REF(int) npow,
                    MLCP_REF(int) ncpu, MLCP_REF(int) nals, MLCP_REF(bool) update, MLCP_REF(int) ishift,
                    MLCP_REF(double) Eshift);

/* Extension beside intertwinecpp_ (no counterpart: the reference requires equal
 * ranks in a block, src/GPUIterate.f90:152-158): the same cycle for a block
 * whose vector v has rank ranks[v] <= rk.  Every vector is stored with rk
 * terms (the layout of intertwinecpp_); terms at or beyond ranks[v] are
 * padding, given zero weight on entry and kept at zero weight, and vector v
 * is fitted as a rank-ranks[v] vector in every stage. */
MLCP_API void intertwineraggedcpp_(double *base, double *coef, int *nbas, MLCP_REF(int) rk, const int *ranks,
                                   MLCP_REF(int) ndof, MLCP_REF(int) nbloc, int *opid, int *mptr, double *Hcoef,
                                   double *mat, MLCP_REF(int) TxD, MLCP_REF(int) nops, MLCP_REF(int) msize,
                                   double *eigv, MLCP_REF(int) npow, MLCP_REF(int) ncpu, MLCP_REF(int) nals,
                                   MLCP_REF(bool) update, MLCP_REF(int) ishift, MLCP_REF(double) Eshift);

/* Replaces src/intertwining.cu:180 (alscpp_): nals ALS sweeps reducing the
 * rank-rG target G (terms rF..rF+rG-1 of coef/base) to the rank-rF vector F
 * (terms 0..rF-1, also the starting guess).  Overwrites terms 0..rF-1. */
MLCP_API void alscpp_(double *coef, double *base, int *nbas, MLCP_REF(int) ndof, MLCP_REF(int) rF, MLCP_REF(int) rG,
             MLCP_REF(int) nals);

/* ---- The update = F path (reference CPU routines, called from the Fortran
 * host through a bind(C) interface) ---------------------------------------- */

/* Replaces GetQHQdiag (src/BlockUtils.f90:385-408) with RayleighQuotient2
 * (:658-688), which the reference's host runs on the CPU after
 * intertwinecpp_ when update is false (src/Solver.f90:499-504):
 * qhqd[i] = <Q_i|H|Q_i> / <Q_i|Q_i> for vectors i = nconv .. nbloc-1 of the
 * block (same layout and operator list as intertwinecpp_), H applied
 * exactly, in FP64 on the GPU.  Entries below nconv are left unchanged. */
MLCP_API void getqhqdiagcpp_(double *base, double *coef, int *nbas, MLCP_REF(int) rk, MLCP_REF(int) ndof,
                             MLCP_REF(int) nbloc, MLCP_REF(int) nconv, int *opid, int *mptr, double *Hcoef,
                             double *mat, MLCP_REF(int) TxD, MLCP_REF(int) nops, MLCP_REF(int) msize,
                             double *qhqd);

/* Replaces GetSpectralRange (src/Solver.f90:563-654): base/coef hold the
 * two starting vectors of rank rk (lower and upper guesses, built by the host
 * as the reference does); ncyc rounds of npow (H - shift) steps -- shift =
 * midpoint of the current bounds for the lower vector, 0 for the upper --
 * each followed by their Rayleigh quotients as the new bounds, all on the
 * GPU.  More than two modes: ALS-fitted steps (ALS_POW_alg).  Two modes:
 * PowrRecurse -- the exact product, its SVD reduction to at most rk terms
 * (redtol 1e-12) and NORMCOEF; the reference starts these vectors at rank 1,
 * so terms past the first carry weight 0, and the result's unused terms are
 * zero.  bounds[2] receives the range padded by 0.1 % of its width on each
 * side; base/coef the final vectors. */
MLCP_API void getspectralrangecpp_(double *base, double *coef, int *nbas, MLCP_REF(int) rk, MLCP_REF(int) ndof,
                                   MLCP_REF(int) npow, MLCP_REF(int) ncyc, int *opid, int *mptr, double *Hcoef,
                                   double *mat, MLCP_REF(int) TxD, MLCP_REF(int) nops, MLCP_REF(int) msize,
                                   double *bounds);

/* Replaces GetQHQ and GetOverlaps (src/BlockUtils.f90:229-264, :347-381) as
 * one call: qhq[i + j*nbloc] = <Q_j|H|Q_i> and s[i + j*nbloc] = <Q_j|Q_i>
 * (full symmetric nbloc x nbloc, column-major, FP64, H applied exactly; s may
 * be NULL), for a block in intertwinecpp_'s layout.  With a one-term operator
 * list it gives the matrix of a product of one-mode operators in the block's
 * basis, which UpdateH/UpdateOperMat (src/Updater.f90:53-151) carry to the
 * next layer of the mode tree. */
MLCP_API void getqhqcpp_(double *base, double *coef, int *nbas, MLCP_REF(int) rk, MLCP_REF(int) ndof,
                         MLCP_REF(int) nbloc, int *opid, int *mptr, double *Hcoef, double *mat, MLCP_REF(int) TxD,
                         MLCP_REF(int) nops, MLCP_REF(int) msize, double *qhq, double *s);

/* Replaces Diagonalize(Q, H, eigv, .FALSE., ...) (src/BlockUtils.f90:184-225),
 * the pre-diagonalisation of the block that the solver runs before its
 * cycles (src/Solver.f90:363-369), on the GPU: A = <Q|H|Q> and S = <Q|Q>
 * with H applied exactly (FP64), the generalised eigenproblem (eigenvalues
 * ascending into eigv), and each vector replaced by the reduction of
 * sum_i U(i, m) Q_i to at most rk terms followed by NORMCOEF: the SVD
 * (redtol 1e-12) for two modes, nals ALS sweeps started from the old Q_m for
 * more (the reference starts from a randomised decomposition; nals = 0
 * keeps the vectors).  Terms the SVD does not need carry weight 0.
 * Same layout and operator list as intertwinecpp_; at most 160 vectors. */
MLCP_API void diagonalizecpp_(double *base, double *coef, int *nbas, MLCP_REF(int) rk, MLCP_REF(int) ndof,
                              MLCP_REF(int) nbloc, int *opid, int *mptr, double *Hcoef, double *mat,
                              MLCP_REF(int) TxD, MLCP_REF(int) nops, MLCP_REF(int) msize, double *eigv,
                              MLCP_REF(int) nals);

/* Replaces UpdateOperMat (src/Updater.f90:110-151) for the nx primitive
 * operators of mode imode (1-based) of the block, on the GPU in FP64:
 * qxq[x] = the nbloc x nbloc matrix <Q_j, X_x Q_i>, each xmats[x] and qxq[x]
 * packed upper-triangular column by column (n(n+1)/2 and
 * nbloc(nbloc+1)/2 entries, back to back), as dspmv('U') reads and
 * SymPackMat2Vec writes them.  UpdateH calls it once per mode with all the
 * operators that the reference passes to UpdateOperMat one at a time. */
MLCP_API void updateopermatcpp_(MLCP_REF(int) imode, double *base, double *coef, int *nbas, MLCP_REF(int) rk,
                                MLCP_REF(int) ndof, MLCP_REF(int) nbloc, MLCP_REF(int) nx, double *xmats,
                                double *qxq);

/* Replaces reduc_SVDa / reduc_SVDb (src/REDUCTIONML.f90:296-392), the
 * reduction of two-mode vectors (reduc with red2D = 'SVD'), batched: each of
 * the nvec vectors of rG terms (base[nvec][rG][nbas[0] + nbas[1]],
 * coef[nvec][rG]) is multiplied out to A = sum_k c_k a_k b_k^T, A's SVD taken
 * (one-sided Jacobi on the GPU: A formed in FP64, sweeps in double-word
 * arithmetic of about 48 bits), and its leading singular triplets
 * written as at most rF terms: obase[nvec][rF][nD], ocoef[nvec][rF] = s_i
 * (mode 1 = U(:, i), mode 2 = V(:, i)), orank[v] = min(nr, nc, rF, ncomp),
 * ncomp = the leading singular values >= redtol * s_1.  Terms past orank[v]
 * are zero.  Limits: min(nr, nc) <= 256, max(nr, nc) <= 4096. */
MLCP_API void reducsvdcpp_(double *base, double *coef, int *nbas, MLCP_REF(int) rG, MLCP_REF(int) nvec,
                           MLCP_REF(int) rF, MLCP_REF(double) redtol, double *obase, double *ocoef, int *orank);

/* Replaces SortVecs (src/BlockUtils.f90:520-583): reorders the block (and
 * eigv alike) by increasing |eigv - Eref|; nconv becomes the position of
 * the first of the first nconv vectors that moved, if any did.  Equal
 * distances keep their order (the reference's dsort leaves ties in an
 * unspecified order).  Host memory only; no GPU work. */
MLCP_API void sortvecscpp_(double *base, double *coef, int *nbas, MLCP_REF(int) rk, MLCP_REF(int) ndof,
                           MLCP_REF(int) nbloc, double *eigv, MLCP_INOUT(int) nconv, MLCP_REF(double) Eref);

/* ---- Extensions (no counterpart in the reference's C layer) ---------- */

/* Message describing the last failure on the calling thread ("" if none). */
MLCP_API const char *mlcp_gb300_last_error(void);

/* Status of the last entry-point call on the calling thread (0 = success). */
MLCP_API int mlcp_gb300_last_status(void);

/* Batched explicit-G ALS on device-resident data: nvec independent
 * reductions with per-vector ranks.  Vector v occupies terms
 * [term_off[v], term_off[v] + rF[v] + rG[v]) of d_coef/d_base: its rF[v]
 * F terms (starting guess, overwritten) followed by its rG[v] target terms.
 * Host arrays: nbas[ndof], rF, rG, term_off [nvec].  stream: a cudaStream_t
 * (NULL = the library's own stream).  Returns 0 or an error code; per-vector
 * numerical flags go to d_status[nvec] when non-NULL (bit 0: a normal-equation
 * matrix was not positive definite; bit 1: an internal pipeline wait timed out
 * and the vector's result is not valid).  Limits: ndof >= 2, rF <= 64,
 * nbas[d] <= 64. */
MLCP_API int mlcp_als_batched(int nvec, int ndof, const int *nbas, const int *rF, const int *rG, const long long *term_off,
                     double *d_coef, double *d_base, int nals, int *d_status, void *stream);

/* Same computation on host buffers, F terms written back in place.  Page-locked
 * mapped arrays (cudaHostAlloc, cudaHostRegister, pinned tensors) are read by
 * the GPU directly: the target terms cross the host link once, inside the
 * FP32 conversion, and only the F terms use device copies.  Other host memory
 * is copied to the device whole.  With a stream the call is asynchronous and
 * the arrays must stay unchanged until the stream reaches the end of the call;
 * with stream NULL it returns when the results are in place. */
MLCP_API int mlcp_als_batched_host(int nvec, int ndof, const int *nbas, const int *rF, const int *rG,
                          const long long *term_off, double *h_coef, double *h_base, int nals, void *stream);

/* Allocation-free explicit-G ALS (no counterpart in the reference): the
 * alscpp_ reduction of one vector held in caller-provided DEVICE buffers
 * (d_coef/d_base in the reference layout: rF F terms, then rG target terms;
 * the F terms are overwritten).  For callers that cannot allocate device
 * memory at call time (a host whose device memory another allocator or pool
 * owns up front, a latency-critical loop that must stay out of the CUDA
 * allocator): all scratch comes from a fixed 32 MiB array inside the library,
 * held by every GPU that loads it.  The first call on a device looks up that
 * array's address.  A call copies a few metadata words from the caller's stack
 * (a pageable copy), so calls are not for stream capture.  Calls share the
 * array: calls whose work overlaps on the GPU race.  Sizes whose scratch
 * exceeds the array return an error; arguments are checked even when
 * nals = 0.  Enqueued on stream (NULL: the legacy default stream).  d_status
 * (required, a device int, cleared by the call) receives bit 0 when a
 * normal-equation matrix was not positive definite and bit 1 when an internal
 * pipeline wait timed out; either bit means the result is not valid. */
MLCP_API int mlcp_als_noalloc(int ndof, const int *nbas, int rF, int rG, double *d_coef, double *d_base, int nals,
                              int *d_status, void *stream);

/* ---- Learned ALS warm start (no counterpart in the reference, whose GPU ALS
 * starts from a random CP vector, GPU_ALS_AA in src/GPUIterate.f90:191-210).
 * Device pointers; stream NULL: the library's stream; each returns a Status.
 * BF16 matrices are row-major with the contracted dimension contiguous. */

/* C[M x N] = A[M x K] B[N x K]^T on the tcgen05 tensor cores (BF16 operands,
 * FP32 accumulation in tensor memory).  M a multiple of 128, N of 16, K of 64,
 * lda/ldb multiples of 8.  Epilogue: x = acc + bias[col] (bias may be NULL);
 * act 0 keeps x, 1 applies max(x, 0), 2 keeps x where mask[row][col] > 0
 * (the ReLU derivative through the forward activations); rows >= valid_m
 * become 0.  Optional outputs C (FP32 [M][ldc]), Cb (BF16 [M][ldcb]), Ct
 * (BF16 transposed, [N][ldct]).  d_status (optional) receives bit 1 if an
 * internal wait timed out (the result is then not valid). */
MLCP_API int mlcp_mlp_gemm(const void *A, const void *B, int M, int N, int K, int lda, int ldb, const float *bias,
                           int act, const void *mask, int ldm, float *C, int ldc, void *Cb, int ldcb, void *Ct,
                           int ldct, int valid_m, int *d_status, void *stream);
/* Mean squared error of Y against T over rows < m, cols < n (both FP32
 * [rows_p][ld]); dY = 2 (Y - T) / (m n) as BF16 [rows_p][ld] and transposed
 * [ld][rows_p] (zero outside the valid block); the loss is added to *loss. */
MLCP_API int mlcp_mlp_loss(const float *Y, const float *T, int m, int n, int ld, int rows_p, void *dY, void *dYt,
                           float *loss, void *stream);
/* db[c] = sum over rows of G[r][c] (BF16 [rows][ld]), c < n. */
MLCP_API int mlcp_mlp_colsum(const void *G, int rows, int n, int ld, float *db, void *stream);
/* One Adam step (bias-corrected, step >= 1) on FP32 parameters w [rows][cols]
 * with gradient g and moments m1, m2; writes the BF16 copy wb and, when wt is
 * not NULL, the transposed BF16 copy [cols][rows]. */
MLCP_API int mlcp_mlp_adam(float *w, const float *g, float *m1, float *m2, int rows, int cols, float lr, float b1,
                           float b2, float eps, int step, void *wb, void *wt, void *stream);
/* Feature rows of a batch of reduction targets (reference layout, every
 * mode of basis size n): row v*ndof + d holds, for the ntop (<= 64)
 * largest-|weight| target terms of vector v (terms d_g_off[v] ..
 * + d_g_rank[v], at most rgmax of them considered), their mode-d factors
 * scaled to unit norm with the largest-magnitude entry positive, then their
 * log10(|c| / |c_max|) / 8.  X: BF16, ldx >= ntop (n + 1). */
MLCP_API int mlcp_ws_features(int nvec, int ndof, int n, int ntop, const long long *d_g_off, const int *d_g_rank,
                              int rgmax, const double *d_base, const double *d_coef, void *X, int ldx, void *stream);
/* Training targets: row v*ndof + d holds, in slot j < rank, the mode-d factor
 * of the term of vector v's reduction (rank terms at d_f_off[v]) that the
 * j-th largest-|weight| target term turned into (greedy matching by the
 * product over modes of the normalised overlaps), unit, with the sign that
 * aligns it with that target term's feature factor.  T: FP32, ldt >= rank n. */
MLCP_API int mlcp_ws_targets(int nvec, int ndof, int n, int rank, const long long *d_g_off, const int *d_g_rank,
                             int rgmax, const long long *d_f_off, const double *d_base, const double *d_coef,
                             float *T, int ldt, void *stream);
/* A proposal: F term j of vector v (at d_f_off[v] + j) gets the normalised
 * slot j of Y's row v*ndof + d (columns j*n ..) as its mode-d factor and the
 * j-th largest |target weight| as its weight. */
MLCP_API int mlcp_ws_apply(int nvec, int ndof, int n, int rank, const long long *d_g_off, const int *d_g_rank,
                           int rgmax, const long long *d_f_off, double *d_base, double *d_coef, const float *Y,
                           int ldy, void *stream);

/* Launch-shape autotuner of the batched ALS (extension; replaces the
 * reference's fixed block-shape rules, PVVkernel::initnew in
 * src/modvecvec.cu:27-94).  Enabled by default (MLCP_GB300_AUTOTUNE=0 in the
 * environment, or enable = 0 here, selects the fixed rule).  The first
 * device-resident reduction of a batch shape times one sweep for every
 * feasible (cluster size, tile-ring depth) pair on the caller's data, F
 * restored after each, and caches the fastest per device and shape; the call
 * synchronises its stream while it tunes.  The same switch covers the power
 * cycle's Gram-Schmidt: the first cycle of a block shape times one sweep with
 * clusters of 16, 12 and 8 CTAs on a scratch copy of the block and keeps the
 * fastest.  The report lists each cached choice with its trial times (lines
 * "als ..." and "gs ..."); returns the report's length. */
MLCP_API void mlcp_gb300_set_autotune(int enable);
MLCP_API int mlcp_gb300_autotune_report(char *buf, int len);

/* Product-pass engine of the batched ALS (extension).  The per-mode dot
 * products of a tile of target terms run either on the CUDA cores (FP32
 * FMAs) or on the tensor cores (one tcgen05 MMA per tile on BF16 three-way
 * splits of both operands, FP32 accumulation; running products held in
 * tensor memory).  0: automatic (the autotuner times both forms among its
 * candidates; without the autotuner the CUDA-core rule applies), 1: CUDA
 * cores only, 2: tensor cores wherever the shape fits (rF <= 32 and the
 * running products of a CTA's terms within 512 tensor-memory columns).
 * MLCP_GB300_ALS_ENGINE=1 or 2 in the environment sets the initial value.
 * Changing it re-tunes shapes on their next call. */
MLCP_API void mlcp_gb300_set_als_engine(int engine);
MLCP_API int mlcp_gb300_als_engine(void);

/* CUDA-graph replay of the power cycle (extension).  intertwinecpp_ and
 * intertwineraggedcpp_ capture the device part of a cycle (POW_ALS,
 * Gram-Schmidt, PRODHV_ALS, Rayleigh-Ritz, vector updates) as a CUDA graph
 * the first time a shape is seen and replay it for later cycles of the same
 * shape (block, ranks, operator table, npow, nals, update, ishift); only the
 * host copies in and out stay outside the graph.  Enabled by default;
 * enable = 0 here, or MLCP_GB300_CYCLE_GRAPH=0, launches the kernels one by
 * one instead.  Results are identical either way. */
MLCP_API void mlcp_gb300_set_cycle_graph(int enable);

/* Kernel timing (extension).  When enabled, the library records CUDA events
 * around its dominant kernel of each call on the call's stream;
 * mlcp_gb300_last_kernel_ms() synchronises on the end event and returns the
 * elapsed milliseconds of the most recent such kernel (negative if none). */
MLCP_API void mlcp_gb300_set_kernel_timing(int enable);
MLCP_API double mlcp_gb300_last_kernel_ms(void);

/* Failure-path self-test (extension): a one-warp kernel sets up the batched
 * ALS kernel's tile ring and waits, with that kernel's bounded wait, for a
 * tile that is never issued.  The wait must give up after its iteration limit
 * (tens of milliseconds); *flags_out receives the status bit the ALS kernel
 * reports for such a vector (2) and the context stays usable.  No GPU fault,
 * trap or hang is involved. */
MLCP_API int mlcp_gb300_wait_selftest(int *flags_out);

/* Full CP inner products out[v] = <X_v, Y_v> for nvec pairs of CP vectors in
 * the reference layout on the device (FP64 arithmetic), used for residuals
 * ||F - G|| = sqrt(<F,F> + <G,G> - 2<F,G>). */
MLCP_API int mlcp_cp_dot_batched(int nvec, int ndof, const int *nbas, const long long *x_off, const int *rx,
                        const long long *y_off, const int *ry, const double *d_coef, const double *d_base,
                        double *d_out, void *stream);

/* Restart files (replace SavePsiFile / ReadPsiFile, src/Restart.f90:614-793;
 * the reference does this I/O in Fortran, so these have no C counterpart).
 * The file is the reference's gfortran unformatted sequential file: records
 * (isavi, nev) | bounds(2) | eigv(nev) | delta(nev), then per vector
 * (ndof, rank) | nbas(ndof) | coef(rank) | base(nD x rank), each framed by
 * its 4-byte length before and after.  Host memory only; no GPU work.
 * ranks[nev]: terms of each vector; coef/base hold the vectors one after the
 * other (sum(ranks) terms, nD = sum(nbas) values per term). */
MLCP_API int mlcp_save_psi(const char *path, int isavi, const double *bounds, int nev, const double *eigv,
                           const double *delta, int ndof, const int *nbas, const int *ranks, const double *coef,
                           const double *base);

/* Reads a restart file written by SavePsiFile or mlcp_save_psi.  As
 * ReadPsiFile, *success = 1 and the caller's isavi, bounds, eigv, delta,
 * ranks, coef and base are replaced only when the whole file was read and
 * its nev, and every vector's ndof and nbas, equal the caller's; otherwise
 * *success = 0 and nothing is changed (a missing file is not an error).
 * max_terms bounds sum(ranks) (the capacity of coef/base in terms); a file
 * with more terms reads as a mismatch. */
MLCP_API int mlcp_read_psi(const char *path, int *isavi, double *bounds, int nev, double *eigv, double *delta,
                           int ndof, const int *nbas, int max_terms, int *ranks, double *coef, double *base,
                           int *success);

#ifdef __cplusplus
}
#endif
#endif
