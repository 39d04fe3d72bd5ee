/*
 * CPU oracle for the MLCP GPU power-iteration hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: tests/, the
 * smoke entry and the CPU-baseline leg of bench.py call it to produce the
 * expected answer.  The product library (libmlcp_gb300.so) never links it.
 *
 * It restates, in plain FP64 C, the algorithm of the reference's CUDA path
 * (src/intertwining.cu, src/als.cu, src/intertw_mvp.cu, src/intertw_lcv.cu,
 * src/modvecvec.cu, src/linalg.cu) with the same loop structure, the same
 * penalty rule and the same normalisations.  Dense solves follow the
 * published LAPACK algorithms the reference calls through cuSOLVER
 * (dgetrf/dgetrs with partial pivoting; dsygvd is replaced by a Cholesky
 * reduction followed by cyclic Jacobi, which yields the same eigenpairs).
 *
 * It also restates the Fortran host's CPU ALS reduction, reduc_ALS
 * (src/REDUCTIONML.f90:593-731), the reference's own CPU implementation of
 * the rank reduction, which the benchmark times as the reference CPU path,
 * and the Fortran host's CPU power solver (solver pals at lowmem 4:
 * ALS_POW3, ALS_ORTHO_2, PRODHV_ALS2, ALS_SUMLCVEC_2), the CPU twin of the
 * GPU power cycle.
 *
 * Pinning: the reference ships no tests, golden vectors or fixtures for
 * this path, and its Fortran host cannot be compiled without a Fortran
 * compiler.  Its CUDA library is built from its own sources on the GPU host
 * (oracle/ref_build.py) and run beside this oracle on the same inputs
 * (tests/test_gpu_reference.py: ALS residuals to 1e-12, one power cycle to
 * 1e-8 relative).  Known-answer tests derived from mathematics (exactly
 * representable reductions, analytically solvable Hamiltonians, a Lanczos
 * reference on the full direct-product basis) cover the host loops.
 *
 * Layout (reference src/cpvector.cu:407-414): a CP vector of rank R over D
 * modes with basis sizes nbas[d] stores term r, mode d, index i at
 * base[r*nD + off_d + i] with off_d = sum_{e<d} nbas[e], nD = off_D, and one
 * weight coef[r] per term.
 */
#ifndef MLCP_ORACLE_H
#define MLCP_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Reference src/intertwining.cu:180 (alscpp_) -> src/als.cu:1021 (ITERATE_ALS).
 * F = first rF terms of (coef, base), G = next rG terms (rG a multiple of rF).
 * Overwrites the first rF terms with the reduced vector. */
void orc_alscpp(double *coef, double *base, const int *nbas, int ndof, int rF, int rG, int nals);

/* Reference src/intertwining.cu:98 (intertwinecpp_): one intertwined power
 * cycle on a block of nbloc vectors of rank rk.  Overwrites base/coef (and
 * eigv when update != 0).  Eigenvectors of the block Rayleigh-Ritz problem
 * are sign-normalised so that their largest-magnitude component is positive. */
void orc_intertwine(double *base, double *coef, const int *nbas, int rk, int ndof, int nbloc,
                    const int *opid, const int *mptr, const double *Hcoef, const double *mat,
                    int TxD, int nops, int msize, double *eigv, int npow, int ncpu, int nals,
                    int update, int ishift, double Eshift);

/* Stages of one cycle, exposed so tests can check each one alone. */
void orc_pow_als_block(double *base, double *coef, const int *nbas, int rk, int ndof, int nbloc,
                       const int *opid, const int *mptr, const double *Hcoef, const double *mat,
                       int T, int npow, int ishift, double Eshift, int nthreads);
void orc_gram_schmidt(double *base, double *coef, const int *nbas, int rk, int ndof, int nbloc, int nals);
/* Fills eigv[nbloc] and U[nbloc*nbloc] (column-major, column i = eigenvector i). */
void orc_gen_eig(const double *base, const double *coef, const int *nbas, int rk, int ndof, int nbloc,
                 const int *opid, const int *mptr, const double *Hcoef, const double *mat, int T,
                 int nals, double *eigv, double *U, int nthreads);
void orc_vector_updates(double *base, double *coef, const int *nbas, int rk, int ndof, int nbloc,
                        const double *U, int nals, int nthreads);

/* Reference src/BlockUtils.f90:658-688 (RayleighQuotient2): <v|H|v>/<v|v>
 * with H applied exactly, term by term. */
double orc_rayleigh_quotient(const double *base, const double *coef, const int *nbas, int rk, int ndof,
                             const int *opid, const int *mptr, const double *Hcoef, const double *mat, int T);
/* Reference src/Updater.f90:110-151 (UpdateOperMat) for nx operators of mode
 * imode (1-based), packed upper-triangular back to back; qxq[x] packed the
 * same way (nbloc x nbloc). */
void orc_update_opermat(int imode, const double *base, const double *coef, const int *nbas, int rk, int ndof,
                        int nbloc, int nx, const double *xmats, double *qxq);
/* Reference src/Solver.f90:563-654 (GetSpectralRange, more than two modes)
 * from the two starting vectors in base/coef (overwritten); padded bounds. */
void orc_spectral_range(double *base, double *coef, const int *nbas, int rk, int ndof, int npow, int ncyc,
                        const int *opid, const int *mptr, const double *Hcoef, const double *mat, int T,
                        double *bounds);
/* Reference src/BlockUtils.f90:385-408 (GetQHQdiag): qhqd[i] for i >= nconv. */
void orc_qhq_diag(const double *base, const double *coef, const int *nbas, int rk, int ndof, int nbloc, int nconv,
                  const int *opid, const int *mptr, const double *Hcoef, const double *mat, int T, double *qhqd,
                  int nthreads);

/* Full inner product <v,w> of two CP vectors (reference src/modvecvec.cu:724
 * constpstot with idof=-1 and both weights, summed). */
double orc_cp_dot(const double *vb, const double *vc, int rv, const double *wb, const double *wc, int rw,
                  const int *nbas, int ndof);

/* Batched explicit-G ALS: nvec independent reductions, OpenMP over vectors. */
void orc_als_batched(int nvec, double *const *coef, double *const *base, const int *nbas, int ndof,
                     const int *rF, const int *rG, int nals, int nthreads);

/* Penalty factor of the normal equations: 1e-10 (reference FP64 build,
 * default) or 1e-5 (reference FP32 build, src/als.cu:248-267).
 * orc_set_penalty_factor sets every stage; orc_set_cycle_penalties sets the
 * power sweeps and H-applications, the Gram-Schmidt and the vector updates of
 * the intertwined cycle separately. */
void orc_set_penalty_factor(double f);
void orc_set_cycle_penalties(double mvp, double gs, double upd);

/* Test knob: round every ALS right-hand side to FP32 before its solve (0 off,
 * the default).  Measures the drift of an FP64 ALS trajectory under
 * FP32-level noise in b, the precision of the GPU's contractions. */
void orc_set_rhs_fp32(int on);

/* Generalised symmetric eigenproblem A x = lambda B x (lower triangles of
 * column-major A, B used).  Eigenvalues ascending; X column-major with
 * X^T B X = I and the largest-magnitude entry of each column positive. */
int orc_sygv(int n, const double *A, const double *B, double *w, double *X);

/* reduc_ALS (src/REDUCTIONML.f90:593-731): F (rF terms, in place) fitted to
 * G (rG terms) by nitn sweeps; penalty 1e-15 max c_G; returns 1 when a
 * weight came out NaN (the reference restarts from a random vector). */
int orc_reduc_als(const double *gcoef, const double *gbase, int rG, double *fcoef, double *fbase, int rF,
                  const int *nbas, int ndof, int nitn);
/* The same over independent vectors, OpenMP over vectors (nthreads < 1: all);
 * returns the number of vectors that hit a NaN weight. */
int orc_reduc_als_batched(int nvec, const double *const *gcoef, const double *const *gbase, const int *rG,
                          double *const *fcoef, double *const *fbase, const int *rF, const int *nbas, int ndof,
                          int nitn, int nthreads);

/* The Fortran host's CPU power cycle, solver pals at lowmem 4 (the _2
 * forms of the Gram-Schmidt, H-application and updates) or lowmem 3 (the
 * least-memory _3 forms) (src/Solver.f90:508-538).  A block holds nbloc vectors; vector v has
 * ranks[v] terms, stored after the terms of vectors 0..v-1 (ragged blocks
 * are allowed, as in ALS_ORTHO_2's ranks table).  Each call returns the
 * number of NaN weights met (the reference aborts on one); the
 * diagonalisation and the cycle return -1 when the eigensolve fails. */
/* ALS_POW3 (src/ALSPow.f90:569-660) on vectors nconv..nbloc-1, OpenMP over vectors. */
int orc_pals_pow3(double *base, double *coef, const int *nbas, int ndof, int nbloc, const int *ranks, int nconv,
                  const int *opid, const int *mptr, const double *Hcoef, const double *mat, int T, int npow,
                  int ishift, double Eshift, int nthreads);
/* ALS_POW_alg (src/ALSPow.f90:83-112): lowmem 0 ALS_POW0, 1 ALS_POW1,
 * 2 ALS_POW2, 3 and 4 ALS_POW3; -2 for another lowmem. */
int orc_pals_pow(double *base, double *coef, const int *nbas, int ndof, int nbloc, const int *ranks, int nconv,
                 const int *opid, const int *mptr, const double *Hcoef, const double *mat, int T, int npow, int ishift,
                 double Eshift, int lowmem, int nthreads);
/* ALS_ORTHO_2 (src/ALSUtils.f90:156-377) and ALS_ORTHO_3 (:381-528). */
int orc_pals_ortho2(double *base, double *coef, const int *nbas, int ndof, int nbloc, const int *ranks, int nitn,
                    int nthreads);
int orc_pals_ortho3(double *base, double *coef, const int *nbas, int ndof, int nbloc, const int *ranks, int nitn,
                    int nthreads);
/* PRODHV_ALS2 (src/ALSPow.f90:664-780): (base, coef) <- ALS fit of
 * (H - Eshift) Fo, rF terms, starting from Fo. */
int orc_pals_prodhv2(const double *fobase, const double *focoef, double *base, double *coef, const int *nbas,
                     int ndof, int rF, const int *opid, const int *mptr, const double *Hcoef, const double *mat,
                     int T, int ishift, double Eshift, int nitn);
/* PRODHV_ALS3 (src/ALSPow.f90:784-865), the same fit without PS. */
int orc_pals_prodhv3(const double *fobase, const double *focoef, double *base, double *coef, const int *nbas,
                     int ndof, int rF, const int *opid, const int *mptr, const double *Hcoef, const double *mat,
                     int T, int ishift, double Eshift, int nitn);
/* UpdateVecs2 (src/BlockUtils.f90:479-516) with ALS_SUMLCVEC_2
 * (src/ALSUtils.f90:731-891): vector v <- fit of sum_l U[v*nbloc + l] Q_l. */
int orc_pals_sumlcvec2(double *base, double *coef, const int *nbas, int ndof, int nbloc, const int *ranks,
                       const double *U, int nitn, int nthreads);
/* The same with ALS_SUMLCVEC_3 (src/ALSUtils.f90:895-1045). */
int orc_pals_sumlcvec3(double *base, double *coef, const int *nbas, int ndof, int nbloc, const int *ranks,
                       const double *U, int nitn, int nthreads);
/* Diagonalize with intertwining (src/BlockUtils.f90:184-225): GetQHQ3,
 * GetOverlaps, SolveGenEigval (upper triangles), UpdateVecs2.  U (optional)
 * receives the eigenvectors, column-major. */
int orc_pals_diagonalize(double *base, double *coef, const int *nbas, int ndof, int nbloc, const int *ranks,
                         const int *opid, const int *mptr, const double *Hcoef, const double *mat, int T, int nitn,
                         int lowmem, double *eigv, double *U, int nthreads);
/* One cycle: ALS_POW_alg, ALS_ORTHO_alg and, with update, the
 * diagonalisation, for lowmem 0-4 (else -2): the _3 forms at lowmem 3, the
 * _2 forms otherwise (the dispatchers' choice). */
int orc_pals_cycle(double *base, double *coef, const int *nbas, int ndof, int nbloc, const int *ranks, int nconv,
                   const int *opid, const int *mptr, const double *Hcoef, const double *mat, int T, int npow,
                   int nals, int lowmem, int update, int ishift, double Eshift, double *eigv, int nthreads);

/* PRODHV (src/MODHVECML.f90:50-110): the explicit (H - Eshift) F, rF T
 * terms (plus rF with a shift) into gbase/gcoef. */
void orc_prodhv(const double *base, const double *coef, const int *nbas, int ndof, int rF, const int *opid,
                const int *mptr, const double *Hcoef, const double *mat, int T, int ishift, double Eshift,
                double *gbase, double *gcoef);
/* The plain power solver (solver powr), reductions by reduc_ALS (more than
 * two modes).  PowrRecurse (src/BlockPower.f90:49-73) on one vector of rF
 * terms. */
int orc_powr_recurse(double *base, double *coef, const int *nbas, int ndof, int rF, const int *opid, const int *mptr,
                     const double *Hcoef, const double *mat, int T, int npow, double Eshift, int nloop);
/* GRAMORTHO (src/BlockUtils.f90:22-68) for k = 0, pGRAMORTHO (:72-123)
 * with vectors 0..k-1 already orthonormal. */
int orc_gramortho(double *base, double *coef, const int *nbas, int ndof, int nbloc, const int *ranks, int k,
                  int nloop, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
