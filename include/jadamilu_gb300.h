/*
 * jadamilu_gb300.h -- C ABI of the GB300 Jacobi-Davidson library.
 *
 * The driver entry points are drop-in replacements for the JADAMILU
 * Fortran drivers: same symbol names (gfortran decoration: lower case plus
 * a trailing underscore), every argument by reference, 1-based indices,
 * the same argument lists, ICNTL/IPRINT/INFO meaning and reverse-
 * communication protocol.  Each declaration cites the reference routine it
 * replaces; the C prototypes of the reference are in
 * src/include/jadamilu1.h:22-118 and the Fortran argument documentation in
 * src/jd/PJD.F and Doc/DPJD_prototypes.f.
 *
 * Integers are 32-bit (the reference's default INTEGER).  Complex arrays are
 * interleaved (re, im) doubles, i.e. COMPLEX*16.
 *
 * Extensions beyond the reference:
 *   ICNTL(5) = 2 stores the preconditioner in bfloat16 (float32 arithmetic);
 *   jdgpu_* entry points expose single kernels for testing and set options.
 */
#ifndef JADAMILU_GB300_H
#define JADAMILU_GB300_H

#ifdef __cplusplus
#include <complex>
typedef std::complex<double> jdg_zcomplex;
typedef std::complex<float> jdg_ccomplex;
#define JDG_API __attribute__((visibility("default")))
extern "C" {
#else
typedef struct { double re, im; } jdg_zcomplex;
typedef struct { float re, im; } jdg_ccomplex;
#define JDG_API
#endif

/* DPJD: replaces PJD_EV (src/jd/PJD.F:5-262) for real symmetric A.
 * Built-in matvec and built-in multilevel ILDL preconditioner. */
JDG_API void dpjd_(int* N, double* A, int* JA, int* IA, double* EIGS, double* RES, double* X, int* LX, int* NEIG,
                   double* SIGMA, int* ISEARCH, int* NINIT, int* MADSPACE, int* ITER, double* TOL, double* SHIFT,
                   double* DROPTOL, double* MEM, int* ICNTL, int* IPRINT, int* INFO, double* GAP);

/* DPJDREVCOM: replaces PJDREVCOM_EV (src/jd/PJD.F:268-362).  Returns with
 * IJOB=1 for X(NDX2) = A*X(NDX1); IJOB=0 when done. */
JDG_API void dpjdrevcom_(int* N, double* A, int* JA, int* IA, double* EIGS, double* RES, double* X, int* LX,
                         int* NEIG, double* SIGMA, int* ISEARCH, int* NINIT, int* MADSPACE, int* ITER, double* TOL,
                         double* SHIFT, double* DROPTOL, double* MEM, int* ICNTL, int* IJOB, int* NDX1, int* NDX2,
                         int* IPRINT, int* INFO, double* GAP);

/* DJDREVCOM: replaces JDREVCOM_EV (src/jd/PJD.F:369-429).  IJOB=1: matvec
 * X(NDX2) = A*X(NDX1); IJOB=2: preconditioner solve Prec*X(NDX1) = X(NDX2). */
JDG_API void djdrevcom_(int* N, double* EIGS, double* RES, double* X, int* LX, int* NEIG, double* SIGMA, int* ISEARCH,
                        int* NINIT, int* MADSPACE, int* ITER, double* TOL, int* IJOB, int* NDX1, int* NDX2,
                        int* IPRINT, int* INFO, double* GAP);

/* DPJD_GEP: replaces PJD_GEP (src/jd/PJD.F:492-572), A x = lambda B x, B SPD. */
JDG_API void dpjd_gep_(int* N, double* A, int* JA, int* IA, double* B, int* JB, int* IB, double* EIGS, double* RES,
                       double* X, int* LX, int* NEIG, double* SIGMA, int* ISEARCH, int* NINIT, int* MADSPACE,
                       int* ITER, double* TOL, double* SHIFT, double* DROPTOL, double* MEM, int* ICNTL, int* IPRINT,
                       int* INFO, double* GAP);

/* DPJDREVCOM_GEP: replaces PJDREVCOM_GEP (src/jd/PJD.F:576-705).  IJOB=1:
 * X(NDX2)=A*X(NDX1) and X(NDX3)=B*X(NDX1); 3: A only; 4: B only. */
JDG_API void dpjdrevcom_gep_(int* N, double* A, int* JA, int* IA, double* B, int* JB, int* IB, double* EIGS,
                             double* RES, double* X, int* LX, int* NEIG, double* SIGMA, int* ISEARCH, int* NINIT,
                             int* MADSPACE, int* ITER, double* TOL, double* SHIFT, double* DROPTOL, double* MEM,
                             int* ICNTL, int* IJOB, int* NDX1, int* NDX2, int* NDX3, int* IPRINT, int* INFO,
                             double* GAP);

/* DJDREVCOM_GEP: replaces JDREVCOM_GEP (src/jd/PJD.F:709-798). */
JDG_API void djdrevcom_gep_(int* N, double* EIGS, double* RES, double* X, int* LX, int* NEIG, double* SIGMA,
                            int* ISEARCH, int* NINIT, int* MADSPACE, int* ITER, double* TOL, int* IJOB, int* NDX1,
                            int* NDX2, int* NDX3, int* IPRINT, int* INFO, double* GAP);

/* DPJDCLEANUP: replaces PJDCLEANUP_EV (src/jd/PJD.F:435-488). */
JDG_API void dpjdcleanup_(void);

/* Legacy drivers PJD, PJDREVCOM, JDREVCOM, PJDCLEANUP (src/jd/PJD_compatible.f:
 * 3-106): the real drivers above with ICNTL(5) forced to 0; ICNTL(1..4) are
 * passed through and copied back. */
JDG_API void pjd_(int* N, double* A, int* JA, int* IA, double* EIGS, double* RES, double* X, int* LX, int* NEIG,
                  double* SIGMA, int* ISEARCH, int* NINIT, int* MADSPACE, int* ITER, double* TOL, double* SHIFT,
                  double* DROPTOL, double* MEM, int* ICNTL, int* IPRINT, int* INFO, double* GAP);
JDG_API void pjdrevcom_(int* N, double* A, int* JA, int* IA, double* EIGS, double* RES, double* X, int* LX, int* NEIG,
                        double* SIGMA, int* ISEARCH, int* NINIT, int* MADSPACE, int* ITER, double* TOL, double* SHIFT,
                        double* DROPTOL, double* MEM, int* ICNTL, int* IJOB, int* NDX1, int* NDX2, int* IPRINT,
                        int* INFO, double* GAP);
JDG_API void jdrevcom_(int* N, double* EIGS, double* RES, double* X, int* LX, int* NEIG, double* SIGMA, int* ISEARCH,
                       int* NINIT, int* MADSPACE, int* ITER, double* TOL, int* IJOB, int* NDX1, int* NDX2, int* IPRINT,
                       int* INFO, double* GAP);
JDG_API void pjdcleanup_(void);

/* Complex Hermitian versions (ZPJD & co.), same argument meaning with
 * COMPLEX*16 A, B and X (reference C prototypes jadamilu1.h:68-118). */
JDG_API void zpjd_(int* N, jdg_zcomplex* A, int* JA, int* IA, double* EIGS, double* RES, jdg_zcomplex* X, int* LX,
                   int* NEIG, double* SIGMA, int* ISEARCH, int* NINIT, int* MADSPACE, int* ITER, double* TOL,
                   double* SHIFT, double* DROPTOL, double* MEM, int* ICNTL, int* IPRINT, int* INFO, double* GAP);
JDG_API void zpjdrevcom_(int* N, jdg_zcomplex* A, int* JA, int* IA, double* EIGS, double* RES, jdg_zcomplex* X,
                         int* LX, int* NEIG, double* SIGMA, int* ISEARCH, int* NINIT, int* MADSPACE, int* ITER,
                         double* TOL, double* SHIFT, double* DROPTOL, double* MEM, int* ICNTL, int* IJOB, int* NDX1,
                         int* NDX2, int* IPRINT, int* INFO, double* GAP);
JDG_API void zjdrevcom_(int* N, double* EIGS, double* RES, jdg_zcomplex* X, int* LX, int* NEIG, double* SIGMA,
                        int* ISEARCH, int* NINIT, int* MADSPACE, int* ITER, double* TOL, int* IJOB, int* NDX1,
                        int* NDX2, int* IPRINT, int* INFO, double* GAP);
JDG_API void zpjd_gep_(int* N, jdg_zcomplex* A, int* JA, int* IA, jdg_zcomplex* B, int* JB, int* IB, double* EIGS,
                       double* RES, jdg_zcomplex* X, int* LX, int* NEIG, double* SIGMA, int* ISEARCH, int* NINIT,
                       int* MADSPACE, int* ITER, double* TOL, double* SHIFT, double* DROPTOL, double* MEM, int* ICNTL,
                       int* IPRINT, int* INFO, double* GAP);
JDG_API void zpjdrevcom_gep_(int* N, jdg_zcomplex* A, int* JA, int* IA, jdg_zcomplex* B, int* JB, int* IB,
                             double* EIGS, double* RES, jdg_zcomplex* X, int* LX, int* NEIG, double* SIGMA,
                             int* ISEARCH, int* NINIT, int* MADSPACE, int* ITER, double* TOL, double* SHIFT,
                             double* DROPTOL, double* MEM, int* ICNTL, int* IJOB, int* NDX1, int* NDX2, int* NDX3,
                             int* IPRINT, int* INFO, double* GAP);
JDG_API void zjdrevcom_gep_(int* N, double* EIGS, double* RES, jdg_zcomplex* X, int* LX, int* NEIG, double* SIGMA,
                            int* ISEARCH, int* NINIT, int* MADSPACE, int* ITER, double* TOL, int* IJOB, int* NDX1,
                            int* NDX2, int* NDX3, int* IPRINT, int* INFO, double* GAP);
JDG_API void zpjdcleanup_(void);

/* ---- single-kernel entry points (host arrays in and out) ---- */

/* Single-precision drivers: SPJD, SPJD_GEP, SPJDREVCOM, SPJDREVCOM_GEP,
 * SJDREVCOM, SJDREVCOM_GEP, SPJDCLEANUP (Doc/SPJD_prototypes.f:3-798) and
 * CPJD ... CPJDCLEANUP (Doc/CPJD_prototypes.f:3-798), which the reference
 * builds from src/jd/PJD.F with _SINGLE_REAL_ / _SINGLE_COMPLEX_
 * (src/include/ilupackmacros.h:379-400).  Arguments and protocol as the
 * double drivers above with REAL (COMPLEX) values.  The iteration runs in
 * double precision on widened copies of the caller's arrays, with the results
 * rounded back; reverse-communication requests convert only their vectors.
 * They share the double drivers' state: an S (C) and a D (Z) reverse-
 * communication solve cannot be in flight together.  The ILP64 library
 * (jadamilu_gb300_ilp64.h) has them with 64-bit integers. */
JDG_API void spjd_(int* N, float* A, int* JA, int* IA, float* EIGS, float* RES, float* X, int* LX, int* NEIG,
                   float* SIGMA, int* ISEARCH, int* NINIT, int* MADSPACE, int* ITER, float* TOL, float* SHIFT,
                   float* DROPTOL, float* MEM, int* ICNTL, int* IPRINT, int* INFO, float* GAP);
JDG_API void spjd_gep_(int* N, float* A, int* JA, int* IA, float* B, int* JB, int* IB, float* EIGS, float* RES,
                       float* X, int* LX, int* NEIG, float* SIGMA, int* ISEARCH, int* NINIT, int* MADSPACE, int* ITER,
                       float* TOL, float* SHIFT, float* DROPTOL, float* MEM, int* ICNTL, int* IPRINT, int* INFO,
                       float* GAP);
JDG_API void spjdrevcom_(int* N, float* A, int* JA, int* IA, float* EIGS, float* RES, float* X, int* LX, int* NEIG,
                         float* SIGMA, int* ISEARCH, int* NINIT, int* MADSPACE, int* ITER, float* TOL, float* SHIFT,
                         float* DROPTOL, float* MEM, int* ICNTL, int* IJOB, int* NDX1, int* NDX2, int* IPRINT,
                         int* INFO, float* GAP);
JDG_API void spjdrevcom_gep_(int* N, float* A, int* JA, int* IA, float* B, int* JB, int* IB, float* EIGS, float* RES,
                             float* X, int* LX, int* NEIG, float* SIGMA, int* ISEARCH, int* NINIT, int* MADSPACE,
                             int* ITER, float* TOL, float* SHIFT, float* DROPTOL, float* MEM, int* ICNTL, int* IJOB,
                             int* NDX1, int* NDX2, int* NDX3, int* IPRINT, int* INFO, float* GAP);
JDG_API void sjdrevcom_(int* N, float* EIGS, float* RES, float* X, int* LX, int* NEIG, float* SIGMA, int* ISEARCH,
                        int* NINIT, int* MADSPACE, int* ITER, float* TOL, int* IJOB, int* NDX1, int* NDX2, int* IPRINT,
                        int* INFO, float* GAP);
JDG_API void sjdrevcom_gep_(int* N, float* EIGS, float* RES, float* X, int* LX, int* NEIG, float* SIGMA, int* ISEARCH,
                            int* NINIT, int* MADSPACE, int* ITER, float* TOL, int* IJOB, int* NDX1, int* NDX2,
                            int* NDX3, int* IPRINT, int* INFO, float* GAP);
JDG_API void spjdcleanup_(void);
JDG_API void cpjd_(int* N, jdg_ccomplex* A, int* JA, int* IA, float* EIGS, float* RES, jdg_ccomplex* X, int* LX,
                   int* NEIG, float* SIGMA, int* ISEARCH, int* NINIT, int* MADSPACE, int* ITER, float* TOL,
                   float* SHIFT, float* DROPTOL, float* MEM, int* ICNTL, int* IPRINT, int* INFO, float* GAP);
JDG_API void cpjd_gep_(int* N, jdg_ccomplex* A, int* JA, int* IA, jdg_ccomplex* B, int* JB, int* IB, float* EIGS,
                       float* RES, jdg_ccomplex* X, int* LX, int* NEIG, float* SIGMA, int* ISEARCH, int* NINIT,
                       int* MADSPACE, int* ITER, float* TOL, float* SHIFT, float* DROPTOL, float* MEM, int* ICNTL,
                       int* IPRINT, int* INFO, float* GAP);
JDG_API void cpjdrevcom_(int* N, jdg_ccomplex* A, int* JA, int* IA, float* EIGS, float* RES, jdg_ccomplex* X, int* LX,
                         int* NEIG, float* SIGMA, int* ISEARCH, int* NINIT, int* MADSPACE, int* ITER, float* TOL,
                         float* SHIFT, float* DROPTOL, float* MEM, int* ICNTL, int* IJOB, int* NDX1, int* NDX2,
                         int* IPRINT, int* INFO, float* GAP);
JDG_API void cpjdrevcom_gep_(int* N, jdg_ccomplex* A, int* JA, int* IA, jdg_ccomplex* B, int* JB, int* IB,
                             float* EIGS, float* RES, jdg_ccomplex* X, int* LX, int* NEIG, float* SIGMA, int* ISEARCH,
                             int* NINIT, int* MADSPACE, int* ITER, float* TOL, float* SHIFT, float* DROPTOL,
                             float* MEM, int* ICNTL, int* IJOB, int* NDX1, int* NDX2, int* NDX3, int* IPRINT,
                             int* INFO, float* GAP);
JDG_API void cjdrevcom_(int* N, float* EIGS, float* RES, jdg_ccomplex* X, int* LX, int* NEIG, float* SIGMA,
                        int* ISEARCH, int* NINIT, int* MADSPACE, int* ITER, float* TOL, int* IJOB, int* NDX1,
                        int* NDX2, int* IPRINT, int* INFO, float* GAP);
JDG_API void cjdrevcom_gep_(int* N, float* EIGS, float* RES, jdg_ccomplex* X, int* LX, int* NEIG, float* SIGMA,
                            int* ISEARCH, int* NINIT, int* MADSPACE, int* ITER, float* TOL, int* IJOB, int* NDX1,
                            int* NDX2, int* NDX3, int* IPRINT, int* INFO, float* GAP);
JDG_API void cpjdcleanup_(void);

/* Number of visible CUDA devices (0 without a GPU). */
JDG_API int jdgpu_device_count(void);

/* y = A x on the GPU for A stored like DPJD's A/JA/IA; replaces one call of
 * MATVECA (src/jd/JDaux.F:3397-3418).  Returns 0 or -1 on a CUDA error. */
JDG_API int jdgpu_dspmv(int n, const int* ia, const int* ja, const double* a, const double* x, double* y);
JDG_API int jdgpu_zspmv(int n, const int* ia, const int* ja, const jdg_zcomplex* a, const jdg_zcomplex* x,
                        jdg_zcomplex* y);

/* Factor A - shift*I with the host ILDLC and apply it on the GPU to nrhs
 * right-hand sides; replaces SYMILUPACKFACTOR + SYMILUPACKSOL /
 * SINGLESYMILUPACKSOL (src/ilupack/symilupacksol.c:60-128,
 * singlesymilupacksol.c:69-104).  spd != 0 applies |D| (SYMSPDCONVERT).
 * precision: 0 float64, 1 float32 (ICNTL(5)=1), 2 bfloat16 storage.
 * info (5 entries, may be NULL): nnz(L), negative pivots, levels, forward
 * and backward schedule depth.  Returns 0, a factorisation error code, or
 * -99 on a CUDA error. */
JDG_API int jdgpu_dildl_apply(int n, const int* ia, const int* ja, const double* a, double shift, double droptol,
                              double condest, int spd, int precision, int nrhs, const double* b, double* x,
                              long* info);

/* Time `reps` GPU applications of the factor of A - shift*I (inputs resident
 * on the device, CUDA events).  out (8): ms per application, nnz(L),
 * forward depth, backward depth, kernels per application, factor seconds,
 * rows of the tail (dense inverse or single-CTA levels), upload seconds
 * (includes the tail inverse). */
JDG_API int jdgpu_dildl_bench(int n, const int* ia, const int* ja, const double* a, double shift, double droptol,
                              double condest, int spd, int precision, int reps, double* out);

/* Device-resident mode (no reference counterpart; used for repeated solves
 * and timing): upload A once, let dpjd_ reuse it and keep eigenvectors on the
 * device, until jdgpu_drelease_matrix(). */
JDG_API int jdgpu_dprepare_matrix(int n, const int* ia, const int* ja, const double* a);
JDG_API void jdgpu_drelease_matrix(void);
JDG_API void jdgpu_dmatrix_info(long* out);

/* Run on the caller's CUDA stream (a cudaStream_t); NULL: the library's own. */
JDG_API void jdgpu_set_stream(void* stream);

/* Kernels launched by the library so far (graph replays count their nodes). */
JDG_API long long jdgpu_launch_count(void);

/* Timing of the last real (d) or complex (z) solve's preconditioner and of
 * SpMV with its matrix, on the solver stream (no reference counterpart;
 * measurement only).  precond out: ms per application, bytes streamed,
 * nnz(L), rows in dense blocks, kernels per application, algorithmic bytes;
 * spmv out: ms per SpMV, algorithmic bytes, nnz, stored entries.  -1: no
 * factor (or matrix) on the device. */
JDG_API int jdgpu_dprecond_bench(int reps, double* out);
JDG_API int jdgpu_dspmv_bench(int reps, double* out);
JDG_API int jdgpu_zprecond_bench(int reps, double* out);
JDG_API int jdgpu_zspmv_bench(int reps, double* out);

/* Copy out the host factor of the last real solve (CPU comparison runs). */
JDG_API int jdgpu_dfactor_export(int* n_out, long long* nnz_out, double* shift_out, int* perm, long long* lp, int* li,
                                 double* lx, signed char* blk, double* dinv, double* doff, double* ainv,
                                 double* aoff);
/* Its level structure (level_start: nlev + 1 elimination steps) and, when
 * coupling_out is 1, the coupling blocks F of its multilevel form as CSR over
 * elimination steps (fp: n + 1 entries, fi/fx: nnzf).  With level_start NULL
 * only the sizes are written.  No reference counterpart (measurement only). */
JDG_API int jdgpu_dfactor_export_levels(int* coupling_out, int* nlev_out, long long* nnzf_out, int* level_start,
                                        long long* fp, int* fi, double* fx);

/* jdgpu_dildl_apply without allocating GPU memory.  No counterpart in the
 * reference.  For callers that cannot call cudaMalloc: applications whose GPU
 * memory is owned by another allocator (a framework's caching pool that must
 * see every byte) or that fix their device-memory budget at start-up and
 * treat any later allocation as an error.  The factor, the staging vectors
 * and the work vector live in one fixed 32 MiB device array compiled into
 * this library (every GPU that loads it keeps those 32 MiB until the process
 * exits); problems that do not fit are rejected with -98 before any kernel
 * runs.  Nothing in the array has to start at zero: each call writes every
 * byte it later reads.  Every call looks the array's address up
 * (cudaGetSymbolAddress) with the caller's device current; the first lookup
 * on a device may load the library's device code, so make the first call on
 * each device before any stream capture.  All calls share the one array:
 * calls that overlap on the GPU race and must not be issued.  Arguments,
 * results and other error codes as jdgpu_dildl_apply. */
JDG_API int jdgpu_dildl_apply_noalloc(int n, const int* ia, const int* ja, const double* a, double shift,
                                      double droptol, double condest, int spd, int precision, int nrhs,
                                      const double* b, double* x, long* info);

/* Gradient of f = sum_k w[k] * lambda_k with respect to every stored entry
 * of A, for eigenpairs of A x = lambda B x (B = I, or B diagonal with its
 * diagonal in bdiag; NULL for B = I).  ia/ja: the one-triangle CSR of A as
 * passed to DPJD / DPJD_GEP (1-based; the order DPJD leaves the entries in
 * is fine).  X: the eigenvectors, n x neig column-major with leading
 * dimension ldx (DPJD's X), any scaling.  grad[q] for stored entry q (i, j):
 * sum_k w_k x_k(i) x_k(j) / (x_k^T B x_k), doubled off the diagonal since the
 * entry stands for a_ij and a_ji (Hellmann-Feynman; B held fixed).  For a
 * cluster of equal eigenvalues give the whole cluster one weight.  An
 * extension with no counterpart in the reference.  neig <= 64.  Returns 0,
 * -1 on bad arguments, -99 on a CUDA error. */
JDG_API int jdgpu_deig_grad(int n, const int* ia, const int* ja, int neig, const double* X, int ldx,
                            const double* w, const double* bdiag, double* grad);

/* Gradient of a loss L(x) of one eigenvector with respect to every stored
 * entry of A: x an eigenvector of A x = lambda B x (B = I, or diagonal with
 * diagonal bdiag; NULL for I), any scale; g = dL/dx at x scaled to
 * x^T B x = 1.  The adjoint mu solves P^T (A - lambda B) P mu = P^T g with
 * P = I - x x^T B (mu B-orthogonal to x) by preconditioned MINRES on the GPU,
 * reusing the SpMV and the ILDLC preconditioner (factor of A - lambda B with
 * DROPTOL droptol, |D| form); stopping at residual tol (relative) or maxit
 * iterations.  grad[q] for stored entry q (i, j): -(mu_i x_j + mu_j x_i), and
 * -mu_i x_i on the diagonal (B held fixed; lambda simple).  out (2, may be
 * NULL): iterations, relative residual.  An extension with no counterpart in
 * the reference.  Returns 0, a factorisation error code, -1 on bad arguments,
 * or -99 on a CUDA error. */
JDG_API int jdgpu_deigvec_grad(int n, const int* ia, const int* ja, const double* a, const double* bdiag,
                               double lambda, const double* x, const double* g, double droptol, double tol,
                               int maxit, double* grad, double* out);

/* Batched DPJD: nprob independent real symmetric problems solved by
 * nworkers host threads, each with its own solver state and CUDA stream, so
 * several solves run on the GPU at once; problems are taken largest first.
 * Per problem q (arrays of pointers / values indexed by q), as in DPJD:
 * n[q], a[q]/ja[q]/ia[q] (modified as by DPJD), eigs[q], res[q], x[q] (LX =
 * lx[q] entries), neig[q] (in: wanted, out: converged), iter[q] (in: MATVEC
 * budget, out: used), info[q], gap[q] (may be NULL).  Shared: sigma,
 * isearch, madspace, tol, droptol, mem and icntl (ICNTL(2) is taken as 0:
 * every problem gets its own preconditioner).  No NINIT, no printing.
 * Extension for the batched configuration; the drop-in drivers keep the
 * reference's one-solve-per-process state.  Returns 0, or -1 on bad
 * arguments. */
JDG_API int jdgpu_dpjd_batch(int nprob, const int* n, double* const* a, int* const* ja, int* const* ia,
                             double* const* eigs, double* const* res, double* const* x, const int* lx, int* neig,
                             int* iter, int* info, double* gap, double sigma, int isearch, int madspace, double tol,
                             double droptol, double mem, const int* icntl, int nworkers);

/* Options: "depth_weight" (ordering key weight of the triangular-solve
 * depth, default 64), "verbose", "dense_tail" (1: solve the deepest levels of
 * the preconditioner with the explicit inverse of their block, default; 0:
 * level by level in one CTA), "dense_max" (most rows of that block, default
 * 32768), "dense_min_saving" (modelled seconds per application the dense
 * blocks must save to be used, default 1e-4), "drop_schur" (drop tolerance of the Schur-complement fill; negative:
 * DROPTOL/10), "apply_graph" (1: jdgpu_dildl_apply replays the captured CUDA
 * graph of the application, as the eigensolver does), "fuse_inner" (1,
 * default: with the built-in matvec the inner CG/sQMR iteration keeps its
 * scalars on the device and synchronises once per iteration, same arithmetic;
 * 0: one synchronisation per scalar), "revcom_device" (1: reverse-
 * communication requests on device pointers, see jdgpu_revcom_device_ptr),
 * "matching" (1: the first level of the factor takes its pivot and dropping
 * decisions in the symmetric scale of a maximum-product matching, the role of
 * the reference's MC64 step; 2: also pivots the matching's 2-cycles of that
 * level as 2x2 blocks first; default 0, the level's max-norm equilibration).
 * Factor form for matrices of at least "coupled_min_n" rows (default 4096),
 * in solves with ISEARCH at least "large_form_isearch" (default 2: interior
 * eigenvalues; the factor-only and gradient entry points count as 2):
 * "coupling" (0, default: one global L, one sweep each way; 1: each level
 * keeps its own L and is coupled to the later levels through the block F of
 * its matrix, applied with two B-solves per level as ILUPACK's multilevel
 * solve, about two thirds of the memory), "drop_rule" (1,
 * default: drop an L entry by its largest Schur-complement contribution; 0:
 * by |l_ik| times the inverse estimate), "lookahead" (1, default: defer a
 * pivot whose column would raise a neighbour's inverse estimate above
 * CONDEST), "last_droptol" (drop tolerance of the last level, default 0: no
 * dropping; negative: DROPTOL) and "last_fill" (a later level whose matrix is
 * at least this full becomes the last level, default 1/3).  "factor_verbose"
 * (1: one line per factor level and per uploaded sub-factor on stderr).
 * "plan_launch_us" (default 4) and "plan_tile_gbs" (default 5000): the cost
 * of one launch and the streaming rate the apply planner weighs when it
 * chooses which runs of sweep levels become dense tiles.  "tri_cluster" (8,
 * default, or 16): CTAs per thread-block cluster of the dense-block tile
 * product for factors uploaded after the call (16 only where the device
 * runs clusters of that size; otherwise 8).  "dense_min_rows" (default
 * 8192): a factor level at least a quarter full is eliminated densely from
 * this many rows on.
 * They apply to factors computed, and solves started, after the call. */
JDG_API void jdgpu_set_option(const char* name, double value);

/* Device-pointer reverse communication (no reference counterpart; extends
 * DPJDREVCOM / DJDREVCOM and their _GEP and Z forms, src/jd/PJD.F:268-429,
 * 576-798, for GPU-resident user operators).  With
 * jdgpu_set_option("revcom_device", 1) before a solve starts (IJOB = 0), its
 * requests are served on the device copy of X instead of the caller's X:
 * after a return with IJOB = 1, 2, 3 or 4, jdgpu_revcom_device_ptr gives the
 * device address XD of X(1) and the solver's CUDA stream; the request reads
 * XD[NDX1-1 ...] (IJOB 1, 3, 4) or XD[NDX2-1 ...] (IJOB 2) and writes
 * XD[NDX2-1 ...], XD[NDX3-1 ...] (B x, GEP) or XD[NDX1-1 ...] (IJOB 2), N
 * entries each, exactly as the host protocol does with X.  The input vectors
 * are complete when the driver returns; the caller's results must be complete
 * when it calls the driver again (work enqueued on the returned stream
 * counts).  The caller's X receives the eigenvectors at the end as usual; it
 * holds no request vectors in between.  Returns 0, or -1 when no solve of
 * that arithmetic (complex_ 0: real, 1: complex) is waiting on a
 * device-mode request. */
JDG_API int jdgpu_revcom_device_ptr(int complex_, void** xd, void** stream);

/* Statistics of the last real (d) or complex (z) solve (12 doubles): factor
 * seconds, upload seconds, preconditioner applications, matvecs, levels,
 * forward depth, backward depth, nnz(L), fill, factorisations, rows of the
 * current device factor solved by dense blocks (or the single-CTA tail), and
 * the number of those blocks.  jdgpu_reset_stats clears the counters and
 * times of both. */
JDG_API void jdgpu_dstats(double* out);
JDG_API void jdgpu_zstats(double* out);
JDG_API void jdgpu_reset_stats(void);

#ifdef __cplusplus
}
#endif
#endif
