/*
 * jadamilu_gb300_ilp64.h -- the drivers of jadamilu_gb300.h with 64-bit
 * integers (libjadamilu_gb300_ilp64.so).
 *
 * The reference builds an ILP64 variant in which every Fortran INTEGER is
 * 8 bytes (src/include/long_integer.h:1-18, makefile.includeINT64YGNU:37,48,
 * gfortran -fdefault-integer-8).  This library exports the same symbols with
 * every integer argument as a 64-bit integer; arguments, ICNTL/IPRINT/INFO
 * meaning and the reverse-communication protocol are those of
 * jadamilu_gb300.h.  N, the nonzero counts and LX must fit in 32 bits (the
 * kernels index with 32-bit integers); larger values return INFO = -1.
 * Reverse communication: as in the reference, only one solve per driver may
 * be in flight, and the caller passes every argument back unchanged.
 * The jdgpu_* extensions of this library keep the 32-bit signatures of
 * jadamilu_gb300.h.
 */
#ifndef JADAMILU_GB300_ILP64_H
#define JADAMILU_GB300_ILP64_H

#include <stdint.h>

#ifdef __cplusplus
#include <complex>
typedef std::complex<double> jdg64_zcomplex;
typedef std::complex<float> jdg64_ccomplex;
#define JDG64_API __attribute__((visibility("default")))
extern "C" {
#else
typedef struct { double re, im; } jdg64_zcomplex;
typedef struct { float re, im; } jdg64_ccomplex;
#define JDG64_API
#endif

typedef int64_t jdg_i8;

/* DPJD (src/jd/PJD.F:5-262), DPJD_GEP (PJD.F:492-572). */
JDG64_API void dpjd_(jdg_i8* N, double* A, jdg_i8* JA, jdg_i8* IA, double* EIGS, double* RES, double* X, jdg_i8* LX,
                     jdg_i8* NEIG, double* SIGMA, jdg_i8* ISEARCH, jdg_i8* NINIT, jdg_i8* MADSPACE, jdg_i8* ITER,
                     double* TOL, double* SHIFT, double* DROPTOL, double* MEM, jdg_i8* ICNTL, jdg_i8* IPRINT,
                     jdg_i8* INFO, double* GAP);
JDG64_API void dpjd_gep_(jdg_i8* N, double* A, jdg_i8* JA, jdg_i8* IA, double* B, jdg_i8* JB, jdg_i8* IB,
                         double* EIGS, double* RES, double* X, jdg_i8* LX, jdg_i8* NEIG, double* SIGMA,
                         jdg_i8* ISEARCH, jdg_i8* NINIT, jdg_i8* MADSPACE, jdg_i8* ITER, double* TOL, double* SHIFT,
                         double* DROPTOL, double* MEM, jdg_i8* ICNTL, jdg_i8* IPRINT, jdg_i8* INFO, double* GAP);
/* DPJDREVCOM (PJD.F:268-362), DPJDREVCOM_GEP (PJD.F:576-705). */
JDG64_API void dpjdrevcom_(jdg_i8* N, double* A, jdg_i8* JA, jdg_i8* IA, double* EIGS, double* RES, double* X,
                           jdg_i8* LX, jdg_i8* NEIG, double* SIGMA, jdg_i8* ISEARCH, jdg_i8* NINIT, jdg_i8* MADSPACE,
                           jdg_i8* ITER, double* TOL, double* SHIFT, double* DROPTOL, double* MEM, jdg_i8* ICNTL,
                           jdg_i8* IJOB, jdg_i8* NDX1, jdg_i8* NDX2, jdg_i8* IPRINT, jdg_i8* INFO, double* GAP);
JDG64_API void dpjdrevcom_gep_(jdg_i8* N, double* A, jdg_i8* JA, jdg_i8* IA, double* B, jdg_i8* JB, jdg_i8* IB,
                               double* EIGS, double* RES, double* X, jdg_i8* LX, jdg_i8* NEIG, double* SIGMA,
                               jdg_i8* ISEARCH, jdg_i8* NINIT, jdg_i8* MADSPACE, jdg_i8* ITER, double* TOL,
                               double* SHIFT, double* DROPTOL, double* MEM, jdg_i8* ICNTL, jdg_i8* IJOB, jdg_i8* NDX1,
                               jdg_i8* NDX2, jdg_i8* NDX3, jdg_i8* IPRINT, jdg_i8* INFO, double* GAP);
/* DJDREVCOM (PJD.F:369-429), DJDREVCOM_GEP (PJD.F:709-798). */
JDG64_API void djdrevcom_(jdg_i8* N, double* EIGS, double* RES, double* X, jdg_i8* LX, jdg_i8* NEIG, double* SIGMA,
                          jdg_i8* ISEARCH, jdg_i8* NINIT, jdg_i8* MADSPACE, jdg_i8* ITER, double* TOL, jdg_i8* IJOB,
                          jdg_i8* NDX1, jdg_i8* NDX2, jdg_i8* IPRINT, jdg_i8* INFO, double* GAP);
JDG64_API void djdrevcom_gep_(jdg_i8* N, double* EIGS, double* RES, double* X, jdg_i8* LX, jdg_i8* NEIG,
                              double* SIGMA, jdg_i8* ISEARCH, jdg_i8* NINIT, jdg_i8* MADSPACE, jdg_i8* ITER,
                              double* TOL, jdg_i8* IJOB, jdg_i8* NDX1, jdg_i8* NDX2, jdg_i8* NDX3, jdg_i8* IPRINT,
                              jdg_i8* INFO, double* GAP);
/* DPJDCLEANUP (PJD.F:435-488). */
JDG64_API void dpjdcleanup_(void);

/* Complex Hermitian drivers (jadamilu1.h:68-118), COMPLEX*16 A, B and X. */
JDG64_API void zpjd_(jdg_i8* N, jdg64_zcomplex* A, jdg_i8* JA, jdg_i8* IA, double* EIGS, double* RES,
                     jdg64_zcomplex* X, jdg_i8* LX, jdg_i8* NEIG, double* SIGMA, jdg_i8* ISEARCH, jdg_i8* NINIT,
                     jdg_i8* MADSPACE, jdg_i8* ITER, double* TOL, double* SHIFT, double* DROPTOL, double* MEM,
                     jdg_i8* ICNTL, jdg_i8* IPRINT, jdg_i8* INFO, double* GAP);
JDG64_API void zpjd_gep_(jdg_i8* N, jdg64_zcomplex* A, jdg_i8* JA, jdg_i8* IA, jdg64_zcomplex* B, jdg_i8* JB,
                         jdg_i8* IB, double* EIGS, double* RES, jdg64_zcomplex* X, jdg_i8* LX, jdg_i8* NEIG,
                         double* SIGMA, jdg_i8* ISEARCH, jdg_i8* NINIT, jdg_i8* MADSPACE, jdg_i8* ITER, double* TOL,
                         double* SHIFT, double* DROPTOL, double* MEM, jdg_i8* ICNTL, jdg_i8* IPRINT, jdg_i8* INFO,
                         double* GAP);
JDG64_API void zpjdrevcom_(jdg_i8* N, jdg64_zcomplex* A, jdg_i8* JA, jdg_i8* IA, double* EIGS, double* RES,
                           jdg64_zcomplex* X, jdg_i8* LX, jdg_i8* NEIG, double* SIGMA, jdg_i8* ISEARCH, jdg_i8* NINIT,
                           jdg_i8* MADSPACE, jdg_i8* ITER, double* TOL, double* SHIFT, double* DROPTOL, double* MEM,
                           jdg_i8* ICNTL, jdg_i8* IJOB, jdg_i8* NDX1, jdg_i8* NDX2, jdg_i8* IPRINT, jdg_i8* INFO,
                           double* GAP);
JDG64_API void zpjdrevcom_gep_(jdg_i8* N, jdg64_zcomplex* A, jdg_i8* JA, jdg_i8* IA, jdg64_zcomplex* B, jdg_i8* JB,
                               jdg_i8* IB, double* EIGS, double* RES, jdg64_zcomplex* X, jdg_i8* LX, jdg_i8* NEIG,
                               double* SIGMA, jdg_i8* ISEARCH, jdg_i8* NINIT, jdg_i8* MADSPACE, jdg_i8* ITER,
                               double* TOL, double* SHIFT, double* DROPTOL, double* MEM, jdg_i8* ICNTL, jdg_i8* IJOB,
                               jdg_i8* NDX1, jdg_i8* NDX2, jdg_i8* NDX3, jdg_i8* IPRINT, jdg_i8* INFO, double* GAP);
JDG64_API void zjdrevcom_(jdg_i8* N, double* EIGS, double* RES, jdg64_zcomplex* X, jdg_i8* LX, jdg_i8* NEIG,
                          double* SIGMA, jdg_i8* ISEARCH, jdg_i8* NINIT, jdg_i8* MADSPACE, jdg_i8* ITER, double* TOL,
                          jdg_i8* IJOB, jdg_i8* NDX1, jdg_i8* NDX2, jdg_i8* IPRINT, jdg_i8* INFO, double* GAP);
JDG64_API void zjdrevcom_gep_(jdg_i8* N, double* EIGS, double* RES, jdg64_zcomplex* X, jdg_i8* LX, jdg_i8* NEIG,
                              double* SIGMA, jdg_i8* ISEARCH, jdg_i8* NINIT, jdg_i8* MADSPACE, jdg_i8* ITER,
                              double* TOL, jdg_i8* IJOB, jdg_i8* NDX1, jdg_i8* NDX2, jdg_i8* NDX3, jdg_i8* IPRINT,
                              jdg_i8* INFO, double* GAP);
JDG64_API void zpjdcleanup_(void);

/* Single-precision drivers (Doc/SPJD_prototypes.f:3-798, Doc/CPJD_prototypes.f:3-798) with 64-bit
 * integers; REAL / COMPLEX values as in jadamilu_gb300.h's spjd_ ... cpjdcleanup_. */
JDG64_API void spjd_(jdg_i8* N, float* A, jdg_i8* JA, jdg_i8* IA, float* EIGS, float* RES, float* X, jdg_i8* LX,
                     jdg_i8* NEIG, float* SIGMA, jdg_i8* ISEARCH, jdg_i8* NINIT, jdg_i8* MADSPACE, jdg_i8* ITER,
                     float* TOL, float* SHIFT, float* DROPTOL, float* MEM, jdg_i8* ICNTL, jdg_i8* IPRINT,
                     jdg_i8* INFO, float* GAP);
JDG64_API void spjd_gep_(jdg_i8* N, float* A, jdg_i8* JA, jdg_i8* IA, float* B, jdg_i8* JB, jdg_i8* IB,
                         float* EIGS, float* RES, float* X, jdg_i8* LX, jdg_i8* NEIG, float* SIGMA,
                         jdg_i8* ISEARCH, jdg_i8* NINIT, jdg_i8* MADSPACE, jdg_i8* ITER, float* TOL, float* SHIFT,
                         float* DROPTOL, float* MEM, jdg_i8* ICNTL, jdg_i8* IPRINT, jdg_i8* INFO, float* GAP);
JDG64_API void spjdrevcom_(jdg_i8* N, float* A, jdg_i8* JA, jdg_i8* IA, float* EIGS, float* RES, float* X,
                           jdg_i8* LX, jdg_i8* NEIG, float* SIGMA, jdg_i8* ISEARCH, jdg_i8* NINIT, jdg_i8* MADSPACE,
                           jdg_i8* ITER, float* TOL, float* SHIFT, float* DROPTOL, float* MEM, jdg_i8* ICNTL,
                           jdg_i8* IJOB, jdg_i8* NDX1, jdg_i8* NDX2, jdg_i8* IPRINT, jdg_i8* INFO, float* GAP);
JDG64_API void spjdrevcom_gep_(jdg_i8* N, float* A, jdg_i8* JA, jdg_i8* IA, float* B, jdg_i8* JB, jdg_i8* IB,
                               float* EIGS, float* RES, float* X, jdg_i8* LX, jdg_i8* NEIG, float* SIGMA,
                               jdg_i8* ISEARCH, jdg_i8* NINIT, jdg_i8* MADSPACE, jdg_i8* ITER, float* TOL,
                               float* SHIFT, float* DROPTOL, float* MEM, jdg_i8* ICNTL, jdg_i8* IJOB, jdg_i8* NDX1,
                               jdg_i8* NDX2, jdg_i8* NDX3, jdg_i8* IPRINT, jdg_i8* INFO, float* GAP);
JDG64_API void sjdrevcom_(jdg_i8* N, float* EIGS, float* RES, float* X, jdg_i8* LX, jdg_i8* NEIG, float* SIGMA,
                          jdg_i8* ISEARCH, jdg_i8* NINIT, jdg_i8* MADSPACE, jdg_i8* ITER, float* TOL, jdg_i8* IJOB,
                          jdg_i8* NDX1, jdg_i8* NDX2, jdg_i8* IPRINT, jdg_i8* INFO, float* GAP);
JDG64_API void sjdrevcom_gep_(jdg_i8* N, float* EIGS, float* RES, float* X, jdg_i8* LX, jdg_i8* NEIG,
                              float* SIGMA, jdg_i8* ISEARCH, jdg_i8* NINIT, jdg_i8* MADSPACE, jdg_i8* ITER,
                              float* TOL, jdg_i8* IJOB, jdg_i8* NDX1, jdg_i8* NDX2, jdg_i8* NDX3, jdg_i8* IPRINT,
                              jdg_i8* INFO, float* GAP);
JDG64_API void spjdcleanup_(void);

JDG64_API void cpjd_(jdg_i8* N, jdg64_ccomplex* A, jdg_i8* JA, jdg_i8* IA, float* EIGS, float* RES,
                     jdg64_ccomplex* X, jdg_i8* LX, jdg_i8* NEIG, float* SIGMA, jdg_i8* ISEARCH, jdg_i8* NINIT,
                     jdg_i8* MADSPACE, jdg_i8* ITER, float* TOL, float* SHIFT, float* DROPTOL, float* MEM,
                     jdg_i8* ICNTL, jdg_i8* IPRINT, jdg_i8* INFO, float* GAP);
JDG64_API void cpjd_gep_(jdg_i8* N, jdg64_ccomplex* A, jdg_i8* JA, jdg_i8* IA, jdg64_ccomplex* B, jdg_i8* JB,
                         jdg_i8* IB, float* EIGS, float* RES, jdg64_ccomplex* X, jdg_i8* LX, jdg_i8* NEIG,
                         float* SIGMA, jdg_i8* ISEARCH, jdg_i8* NINIT, jdg_i8* MADSPACE, jdg_i8* ITER, float* TOL,
                         float* SHIFT, float* DROPTOL, float* MEM, jdg_i8* ICNTL, jdg_i8* IPRINT, jdg_i8* INFO,
                         float* GAP);
JDG64_API void cpjdrevcom_(jdg_i8* N, jdg64_ccomplex* A, jdg_i8* JA, jdg_i8* IA, float* EIGS, float* RES,
                           jdg64_ccomplex* X, jdg_i8* LX, jdg_i8* NEIG, float* SIGMA, jdg_i8* ISEARCH, jdg_i8* NINIT,
                           jdg_i8* MADSPACE, jdg_i8* ITER, float* TOL, float* SHIFT, float* DROPTOL, float* MEM,
                           jdg_i8* ICNTL, jdg_i8* IJOB, jdg_i8* NDX1, jdg_i8* NDX2, jdg_i8* IPRINT, jdg_i8* INFO,
                           float* GAP);
JDG64_API void cpjdrevcom_gep_(jdg_i8* N, jdg64_ccomplex* A, jdg_i8* JA, jdg_i8* IA, jdg64_ccomplex* B, jdg_i8* JB,
                               jdg_i8* IB, float* EIGS, float* RES, jdg64_ccomplex* X, jdg_i8* LX, jdg_i8* NEIG,
                               float* SIGMA, jdg_i8* ISEARCH, jdg_i8* NINIT, jdg_i8* MADSPACE, jdg_i8* ITER,
                               float* TOL, float* SHIFT, float* DROPTOL, float* MEM, jdg_i8* ICNTL, jdg_i8* IJOB,
                               jdg_i8* NDX1, jdg_i8* NDX2, jdg_i8* NDX3, jdg_i8* IPRINT, jdg_i8* INFO, float* GAP);
JDG64_API void cjdrevcom_(jdg_i8* N, float* EIGS, float* RES, jdg64_ccomplex* X, jdg_i8* LX, jdg_i8* NEIG,
                          float* SIGMA, jdg_i8* ISEARCH, jdg_i8* NINIT, jdg_i8* MADSPACE, jdg_i8* ITER, float* TOL,
                          jdg_i8* IJOB, jdg_i8* NDX1, jdg_i8* NDX2, jdg_i8* IPRINT, jdg_i8* INFO, float* GAP);
JDG64_API void cjdrevcom_gep_(jdg_i8* N, float* EIGS, float* RES, jdg64_ccomplex* X, jdg_i8* LX, jdg_i8* NEIG,
                              float* SIGMA, jdg_i8* ISEARCH, jdg_i8* NINIT, jdg_i8* MADSPACE, jdg_i8* ITER,
                              float* TOL, jdg_i8* IJOB, jdg_i8* NDX1, jdg_i8* NDX2, jdg_i8* NDX3, jdg_i8* IPRINT,
                              jdg_i8* INFO, float* GAP);
JDG64_API void cpjdcleanup_(void);

/* Legacy PJD, PJDREVCOM, JDREVCOM, PJDCLEANUP (src/jd/PJD_compatible.f:3-106). */
JDG64_API void pjd_(jdg_i8* N, double* A, jdg_i8* JA, jdg_i8* IA, double* EIGS, double* RES, double* X, jdg_i8* LX,
                    jdg_i8* NEIG, double* SIGMA, jdg_i8* ISEARCH, jdg_i8* NINIT, jdg_i8* MADSPACE, jdg_i8* ITER,
                    double* TOL, double* SHIFT, double* DROPTOL, double* MEM, jdg_i8* ICNTL, jdg_i8* IPRINT,
                    jdg_i8* INFO, double* GAP);
JDG64_API void pjdrevcom_(jdg_i8* N, double* A, jdg_i8* JA, jdg_i8* IA, double* EIGS, double* RES, double* X,
                          jdg_i8* LX, jdg_i8* NEIG, double* SIGMA, jdg_i8* ISEARCH, jdg_i8* NINIT, jdg_i8* MADSPACE,
                          jdg_i8* ITER, double* TOL, double* SHIFT, double* DROPTOL, double* MEM, jdg_i8* ICNTL,
                          jdg_i8* IJOB, jdg_i8* NDX1, jdg_i8* NDX2, jdg_i8* IPRINT, jdg_i8* INFO, double* GAP);
JDG64_API void jdrevcom_(jdg_i8* N, double* EIGS, double* RES, double* X, jdg_i8* LX, jdg_i8* NEIG, double* SIGMA,
                         jdg_i8* ISEARCH, jdg_i8* NINIT, jdg_i8* MADSPACE, jdg_i8* ITER, double* TOL, jdg_i8* IJOB,
                         jdg_i8* NDX1, jdg_i8* NDX2, jdg_i8* IPRINT, jdg_i8* INFO, double* GAP);
JDG64_API void pjdcleanup_(void);

#ifdef __cplusplus
}
#endif
#endif
