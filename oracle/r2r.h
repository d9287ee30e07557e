/*
 * CPU reference transforms — TEST INFRASTRUCTURE ONLY (oracle).
 *
 * The reference solver does its Poisson transforms with FFTW3 (third-party,
 * not vendored, no pinned version: any `fftw3` found by pkg-config,
 * CMakeLists.txt:13-16; system default paths in Makefile:52-57). It uses three
 * real-to-real kinds, planned in src/PressureSolverStructures.cpp:19-41:
 *   REDFT00 (DCT-I) for Neumann axes, R2HC/HC2R for periodic axes.
 * These functions restate FFTW's published definitions of those kinds
 * (FFTW manual, "1d Real-even DFTs (DCTs)" and "The Halfcomplex-format DFT"),
 * unnormalised exactly as FFTW computes them:
 *   REDFT00, n points:  Y_k = X_0 + (-1)^k X_{n-1} + 2 sum_{j=1}^{n-2} X_j cos(pi j k/(n-1))
 *   R2HC,    n points:  r_k = sum_j X_j cos(2 pi j k/n),  i_k = -sum_j X_j sin(2 pi j k/n),
 *                       out = r_0, r_1, ..., r_{n/2}, i_{(n+1)/2-1}, ..., i_1
 *   HC2R,    n points:  the inverse of R2HC without the 1/n factor.
 * Internally each is a mixed-radix complex FFT (O(n log n) for smooth n) of
 * the even extension (REDFT00, length 2(n-1)) or of the real line (R2HC/HC2R).
 */
#ifndef ORACLE_R2R_H
#define ORACLE_R2R_H

#ifdef __cplusplus
extern "C" {
#endif

enum oracle_r2r_kind { ORACLE_R2HC = 0, ORACLE_HC2R = 1, ORACLE_REDFT00 = 3 };

/* in and out may alias. Returns 0 on success, -1 on invalid arguments. */
int oracle_r2r_1d(int n, int kind, const double *in, double *out);

/* Direct O(n^2) evaluation of the same definitions, for known-answer tests. */
int oracle_r2r_1d_direct(int n, int kind, const double *in, double *out);

#ifdef __cplusplus
}
#endif

#endif
