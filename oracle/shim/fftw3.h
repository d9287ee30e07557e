/*
 * Stand-in for <fftw3.h> — TEST INFRASTRUCTURE ONLY.
 *
 * FFTW3 is not installed in this image. The reference's Poisson solver
 * (src/PressureSolverStructures.cpp:19-41, src/PressureEquation.cpp:71-261)
 * is compiled against this header to build the oracle library under
 * oracle/_ref/. It declares the subset of FFTW's double-precision API the
 * reference calls and routes execution to oracle/r2r.c, which restates the
 * three r2r kinds from FFTW's documented definitions.
 */
#ifndef ORACLE_SHIM_FFTW3_H
#define ORACLE_SHIM_FFTW3_H

#include <stdint.h>
#include <stdlib.h>

#include "../r2r.h"

typedef enum { FFTW_R2HC = 0, FFTW_HC2R = 1, FFTW_REDFT00 = 3 } fftw_r2r_kind;
#define FFTW_ESTIMATE (1U << 6)

typedef struct oracle_fftw_plan_s {
  int n;
  int kind;
  double *in;
  double *out;
} *fftw_plan;

static inline fftw_plan fftw_plan_r2r_1d(int n, double *in, double *out, fftw_r2r_kind kind,
                                         unsigned) {
  fftw_plan p = (fftw_plan)malloc(sizeof(*p));
  p->n = n;
  p->kind = (int)kind;
  p->in = in;
  p->out = out;
  return p;
}
static inline void fftw_execute_r2r(const fftw_plan p, double *in, double *out) {
  if (oracle_r2r_1d(p->n, p->kind, in, out) != 0) abort();
}
static inline void fftw_execute(const fftw_plan p) { fftw_execute_r2r(p, p->in, p->out); }
static inline void fftw_destroy_plan(fftw_plan p) { free(p); }
static inline void fftw_cleanup(void) {}
static inline void *fftw_malloc(size_t n) {
  void *ptr = NULL;
  if (posix_memalign(&ptr, 64, n ? n : 64) != 0) return NULL;
  return ptr;
}
static inline void fftw_free(void *p) { free(p); }
/* The reference asserts equal alignment classes; 64-byte allocations share one. */
static inline int fftw_alignment_of(double *p) { return (int)(((uintptr_t)p) % 16); }

#endif /* ORACLE_SHIM_FFTW3_H */
