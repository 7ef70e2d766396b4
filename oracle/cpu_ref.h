/*
 * cpu_ref.h — CPU oracle (test infrastructure only; see cpu_ref.c).
 */
#ifndef OREF_CPU_REF_H_
#define OREF_CPU_REF_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* GLPK status codes, as blpg.h. */
enum { OREF_UNDEF = 1, OREF_NOFEAS = 4, OREF_OPT = 5, OREF_UNBND = 6 };
enum { OREF_FP64 = 0, OREF_FP32 = 1 };

typedef struct {
  int precision;
  int max_pivots;  /* <= 0: 50 (m + n) + 1000 */
  int bland_after; /* consecutive degenerate pivots before Bland's rule */
  int refactor_period;
  double opt_tol, piv_tol, phase1_tol;
  double deg_tol; /* a pivot with ratio <= deg_tol counts as degenerate */
  double feas_tol; /* Harris ratio-test relaxation */
  int harris;      /* 1: Harris two-pass ratio test outside Bland mode */
  double ptol;     /* primal feasibility tolerance of the warm-start checks */
  int composite;   /* 1: a hinted basis infeasible both ways is finished by a
                      cost-shifted dual phase instead of a cold solve */
  double shift;    /* size of the cost shift (the shifted d_j lie in [shift, 2 shift)) */
  int pricing;     /* 0: Dantzig (the reference); 1: steepest edge, exact norms */
  const float* weight; /* steepest edge: score factor per variable (n + m), or null */
} oref_opts;

void oref_opts_init(oref_opts* o, int precision);
int oref_default_max_pivots(int m, int n);

int oref_solve_one(int m, int n, const double* A, const double* b,
                   const double* c, const oref_opts* o, const int* hint,
                   double* obj, double* x, int* basis, int* pivots, int* info);

/* Null offsets = packed.  x (nullable) follows off_c; basis and hint
 * (nullable) are packed m per LP; info (nullable) gets the warm-start bits
 * (1 warm, 2 fallback, 4 partial, 8 dual); weight (nullable, steepest edge)
 * is packed n + m per LP.  threads = POSIX threads. */
int oref_solve_batch(int count, const int* m, const int* n, const int64_t* offA,
                     const int64_t* offb, const int64_t* offc, const double* A,
                     const double* b, const double* c, const oref_opts* o,
                     int threads, const int* hint, int* status, double* obj,
                     double* x, int* pivots, int* basis, int* info, const float* weight);

#ifdef __cplusplus
}
#endif

#endif
