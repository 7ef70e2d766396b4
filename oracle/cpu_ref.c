/*
 * cpu_ref.c — CPU oracle for the GB300 batched LP solver.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * method (BLPG-Solver/src/simplex.cu, dense-tableau primal simplex from the
 * slack basis) with the pivot rules of the CUDA kernels; see cpu_ref_impl.h
 * for the rule-by-rule citations.  Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg load it, as the checker or the timed CPU
 * baseline; the product library never does.
 *
 * Build (oracle/Makefile): gcc -O2 -ffp-contract=off -fPIC -shared -pthread.
 * -ffp-contract=off matters: every multiply-add that must be fused is an
 * explicit fma()/fmaf() call, and no other expression may be contracted, so
 * the FP64 oracle and the FP64 GPU kernel agree bit for bit.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "cpu_ref.h"

#define REAL double
#define SUFFIX _d
#define FMA fma
#include "cpu_ref_impl.h"
#undef REAL
#undef SUFFIX
#undef FMA

#define REAL float
#define SUFFIX _f
#define FMA fmaf
#include "cpu_ref_impl.h"
#undef REAL
#undef SUFFIX
#undef FMA

void oref_opts_init(oref_opts* o, int precision) {
  memset(o, 0, sizeof(*o));
  o->precision = precision;
  o->max_pivots = 0;
  o->bland_after = 64;
  o->opt_tol = precision == OREF_FP32 ? 1e-5 : 1e-9;
  o->piv_tol = precision == OREF_FP32 ? 1e-5 : 1e-7;
  o->phase1_tol = precision == OREF_FP32 ? 1e-4 : 1e-7;
  o->deg_tol = precision == OREF_FP32 ? 1e-7 : 1e-12;
  o->feas_tol = precision == OREF_FP32 ? 1e-6 : 1e-9;
  o->harris = 1;
  o->ptol = precision == OREF_FP32 ? 1e-7 : 1e-9;
  o->shift = 0.1;
  o->composite = 1;
}

int oref_default_max_pivots(int m, int n) { return 50 * (m + n) + 1000; }

int oref_solve_one(int m, int n, const double* A, const double* b,
                   const double* c, const oref_opts* o_in, const int* hint,
                   double* obj, double* x, int* basis, int* pivots, int* info) {
  oref_opts o = *o_in;
  if (o.max_pivots <= 0) o.max_pivots = oref_default_max_pivots(m, n);
  if (o.precision == OREF_FP32)
    return solve_one_f(m, n, A, b, c, &o, hint, obj, x, basis, pivots, info);
  return solve_one_d(m, n, A, b, c, &o, hint, obj, x, basis, pivots, info);
}

typedef struct {
  int count;
  const int *m, *n;
  const int64_t *offA, *offb, *offc, *offx, *offbasis;
  const double *A, *b, *c;
  const oref_opts* o;
  const int* hint;
  const float* weight;
  const int64_t* offw;
  int* info;
  int* status;
  double* obj;
  double* x;
  int* pivots;
  int* basis;
  int next; /* work counter, taken under the lock */
  pthread_mutex_t lock;
} batch_job;

static void* worker(void* arg) {
  batch_job* J = (batch_job*)arg;
  for (;;) {
    pthread_mutex_lock(&J->lock);
    int k = J->next++;
    pthread_mutex_unlock(&J->lock);
    if (k >= J->count) break;
    int piv = 0;
    double ob = 0.0;
    int inf = 0;
    oref_opts o = *J->o;
    o.weight = J->weight ? J->weight + J->offw[k] : NULL;
    int st = oref_solve_one(J->m[k], J->n[k], J->A + J->offA[k], J->b + J->offb[k],
                            J->c + J->offc[k], &o,
                            J->hint ? J->hint + J->offbasis[k] : NULL, &ob,
                            J->x ? J->x + J->offx[k] : NULL,
                            J->basis ? J->basis + J->offbasis[k] : NULL, &piv, &inf);
    if (J->info) J->info[k] = inf;
    J->status[k] = st;
    J->obj[k] = ob;
    if (J->pivots) J->pivots[k] = piv;
  }
  return NULL;
}

int oref_solve_batch(int count, const int* m, const int* n, const int64_t* offA,
                     const int64_t* offb, const int64_t* offc, const double* A,
                     const double* b, const double* c, const oref_opts* o,
                     int threads, const int* hint, int* status, double* obj,
                     double* x, int* pivots, int* basis, int* info, const float* weight) {
  if (count < 0 || !m || !n || !A || !b || !c || !o || !status || !obj) return -1;
  int64_t* own = (int64_t*)malloc(sizeof(int64_t) * 6 * (size_t)(count + 1));
  if (!own) return -1;
  int64_t *pA = own, *pb = own + (count + 1), *pc = own + 2 * (count + 1);
  int64_t *px = own + 3 * (count + 1), *pbs = own + 4 * (count + 1);
  int64_t* pw = own + 5 * (count + 1);
  pA[0] = pb[0] = pc[0] = px[0] = pbs[0] = pw[0] = 0;
  for (int k = 0; k < count; ++k) {
    pA[k + 1] = pA[k] + (int64_t)m[k] * n[k];
    pb[k + 1] = pb[k] + m[k];
    pc[k + 1] = pc[k] + n[k];
    pbs[k + 1] = pbs[k] + m[k];
    pw[k + 1] = pw[k] + m[k] + n[k];
  }
  batch_job J;
  memset(&J, 0, sizeof(J));
  J.count = count;
  J.m = m;
  J.n = n;
  J.offA = offA ? offA : pA;
  J.offb = offb ? offb : pb;
  J.offc = offc ? offc : pc;
  J.offx = offc ? offc : pc;
  J.offbasis = pbs;
  J.A = A;
  J.b = b;
  J.c = c;
  J.o = o;
  J.status = status;
  J.obj = obj;
  J.x = x;
  J.pivots = pivots;
  J.basis = basis;
  J.hint = hint;
  J.weight = weight;
  J.offw = pw;
  J.info = info;
  pthread_mutex_init(&J.lock, NULL);
  if (threads < 1) threads = 1;
  if (threads > count) threads = count > 0 ? count : 1;
  if (threads == 1) {
    worker(&J);
  } else {
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)threads);
    int started = 0;
    for (int t = 0; t < threads; ++t)
      if (pthread_create(&th[t], NULL, worker, &J) == 0) ++started;
    if (started == 0) worker(&J);
    for (int t = 0; t < started; ++t) pthread_join(th[t], NULL);
    free(th);
  }
  pthread_mutex_destroy(&J.lock);
  free(own);
  return 0;
}
