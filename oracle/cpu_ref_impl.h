/*
 * cpu_ref_impl.h — body of the CPU restatement, instantiated twice by
 * cpu_ref.c: once with REAL = double (suffix _d) and once with REAL = float
 * (suffix _f).  TEST INFRASTRUCTURE ONLY: this is the oracle the CUDA solver
 * is checked against; nothing in the product links it.
 *
 * Method (reference: BLPG-Solver/src/simplex.cu, kernel mykernel):
 *   tableau from the slack basis ........ simplex.cu:463-550, :880-890
 *   pricing, most negative z_j - c_j .... simplex.cu:97-167
 *   minimum-ratio test, pivot tol ........ simplex.cu:171-260
 *   pivot-row scale ...................... simplex.cu:292-300
 *   rank-1 elimination incl. objective ... simplex.cu:302-319
 *   termination, objective = T[m][last] .. simplex.cu:334-342, :379-383
 *   phase I with artificial columns ...... simplex.cu:602-826
 * Deliberate, documented deviations from the reference kernel (which the
 * CUDA kernels share bit for bit):
 *   - ties: pricing takes the lowest column index, the ratio test the row
 *     whose basic variable has the lowest index (the reference's tree
 *     reduction picks tree-order winners, simplex.cu:126, :225);
 *   - reduced costs count as negative only below -opt_tol (reference: < 0);
 *   - a non-positive RHS gives ratio 0 instead of excluding the row
 *     (reference requires b_k >= 0, simplex.cu:193);
 *   - no positive pivot entry => status UNBOUNDED (the reference just stops,
 *     simplex.cu:344-347); a pivot cap => status UNDEF;
 *   - after bland_after consecutive degenerate pivots the entering column
 *     becomes the lowest eligible index (Bland's rule) for the rest of the
 *     solve, so degenerate LPs cannot cycle;
 *   - every elimination is one fused multiply-add, fma(-f, p_j, t_ij),
 *     applied to every row whose multiplier f is non-zero (the GPU kernels
 *     do the same, so the results are bit-identical).
 */

#define CAT2(a, b) a##b
#define CAT(a, b) CAT2(a, b)
#define FN(name) CAT(name, SUFFIX)

typedef struct {
  int m, n, na;   /* rows, structural columns, artificial columns */
  int W;          /* n + m + na + 1 (last column = RHS) */
  REAL* T;        /* (m + 1) x W, row-major; row m = objective row */
  int* basis;     /* m basic column ids */
} FN(tab_t);

#define TT(t, i, j) ((t)->T[(size_t)(i) * (t)->W + (j)])

/* Entering column over [0, ncols): Dantzig (most negative, lowest index on
 * ties) or Bland (lowest eligible index). -1 if none is below -opt_tol. */
static int FN(price)(const FN(tab_t) * t, int ncols, int bland, REAL opt_tol) {
  const REAL* d = &TT(t, t->m, 0);
  int q = -1;
  REAL best = (REAL)0;
  for (int j = 0; j < ncols; ++j) {
    REAL v = d[j];
    if (!(v < -opt_tol)) continue;
    if (bland) return j;
    if (q < 0 || v < best) {
      q = j;
      best = v;
    }
  }
  return q;
}

/* Steepest-edge pricing (a rule the reference does not have; the published
 * Goldfarb-Reid criterion with exact norms): among d_j < -opt_tol the
 * largest d_j^2 / (1 + sum_{i<m} T_ij^2), times weight[j] when given,
 * lowest index on ties.  The score is rounded to float as on the GPU, whose
 * norms are fixed-point sums; near-ties may therefore resolve differently
 * there, so this mode is checked on statuses and objectives, not bit for
 * bit. */
static int FN(price_se)(const FN(tab_t) * t, int ncols, REAL opt_tol, const float* weight) {
  const REAL* d = &TT(t, t->m, 0);
  int q = -1;
  float best = 0.f;
  for (int j = 0; j < ncols; ++j) {
    const REAL v = d[j];
    if (!(v < -opt_tol)) continue;
    double g = 1.0;
    for (int i = 0; i < t->m; ++i) {
      const double a = (double)TT(t, i, j);
      g += a * a;
    }
    const float vf = (float)v;
    float sc = (float)((double)vf * (double)vf / g);
    if (weight) sc *= weight[j];
    if (q < 0 || sc > best) {
      q = j;
      best = sc;
    }
  }
  return q;
}

/* Leaving row for entering column q; -1 if no entry exceeds piv_tol.
 * Textbook rule (Bland mode): minimum ratio, ties by lowest basic variable.
 * Harris rule (default): pass 1 bounds the step by the ratios relaxed by
 * feas_tol, pass 2 takes the LARGEST pivot entry among rows whose ratio is
 * within that bound (ties by lowest basic variable), so a tiny pivot never
 * wins a tie of degenerate rows. */
static int FN(ratio)(const FN(tab_t) * t, int q, REAL piv_tol, REAL feas_tol, int harris,
                     REAL* theta_out) {
  int r = -1, rb = 0;
  REAL best = (REAL)0;
  if (!harris) {
    for (int i = 0; i < t->m; ++i) {
      REAL a = TT(t, i, q);
      if (!(a > piv_tol)) continue;
      REAL rhs = TT(t, i, t->W - 1);
      REAL th = rhs > (REAL)0 ? rhs / a : (REAL)0;
      if (r < 0 || th < best || (th == best && t->basis[i] < rb)) {
        r = i;
        best = th;
        rb = t->basis[i];
      }
    }
    *theta_out = best;
    return r;
  }
  REAL tmax = (REAL)0;
  int any = 0;
  for (int i = 0; i < t->m; ++i) {
    REAL a = TT(t, i, q);
    if (!(a > piv_tol)) continue;
    REAL rhs = TT(t, i, t->W - 1);
    REAL rr = rhs > (REAL)0 ? rhs : (REAL)0;
    REAL th = (rr + feas_tol) / a;
    if (!any || th < tmax) tmax = th;
    any = 1;
  }
  if (!any) return -1;
  REAL amax = (REAL)0;
  for (int i = 0; i < t->m; ++i) {
    REAL a = TT(t, i, q);
    if (!(a > piv_tol)) continue;
    REAL rhs = TT(t, i, t->W - 1);
    REAL th = rhs > (REAL)0 ? rhs / a : (REAL)0;
    if (!(th <= tmax)) continue;
    if (r < 0 || a > amax || (a == amax && t->basis[i] < rb)) {
      r = i;
      amax = a;
      best = th;
      rb = t->basis[i];
    }
  }
  *theta_out = best;
  return r;
}

static void FN(pivot)(FN(tab_t) * t, int r, int q, REAL* f) {
  const int W = t->W, m = t->m;
  REAL* pr = &TT(t, r, 0);
  const REAL piv = pr[q];
  for (int j = 0; j < W; ++j) pr[j] = pr[j] / piv;
  for (int i = 0; i <= m; ++i) f[i] = TT(t, i, q);
  for (int i = 0; i <= m; ++i) {
    if (i == r) continue;
    REAL* row = &TT(t, i, 0);
    const REAL fi = f[i];
    if (fi == (REAL)0) continue; /* a zero multiplier leaves the row as it is */
    for (int j = 0; j < W; ++j) row[j] = FMA(-fi, pr[j], row[j]);
  }
  t->basis[r] = q;
}

/* The pivot loop shared by phase I and phase II. */
static int FN(simplex_loop)(FN(tab_t) * t, int ncols, const oref_opts* o,
                            int* pivots, int* bland, int* degen, REAL* f) {
  const REAL opt_tol = (REAL)o->opt_tol, piv_tol = (REAL)o->piv_tol;
  for (;;) {
    int q = o->pricing == 1 && !*bland ? FN(price_se)(t, ncols, opt_tol, o->weight)
                                       : FN(price)(t, ncols, *bland, opt_tol);
    if (q < 0) return OREF_OPT;
    if (*pivots >= o->max_pivots) return OREF_UNDEF;
    REAL theta;
    int r = FN(ratio)(t, q, piv_tol, (REAL)o->feas_tol, o->harris && !*bland, &theta);
    if (r < 0) return OREF_UNBND;
    FN(pivot)(t, r, q, f);
    *pivots += 1;
    if (theta <= (REAL)o->deg_tol) {
      *degen += 1;
      if (*degen > o->bland_after) *bland = 1;
    } else {
      *degen = 0;
    }
  }
}

/* Objective row from the current basis: d_j = sum_i cB_i T_ij - c_j,
 * z = sum_i cB_i rhs_i (sums over rows in increasing order). */
static void FN(objective_row)(FN(tab_t) * t, const double* c) {
  const int m = t->m, n = t->n, rhs = t->W - 1;
  for (int j = 0; j < t->W; ++j) {
    REAL acc = (REAL)0;
    for (int i = 0; i < m; ++i) {
      const int bi = t->basis[i];
      const REAL cb = bi < n ? (REAL)c[bi] : (REAL)0;
      acc = FMA(cb, TT(t, i, j), acc);
    }
    const REAL cj = j < n ? (REAL)c[j] : (REAL)0;
    TT(t, m, j) = j == rhs ? acc : acc - cj;
  }
}

/* Feasibility of the tableau: bit 0 when every RHS >= -ptol, bit 1 when
 * every reduced cost d_j (j < n+m) >= -opt_tol (the GPU's check_feasible). */
static int FN(check)(const FN(tab_t) * t, REAL ptol, REAL opt_tol) {
  int ok = 3;
  for (int i = 0; i < t->m; ++i)
    if (TT(t, i, t->W - 1) < -ptol) ok &= ~1;
  for (int j = 0; j < t->n + t->m; ++j)
    if (TT(t, t->m, j) < -opt_tol) ok &= ~2;
  return ok;
}

/* Dual simplex from a dual-feasible basis: leaving row = most negative RHS
 * below -ptol (ties lowest basic variable), entering column = minimum
 * max(d_j, 0) / -T_rj over T_rj < -piv_tol (ties lowest column). */
static int FN(dual_loop)(FN(tab_t) * t, const oref_opts* o, int* pivots, REAL* f, REAL ptol) {
  const REAL piv_tol = (REAL)o->piv_tol;
  const int m = t->m, ncols = t->n + t->m;
  for (;;) {
    int r = -1, rb = 0;
    REAL best = (REAL)0;
    for (int i = 0; i < m; ++i) {
      const REAL v = TT(t, i, t->W - 1);
      if (!(v < -ptol)) continue;
      if (r < 0 || v < best || (v == best && t->basis[i] < rb)) {
        r = i;
        best = v;
        rb = t->basis[i];
      }
    }
    if (r < 0) return OREF_OPT;
    if (*pivots >= o->max_pivots) return OREF_UNDEF;
    int q = -1;
    if (!o->harris) {
      REAL bth = (REAL)0;
      for (int j = 0; j < ncols; ++j) {
        const REAL a = TT(t, r, j);
        if (!(a < -piv_tol)) continue;
        const REAL dj = TT(t, m, j);
        const REAL th = dj > (REAL)0 ? dj / (-a) : (REAL)0;
        if (q < 0 || th < bth) {
          q = j;
          bth = th;
        }
      }
    } else {
      /* Harris: bound by ratios relaxed by opt_tol, then the largest |T_rj| */
      REAL tmax = (REAL)0;
      int any = 0;
      for (int j = 0; j < ncols; ++j) {
        const REAL a = TT(t, r, j);
        if (!(a < -piv_tol)) continue;
        const REAL dj = TT(t, m, j);
        const REAL th = ((dj > (REAL)0 ? dj : (REAL)0) + (REAL)o->opt_tol) / (-a);
        if (!any || th < tmax) tmax = th;
        any = 1;
      }
      REAL amax = (REAL)0;
      for (int j = 0; any && j < ncols; ++j) {
        const REAL a = TT(t, r, j);
        if (!(a < -piv_tol)) continue;
        const REAL dj = TT(t, m, j);
        const REAL th = dj > (REAL)0 ? dj / (-a) : (REAL)0;
        if (th <= tmax && (q < 0 || -a > amax)) {
          q = j;
          amax = -a;
        }
      }
    }
    if (q < 0) return OREF_NOFEAS;
    FN(pivot)(t, r, q, f);
    *pivots += 1;
  }
}

/* Warm start: pivot each hinted structural column into the basis on the
 * row, among rows whose basic variable is a slack the hint does not keep,
 * with the largest |T_ij| (ties lowest row).  Returns how many hinted
 * columns found no pivot. */
static int FN(crash)(FN(tab_t) * t, const int* hint, const oref_opts* o, int* pivots, REAL* f) {
  const int m = t->m, n = t->n;
  const REAL piv_tol = (REAL)o->piv_tol;
  int* keep = (int*)calloc((size_t)(m > 0 ? m : 1), sizeof(int));
  for (int k = 0; k < m; ++k)
    if (hint[k] >= n && hint[k] < n + m) keep[hint[k] - n] = 1;
  int missing = 0;
  for (int k = 0; k < m; ++k) {
    const int h = hint[k];
    if (h < 0 || h >= n) continue;
    int isbasic = 0;
    for (int i = 0; i < m; ++i) isbasic |= t->basis[i] == h;
    if (isbasic) continue;
    int r = -1;
    REAL best = (REAL)0;
    for (int i = 0; i < m; ++i) {
      const int bi = t->basis[i];
      if (bi < n || bi >= n + m || keep[bi - n]) continue;
      const REAL v = TT(t, i, h);
      const REAL av = v < (REAL)0 ? -v : v;
      if (av > piv_tol && (r < 0 || av > best)) {
        r = i;
        best = av;
      }
    }
    if (r < 0) {
      ++missing;
      continue;
    }
    FN(pivot)(t, r, h, f);
    *pivots += 1;
  }
  free(keep);
  return missing;
}

/* Solve one LP.  Returns the status; fills objective, x (n, nullable),
 * basis (m, nullable), pivot count. */
static int FN(solve_one)(int m, int n, const double* A, const double* b,
                         const double* c, const oref_opts* o, const int* hint,
                         double* obj, double* x, int* basis_out, int* pivots_out,
                         int* info_out) {
  int na = 0;
  for (int i = 0; i < m; ++i)
    if (b[i] < 0) ++na;
  FN(tab_t) t;
  t.m = m;
  t.n = n;
  t.na = na;
  t.W = n + m + na + 1;
  t.T = (REAL*)calloc((size_t)(m + 1) * t.W, sizeof(REAL));
  t.basis = (int*)malloc(sizeof(int) * (size_t)(m > 0 ? m : 1));
  REAL* f = (REAL*)malloc(sizeof(REAL) * (size_t)(m + 1));
  if (!t.T || !t.basis || !f) {
    free(t.T);
    free(t.basis);
    free(f);
    return -1;
  }
  const int rhs = t.W - 1;
  int info = 0;
  int pivots = 0, bland = 0, degen = 0, st;
reload:;
  bland = 0; /* a cold reload restarts the rule state; pivots keep counting */
  degen = 0;
  /* slack-basis tableau (simplex.cu:506-534); rows with b_i < 0 are negated
   * and get an artificial column (simplex.cu:642-686). */
  memset(t.T, 0, sizeof(REAL) * (size_t)(m + 1) * t.W);
  int k = 0;
  for (int i = 0; i < m; ++i) {
    const REAL sgn = b[i] < 0 ? (REAL)-1 : (REAL)1;
    for (int j = 0; j < n; ++j) {
      const REAL av = (REAL)A[(size_t)i * n + j];
      TT(&t, i, j) = b[i] < 0 ? -av : av;
    }
    TT(&t, i, n + i) = sgn;
    TT(&t, i, rhs) = b[i] < 0 ? -(REAL)b[i] : (REAL)b[i];
    if (b[i] < 0) {
      TT(&t, i, n + m + k) = (REAL)1;
      t.basis[i] = n + m + k;
      ++k;
    } else {
      t.basis[i] = n + i;
    }
  }
  if (na > 0) {
    /* phase I: maximise -sum(artificials); row m = -sum of artificial rows */
    for (int j = 0; j < t.W; ++j) {
      if (j >= n + m && j < rhs) continue;
      REAL acc = (REAL)0;
      for (int i = 0; i < m; ++i)
        if (t.basis[i] >= n + m) acc = acc - TT(&t, i, j);
      TT(&t, m, j) = acc;
    }
    st = FN(simplex_loop)(&t, n + m, o, &pivots, &bland, &degen, f);
    if (st == OREF_OPT) {
      const double z = (double)TT(&t, m, rhs);
      if (z < -o->phase1_tol) st = OREF_NOFEAS;
    } else if (st == OREF_UNBND) {
      st = OREF_UNDEF; /* phase I is bounded; only numerical trouble gets here */
    }
    if (st == OREF_OPT) {
      /* drive zero-level artificials out of the basis */
      for (int i = 0; i < m; ++i) {
        if (t.basis[i] < n + m) continue;
        for (int j = 0; j < n + m; ++j) {
          REAL a = TT(&t, i, j);
          if (a > (REAL)o->piv_tol || a < -(REAL)o->piv_tol) {
            FN(pivot)(&t, i, j, f);
            ++pivots;
            break;
          }
        }
      }
      /* phase II objective row: d_j = sum_i cB_i T_ij - c_j, z = sum cB_i rhs_i */
      FN(objective_row)(&t, c);
      bland = 0;
      degen = 0;
      st = FN(simplex_loop)(&t, n + m, o, &pivots, &bland, &degen, f);
    }
  } else {
    for (int j = 0; j < n; ++j) TT(&t, m, j) = -(REAL)c[j];
    st = -1;
    if (hint && !(info & 2)) {
      const REAL ptol = (REAL)o->ptol, opt_tol = (REAL)o->opt_tol;
      info |= 1;
      if (FN(crash)(&t, hint, o, &pivots, f) > 0) info |= 4;
      const int fl = FN(check)(&t, ptol, opt_tol);
      if (fl & 1) {
        st = FN(simplex_loop)(&t, n + m, o, &pivots, &bland, &degen, f);
      } else if (fl & 2) {
        info |= 8;
        st = FN(dual_loop)(&t, o, &pivots, f, ptol);
        if (st == OREF_OPT) st = FN(simplex_loop)(&t, n + m, o, &pivots, &bland, &degen, f);
      } else if (o->composite) {
        /* infeasible both ways: shift the costs of the columns with
         * d_j < -opt_tol to make d_j = 0 (dual feasible), dual simplex to a
         * primal-feasible basis, restore the true costs, primal simplex */
        info |= 8 | 64;
        for (int j = 0; j < n + m; ++j)
          if (TT(&t, m, j) < -opt_tol)
            TT(&t, m, j) = (REAL)o->shift * ((REAL)1 + (REAL)((j * 7919) % 1000) / (REAL)1000);
        st = FN(dual_loop)(&t, o, &pivots, f, ptol);
        if (st == OREF_OPT) {
          FN(objective_row)(&t, c);
          st = FN(simplex_loop)(&t, n + m, o, &pivots, &bland, &degen, f);
        }
      }
      if (st < 0 || st == OREF_NOFEAS) {
        info |= 2; /* infeasible both ways: cold solve from the slack basis */
        goto reload;
      }
    }
    if (st < 0) st = FN(simplex_loop)(&t, n + m, o, &pivots, &bland, &degen, f);
  }
  *obj = (double)TT(&t, m, rhs);
  if (x) {
    for (int j = 0; j < n; ++j) x[j] = 0.0;
    for (int i = 0; i < m; ++i)
      if (t.basis[i] < n) x[t.basis[i]] = (double)TT(&t, i, rhs);
  }
  if (basis_out)
    for (int i = 0; i < m; ++i) basis_out[i] = t.basis[i];
  *pivots_out = pivots;
  if (info_out) *info_out = info;
  free(t.T);
  free(t.basis);
  free(f);
  return st;
}

#undef TT
#undef FN
#undef CAT
#undef CAT2
