// Batched dense-tableau primal simplex for sm_103a.
//
// One LP per CTA, or per thread-block cluster of K CTAs when the tableau does
// not fit one CTA's shared memory (K in {1,2,4,8}).  The kernel is
// persistent: each CTA (cluster) takes LP tickets from a device work queue
// until the class's queue is empty.
//
// Reference kernel: BLPG-Solver/src/simplex.cu:35-385 (mykernel).  Same
// method, rebuilt for Blackwell:
//   - the whole tableau lives in shared memory (the reference keeps it in
//     global memory and reduces through global scratch, simplex.cu:108-143);
//   - pricing and the ratio test are warp argmins with __reduce_min_sync on
//     lexicographic 32-bit key words (value, tie index, payload), so ties are
//     broken by lowest index deterministically (reference: tree order);
//   - the next pivot column is priced from the updated objective row BEFORE
//     the body update, so the body sweep also extracts the next pivot column
//     and RHS into contiguous buffers (no strided column reads);
//   - rows are swept as 16-byte vectors (double2 / float4), one vector lane
//     per thread, the pivot-row vector held in registers;
//   - with K > 1 the columns are split into K blocks, the RHS column is
//     replicated in every block, and the pivot column and both argmins are
//     exchanged through distributed shared memory with two cluster barriers
//     per pivot.
// Every elimination is fma(-f, p_j, t_ij) and the pivot row is divided
// (IEEE division), exactly as the CPU oracle does, so the FP64 path is
// bit-identical to it.
#pragma once

#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace blpg {
namespace dev {

namespace cg = cooperative_groups;

// ---------------------------------------------------------------------------
// Arguments
// ---------------------------------------------------------------------------

struct LpArgs {
  const int32_t* m;
  const int32_t* n;
  const int64_t* offA;
  const int64_t* offb;
  const int64_t* offc;
  const int64_t* offx;
  const int64_t* offbasis;
  const double* A;
  const double* b;
  const double* c;
  int32_t* status;
  double* obj;
  double* x;        // nullable
  int32_t* pivots;  // nullable
  int32_t* basis;   // nullable
  double opt_tol;
  double piv_tol;
  double phase1_tol;
  double feas_tol;  // Harris ratio-test relaxation
  double deg_tol;   // a step <= deg_tol counts as degenerate
  int32_t harris;   // 1: Harris two-pass ratio test outside Bland mode
  int32_t max_pivots;  // <= 0: 50 (m + n) + 1000
  int32_t bland_after;
};

struct ClassArgs {
  const int32_t* order;  // LP ids of this class, heaviest first
  int32_t count;
  int32_t* ticket;  // queue head, zeroed before the launch
  int32_t K;        // CTAs per LP (cluster size)
  int32_t max_m;    // smem layout is sized for these
  int32_t max_ldw;
  int32_t max_na;   // artificial columns (two-phase LPs)
};

template <typename T>
struct VecT;
template <>
struct VecT<double> {
  using type = double2;
  static constexpr int V = 2;
};
template <>
struct VecT<float> {
  using type = float4;
  static constexpr int V = 4;
};

__host__ __device__ inline int ceil_div(int a, int b) { return (a + b - 1) / b; }
__host__ __device__ inline int round_up(int a, int b) { return ceil_div(a, b) * b; }

// Per-LP column geometry.  Columns 0..n-1 structural, n..n+m-1 slacks,
// n+m..n+m+na-1 artificials (two-phase only); CTA k of the cluster holds
// global columns [k*cw, k*cw + cw) at local 0..cw-1, the RHS at local cw,
// zero padding after it; rows 0..m-1 constraints, row m objective.
struct Geom {
  int m, n, na, Wc, cw, ldw, nl;
  __host__ __device__ Geom(int m_, int n_, int na_, int K, int V) {
    m = m_;
    n = n_;
    na = na_;
    Wc = n + m + na;
    cw = round_up(ceil_div(Wc, K), V);
    ldw = cw + V;
    nl = ldw / V;
  }
};

// Shared-memory layout of a class (bytes).  Identical on host and device.
struct Layout {
  int tab, colA, colB, rhsx, basis, red, state, total;
  __host__ __device__ Layout(int max_m, int max_ldw, int elem) {
    int mp1 = round_up(max_m + 1, 4);
    tab = 0;
    int off = round_up((max_m + 1) * max_ldw * elem, 16);
    colA = off;
    off += round_up(mp1 * elem, 16);
    colB = off;
    off += round_up(mp1 * elem, 16);
    rhsx = off;
    off += round_up(mp1 * elem, 16);
    basis = off;
    off += round_up(mp1 * 4, 16);
    red = off;
    off += 3 * 32 * 16;  // three argmin scratch buffers (pricing, ratio, Harris)
    state = off;
    off += 64;
    total = off;
  }
};

// ---------------------------------------------------------------------------
// Argmin keys: words compared lexicographically (w0, w1, w2); w3 is a
// payload carried with the winner.  Unused lanes hold all-ones.
// ---------------------------------------------------------------------------

struct Key {
  unsigned w0, w1, w2, w3;
};

__device__ __forceinline__ Key key_none() { return Key{~0u, ~0u, ~0u, ~0u}; }

__device__ __forceinline__ bool key_less(const Key& a, const Key& b) {
  if (a.w0 != b.w0) return a.w0 < b.w0;
  if (a.w1 != b.w1) return a.w1 < b.w1;
  return a.w2 < b.w2;
}

__device__ __forceinline__ Key warp_min(const Key& k) {
  const unsigned full = 0xffffffffu;
  Key r;
  r.w0 = __reduce_min_sync(full, k.w0);
  bool e0 = k.w0 == r.w0;
  r.w1 = __reduce_min_sync(full, e0 ? k.w1 : ~0u);
  bool e1 = e0 && k.w1 == r.w1;
  r.w2 = __reduce_min_sync(full, e1 ? k.w2 : ~0u);
  bool e2 = e1 && k.w2 == r.w2;
  r.w3 = __reduce_min_sync(full, e2 ? k.w3 : ~0u);
  return r;
}

// Block-wide argmin: every thread returns the winner.  Contains exactly one
// __syncthreads; `red` (32 keys) must not be reused before another barrier.
__device__ __forceinline__ Key block_min(const Key& k, Key* red) {
  Key w = warp_min(k);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) red[warp] = w;
  __syncthreads();
  const int nw = (int)(blockDim.x >> 5);
  Key v = lane < nw ? red[lane] : key_none();
  return warp_min(v);
}

// Pricing key of reduced cost d at global column j (only d < -tol is
// eligible).  For negative numbers ~bits is increasing in the value, so the
// most negative d has the smallest key; Bland's rule zeroes the value words
// so the lowest index wins.
__device__ __forceinline__ Key price_key(double d, int j, bool bland) {
  unsigned long long u = ~(unsigned long long)__double_as_longlong(d);
  if (bland) u = 0ull;
  return Key{(unsigned)(u >> 32), (unsigned)u, (unsigned)j, 0u};
}
__device__ __forceinline__ Key price_key(float d, int j, bool bland) {
  unsigned u = ~__float_as_uint(d);
  if (bland) u = 0u;
  return Key{u, 0u, (unsigned)j, 0u};
}
// Ratio key of theta >= 0 (IEEE bits are increasing for non-negative values),
// ties by lowest basic-variable id, payload = row.
__device__ __forceinline__ Key ratio_key(double th, int bid, int row) {
  unsigned long long u = (unsigned long long)__double_as_longlong(th);
  return Key{(unsigned)(u >> 32), (unsigned)u, (unsigned)bid, (unsigned)row};
}
__device__ __forceinline__ Key ratio_key(float th, int bid, int row) {
  return Key{__float_as_uint(th), 0u, (unsigned)bid, (unsigned)row};
}
// Largest positive value first: ~bits is decreasing in a positive value.
__device__ __forceinline__ Key big_key(double a, int bid, int row) {
  unsigned long long u = ~(unsigned long long)__double_as_longlong(a);
  return Key{(unsigned)(u >> 32), (unsigned)u, (unsigned)bid, (unsigned)row};
}
__device__ __forceinline__ Key big_key(float a, int bid, int row) {
  return Key{~__float_as_uint(a), 0u, (unsigned)bid, (unsigned)row};
}
__device__ __forceinline__ double key_theta(const Key& k, double) {
  return __hiloint2double((int)k.w0, (int)k.w1);
}
__device__ __forceinline__ float key_theta(const Key& k, float) {
  return __uint_as_float(k.w0);
}

template <typename VT, typename T>
__device__ __forceinline__ T vget(const VT& v, int e);
template <>
__device__ __forceinline__ double vget<double2, double>(const double2& v, int e) {
  return e == 0 ? v.x : v.y;
}
template <>
__device__ __forceinline__ float vget<float4, float>(const float4& v, int e) {
  return e == 0 ? v.x : (e == 1 ? v.y : (e == 2 ? v.z : v.w));
}

__device__ __forceinline__ double2 v_fma(double f, const double2& p, const double2& t) {
  return make_double2(fma(-f, p.x, t.x), fma(-f, p.y, t.y));
}
__device__ __forceinline__ float4 v_fma(float f, const float4& p, const float4& t) {
  return make_float4(fmaf(-f, p.x, t.x), fmaf(-f, p.y, t.y), fmaf(-f, p.z, t.z),
                     fmaf(-f, p.w, t.w));
}
__device__ __forceinline__ double2 v_div(const double2& a, double d) {
  return make_double2(a.x / d, a.y / d);
}
__device__ __forceinline__ float4 v_div(const float4& a, float d) {
  return make_float4(__fdiv_rn(a.x, d), __fdiv_rn(a.y, d), __fdiv_rn(a.z, d),
                     __fdiv_rn(a.w, d));
}

// Status codes (GLPK numbering, as blpg.h)
constexpr int kUndef = 1, kNoFeas = 4, kOpt = 5, kUnbnd = 6;

struct SharedState {
  int ticket;
  int r;
  int pad0, pad1;
  double theta;
  Key pslot;
  Key aux;
};

// ---------------------------------------------------------------------------
// The solver kernel
// ---------------------------------------------------------------------------

template <typename T, bool CLUSTER>
struct Solver {
  using VT = typename VecT<T>::type;
  static constexpr int V = VecT<T>::V;

  unsigned char* smem;
  T* tab;
  T* col0;
  T* col1;
  __device__ T* colbuf(int k) const { return k ? col1 : col0; }
  T* rhsx;
  int* basis;
  Key* redP;
  Key* redR;
  Key* redH;
  SharedState* sh;
  int K, rank;

  __device__ void csync() {
    if (CLUSTER)
      cg::this_cluster().sync();
    else
      __syncthreads();
  }
  template <typename P>
  __device__ P* remote(P* p, int r) {
    if (CLUSTER) return cg::this_cluster().map_shared_rank(p, (unsigned)r);
    return p;
  }

  // Cluster-wide argmin of a pricing candidate that is already block-reduced.
  __device__ Key cluster_min(const Key& mine) {
    if (!CLUSTER) return mine;
    if (threadIdx.x == 0) sh->pslot = mine;
    csync();
    Key best = key_none();
    for (int k = 0; k < K; ++k) {
      Key o = *remote(&sh->pslot, k);
      if (key_less(o, best)) best = o;
    }
    return best;
  }

  // Local pricing over the objective row (no update): block + cluster min.
  __device__ Key price_only(const Geom& g, int c0, int lc, bool bland, T opt_tol,
                            int price_cols) {
    Key k = key_none();
    const T* d = tab + (size_t)g.m * g.ldw;
    for (int lj = threadIdx.x; lj < lc; lj += blockDim.x) {
      const int j = c0 + lj;
      const T v = d[lj];
      if (j < price_cols && v < -opt_tol) {
        Key kk = price_key(v, j, bland);
        if (key_less(kk, k)) k = kk;
      }
    }
    k = block_min(k, redP);
    return cluster_min(k);
  }

  // Owner of column q copies it (rows 0..m) and the RHS column into the
  // extraction buffers.
  __device__ void extract(const Geom& g, int q, int c0, T* colx) {
    const int ql = q - c0;
    for (int i = threadIdx.x; i <= g.m; i += blockDim.x) {
      colx[i] = tab[(size_t)i * g.ldw + ql];
      rhsx[i] = tab[(size_t)i * g.ldw + g.cw];
    }
  }

  // Ratio test on the owner CTA: every thread returns the winning key
  // (payload = row) and theta.  Textbook rule: minimum ratio, ties by lowest
  // basic variable.  Harris rule: pass 1 bounds the step by the ratios
  // relaxed by feas_tol, pass 2 takes the largest pivot entry among rows
  // within the bound (ties by lowest basic variable).  The oracle's ratio()
  // performs the same operations.
  __device__ Key ratio(const Geom& g, const T* colx, T piv_tol, T feas_tol, bool harris,
                       T& theta) {
    Key k = key_none();
    if (!harris) {
      for (int i = threadIdx.x; i < g.m; i += blockDim.x) {
        const T a = colx[i];
        if (a > piv_tol) {
          const T rh = rhsx[i];
          const T th = rh > T(0) ? rh / a : T(0);
          Key kk = ratio_key(th, basis[i], i);
          if (key_less(kk, k)) k = kk;
        }
      }
      k = block_min(k, redR);
      theta = key_theta(k, T(0));
      return k;
    }
    for (int i = threadIdx.x; i < g.m; i += blockDim.x) {
      const T a = colx[i];
      if (a > piv_tol) {
        const T rh = rhsx[i];
        const T rr = rh > T(0) ? rh : T(0);
        const T th1 = (rr + feas_tol) / a;
        Key kk = ratio_key(th1, 0, i);
        if (key_less(kk, k)) k = kk;
      }
    }
    k = block_min(k, redR);
    if (k.w2 == ~0u) return k;
    const T tmax = key_theta(k, T(0));
    Key k2 = key_none();
    for (int i = threadIdx.x; i < g.m; i += blockDim.x) {
      const T a = colx[i];
      if (a > piv_tol) {
        const T rh = rhsx[i];
        const T th = rh > T(0) ? rh / a : T(0);
        if (th <= tmax) {
          Key kk = big_key(a, basis[i], i);
          if (key_less(kk, k2)) k2 = kk;
        }
      }
    }
    k2 = block_min(k2, redH);
    const int r = (int)k2.w3;
    const T a = colx[r], rh = rhsx[r];
    theta = rh > T(0) ? rh / a : T(0);
    return k2;
  }

  // Pivot row scale + objective-row update + pricing of the next column.
  __device__ Key pivot_rows(const Geom& g, int r, const T* pcol, int c0, int lc,
                            bool bland, T opt_tol, int price_cols) {
    const T piv = pcol[r];
    const T dq = pcol[g.m];
    T* prow = tab + (size_t)r * g.ldw;
    T* drow = tab + (size_t)g.m * g.ldw;
    Key k = key_none();
    for (int v = threadIdx.x; v < g.nl; v += blockDim.x) {
      VT p = *reinterpret_cast<const VT*>(prow + v * V);
      p = v_div(p, piv);
      *reinterpret_cast<VT*>(prow + v * V) = p;
      VT d = *reinterpret_cast<const VT*>(drow + v * V);
      if (dq != T(0)) {
        d = v_fma(dq, p, d);
        *reinterpret_cast<VT*>(drow + v * V) = d;
      }
#pragma unroll
      for (int e = 0; e < V; ++e) {
        const int lj = v * V + e;
        const T dv = vget<VT, T>(d, e);
        const int j = c0 + lj;
        if (lj < lc && j < price_cols && dv < -opt_tol) {
          Key kk = price_key(dv, j, bland);
          if (key_less(kk, k)) k = kk;
        }
      }
    }
    k = block_min(k, redP);
    return cluster_min(k);
  }

  // Rank-1 update of rows 0..m-1 except r; the owner of the next column qn
  // extracts it into colx_next, every CTA extracts its RHS replica.
  __device__ void update_body(const Geom& g, int r, const T* pcol, int qn,
                              int owner_n, int c0, T* colx_next) {
    const int nt = (int)blockDim.x;
    const int G = nt / g.nl;
    const int grp = threadIdx.x / g.nl;
    const int lane = threadIdx.x - grp * g.nl;
    if (grp >= G) return;
    const VT p = *reinterpret_cast<const VT*>(tab + (size_t)r * g.ldw + lane * V);
    const int qloc = qn - c0;
    const bool has_q = qn >= 0 && owner_n == rank && (qloc / V) == lane;
    const int qe = qloc - lane * V;
    const bool has_rhs = lane == g.cw / V;
    for (int i = grp; i < g.m; i += G) {
      VT t;
      if (i != r) {
        const T f = pcol[i];
        VT* tp = reinterpret_cast<VT*>(tab + (size_t)i * g.ldw + lane * V);
        if (f != T(0)) {
          t = v_fma(f, p, *tp);
          *tp = t;
        } else {
          t = *tp;  // fma(-0, p, t) would only flip the sign of a zero t
        }
      } else {
        t = p;
      }
      if (has_q) colx_next[i] = vget<VT, T>(t, qe);
      if (has_rhs) rhsx[i] = vget<VT, T>(t, 0);
    }
    if (has_q && grp == 0) colx_next[g.m] = tab[(size_t)g.m * g.ldw + qloc];
  }

  // The primal simplex loop from the current tableau (the oracle's
  // simplex_loop).  Pricing covers global columns [0, price_cols).
  __device__ int loop(const Geom& g, int c0, int lc, int price_cols, const LpArgs& a,
                      int max_piv, int& pivots, bool& bland, int& degen, int& cur) {
    const T opt_tol = (T)a.opt_tol, piv_tol = (T)a.piv_tol, feas_tol = (T)a.feas_tol;
    const T deg_tol = (T)a.deg_tol;
    Key kq = price_only(g, c0, lc, bland, opt_tol, price_cols);
    int q = kq.w2 == ~0u ? -1 : (int)kq.w2;
    if (q < 0) return kOpt;
    if (pivots >= max_piv) return kUndef;
    int owner = q / g.cw;
    if (owner == rank) extract(g, q, c0, colbuf(cur));
    __syncthreads();
    for (;;) {
      // A: ratio test on the owner of q
      int r = -1;
      T theta = T(0);
      if (owner == rank) {
        Key kr = ratio(g, colbuf(cur), piv_tol, feas_tol, a.harris && !bland, theta);
        r = kr.w2 == ~0u ? -1 : (int)kr.w3;
        if (CLUSTER && threadIdx.x == 0) {
          sh->r = r;
          sh->theta = (double)theta;
        }
      }
      if (CLUSTER) {
        csync();  // B1
        if (owner != rank) {
          const SharedState* os = remote(sh, owner);
          r = os->r;
          theta = (T)os->theta;
        }
      }
      if (r < 0) return kUnbnd;
      if (CLUSTER && owner != rank) {
        const T* src = remote(colbuf(cur), owner);
        for (int i = threadIdx.x; i <= g.m; i += blockDim.x) colbuf(cur)[i] = src[i];
        __syncthreads();
      }
      if (theta <= deg_tol) {
        if (++degen > a.bland_after) bland = true;
      } else {
        degen = 0;
      }
      // C: pivot row, objective row, next pricing (cluster barrier B2 inside)
      const T* pcol = colbuf(cur);
      Key kn = pivot_rows(g, r, pcol, c0, lc, bland, opt_tol, price_cols);
      const int qn = kn.w2 == ~0u ? -1 : (int)kn.w2;
      const int owner_n = qn >= 0 ? qn / g.cw : -1;
      if (threadIdx.x == 0) basis[r] = q;
      // D: body update, extraction of the next pivot column
      update_body(g, r, pcol, qn, owner_n, c0, colbuf(cur ^ 1));
      __syncthreads();
      cur ^= 1;
      ++pivots;
      if (qn < 0) return kOpt;
      if (pivots >= max_piv) return kUndef;
      q = qn;
      owner = owner_n;
    }
  }

  // Objective row from the current basis: d_j = sum_i cB_i T_ij - c_j over
  // local columns (phase II after phase I), or the phase I row
  // -sum_{artificial rows} T_ij.  Sums run over rows in increasing order, as
  // the oracle does.
  __device__ void objective_row(const Geom& g, int c0, int lc, const double* c,
                                bool phase1) {
    const int nart0 = g.n + g.m;
    for (int lj = threadIdx.x; lj <= g.cw; lj += blockDim.x) {
      const bool is_rhs = lj == g.cw;
      if (!is_rhs && lj >= lc) continue;
      const int j = is_rhs ? -1 : c0 + lj;
      T acc = T(0);
      if (phase1) {
        if (!is_rhs && j >= nart0) continue;  // artificial: stays 0
        for (int i = 0; i < g.m; ++i)
          if (basis[i] >= nart0) acc = acc - tab[(size_t)i * g.ldw + lj];
        tab[(size_t)g.m * g.ldw + lj] = acc;
      } else {
        for (int i = 0; i < g.m; ++i) {
          const int bi = basis[i];
          const T cb = bi < g.n ? (T)c[bi] : T(0);
          acc = fma_t(cb, tab[(size_t)i * g.ldw + lj], acc);
        }
        const T cj = (!is_rhs && j < g.n) ? (T)c[j] : T(0);
        tab[(size_t)g.m * g.ldw + lj] = is_rhs ? acc : acc - cj;
      }
    }
  }
  __device__ static double fma_t(double a, double b, double c) { return fma(a, b, c); }
  __device__ static float fma_t(float a, float b, float c) { return fmaf(a, b, c); }

  // Drive zero-level artificials out of the basis after phase I: for each
  // such row, pivot on the lowest column j < n+m with |T_ij| > piv_tol.
  __device__ void drive_out(const Geom& g, int c0, int lc, const LpArgs& a, int& pivots,
                            int& cur) {
    const T piv_tol = (T)a.piv_tol;
    const int nart0 = g.n + g.m;
    for (int i = 0; i < g.m; ++i) {
      if (basis[i] < nart0) continue;  // uniform across the block and cluster
      Key k = key_none();
      const T* row = tab + (size_t)i * g.ldw;
      for (int lj = threadIdx.x; lj < lc; lj += blockDim.x) {
        const int j = c0 + lj;
        const T v = row[lj];
        if (j < nart0 && (v > piv_tol || v < -piv_tol)) {
          Key kk{0u, 0u, (unsigned)j, 0u};
          if (key_less(kk, k)) k = kk;
        }
      }
      k = block_min(k, redP);
      k = cluster_min(k);
      if (CLUSTER) csync();  // pslot reads done before the next write
      if (k.w2 == ~0u) continue;  // redundant row: artificial stays basic at 0
      const int q = (int)k.w2;
      const int owner = q / g.cw;
      if (owner == rank) extract(g, q, c0, colbuf(cur));
      if (CLUSTER) {
        csync();
        if (owner != rank) {
          const T* src = remote(colbuf(cur), owner);
          for (int e = threadIdx.x; e <= g.m; e += blockDim.x) colbuf(cur)[e] = src[e];
        }
      }
      __syncthreads();
      const T* pcol = colbuf(cur);
      // pivot without pricing: reuse pivot_rows with an impossible tolerance
      pivot_rows(g, i, pcol, c0, lc, false, T(0), 0);
      if (threadIdx.x == 0) basis[i] = q;
      update_body(g, i, pcol, -1, -1, c0, colbuf(cur ^ 1));
      __syncthreads();
      if (CLUSTER) csync();  // column copies done before the owner's next extract
      ++pivots;
    }
  }

  __device__ void run(const LpArgs& a, const ClassArgs& ca) {
    const int tid = threadIdx.x, nt = blockDim.x;
    for (;;) {
      if (rank == 0 && tid == 0) sh->ticket = atomicAdd(ca.ticket, 1);
      csync();
      const int t = *remote(&sh->ticket, 0);
      if (t >= ca.count) break;
      const int lp = ca.order[t];
      const int m = a.m[lp], n = a.n[lp];
      const double* A = a.A + a.offA[lp];
      const double* b = a.b + a.offb[lp];
      const double* c = a.c + a.offc[lp];
      // two-phase when any b_i < 0 (the reference's rem list, simplex.cu:574-583)
      int na = 0;
      for (int i = tid; i < m; i += nt) na += b[i] < 0.0 ? 1 : 0;
      na = block_sum(na);
      const Geom g(m, n, na, K, V);
      if (m > ca.max_m || g.ldw > ca.max_ldw) {
        // the LP does not fit the layout this plan was built for (e.g. a
        // plan made without b has no room for phase-I columns): refuse it
        if (rank == 0 && tid == 0) {
          a.status[lp] = kUndef;
          a.obj[lp] = 0.0;
          if (a.pivots) a.pivots[lp] = -1;
        }
        __syncthreads();
        continue;
      }
      const int c0 = rank * g.cw;
      const int lc = max(0, min(g.cw, g.Wc - c0));
      // load the slack-basis tableau (rows with b_i < 0 negated, with an
      // artificial column each); coalesced along rows of A
      const int warp = tid >> 5, lane = tid & 31, nw = nt >> 5;
      for (int i = warp; i <= m; i += nw) {
        const bool neg = i < m && b[i] < 0.0;
        const T sgn = neg ? T(-1) : T(1);
        // index of this row's artificial column (rank among negative rows)
        int aidx = -1;
        if (neg && na > 0) {
          int cnt = 0;
          for (int i2 = lane; i2 < i; i2 += 32) cnt += b[i2] < 0.0 ? 1 : 0;
          cnt = __reduce_add_sync(0xffffffffu, cnt);
          aidx = cnt;
        }
        T* row = tab + (size_t)i * g.ldw;
        for (int lj = lane; lj < g.ldw; lj += 32) {
          T v = T(0);
          if (lj < lc) {
            const int j = c0 + lj;
            if (i < m) {
              if (j < n)
                {
                const T av = (T)A[(size_t)i * n + j];
                v = neg ? -av : av;
              }
              else if (j < n + m)
                v = (j - n == i) ? sgn : T(0);
              else
                v = (aidx >= 0 && j - n - m == aidx) ? T(1) : T(0);
            } else if (na == 0 && j < n) {
              v = -(T)c[j];
            }
          } else if (lj == g.cw && i < m) {
            {
            const T bv = (T)b[i];
            v = neg ? -bv : bv;
          }
          }
          row[lj] = v;
        }
        if (i < m && lane == 0) basis[i] = neg ? n + m + aidx : n + i;
      }
      __syncthreads();
      int pivots = 0, degen = 0, cur = 0, st;
      bool bland = false;
      const int max_piv = a.max_pivots > 0 ? a.max_pivots : 50 * (m + n) + 1000;
      if (na > 0) {
        objective_row(g, c0, lc, c, true);
        __syncthreads();
        st = loop(g, c0, lc, n + m, a, max_piv, pivots, bland, degen, cur);
        if (CLUSTER) csync();
        if (st == kOpt) {
          const double z = (double)tab[(size_t)m * g.ldw + g.cw];
          if (z < -a.phase1_tol) st = kNoFeas;
        } else if (st == kUnbnd) {
          st = kUndef;
        }
        if (st == kOpt) {
          drive_out(g, c0, lc, a, pivots, cur);
          objective_row(g, c0, lc, c, false);
          __syncthreads();
          bland = false;
          degen = 0;
          st = loop(g, c0, lc, n + m, a, max_piv, pivots, bland, degen, cur);
        }
      } else {
        st = loop(g, c0, lc, n + m, a, max_piv, pivots, bland, degen, cur);
      }
      // outputs (rank 0 holds a replica of the RHS column)
      if (rank == 0) {
        if (tid == 0) {
          a.status[lp] = st;
          a.obj[lp] = (double)tab[(size_t)m * g.ldw + g.cw];
          if (a.pivots) a.pivots[lp] = pivots;
        }
        if (a.basis)
          for (int i = tid; i < m; i += nt) a.basis[a.offbasis[lp] + i] = basis[i];
        if (a.x) {
          double* x = a.x + a.offx[lp];
          for (int j = tid; j < n; j += nt) x[j] = 0.0;
          __syncthreads();
          for (int i = tid; i < m; i += nt)
            if (basis[i] < n) x[basis[i]] = (double)tab[(size_t)i * g.ldw + g.cw];
        }
      }
      __syncthreads();
    }
    if (CLUSTER) csync();  // no CTA leaves while others may read its smem
  }

  __device__ int block_sum(int v) {
    v = __reduce_add_sync(0xffffffffu, v);
    int* red = reinterpret_cast<int*>(redR);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) red[warp] = v;
    __syncthreads();
    const int nw = (int)(blockDim.x >> 5);
    int s = lane < nw ? red[lane] : 0;
    s = __reduce_add_sync(0xffffffffu, s);
    __syncthreads();
    return s;
  }
};

template <typename T, bool CLUSTER>
__global__ void __launch_bounds__(512, 1) solve_kernel(const LpArgs a, const ClassArgs ca) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Solver<T, CLUSTER> s;
  const Layout L(ca.max_m, ca.max_ldw, (int)sizeof(T));
  s.smem = smem_raw;
  s.tab = reinterpret_cast<T*>(smem_raw + L.tab);
  s.col0 = reinterpret_cast<T*>(smem_raw + L.colA);
  s.col1 = reinterpret_cast<T*>(smem_raw + L.colB);
  s.rhsx = reinterpret_cast<T*>(smem_raw + L.rhsx);
  s.basis = reinterpret_cast<int*>(smem_raw + L.basis);
  s.redP = reinterpret_cast<Key*>(smem_raw + L.red);
  s.redR = s.redP + 32;
  s.redH = s.redP + 64;
  s.sh = reinterpret_cast<SharedState*>(smem_raw + L.state);
  s.K = ca.K;
  s.rank = CLUSTER ? (int)cg::this_cluster().block_rank() : 0;
  s.run(a, ca);
}

}  // namespace dev
}  // namespace blpg
