// Batched dense-tableau primal simplex for sm_103a.
//
// One LP per CTA, or per thread-block cluster of K CTAs when the tableau does
// not fit one CTA's shared memory (K in {1,2,4,8}).  The kernel is
// persistent: each CTA (cluster) takes LP tickets from a device work queue
// until the class's queue is empty.
//
// Reference kernel: BLPG-Solver/src/simplex.cu:35-385 (mykernel).  Same
// method, rebuilt for Blackwell:
//   - the tableau is condensed: basic columns are unit vectors, so only the
//     nonbasic columns and the RHS are stored, (m + 1) x (n + na + 1)
//     instead of (m + 1) x (n + m + na + 1).  A pivot on (r, q) puts the
//     leaving variable into q's column slot with entries 1/a_rq in row r and
//     -t_iq / a_rq elsewhere, which are the values the full tableau's
//     elimination writes into that variable's unit column; slot labels
//     (cvar) and variable positions (vpos) are kept beside the tableau, and
//     ties are broken on variable ids, so every decision and every output
//     matches the full-tableau oracle (only signs of zero entries inside the
//     tableau may differ, and a zero never decides anything);
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
  const int32_t* hint;  // nullable: m basic column ids per LP (offbasis layout)
  int32_t* info;        // nullable: per-LP flags (kInfo*)
  double ptol;          // primal feasibility tolerance of the final checks
  int32_t refresh_period;  // FP32: FP64 refresh every k pivots (0: at the end)
  int32_t warm_mode;       // 0: hinted basis infeasible both ways -> cold; 1: cost-shifted dual
  double shift;            // cost shift of warm_mode 1
  int32_t pricing;         // 0: Dantzig, 1: steepest edge (exact column norms)
  const float* weight;     // nullable: steepest-edge score weight per variable (n + m per LP)
  const int64_t* offw;     // offsets of `weight`
  const float* A32;        // nullable: A rounded to FP32, rows padded to a32_pitch(n)
  const int64_t* off32;    // offsets of A32 (with A32)
  int32_t* fb;             // nullable (FP32 plans): [0] count, [1..] LPs handed to the FP64 pass
  int32_t info_or;         // bits OR'ed into every info written (the FP64 pass: kInfoFp64)
};

// Bits of the per-LP info output.
constexpr int kInfoWarm = 1;       // a basis hint was used
constexpr int kInfoFallback = 2;   // hinted basis infeasible both ways: cold solve
constexpr int kInfoPartial = 4;    // some hinted columns found no pivot
constexpr int kInfoDual = 8;       // dual simplex pivots were taken
constexpr int kInfoRefresh = 16;   // FP64 refresh of the FP32 tableau ran
constexpr int kInfoRepair = 32;    // a refresh found a violation (more pivots)
constexpr int kInfoShift = 64;     // hinted basis infeasible both ways: cost-shifted dual phase
constexpr int kInfoUnverified = 128;  // FP32: the FP64 refresh could not verify the final basis
constexpr int kInfoReinvert = 256;    // the tableau was rebuilt from an FP64 factorisation
constexpr int kInfoFactor = 512;      // an FP64 refresh used the LU factorisation (refresh_lu)
constexpr int kInfoFp64 = 1024;       // re-solved on an FP64 tableau (the FP64 pass of an FP32 plan)
constexpr int kInfoRetry = 2048;      // a warm start ended unverified or at the pivot cap: re-run cold
constexpr int kInfoLoad = 4096;       // a tableau load's bulk copies did not complete: LP given up

struct ClassArgs {
  const int32_t* order;  // LP ids of this class, heaviest first
  int32_t count;
  const int32_t* count_dev;  // nullable: the count in device memory (the FP64 pass's list)
  int32_t* ticket;  // queue head, zeroed before the launch
  int32_t K;        // CTAs per LP (cluster size)
  int32_t max_na;   // artificial columns (two-phase LPs); LPs with more are refused
  int32_t se;       // steepest-edge pricing: the layout holds column norms
  int32_t smem;     // dynamic shared memory per CTA; LPs whose layout is larger are refused
  double* lu;          // nullable: FP64 scratch of the LU refresh, lu_stride doubles per
  long long lu_stride; // CTA (per cluster: the cluster's index blockIdx.x / K)
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
// Row pitch of the FP32 copy of A (elements): the row length of a
// single-CTA phase-II FP32 tableau (Geom with K = 1, na = 0, V = 4), so that
// such an LP's whole block is one contiguous copy; every row 16-byte aligned.
__host__ __device__ inline int a32_pitch(int n) { return round_up(n, 4) + 4; }

// Per-LP column geometry.  Variables 0..n-1 structural, n..n+m-1 slacks,
// n+m..n+m+na-1 artificials (two-phase only).  The tableau stores Wc = n + na
// column slots (one per nonbasic variable); CTA k of the cluster holds slots
// [k*cw, k*cw + cw) at local 0..cw-1, the RHS at local cw, zero padding after
// it; rows 0..m-1 constraints, row m objective.
struct Geom {
  int m, n, na, Wc, cw, ldw, nl;
  __host__ __device__ Geom(int m_, int n_, int na_, int K, int V) {
    m = m_;
    n = n_;
    na = na_;
    Wc = n + na;
    cw = round_up(ceil_div(Wc, K), V);
    ldw = cw + V;
    nl = ldw / V;
  }
};

// Shared-memory layout of one LP (bytes), identical on host and device.  A
// fixed header (the CTA's state and argmin scratch) comes first; the LP's
// regions follow, sized for its own m, column width ldw and variable count
// nv, so a CTA lays out each LP it takes within its allocation and a class
// only needs the largest member's total.
struct Layout {
  int tab, colA, colB, rhsx, basis, flags, cvar, vpos, ext, red, state, gam, gbytes, total;
  // pbytes: bytes the norm region must hold for partial sums (0: the counters
  // and whatever the region has anyway)
  __host__ __device__ Layout(int m, int ldw, int nv, int elem, int se = 0, int pbytes = 0) {
    const int mp1 = round_up(m + 1, 4);
    const int nvp = round_up(nv, 4);
    state = 0;
    int off = 224;
    red = off;
    off += 3 * 32 * 16;  // three argmin scratch buffers (pricing, ratio, Harris)
    tab = off;
    off += round_up((m + 1) * ldw * elem, 16);
    colA = off;
    off += round_up(mp1 * elem, 16);
    colB = off;
    off += round_up(mp1 * elem, 16);
    rhsx = off;
    off += round_up(mp1 * elem, 16);
    basis = off;
    off += round_up(mp1 * 4, 16);
    flags = off;
    off += round_up(mp1 * 4, 16);
    cvar = off;  // variable id of every column slot
    off += nvp * 4;
    vpos = off;  // slot of every nonbasic variable, -1 - row of a basic one
    off += nvp * 4;
    ext = off;
    // FP64 x_B, duals and a 32-bit list of the refresh (FP32 tableaux, and
    // FP64 ones with steepest edge, which are verified in FP64 too)
    const int ext_bytes = (elem == 4 || se) ? 2 * mp1 * 8 + mp1 * 4 : 0;
    off += ext_bytes;
    // steepest edge: two 32-bit fixed-point norm counters per local column slot,
    // sharing the refresh's region when it is large enough (the norms are
    // recomputed after every refresh)
    gam = -1;
    gbytes = 0;
    if (se) {
      if (ext_bytes >= ldw * 8) {
        // over the refresh's region, extended past it for partial sums
        gam = ext;
        gbytes = ext_bytes;
        if (pbytes > gbytes) {
          off += round_up(pbytes - gbytes, 16);
          gbytes += round_up(pbytes - gbytes, 16);
        }
      } else {
        off = round_up(off, 16);
        gam = off;
        gbytes = round_up(ldw * 8 > pbytes ? ldw * 8 : pbytes, 16);
        off += gbytes;
      }
    }
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

// W1 = false: every real key has w1 == 0 (FP32 values fit w0), so that word
// is not reduced (an all-empty warp then returns w1 = 0, still empty by w2).
template <bool W1 = true>
__device__ __forceinline__ Key warp_min(const Key& k) {
  const unsigned full = 0xffffffffu;
  Key r;
  r.w0 = __reduce_min_sync(full, k.w0);
  bool e0 = k.w0 == r.w0;
  r.w1 = W1 ? __reduce_min_sync(full, e0 ? k.w1 : ~0u) : 0u;
  bool e1 = e0 && (!W1 || k.w1 == r.w1);
  r.w2 = __reduce_min_sync(full, e1 ? k.w2 : ~0u);
  bool e2 = e1 && k.w2 == r.w2;
  r.w3 = __reduce_min_sync(full, e2 ? k.w3 : ~0u);
  return r;
}

// Block-wide argmin: every thread returns the winner.  Contains exactly one
// __syncthreads; `red` (32 keys) must not be reused before another barrier.
template <bool W1 = true>
__device__ __forceinline__ Key block_min(const Key& k, Key* red) {
  Key w = warp_min<W1>(k);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) red[warp] = w;
  __syncthreads();
  const int nw = (int)(blockDim.x >> 5);
  Key v = lane < nw ? red[lane] : key_none();
  return warp_min<W1>(v);
}

// Block-wide minimum of the value words only (w0, and w1 with W1): every
// thread returns them, w2 = w3 = 0, or key_none() when no thread had a
// value.  For a minimum whose ties do not matter (Harris's first pass).  One
// __syncthreads, `red` as block_min.
template <bool W1 = true>
__device__ __forceinline__ Key block_min_value(const Key& k, Key* red) {
  const unsigned full = 0xffffffffu;
  auto vmin = [&](unsigned a0, unsigned a1, unsigned& r0, unsigned& r1) {
    r0 = __reduce_min_sync(full, a0);
    r1 = W1 ? __reduce_min_sync(full, a0 == r0 ? a1 : ~0u) : 0u;
  };
  unsigned w0, w1;
  vmin(k.w0, k.w1, w0, w1);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) red[warp] = Key{w0, w1, 0u, 0u};
  __syncthreads();
  const int nw = (int)(blockDim.x >> 5);
  const Key v = lane < nw ? red[lane] : key_none();
  vmin(v.w0, v.w1, w0, w1);
  return w0 == ~0u ? key_none() : Key{w0, w1, 0u, 0u};
}

// Pricing key of reduced cost d of variable j in column slot s (only
// d < -tol is eligible).  For negative numbers ~bits is increasing in the
// value, so the most negative d has the smallest key; ties go to the lowest
// variable id; Bland's rule zeroes the value words so the lowest variable id
// wins.  The payload is the slot.
__device__ __forceinline__ Key price_key(double d, int j, int s, bool bland) {
  unsigned long long u = ~(unsigned long long)__double_as_longlong(d);
  if (bland) u = 0ull;
  return Key{(unsigned)(u >> 32), (unsigned)u, (unsigned)j, (unsigned)s};
}
__device__ __forceinline__ Key price_key(float d, int j, int s, bool bland) {
  unsigned u = ~__float_as_uint(d);
  if (bland) u = 0u;
  return Key{u, 0u, (unsigned)j, (unsigned)s};
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
// Most negative value first (as price_key), ties by `tie`, payload `row`.
__device__ __forceinline__ Key neg_key(double v, int tie, int row) {
  unsigned long long u = ~(unsigned long long)__double_as_longlong(v);
  return Key{(unsigned)(u >> 32), (unsigned)u, (unsigned)tie, (unsigned)row};
}
__device__ __forceinline__ Key neg_key(float v, int tie, int row) {
  return Key{~__float_as_uint(v), 0u, (unsigned)tie, (unsigned)row};
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

// Bulk (TMA) copies from global to this CTA's shared memory, completing on
// an mbarrier in shared memory: both addresses 16-byte aligned, the size a
// multiple of 16 (the callers check both).  No cluster multicast.
__device__ __forceinline__ unsigned smem_addr(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_inval(unsigned long long* bar) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
  unsigned done;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(done)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return done != 0;
}
// Bounded wait for phase `parity` of an mbarrier (every thread that reads
// the copied data waits itself): false when it did not complete.
constexpr int kBarWaitLimit = 1 << 22;
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity) {
  for (int it = 0; it < kBarWaitLimit; ++it)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes,
                                         unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}
// Orders this thread's earlier generic-proxy accesses to shared memory
// before later bulk copies into it.
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ double sdiv(double a, double b) { return a / b; }
__device__ __forceinline__ float sdiv(float a, float b) { return __fdiv_rn(a, b); }
// Local index of global slot s on the CTA holding slots [c0, c0 + cw), -1 on
// the other CTAs.
__device__ __forceinline__ int local_slot(int s, int c0, int cw) {
  return s >= c0 && s < c0 + cw ? s - c0 : -1;
}

__device__ __forceinline__ void vset(double2& v, int e, double x) {
  if (e == 0) v.x = x; else v.y = x;
}
__device__ __forceinline__ void vset(float4& v, int e, float x) {
  if (e == 0) v.x = x; else if (e == 1) v.y = x; else if (e == 2) v.z = x; else v.w = x;
}

__device__ __forceinline__ double2 v_fma(double f, const double2& p, const double2& t) {
  return make_double2(fma(-f, p.x, t.x), fma(-f, p.y, t.y));
}
__device__ __forceinline__ float4 v_fma(float f, const float4& p, const float4& t) {
  return make_float4(fmaf(-f, p.x, t.x), fmaf(-f, p.y, t.y), fmaf(-f, p.z, t.z),
                     fmaf(-f, p.w, t.w));
}
// Steepest-edge norm accumulation.  Pricing only needs the norms' size, so
// an FP64 value enters as an FP32 approximation of its magnitude built from
// its exponent and top 20 mantissa bits with integer operations (values
// below FLT_MIN count as 0, above FLT_MAX as FLT_MAX): the squares then run
// on the FP32 pipe, not GB300's slow FP64 pipe.  FP32 values are squared as
// they are.
__device__ __forceinline__ float mag_f32(double x) {
  const unsigned hi = (unsigned)((unsigned long long)__double_as_longlong(x) >> 32) & 0x7FFFFFFFu;
  const int e = (int)(hi >> 20) - 896;  // biased FP32 exponent
  const unsigned bits = ((unsigned)e << 23) | ((hi & 0xFFFFFu) << 3);
  return e <= 0 ? 0.f : (e >= 255 ? 3.4e38f : __uint_as_float(bits));
}
// FP64 -> FP32 for the tableau, built with integer operations and selects
// (the FP64-to-FP32 conversion instruction runs at GB300's low FP64 rate, and
// per-element branches would diverge on every mix of zeros and nonzeros).  A
// funnel shift of the two halves left by 3 puts the low 8 bits of the FP64
// exponent e and the top 23 fraction bits where FP32 keeps its exponent and
// fraction; for e in [897, 1150] the FP32 exponent e - 896 equals those 8
// bits with the top one flipped.  The 29 dropped bits round up above one half
// and at one half when the kept bits are odd: their sum with 2^28 - 1 plus
// the kept lowest bit carries out of bit 29 exactly then (a carry into the
// exponent is the correctly rounded result, up to infinity).  Larger values
// give infinity (NaN stays NaN); values below FP32's normal range (below
// 1.2e-38, where FP32 would have subnormals) give zero of their sign.
__device__ __forceinline__ float f64_to_f32_rn(double x) {
  const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  const unsigned e = (hi >> 20) & 0x7FFu, sign = hi & 0x80000000u;
  unsigned bits = (__funnelshift_l(lo, hi, 3) & 0x7FFFFFFFu) ^ 0x40000000u;
  bits += ((lo & 0x1FFFFFFFu) + 0x0FFFFFFFu + (bits & 1u)) >> 29;
  const bool nan = e == 0x7FFu && ((hi & 0xFFFFFu) | lo) != 0u;
  const unsigned big = nan ? 0x7FC00000u : 0x7F800000u;
  const unsigned out = e - 897u < 254u ? bits : (e >= 897u ? big : 0u);
  return __uint_as_float(sign | out);
}
__device__ __forceinline__ float to_tab(double x, float) { return f64_to_f32_rn(x); }
__device__ __forceinline__ double to_tab(double x, double) { return x; }

template <typename T>
struct SqT;
template <>
struct SqT<double> {
  using type = float2;
};
template <>
struct SqT<float> {
  using type = float4;
};
__device__ __forceinline__ float2 v_sq(const double2& t, const float2& a) {
  const float x = mag_f32(t.x), y = mag_f32(t.y);
  return make_float2(fmaf(x, x, a.x), fmaf(y, y, a.y));
}
__device__ __forceinline__ float4 v_sq(const float4& t, const float4& a) {
  return make_float4(fmaf(t.x, t.x, a.x), fmaf(t.y, t.y, a.y), fmaf(t.z, t.z, a.z),
                     fmaf(t.w, t.w, a.w));
}
__device__ __forceinline__ float sq_get(const float2& a, int e) { return e == 0 ? a.x : a.y; }
__device__ __forceinline__ float sq_get(const float4& a, int e) {
  return e == 0 ? a.x : (e == 1 ? a.y : (e == 2 ? a.z : a.w));
}
__device__ __forceinline__ double2 v_div(const double2& a, double d) {
  return make_double2(a.x / d, a.y / d);
}
__device__ __forceinline__ float4 v_div(const float4& a, float d) {
  return make_float4(__fdiv_rn(a.x, d), __fdiv_rn(a.y, d), __fdiv_rn(a.z, d),
                     __fdiv_rn(a.w, d));
}

// Steepest-edge column norms gamma_j = 1 + sum_i T_ij^2 are summed as
// fixed-point integers with 2^-24 resolution, in two 32-bit shared counters
// per column (x: the 24-bit fractions, y: the integer parts): integer sums do
// not depend on the order of the additions, and a 32-bit shared atomic add
// is one instruction where a 64-bit one is a compare-and-swap loop.  At most
// kMaxNormGroups partial sums reach a column, each clamped to 2^25, so the
// integer counter stays below 2^31 and the fraction counter below 2^30.
constexpr int kMaxNormGroups = 64;
// The two parts of RN(v * 2^24) come from 32-bit conversions: v * 2^24 is
// exact, an integer from v = 1/2 up, so truncating v gives the integer part
// exactly and the remainder v - trunc(v) is exact too.
__device__ __forceinline__ void norm_add(uint2* gcol, float v) {
  v = fminf(v, 33554432.f);
  const unsigned ip = __float2uint_rz(v);
  atomicAdd(&gcol->x, __float2uint_rn((v - (float)ip) * 16777216.f));
  atomicAdd(&gcol->y, ip);
}
__device__ __forceinline__ float norm_gamma(uint2 gv) {
  return 1.f + ((float)gv.y + (float)gv.x * (1.f / 16777216.f));
}
// The FP32 single-CTA steepest-edge loop keeps the norms as partial sums
// instead, when they fit the norm region: row group g of the sweep stores its
// sums of squares of local slots [0, cw) in row g of a G x cw float array
// (one 16-byte store per thread, no atomics), clamped like the counters, and
// pricing adds the G partials of a column in group order, so the sum is the
// same on every run.
__device__ __forceinline__ float norm_clamp(float v) { return fminf(v, 33554432.f); }

// Status codes (GLPK numbering, as blpg.h)
constexpr int kUndef = 1, kNoFeas = 4, kOpt = 5, kUnbnd = 6;
constexpr int kRefresh = 100;  // internal: the primal loop paused for a refresh
constexpr int kUnverified = 101;  // internal: the FP64 refresh could not verify the basis
// Iterative-refinement steps of the FP64 refresh; a refresh whose last
// correction is still above 1e-10 of the values reports no convergence (the
// FP32 B^-1 is too inaccurate to verify the basis).
constexpr int kRefineIters = 4;

struct SharedState {
  int ticket;
  int r;
  int pad0, pad1;
  double theta;
  Key pslot;
  Key aux;
  double z;       // FP64 objective of the last refresh
  unsigned long long bar;  // mbarrier of the tableau's bulk loads (valid only during a load)
  Key gather[8];  // the cluster's pricing candidates, fetched once per CTA
};

// ---------------------------------------------------------------------------
// The solver kernel
// ---------------------------------------------------------------------------

template <typename T, bool CLUSTER>
struct Solver {
  using VT = typename VecT<T>::type;
  static constexpr int V = VecT<T>::V;
  static constexpr bool kW1 = sizeof(T) == 8;  // keys use w1 only for FP64 values

  unsigned char* smem;
  T* tab;
  T* col0;
  T* col1;
  __device__ T* colbuf(int k) const { return k ? col1 : col0; }
  T* rhsx;
  int* basis;
  int* flags;
  int* cvar;   // slot -> variable id (every slot of the LP, replicated per CTA)
  int* vpos;   // variable -> slot if nonbasic, -1 - row if basic
  uint2* gam;  // steepest edge: fixed-point column norms of the local slots
  int ngrp;     // or, when > 0, that many rows of per-row-group partial sums
                // of slots [0, cw) in the same region (row pitch cw)
  double* xr;  // FP64 x_B of the refresh (FP32 tableaux, FP64 ones with steepest edge)
  double* yr;  // FP64 duals of the refresh
  float* rf;   // the refresh's residuals rounded to FP32 / a 32-bit list
  double* lu;  // nullable: this CTA's FP64 scratch for the LU refresh (global memory)
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
    // K threads fetch one remote candidate each; the CTA reduces locally
    if (threadIdx.x < K) sh->gather[threadIdx.x] = *remote(&sh->pslot, threadIdx.x);
    __syncthreads();
    Key best = key_none();
    for (int k = 0; k < K; ++k) {
      const Key o = sh->gather[k];
      if (key_less(o, best)) best = o;
    }
    return best;
  }

  // Local pricing over the objective row (no update): block + cluster min.
  // Variables below price_cols are eligible.
  __device__ Key price_only(const Geom& g, int c0, int lc, bool bland, T opt_tol,
                            int price_cols) {
    Key k = key_none();
    const T* d = tab + (size_t)g.m * g.ldw;
    for (int lj = threadIdx.x; lj < lc; lj += blockDim.x) {
      const int j = cvar[c0 + lj];
      const T v = d[lj];
      if (j < price_cols && v < -opt_tol) {
        Key kk = price_key(v, j, c0 + lj, bland);
        if (key_less(kk, k)) k = kk;
      }
    }
    k = block_min<kW1>(k, redP);
    return cluster_min(k);
  }

  // Owner of slot s copies its column (rows 0..m) and the RHS column into
  // the extraction buffers.
  __device__ void extract(const Geom& g, int s, int c0, T* colx) {
    const int ql = s - c0;
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
  // With fuse_sl >= 0 the entering column (local slot fuse_sl) and the RHS
  // are read from the tableau and copied into colx / rhsx on the way, the
  // first pass's barrier publishing them (single-CTA steepest-edge loop);
  // with zero_sl the tableau's slot is also cleared in rows 0..m-1, as the
  // FP32 steepest-edge sweep expects, and the RHS is not copied into rhsx
  // (that loop reads it from the tableau).  With recip the ratios are formed with
  // one reciprocal per row (the FP32 steepest-edge loops, which are not held
  // to the oracle's pivot sequence; the Dantzig loops divide, as it does).
  __device__ Key ratio(const Geom& g, T* colx, T piv_tol, T feas_tol, bool harris, T& theta,
                       int fuse_sl = -1, bool zero_sl = false, bool recip = false) {
    auto fetch = [&](int i, T& a, T& rh) {
      if (fuse_sl >= 0) {
        a = tab[(size_t)i * g.ldw + fuse_sl];
        rh = tab[(size_t)i * g.ldw + g.cw];
        colx[i] = a;
        if (zero_sl)
          tab[(size_t)i * g.ldw + fuse_sl] = T(0);
        else
          rhsx[i] = rh;
      } else {
        a = colx[i];
        rh = rhsx[i];
      }
    };
    if (fuse_sl >= 0 && threadIdx.x == 0) colx[g.m] = tab[(size_t)g.m * g.ldw + fuse_sl];
    Key k = key_none();
    if (!harris) {
      for (int i = threadIdx.x; i < g.m; i += blockDim.x) {
        T a, rh;
        fetch(i, a, rh);
        if (a > piv_tol) {
          const T th = rh > T(0) ? rh / a : T(0);
          Key kk = ratio_key(th, basis[i], i);
          if (key_less(kk, k)) k = kk;
        }
      }
      k = block_min<kW1>(k, redR);
      theta = key_theta(k, T(0));
      return k;
    }
    // pass 1 also keeps every eligible row's ratio rh / a (0 when rh <= 0),
    // so that pass 2 and theta reuse it: in the other column buffer, or with
    // zero_sl in rhsx (that loop writes its next multipliers into the other
    // column buffer right after this returns, with no barrier between, and
    // does not read rhsx)
    T* thx = zero_sl ? rhsx : (colx == col0 ? col1 : col0);
    for (int i = threadIdx.x; i < g.m; i += blockDim.x) {
      T a, rh;
      fetch(i, a, rh);
      if (a > piv_tol) {
        const T rr = rh > T(0) ? rh : T(0);
        T th1, th;
        if (recip) {
          const T ra = sdiv(T(1), a);
          th1 = (rr + feas_tol) * ra;
          th = rr * ra;
        } else {
          th1 = (rr + feas_tol) / a;
          th = rr / a;
        }
        thx[i] = th;
        Key kk = ratio_key(th1, 0, i);
        if (key_less(kk, k)) k = kk;
      }
    }
    // only the bound matters here, not which row gives it
    k = block_min_value<kW1>(k, redR);
    if (k.w2 == ~0u) return k;
    const T tmax = key_theta(k, T(0));
    Key k2 = key_none();
    for (int i = threadIdx.x; i < g.m; i += blockDim.x) {
      const T a = colx[i];
      if (a > piv_tol && thx[i] <= tmax) {
        Key kk = big_key(a, basis[i], i);
        if (key_less(kk, k2)) k2 = kk;
      }
    }
    k2 = block_min<kW1>(k2, redH);
    theta = thx[(int)k2.w3];
    return k2;
  }

  // Pivot on (r, slot s): the pivot row is divided by the pivot and its slot
  // s entry becomes 1/pivot (the leaving variable's column), the objective
  // row is updated with its slot s entry taken as 0 (the leaving variable's
  // reduced cost before the pivot), and the next column is priced; lv is the
  // leaving variable, now the label of slot s.
  // recip: the pivot row times 1/pivot (the FP32 steepest-edge loop, not
  // held to the oracle's pivot sequence) instead of divided by the pivot.
  __device__ Key pivot_rows(const Geom& g, int r, int s, int lv, const T* pcol, int c0,
                            int lc, bool bland, T opt_tol, int price_cols, bool recip = false) {
    const T piv = pcol[r];
    const T dq = pcol[g.m];
    const T rcp = sdiv(T(1), piv);
    T* prow = tab + (size_t)r * g.ldw;
    T* drow = tab + (size_t)g.m * g.ldw;
    const int sl = local_slot(s, c0, g.cw);
    const bool price = price_cols > 0;
    Key k = key_none();
    // one element per thread (the row is short: a few hundred entries), so
    // that each thread waits on one division, not a vector of them
    for (int lj = threadIdx.x; lj < g.ldw; lj += blockDim.x) {
      const T p = lj == sl ? rcp : (recip ? prow[lj] * rcp : sdiv(prow[lj], piv));
      prow[lj] = p;
      T d = drow[lj];
      if (dq != T(0)) {
        d = fma_t(-dq, p, lj == sl ? T(0) : d);
        drow[lj] = d;
      }
      if (price && lj < lc && d < -opt_tol) {
        const int j = lj == sl ? lv : cvar[c0 + lj];
        if (j < price_cols) {
          Key kk = price_key(d, j, c0 + lj, bland);
          if (key_less(kk, k)) k = kk;
        }
      }
    }
    if (!price) {  // no pricing: the pivot row only has to be visible
      __syncthreads();
      return k;
    }
    k = block_min<kW1>(k, redP);
    return cluster_min(k);
  }

  // Labels after a pivot on (r, slot s) that brought q in for lv (one
  // thread; every CTA of a cluster updates its own replica).
  __device__ void relabel(int r, int s, int q, int lv) {
    if (threadIdx.x == 0) {
      basis[r] = q;
      cvar[s] = lv;
      vpos[lv] = s;
      vpos[q] = -1 - r;
    }
  }

  // Rank-1 update of rows 0..m-1 except r; the owner of the next slot sn
  // extracts its column into colx_next, every CTA extracts its RHS replica.
  __device__ void update_body(const Geom& g, int r, int s, const T* pcol, int sn, int owner_n,
                              int c0, T* colx_next) {
    update_rows<false>(tab, rhsx, rank, g.m, g.ldw, g.nl, g.cw, r, s, pcol, sn, owner_n, c0,
                       colx_next, nullptr, 0);
  }
  // The same sweep, also summing the squares of every row's final values
  // into the column norms (steepest-edge pricing).
  __device__ void update_body_se(const Geom& g, int r, int s, const T* pcol, int c0, int lc) {
    update_rows<true>(tab, rhsx, rank, g.m, g.ldw, g.nl, g.cw, r, s, pcol, -1, -1, c0, nullptr,
                      gam, lc);
  }
  // The FP32 single-CTA steepest-edge sweep: the entering slot was cleared
  // by the ratio test and fcol is the pivot column with row r's entry 0, so
  // every row is t + f * p, stored where f != 0.  A row with f == 0 computes
  // t back (p is finite), so the norms take every computed row as it is.
  // The RHS replica is not extracted: the next ratio test reads the tableau.
  __device__ void update_body_se32(const Geom& g, int r, const T* fcol, int lc) {
    update_rows<true, true>(tab, rhsx, rank, g.m, g.ldw, g.nl, g.cw, r, -1, fcol, -1, -1, 0,
                            nullptr, gam, lc, ngrp ? reinterpret_cast<float*>(gam) : nullptr);
  }
  // Kept out of line with plain arguments (no `this`, no structs by
  // reference) so that the unrolled sweep has its own register budget and
  // nothing in its loop lives in local memory.  The slot s entry of every
  // updated row is taken as 0 before the elimination (it held the entering
  // column, whose slot now carries the leaving variable's unit column).
  template <bool SE, bool PRE = false>
  static __device__ __noinline__ void update_rows(T* const tb, T* const rhsx, const int rank,
                                                  const int m, const int ldw, const int nl,
                                                  const int cw, const int r, const int s,
                                                  const T* pcol, const int qn, const int owner_n,
                                                  const int c0, T* colx_next,
                                                  uint2* gam, const int lc,
                                                  float* part = nullptr) {
    const int nt = (int)blockDim.x;
    const int G = SE ? min(nt / nl, kMaxNormGroups) : nt / nl;  // rows of lanes
    const int grp = threadIdx.x / nl;
    const int lane = threadIdx.x - grp * nl;
    if (grp >= G) return;
    const VT p = *reinterpret_cast<const VT*>(tb + (size_t)r * ldw + lane * V);
    const int qloc = qn - c0;
    const bool has_q = qn >= 0 && owner_n == rank && (qloc / V) == lane;
    const int qe = qloc - lane * V;
    const bool has_rhs = lane == cw / V;
    const int sl = local_slot(s, c0, cw);
    const bool has_s = sl >= lane * V && sl < lane * V + V;
    const int se = sl - lane * V;
    // Elements of the entering slot, taken as 0 before the elimination.
    bool zs[V];
#pragma unroll
    for (int e = 0; e < V; ++e) zs[e] = has_s && se == e;
    typename SqT<T>::type sq{};  // steepest edge: sum of squares of this lane's final values
    // One row: the elimination is computed unconditionally and stored only
    // where it applies (a zero multiplier leaves the row as it is; row r
    // already holds the divided pivot row), so the body has no divergent
    // branch, only predicated stores.
    auto row = [&](const int i, const T f, const VT t) {
      if constexpr (PRE) {
        // slot s and row r were prepared by the caller; the RHS is not
        // extracted (that loop's ratio test reads it from the tableau)
        const VT tn = v_fma(f, p, t);
        if (f != T(0)) *reinterpret_cast<VT*>(tb + (size_t)i * ldw + lane * V) = tn;
        sq = v_sq(tn, sq);
        return;
      }
      const bool upd = f != T(0) && i != r;
      VT tz = t;
#pragma unroll
      for (int e = 0; e < V; ++e)
        if (zs[e]) vset(tz, e, T(0));
      const VT tn = v_fma(f, p, tz);
      if (upd) *reinterpret_cast<VT*>(tb + (size_t)i * ldw + lane * V) = tn;
      const VT tf = upd ? tn : t;
      if (has_q) colx_next[i] = vget<VT, T>(tf, qe);
      if (has_rhs) rhsx[i] = vget<VT, T>(tf, 0);
      if (SE) sq = v_sq(tf, sq);
    };
    // kU rows per step, every load issued before any store (rows grp,
    // grp + G, ... are disjoint, so this only adds parallelism)
    constexpr int kU = 4;
    int i0 = grp;
    for (; i0 + (kU - 1) * G < m; i0 += kU * G) {
      T f[kU];
      VT t[kU];
#pragma unroll
      for (int u = 0; u < kU; ++u) {
        const int i = i0 + u * G;
        f[u] = pcol[i];
        t[u] = *reinterpret_cast<const VT*>(tb + (size_t)i * ldw + lane * V);
      }
#pragma unroll
      for (int u = 0; u < kU; ++u) row(i0 + u * G, f[u], t[u]);
    }
    for (; i0 < m; i0 += G)
      row(i0, pcol[i0], *reinterpret_cast<const VT*>(tb + (size_t)i0 * ldw + lane * V));
    if (SE) {
      if (PRE && part) {
        // this row group's partial sums of slots [0, cw), one store
        if (lane * V < cw) store_partials(part + (size_t)grp * cw + lane * V, sq);
      } else {
        // columns visited in a rotated order, so that the counter pairs of one
        // instruction fall in distinct banks (two wavefronts, not eight)
#pragma unroll
        for (int e2 = 0; e2 < V; ++e2) {
          const int e = (e2 + (lane >> 2)) & (V - 1);
          const int lj = lane * V + e;
          if (lj < lc) norm_add(&gam[lj], sq_get(sq, e));
        }
      }
    }
    if (has_q && grp == 0) colx_next[m] = tb[(size_t)m * ldw + qloc];
  }

  // The primal simplex loop from the current tableau (the oracle's
  // simplex_loop).  Pricing covers global columns [0, price_cols).
  __device__ int loop(const Geom& g, int c0, int lc, int price_cols, const LpArgs& a,
                      int max_piv, int& pivots, bool& bland, int& degen, int& cur,
                      int period = 0) {
    const T opt_tol = (T)a.opt_tol, piv_tol = (T)a.piv_tol, feas_tol = (T)a.feas_tol;
    const T deg_tol = (T)a.deg_tol;
    Key kq = price_only(g, c0, lc, bland, opt_tol, price_cols);
    int q = kq.w2 == ~0u ? -1 : (int)kq.w2;  // entering variable
    if (q < 0) return kOpt;
    if (pivots >= max_piv) return kUndef;
    int s = (int)kq.w3;  // its slot
    int owner = s / g.cw;
    if (owner == rank) extract(g, s, c0, colbuf(cur));
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
          // one thread fetches the owner's verdict; every thread copies part
          // of the pivot column (unused if the LP turns out unbounded)
          if (threadIdx.x == 0) {
            const SharedState* os = remote(sh, owner);
            sh->r = os->r;
            sh->theta = os->theta;
          }
          const T* src = remote(colbuf(cur), owner);
          for (int i = threadIdx.x; i <= g.m; i += blockDim.x) colbuf(cur)[i] = src[i];
          __syncthreads();
          r = sh->r;
          theta = (T)sh->theta;
        }
      }
      if (r < 0) return kUnbnd;
      if (theta <= deg_tol) {
        if (++degen > a.bland_after) bland = true;
      } else {
        degen = 0;
      }
      // C: pivot row, objective row, next pricing (cluster barrier B2 inside)
      const T* pcol = colbuf(cur);
      const int lv = basis[r];
      Key kn = pivot_rows(g, r, s, lv, pcol, c0, lc, bland, opt_tol, price_cols);
      const int qn = kn.w2 == ~0u ? -1 : (int)kn.w2;
      const int sn = qn >= 0 ? (int)kn.w3 : -1;
      const int owner_n = qn >= 0 ? sn / g.cw : -1;
      relabel(r, s, q, lv);
      // D: body update, extraction of the next pivot column
      update_body(g, r, s, pcol, sn, owner_n, c0, colbuf(cur ^ 1));
      __syncthreads();
      cur ^= 1;
      ++pivots;
      if (qn < 0) return kOpt;
      if (pivots >= max_piv) return kUndef;
      if (period > 0 && pivots % period == 0) return kRefresh;
      q = qn;
      s = sn;
      owner = owner_n;
    }
  }

  // ---- steepest-edge pricing --------------------------------------------
  // Column norms gamma_j = 1 + sum_{i<m} T_ij^2 of the current tableau,
  // recomputed with a full pass (at the start of a pricing loop, after
  // loads, crashes, refreshes and pivots made without norms).
  // Partial sums of squares of one lane's V slots, clamped as the counters are.
  static __device__ __forceinline__ void store_partials(float* dst, const float4& sq) {
    *reinterpret_cast<float4*>(dst) = make_float4(norm_clamp(sq.x), norm_clamp(sq.y),
                                                  norm_clamp(sq.z), norm_clamp(sq.w));
  }
  static __device__ __forceinline__ void store_partials(float* dst, const float2& sq) {
    *reinterpret_cast<float2*>(dst) = make_float2(norm_clamp(sq.x), norm_clamp(sq.y));
  }
  // gamma_j of local slot lj from the partial sums, added in row-group order
  // (the first eight loaded together; the zeros past ngrp add exactly, the
  // partials being >= 0).
  __device__ __forceinline__ float part_gamma(int lj, int cw) const {
    const float* p = reinterpret_cast<const float*>(gam) + lj;
    float v[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) v[q] = q < ngrp ? p[q * cw] : 0.f;
    float acc = 0.f;
#pragma unroll
    for (int q = 0; q < 8; ++q) acc += v[q];
    for (int q = 8; q < ngrp; ++q) acc += p[q * cw];
    return 1.f + acc;
  }
  __device__ void norms_full(const Geom& g, int lc) {
    if (ngrp) {
      // the partial sums of every row group, grouped as the sweep groups
      // them; each group's row overwrites the last pivot's
      const int grp = threadIdx.x / g.nl, lane = threadIdx.x - grp * g.nl;
      if (grp < ngrp && lane * V < g.cw) {
        typename SqT<T>::type sq{};
        for (int i = grp; i < g.m; i += ngrp)
          sq = v_sq(*reinterpret_cast<const VT*>(tab + (size_t)i * g.ldw + lane * V), sq);
        store_partials(reinterpret_cast<float*>(gam) + (size_t)grp * g.cw + lane * V, sq);
      }
      __syncthreads();
      return;
    }
    for (int lj = threadIdx.x; lj < g.ldw; lj += blockDim.x) gam[lj] = make_uint2(0u, 0u);
    __syncthreads();
    const int nt = (int)blockDim.x, G = min(nt / g.nl, kMaxNormGroups);
    const int grp = threadIdx.x / g.nl, lane = threadIdx.x - grp * g.nl;
    if (grp < G) {
      typename SqT<T>::type sq{};
      for (int i = grp; i < g.m; i += G)
        sq = v_sq(*reinterpret_cast<const VT*>(tab + (size_t)i * g.ldw + lane * V), sq);
#pragma unroll
      for (int e = 0; e < V; ++e) {
        const int lj = lane * V + e;
        if (lj < lc) norm_add(&gam[lj], sq_get(sq, e));
      }
    }
    __syncthreads();
  }

  // Steepest-edge pricing: among d_j < -opt_tol (variables below
  // price_cols), the largest d_j^2 / gamma_j, times weight[j] when weights
  // are given; ties to the lowest variable id.  Bland's rule (after a
  // degenerate streak) takes the lowest eligible id as in Dantzig mode.
  __device__ Key price_se(const Geom& g, int c0, int lc, bool bland, T opt_tol, int price_cols,
                          const float* w) {
    Key k = key_none();
    const T* d = tab + (size_t)g.m * g.ldw;
    for (int lj = threadIdx.x; lj < lc; lj += blockDim.x) {
      const int j = cvar[c0 + lj];
      const T v = d[lj];
      if (j < price_cols && v < -opt_tol) {
        Key kk;
        if (bland) {
          kk = price_key(v, j, c0 + lj, true);
        } else {
          const float gm = ngrp ? part_gamma(lj, g.cw) : norm_gamma(gam[lj]);
          const float vf = (float)v;
          float sc = __fdividef(vf * vf, gm);
          if (w) sc *= w[j];
          kk = Key{~__float_as_uint(sc), 0u, (unsigned)j, (unsigned)(c0 + lj)};
        }
        if (key_less(kk, k)) k = kk;
      }
    }
    k = block_min<kW1>(k, redP);
    return cluster_min(k);
  }

  // The primal loop with the plan's pricing rule over variables < n + m.
  __device__ int primal(const Geom& g, int c0, int lc, const LpArgs& a, const float* w,
                        int max_piv, int& pivots, bool& bland, int& degen, int& cur,
                        int period = 0) {
    if (a.pricing == 1 && gam)
      return loop_se(g, c0, lc, g.n + g.m, a, w, max_piv, pivots, bland, degen, cur, period);
    return loop(g, c0, lc, g.n + g.m, a, max_piv, pivots, bland, degen, cur, period);
  }

  // The primal loop with steepest-edge pricing.  Pricing needs the norms of
  // the updated tableau, so it runs after the sweep (which sums them), and
  // the entering column is then extracted by its owner.
  __device__ int loop_se(const Geom& g, int c0, int lc, int price_cols, const LpArgs& a,
                         const float* w, int max_piv, int& pivots, bool& bland, int& degen,
                         int& cur, int period = 0) {
    const T opt_tol = (T)a.opt_tol, piv_tol = (T)a.piv_tol, feas_tol = (T)a.feas_tol;
    const T deg_tol = (T)a.deg_tol;
    // FP32 on one CTA: the sweep with the entering slot and row r prepared;
    // FP32: ratios and the pivot row with reciprocals (on any cluster size, so
    // that a split tableau gives the same bits)
    constexpr bool kPre = sizeof(T) == 4 && !CLUSTER;
    constexpr bool kRecip = sizeof(T) == 4;
    norms_full(g, lc);
    for (;;) {
      Key kq = price_se(g, c0, lc, bland, opt_tol, price_cols, w);
      const int q = kq.w2 == ~0u ? -1 : (int)kq.w2;
      if (q < 0) return kOpt;
      if (pivots >= max_piv) return kUndef;
      const int s = (int)kq.w3;
      T theta = T(0);
      Key kr;
      if (!CLUSTER) {
        // the norms are summed afresh by this pivot's sweep (the pricing
        // reads are done: its argmin ended with a barrier); the column is
        // extracted inside the ratio test's first pass (FP32: and cleared)
        if (!ngrp)
          for (int lj = threadIdx.x; lj < g.ldw; lj += blockDim.x) gam[lj] = make_uint2(0u, 0u);
        kr = ratio(g, colbuf(cur), piv_tol, feas_tol, a.harris && !bland, theta, s, kPre, kRecip);
      } else {
        const int owner = s / g.cw;
        if (owner == rank) extract(g, s, c0, colbuf(cur));
        csync();
        if (owner != rank) {
          // the column from its owner, the RHS from this CTA's own replica
          // (replicas are bit-identical, so every CTA's ratio test agrees)
          const T* src = remote(colbuf(cur), owner);
          for (int i = threadIdx.x; i <= g.m; i += blockDim.x) {
            colbuf(cur)[i] = src[i];
            rhsx[i] = tab[(size_t)i * g.ldw + g.cw];
          }
        }
        __syncthreads();
        for (int lj = threadIdx.x; lj < g.ldw; lj += blockDim.x) gam[lj] = make_uint2(0u, 0u);
        // ratio test: every CTA holds the column, so each computes it
        kr = ratio(g, colbuf(cur), piv_tol, feas_tol, a.harris && !bland, theta, -1, false,
                   kRecip);
      }
      const int r = kr.w2 == ~0u ? -1 : (int)kr.w3;
      if (r < 0) {
        if (kPre) {  // the entering column goes back where the ratio test cleared it
          for (int i = threadIdx.x; i < g.m; i += blockDim.x)
            tab[(size_t)i * g.ldw + s] = colbuf(cur)[i];
          __syncthreads();
        }
        return kUnbnd;
      }
      if (theta <= deg_tol) {
        if (++degen > a.bland_after) bland = true;
      } else {
        degen = 0;
      }
      const T* pcol = colbuf(cur);
      const int lv = basis[r];
      if (kPre) {
        // the sweep's multipliers: the pivot column with row r's entry 0
        // (published by the pivot row's barrier)
        T* fcol = colbuf(cur ^ 1);
        for (int i = threadIdx.x; i < g.m; i += blockDim.x) fcol[i] = i == r ? T(0) : pcol[i];
      }
      pivot_rows(g, r, s, lv, pcol, c0, lc, false, T(0), 0, kRecip);
      relabel(r, s, q, lv);
      if (kPre)
        update_body_se32(g, r, colbuf(cur ^ 1), lc);
      else
        update_body_se(g, r, s, pcol, c0, lc);
      __syncthreads();
      ++pivots;
      if (pivots >= max_piv) return kUndef;
      if (period > 0 && pivots % period == 0) return kRefresh;
    }
  }

  // Objective row from the current basis: d_j = sum_i cB_i T_ij - c_j over
  // local slots (phase II after phase I), or the phase I row
  // -sum_{artificial rows} T_ij.  Sums run over rows in increasing order, as
  // the oracle does.
  __device__ void objective_row(const Geom& g, int c0, int lc, const double* c,
                                bool phase1) {
    const int nart0 = g.n + g.m;
    for (int lj = threadIdx.x; lj <= g.cw; lj += blockDim.x) {
      const bool is_rhs = lj == g.cw;
      if (!is_rhs && lj >= lc) continue;
      const int j = is_rhs ? -1 : cvar[c0 + lj];
      T acc = T(0);
      if (phase1) {
        if (!is_rhs && j >= nart0) {  // artificial: stays 0
          tab[(size_t)g.m * g.ldw + lj] = T(0);
          continue;
        }
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
  // such row, pivot on the lowest variable j < n+m with |T_ij| > piv_tol.
  __device__ void drive_out(const Geom& g, int c0, int lc, const LpArgs& a, int& pivots,
                            int& cur) {
    const T piv_tol = (T)a.piv_tol;
    const int nart0 = g.n + g.m;
    for (int i = 0; i < g.m; ++i) {
      if (basis[i] < nart0) continue;  // uniform across the block and cluster
      Key k = key_none();
      const T* row = tab + (size_t)i * g.ldw;
      for (int lj = threadIdx.x; lj < lc; lj += blockDim.x) {
        const int j = cvar[c0 + lj];
        const T v = row[lj];
        if (j < nart0 && (v > piv_tol || v < -piv_tol)) {
          Key kk{0u, 0u, (unsigned)j, (unsigned)(c0 + lj)};
          if (key_less(kk, k)) k = kk;
        }
      }
      k = block_min<kW1>(k, redP);
      k = cluster_min(k);
      if (CLUSTER) csync();  // pslot reads done before the next write
      if (k.w2 == ~0u) continue;  // redundant row: artificial stays basic at 0
      pivot_on(g, i, (int)k.w2, (int)k.w3, c0, lc, cur);
      ++pivots;
    }
  }

  // Pivot on (r, q in slot s) without pricing (phase-I drive-out, warm-start
  // crash, dual simplex).  The column is extracted by its owner and copied by
  // the other CTAs of the cluster; returns with every copy done.
  __device__ void pivot_on(const Geom& g, int r, int q, int s, int c0, int lc, int cur) {
    const int owner = s / g.cw;
    if (owner == rank) extract(g, s, c0, colbuf(cur));
    if (CLUSTER) {
      csync();
      if (owner != rank) {
        const T* src = remote(colbuf(cur), owner);
        for (int e = threadIdx.x; e <= g.m; e += blockDim.x) colbuf(cur)[e] = src[e];
      }
    }
    __syncthreads();
    const T* pcol = colbuf(cur);
    const int lv = basis[r];
    pivot_rows(g, r, s, lv, pcol, c0, lc, false, T(0), 0);
    relabel(r, s, q, lv);
    update_body(g, r, s, pcol, -1, -1, c0, colbuf(cur ^ 1));
    __syncthreads();
    if (CLUSTER) csync();
  }

  // Cluster-wide OR of a block-level flag.
  __device__ bool cluster_any(bool v) {
    v = __syncthreads_or(v ? 1 : 0) != 0;
    if (!CLUSTER) return v;
    if (threadIdx.x == 0) sh->aux.w0 = v ? 1u : 0u;
    csync();
    bool any = false;
    for (int k = 0; k < K; ++k) any = any || remote(&sh->aux, k)->w0 != 0u;
    csync();
    return any;
  }

  // Feasibility of the current tableau: bit 0 when every x_B >= -ptol,
  // bit 1 when every reduced cost d_j (j < n+m) >= -opt_tol.
  __device__ int check_feasible(const Geom& g, int c0, int lc, T ptol, T opt_tol) {
    bool badp = false, badd = false;
    for (int i = threadIdx.x; i < g.m; i += blockDim.x)
      badp = badp || tab[(size_t)i * g.ldw + g.cw] < -ptol;
    const T* d = tab + (size_t)g.m * g.ldw;
    for (int lj = threadIdx.x; lj < lc; lj += blockDim.x)
      badd = badd || (cvar[c0 + lj] < g.n + g.m && d[lj] < -opt_tol);
    badp = __syncthreads_or(badp ? 1 : 0) != 0;  // RHS is replicated: no exchange
    badd = cluster_any(badd);
    return (badp ? 0 : 1) | (badd ? 0 : 2);
  }

  // Dual simplex from a dual-feasible basis (the oracle's dual_loop):
  // leaving row = most negative RHS below -ptol (ties lowest basic
  // variable); entering column = minimum max(d_j, 0) / -T_rj over
  // T_rj < -piv_tol (ties lowest variable).  kOpt once x_B >= -ptol; kNoFeas
  // when no column can enter (the LP would be primal infeasible).
  __device__ int dual_loop(const Geom& g, int c0, int lc, const LpArgs& a, int max_piv,
                           int& pivots, int cur, T ptol) {
    const T piv_tol = (T)a.piv_tol;
    for (;;) {
      Key kr = key_none();
      for (int i = threadIdx.x; i < g.m; i += blockDim.x) {
        const T v = tab[(size_t)i * g.ldw + g.cw];
        if (v < -ptol) {
          Key kk = neg_key(v, basis[i], i);
          if (key_less(kk, kr)) kr = kk;
        }
      }
      kr = block_min<kW1>(kr, redR);  // RHS replicated: every CTA finds the same row
      if (kr.w2 == ~0u) return kOpt;
      if (pivots >= max_piv) return kUndef;
      const int r = (int)kr.w3;
      const T* row = tab + (size_t)r * g.ldw;
      const T* drow = tab + (size_t)g.m * g.ldw;
      const T dual_tol = (T)a.opt_tol;
      // Harris (as the primal test): pass 1 bounds the dual step by the
      // ratios relaxed by opt_tol, pass 2 takes the largest |T_rj| within it
      // (ties lowest variable).  Textbook rule when Harris is off.
      Key kq = key_none();
      for (int lj = threadIdx.x; lj < lc; lj += blockDim.x) {
        const int j = cvar[c0 + lj];
        const T arj = row[lj];
        if (j < g.n + g.m && arj < -piv_tol) {
          const T dj = drow[lj];
          const T th = a.harris ? ((dj > T(0) ? dj : T(0)) + dual_tol) / (-arj)
                                : (dj > T(0) ? dj / (-arj) : T(0));
          Key kk = ratio_key(th, j, c0 + lj);
          if (key_less(kk, kq)) kq = kk;
        }
      }
      kq = block_min<kW1>(kq, redH);
      kq = cluster_min(kq);
      if (CLUSTER) csync();  // pslot reads done before the next cluster_min
      if (kq.w2 == ~0u) return kNoFeas;
      if (a.harris) {
        const T tmax = key_theta(kq, T(0));
        Key k2 = key_none();
        for (int lj = threadIdx.x; lj < lc; lj += blockDim.x) {
          const int j = cvar[c0 + lj];
          const T arj = row[lj];
          if (j < g.n + g.m && arj < -piv_tol) {
            const T dj = drow[lj];
            const T th = dj > T(0) ? dj / (-arj) : T(0);
            if (th <= tmax) {
              Key kk = big_key(-arj, j, c0 + lj);
              if (key_less(kk, k2)) k2 = kk;
            }
          }
        }
        k2 = block_min<kW1>(k2, redP);
        kq = cluster_min(k2);
        if (CLUSTER) csync();
      }
      pivot_on(g, r, (int)kq.w2, (int)kq.w3, c0, lc, cur);
      ++pivots;
    }
  }

  // Warm start: pivot each hinted structural column into the basis on the
  // row, among rows whose basic variable is a slack the hint does not keep,
  // with the largest |T_ij| (ties lowest row).  Returns how many hinted
  // columns found no pivot (the hinted basis is singular on them).
  __device__ int crash(const Geom& g, int c0, const int32_t* hint, const LpArgs& a,
                       int& pivots, int cur, int lc) {
    const T piv_tol = (T)a.piv_tol;
    for (int i = threadIdx.x; i < g.m; i += blockDim.x) flags[i] = 0;
    __syncthreads();
    for (int k = threadIdx.x; k < g.m; k += blockDim.x) {
      const int h = hint[k];
      if (h >= g.n && h < g.n + g.m) flags[h - g.n] = 1;
    }
    __syncthreads();
    int missing = 0;
    for (int k = 0; k < g.m; ++k) {
      const int h = hint[k];
      if (h < 0 || h >= g.n) continue;
      const int s = vpos[h];
      if (s < 0) continue;  // already basic (duplicate hint entry)
      const int owner = s / g.cw;
      int r = -1;
      if (owner == rank) {
        Key kk = key_none();
        const int hl = s - c0;
        for (int i = threadIdx.x; i < g.m; i += blockDim.x) {
          const int bi = basis[i];
          if (bi >= g.n && bi < g.n + g.m && !flags[bi - g.n]) {
            const T v = tab[(size_t)i * g.ldw + hl];
            const T av = v < T(0) ? -v : v;
            if (av > piv_tol) {
              Key c = big_key(av, i, i);
              if (key_less(c, kk)) kk = c;
            }
          }
        }
        kk = block_min<kW1>(kk, redR);
        r = kk.w2 == ~0u ? -1 : (int)kk.w3;
        if (CLUSTER && threadIdx.x == 0) sh->r = r;
      }
      if (CLUSTER) {
        csync();
        if (owner != rank) r = remote(sh, owner)->r;
        csync();
      }
      if (r < 0) {
        __syncthreads();  // redR is read again by the next column's search
        ++missing;
        continue;
      }
      pivot_on(g, r, h, s, c0, lc, cur);
      ++pivots;
    }
    return missing;
  }

  // Tableau element (row i, global slot s) wherever it lives.
  __device__ T* elem(const Geom& g, int i, int s) {
    if (!CLUSTER) return tab + (size_t)i * g.ldw + s;
    const int o = s / g.cw;
    T* p = tab + (size_t)i * g.ldw + (s - o * g.cw);
    return o == rank ? p : remote(p, o);
  }
  // Element (i, k) of B^-1 = column of slack k: a stored column when the
  // slack is nonbasic, the unit vector of its row when it is basic.
  __device__ T binv(const Geom& g, int i, int k) {
    const int v = vpos[g.n + k];
    if (v >= 0) return *elem(g, i, v);
    return i == -1 - v ? T(1) : T(0);
  }

  // FP64 refresh by refactorisation of the basis.  With the basis's
  // structural columns J (ns of them, in tableau-row order) and the
  // constraints R not covered by a basic slack or a basic artificial (ns of
  // them, in increasing order), the basis matrix in the original coordinates
  // is, up to a permutation, [[K, 0], [A[C, J], D]] with K = A[R, J] and D
  // diagonal (+1 for a basic slack, -1 for a basic artificial: the
  // artificial of a row with b_i < 0 carries +1 in the negated row).  So
  //   K x_J = b_R,  x of the basic slack (artificial) of constraint k =
  //   +(-)(b_k - A[k, J] x_J);   K^T y_R = c_J,  y = 0 off R;
  //   d_j = y_R^T A[R, j] - c_j (structural),  d = y_k (slack k),
  //   z = c_J^T x_J.
  // K is factorised in FP64 with partial pivoting (one warp, K in the CTA's
  // global scratch, rows permuted through a list), each solve is refined once
  // from an FP64 residual on the original A, and the correction judges the
  // factorisation: it must be <= 1e-9 of the values, else bit 2 is clear (the
  // basis is singular or too ill-conditioned to verify).  Nothing is read
  // from the tableau except the basis, so the accuracy of x, y and d does not
  // depend on the FP32 values, and rows negated for phase I need no special
  // case.  The RHS column (every replica) and the objective row are
  // overwritten as in refresh_refine; the artificials' reduced costs are not
  // (they are never priced after phase I).  Rank 0 computes; every sum runs
  // in a fixed order, independent of the thread count and the cluster split.
  // Returns the bits of refresh_refine.  Out of line with the geometry by
  // value: it runs once or twice per LP.
  __device__ __forceinline__ int refresh_lu_body(const Geom g, const double* A,
                                                 const double* b, const double* c,
                                                 const double opt_tol, const double ptol) {
    const int m = g.m, n = g.n, na = g.na;
    const int tid = threadIdx.x, nt = blockDim.x;
    const int lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
    const unsigned full = 0xffffffffu;
    if (CLUSTER) csync();
    int ok = 0;
    if (rank == 0) {
      int* slist = flags;                          // rows of the structural basics
      int* rlist = reinterpret_cast<int*>(rhsx);   // uncovered constraints R
      int* perm = reinterpret_cast<int*>(rf);      // LU row order (positions in R)
      int* arow = reinterpret_cast<int*>(col0);    // constraint of each artificial
      int* wcount = reinterpret_cast<int*>(redH);  // chunk offsets: [0,33) rows, [64,97) R
      const int nch = ceil_div(m, 32);
      // artificial a belongs to the a-th constraint with b_i < 0 (load())
      if (na > 0) {
        for (int ch = warp; ch < nch; ch += nw) {
          const int i = ch * 32 + lane;
          const unsigned bal = __ballot_sync(full, i < m && b[i] < 0.0);
          if (lane == 0) wcount[ch] = __popc(bal);
        }
        __syncthreads();
        if (tid == 0) {
          int acc = 0;
          for (int ch = 0; ch < nch; ++ch) {
            const int v = wcount[ch];
            wcount[ch] = acc;
            acc += v;
          }
        }
        __syncthreads();
        for (int ch = warp; ch < nch; ch += nw) {
          const int i = ch * 32 + lane;
          const bool neg = i < m && b[i] < 0.0;
          const unsigned bal = __ballot_sync(full, neg);
          if (neg) arow[wcount[ch] + __popc(bal & ((1u << lane) - 1u))] = i;
        }
        __syncthreads();
      }
      // yr[k] = 1 marks constraint k covered: its slack, or its artificial, is basic
      for (int k = tid; k < m; k += nt) yr[k] = vpos[n + k] < 0 ? 1.0 : 0.0;
      __syncthreads();
      for (int i = tid; i < m; i += nt) {
        const int v = basis[i];
        if (v >= n + m) yr[arow[v - n - m]] = 1.0;
      }
      __syncthreads();
      // the lists, by ballots and prefix sums over 32-row chunks
      for (int ch = warp; ch < 2 * nch; ch += nw) {
        const bool rows = ch < nch;
        const int i = (rows ? ch : ch - nch) * 32 + lane;
        const bool st = i < m && (rows ? basis[i] < n : yr[i] == 0.0);
        const unsigned bal = __ballot_sync(full, st);
        if (lane == 0) wcount[rows ? ch : 64 + ch - nch] = __popc(bal);
      }
      __syncthreads();
      if (tid < 2) {
        int acc = 0;
        for (int ch = 0; ch < nch; ++ch) {
          const int v = wcount[64 * tid + ch];
          wcount[64 * tid + ch] = acc;
          acc += v;
        }
        wcount[64 * tid + nch] = acc;
      }
      __syncthreads();
      for (int ch = warp; ch < 2 * nch; ch += nw) {
        const bool rows = ch < nch;
        const int i = (rows ? ch : ch - nch) * 32 + lane;
        const bool st = i < m && (rows ? basis[i] < n : yr[i] == 0.0);
        const unsigned bal = __ballot_sync(full, st);
        const int pos = __popc(bal & ((1u << lane) - 1u));
        if (st) {
          if (rows)
            slist[wcount[ch] + pos] = i;
          else
            rlist[wcount[64 + ch - nch] + pos] = i;
        }
      }
      __syncthreads();
      const int ns = wcount[nch], nr = wcount[64 + nch];
      // global scratch: K (ns x ns, row-major, rows in R order), then vectors
      double* Km = lu;
      double* xJ = Km + (size_t)ns * ns;  // x_J (J order)
      double* yR = xJ + ns;               // y_R (R order)
      double* v1 = yR + ns;               // right-hand sides, then corrections
      double* v2 = v1 + ns;
      double* v3 = v2 + ns;               // solve scratch
      bool good = ns == nr;
      if (good) {
        for (int e = tid; e < ns * ns; e += nt) {
          const int r = e / ns, cc = e - r * ns;
          Km[e] = __ldg(A + (size_t)rlist[r] * n + basis[slist[cc]]);
        }
        for (int t = tid; t < ns; t += nt) {
          v1[t] = __ldg(b + rlist[t]);
          v2[t] = __ldg(c + basis[slist[t]]);
        }
      }
      __syncthreads();
      // ---- LU with partial pivoting and the solves, by warp 0
      if (warp == 0) {
        bool conv = false;
        if (good) {
          for (int r = lane; r < ns; r += 32) perm[r] = r;
          __syncwarp();
          double kmax = 0.0;  // largest |K| entry, for the singularity threshold
          for (int e = lane; e < ns * ns; e += 32) kmax = fmax(kmax, fabs(Km[e]));
          for (int o = 16; o > 0; o >>= 1) kmax = fmax(kmax, __shfl_xor_sync(full, kmax, o));
          const double tiny = 1e-13 * kmax;
          for (int kk = 0; kk < ns; ++kk) {
            double bv = -1.0;
            int bi = ns;
            for (int i = kk + lane; i < ns; i += 32) {
              const double v = fabs(Km[(size_t)perm[i] * ns + kk]);
              if (v > bv) {
                bv = v;
                bi = i;
              }
            }
            for (int o = 16; o > 0; o >>= 1) {
              const double ov = __shfl_xor_sync(full, bv, o);
              const int oi = __shfl_xor_sync(full, bi, o);
              if (ov > bv || (ov == bv && oi < bi)) {
                bv = ov;
                bi = oi;
              }
            }
            if (!(bv > tiny)) {  // singular (warp-uniform)
              good = false;
              break;
            }
            const int pb = perm[bi];
            __syncwarp();
            if (lane == 0) {
              perm[bi] = perm[kk];
              perm[kk] = pb;
            }
            __syncwarp();
            const double* urow = Km + (size_t)pb * ns;
            const double rinv = 1.0 / urow[kk];
            for (int i = kk + 1 + lane; i < ns; i += 32)
              Km[(size_t)perm[i] * ns + kk] *= rinv;  // the multiplier, in L's place
            __syncwarp();
            const int w = ns - kk - 1;
            for (int e = lane; e < w * w; e += 32) {
              const int i = kk + 1 + e / w, cc = kk + 1 + e % w;
              double* row = Km + (size_t)perm[i] * ns;
              row[cc] = fma(-row[kk], urow[cc], row[cc]);
            }
            __syncwarp();
          }
        }
        if (good) {
          // K x = v1 (x_J) and K^T y = v2 (y_R), refined from residuals on
          // the original A until the correction is below 1e-12 of the values
          // (at most three refinement steps); converged when the last one is
          // below 1e-9
          double cx = 0.0, mx = 0.0, cy = 0.0, my = 0.0;
          for (int pass = 0; pass < 4; ++pass) {
            lu_solve(Km, perm, ns, v1, v3, lane);    // v1 <- K^-1 v1
            lu_solve_t(Km, perm, ns, v2, v3, lane);  // v2 <- K^-T v2
            for (int t = lane; t < ns; t += 32) {
              if (pass == 0) {
                xJ[t] = v1[t];
                yR[t] = v2[t];
              } else {
                xJ[t] += v1[t];
                yR[t] += v2[t];
              }
            }
            __syncwarp();
            if (pass > 0) {
              cx = cy = mx = my = 0.0;
              for (int t = lane; t < ns; t += 32) {
                cx = fmax(cx, fabs(v1[t]));
                cy = fmax(cy, fabs(v2[t]));
                mx = fmax(mx, fabs(xJ[t]));
                my = fmax(my, fabs(yR[t]));
              }
              for (int o = 16; o > 0; o >>= 1) {
                cx = fmax(cx, __shfl_xor_sync(full, cx, o));
                cy = fmax(cy, __shfl_xor_sync(full, cy, o));
                mx = fmax(mx, __shfl_xor_sync(full, mx, o));
                my = fmax(my, __shfl_xor_sync(full, my, o));
              }
              if (pass == 3 || (cx <= 1e-12 * fmax(1.0, mx) && cy <= 1e-12 * fmax(1.0, my)))
                break;
            }
            // residuals b_R - K x_J and c_J - K^T y_R from the original A
            for (int t = lane; t < ns; t += 32) {
              const double* Ar = A + (size_t)rlist[t] * n;
              const int jt = basis[slist[t]];
              double s0 = 0.0, s1 = 0.0;
              for (int u = 0; u < ns; ++u) {
                s0 = fma(__ldg(Ar + basis[slist[u]]), xJ[u], s0);
                s1 = fma(__ldg(A + (size_t)rlist[u] * n + jt), yR[u], s1);
              }
              v1[t] = __ldg(b + rlist[t]) - s0;
              v2[t] = __ldg(c + jt) - s1;
            }
            __syncwarp();
          }
          conv = cx <= 1e-9 * fmax(1.0, mx) && cy <= 1e-9 * fmax(1.0, my);
        }
        if (lane == 0) sh->aux.w1 = (good ? 1u : 0u) | (conv ? 2u : 0u);
      }
      __syncthreads();
      good = (sh->aux.w1 & 1u) != 0u;
      const bool conv = (sh->aux.w1 & 2u) != 0u;
      bool badd = false, badp = false;
      if (good) {
        // y per constraint (0 off R) and x per tableau row
        for (int k = tid; k < m; k += nt) yr[k] = 0.0;
        __syncthreads();
        for (int t = tid; t < ns; t += nt) {
          yr[rlist[t]] = yR[t];
          xr[slist[t]] = xJ[t];
        }
        for (int i = tid; i < m; i += nt) {
          const int v = basis[i];
          if (v < n) continue;
          const bool art = v >= n + m;
          const int k = art ? arow[v - n - m] : v - n;
          const double* Ak = A + (size_t)k * n;
          double s0 = 0.0;
          for (int u = 0; u < ns; ++u) s0 = fma(__ldg(Ak + basis[slist[u]]), xJ[u], s0);
          const double xv = __ldg(b + k) - s0;
          xr[i] = art ? -xv : xv;
        }
        __syncthreads();
        // reduced costs of the nonbasic structurals and slacks
        for (int j = tid; j < n; j += nt) {
          const int sv = vpos[j];
          if (sv < 0) continue;
          double s0 = 0.0;
          for (int t = 0; t < ns; ++t) s0 = fma(__ldg(A + (size_t)rlist[t] * n + j), yR[t], s0);
          const double d = s0 - __ldg(c + j);
          *elem(g, m, sv) = (T)d;
          badd = badd || d < -opt_tol;
        }
        for (int k = tid; k < m; k += nt) {
          const int sv = vpos[n + k];
          if (sv < 0) continue;
          const double d = yr[k];
          *elem(g, m, sv) = (T)d;
          badd = badd || d < -opt_tol;
        }
        for (int i = tid; i < m; i += nt) {
          const T xv = (T)xr[i];
          for (int o = 0; o < K; ++o) {
            T* p = tab + (size_t)i * g.ldw + g.cw;
            *(o == rank ? p : remote(p, o)) = xv;
          }
          badp = badp || xr[i] < -ptol;
        }
        if (warp == 0) {  // z = c_J^T x_J, lane-strided partial sums and a butterfly
          double z = 0.0;
          for (int t = lane; t < ns; t += 32) z = fma(__ldg(c + basis[slist[t]]), xJ[t], z);
          for (int o = 16; o > 0; o >>= 1) z += __shfl_xor_sync(full, z, o);
          if (lane == 0) {
            sh->z = z;
            for (int o = 0; o < K; ++o) {
              T* p = tab + (size_t)m * g.ldw + g.cw;
              *(o == rank ? p : remote(p, o)) = (T)z;
            }
          }
        }
      }
      badd = __syncthreads_or(badd ? 1 : 0) != 0;
      badp = __syncthreads_or(badp ? 1 : 0) != 0;
      ok = good ? ((badp ? 0 : 1) | (badd ? 0 : 2) | (conv ? 4 : 0)) : 0;
      if (tid == 0) sh->aux.w1 = (unsigned)ok;
    }
    if (CLUSTER) {
      csync();
      ok = (int)remote(&sh->aux, 0)->w1;
      csync();
    }
    return ok;
  }

  // x <- K^-1 x with PK = LU stored in K (the multipliers of L below the
  // diagonal, unit diagonal implied; row i of PK is row perm[i] of K); one
  // warp, column-oriented substitutions, w (ns doubles) scratch.
  static __device__ void lu_solve(const double* K, const int* perm, int ns, double* x, double* w,
                                  int lane) {
    for (int i = lane; i < ns; i += 32) w[i] = x[perm[i]];
    __syncwarp();
    for (int k = 0; k < ns; ++k) {  // L z = P x
      const double wk = w[k];
      for (int i = k + 1 + lane; i < ns; i += 32)
        w[i] = fma(-K[(size_t)perm[i] * ns + k], wk, w[i]);
      __syncwarp();
    }
    for (int k = ns - 1; k >= 0; --k) {  // U x = z
      const double wk = w[k] / K[(size_t)perm[k] * ns + k];
      __syncwarp();
      if (lane == 0) w[k] = wk;
      for (int i = lane; i < k; i += 32) w[i] = fma(-K[(size_t)perm[i] * ns + k], wk, w[i]);
      __syncwarp();
    }
    for (int i = lane; i < ns; i += 32) x[i] = w[i];
    __syncwarp();
  }

  // x <- K^-T x: K^T = U^T L^T P, so U^T s = x (forward), L^T u = s
  // (backward) and x[perm[i]] = u[i]; one warp, w (ns doubles) scratch.
  static __device__ void lu_solve_t(const double* K, const int* perm, int ns, double* x,
                                    double* w, int lane) {
    for (int i = lane; i < ns; i += 32) w[i] = x[i];
    __syncwarp();
    for (int k = 0; k < ns; ++k) {
      const double* urow = K + (size_t)perm[k] * ns;
      const double wk = w[k] / urow[k];
      __syncwarp();
      if (lane == 0) w[k] = wk;
      for (int j = k + 1 + lane; j < ns; j += 32) w[j] = fma(-urow[j], wk, w[j]);
      __syncwarp();
    }
    for (int k = ns - 1; k >= 0; --k) {
      const double* lrow = K + (size_t)perm[k] * ns;
      const double wk = w[k];
      for (int i = lane; i < k; i += 32) w[i] = fma(-lrow[i], wk, w[i]);
      __syncwarp();
    }
    for (int i = lane; i < ns; i += 32) x[perm[i]] = w[i];
    __syncwarp();
  }

  // Out-of-line entries of the rarely run FP64 refreshes and the rebuild.
  // They are static and take a copy of the solver (its shared-memory
  // pointers), so that no member function's `this` escapes and the kernel
  // keeps every pointer of its hot loops in registers.
  static __device__ __noinline__ int refresh_lu_call(Solver self, const Geom g, const double* A,
                                                     const double* b, const double* c,
                                                     const double opt_tol, const double ptol) {
    return self.refresh_lu_body(g, A, b, c, opt_tol, ptol);
  }
  static __device__ __noinline__ int refresh_refine_call(Solver self, const Geom g,
                                                         const double* A, const double* b,
                                                         const double* c, const double opt_tol,
                                                         const double ptol) {
    return self.refresh_refine_body(g, A, b, c, opt_tol, ptol);
  }
  static __device__ __noinline__ void reinvert_call(Solver self, const Geom g, const double* A) {
    self.reinvert_body(g, A);
  }
  __device__ __forceinline__ int refresh_lu(const Geom& g, const double* A, const double* b,
                                            const double* c, double opt_tol, double ptol) {
    return refresh_lu_call(*this, g, A, b, c, opt_tol, ptol);
  }
  __device__ __forceinline__ int refresh_refine(const Geom& g, const double* A, const double* b,
                                                const double* c, double opt_tol, double ptol) {
    return refresh_refine_call(*this, g, A, b, c, opt_tol, ptol);
  }
  __device__ __forceinline__ void reinvert(const Geom& g, const double* A) {
    reinvert_call(*this, g, A);
  }

  // The FP64 refresh: iterative refinement through the tableau's B^-1 (the
  // fast path, FP64 work proportional to the structural basics), or, with LU
  // scratch (plans; the allocation-free entry point has none), the
  // factorisation of refresh_lu for every phase-I LP and whenever the
  // refinement does not converge.  Bit 3 of the result: the LU factors of
  // the current basis are in the scratch (reinvert may use them).
  __device__ int refresh(const Geom& g, const double* A, const double* b, const double* c,
                         const LpArgs& a) {
    if (g.na == 0 || !lu) {
      const int ok = refresh_refine(g, A, b, c, a.opt_tol, a.ptol);
      if ((ok & 4) || !lu) return ok;
    }
    const int ok = refresh_lu(g, A, b, c, a.opt_tol, a.ptol);
    return ok | ((ok & 4) ? 8 : 0);
  }

  // Rebuild the tableau of the current basis from its FP64 factorisation
  // (left in the scratch and the lists by refresh_lu): every slot's column
  // is B^-1 a_j in the original coordinates (the negated phase-I rows cancel
  // out: (D B)^-1 D a_j = B^-1 a_j), i.e. u_J = K^-1 a_j[R] on the rows of
  // the structural basics and +-(a_jk - A[k, J] u_J) on the row holding the
  // slack (+) or artificial (-) of constraint k.  One warp per column, FP64
  // solves, entries rounded to the tableau's type; the RHS and the objective
  // row were set by refresh_lu.  Used before repair pivots, when the tableau
  // has drifted too far from its basis for the repairs to be trusted.
  __device__ __forceinline__ void reinvert_body(const Geom g, const double* A) {
    const int m = g.m, n = g.n;
    const int tid = threadIdx.x, nt = blockDim.x;
    const int lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
    if (CLUSTER) csync();
    if (rank == 0) {
      const int* slist = flags;
      const int* rlist = reinterpret_cast<const int*>(rhsx);
      const int* perm = reinterpret_cast<const int*>(rf);
      const int* arow = reinterpret_cast<const int*>(col0);
      int* rowpos = reinterpret_cast<int*>(yr);  // tableau row -> position in J (or -1)
      int ns = 0;
      for (int i = tid; i < m; i += nt) ns += basis[i] < n ? 1 : 0;
      ns = block_sum(ns);
      for (int i = tid; i < m; i += nt) rowpos[i] = -1;
      __syncthreads();
      for (int t = tid; t < ns; t += nt) rowpos[slist[t]] = t;
      __syncthreads();
      const double* Km = lu;
      double* v = lu + (size_t)ns * ns + 5 * (size_t)ns + (size_t)warp * 2 * ns;
      double* w = v + ns;
      for (int sl = warp; sl < g.Wc; sl += nw) {
        const int j = cvar[sl];
        // a_j on the uncovered constraints R
        for (int t = lane; t < ns; t += 32) {
          const int k = rlist[t];
          v[t] = j < n ? __ldg(A + (size_t)k * n + j)
                       : (j < n + m ? (j - n == k ? 1.0 : 0.0) : (arow[j - n - m] == k ? -1.0 : 0.0));
        }
        __syncwarp();
        lu_solve(Km, perm, ns, v, w, lane);
        for (int i = lane; i < m; i += 32) {
          const int bi = basis[i];
          double u;
          if (bi < n) {
            u = v[rowpos[i]];
          } else {
            const bool art = bi >= n + m;
            const int k = art ? arow[bi - n - m] : bi - n;
            const double ajk =
                j < n ? __ldg(A + (size_t)k * n + j)
                      : (j < n + m ? (j - n == k ? 1.0 : 0.0) : (arow[j - n - m] == k ? -1.0 : 0.0));
            double s0 = 0.0;
            for (int t = 0; t < ns; ++t)
              s0 = fma(__ldg(A + (size_t)k * n + basis[slist[t]]), v[t], s0);
            u = art ? -(ajk - s0) : ajk - s0;
          }
          *elem(g, i, sl) = (T)u;
        }
        __syncwarp();
      }
    }
    __syncthreads();
    if (CLUSTER) csync();
  }

  // FP64 refresh of the FP32 tableau: x_B and the duals y are recomputed
  // from the original A, b, c with iterative refinement (residual in FP64,
  // correction through B^-1 in FP32; the columns of B^-1 are the slack
  // columns: stored ones for nonbasic slacks, unit vectors for basic ones),
  // then d_j = y^T a_j - c_j for the nonbasic columns and z = c_B^T x_B in
  // FP64.  The FP32 RHS column (every replica) and objective row are
  // overwritten.  Rank 0 computes, reading and writing the other CTAs'
  // columns through distributed shared memory.  Every sum runs in a fixed
  // order, so the result does not depend on the thread count or the cluster
  // split.  All work is proportional to ns, the number of structural basics
  // (= the number of nonbasic slacks), except the reduced costs, one FP64
  // dot product per nonbasic structural column.  Returns bit 0: x_B >= -ptol,
  // bit 1: d >= -opt_tol (both judged in FP64), bit 2: both refinements
  // converged (without it bits 0 and 1 prove nothing).  Single-phase LPs only.
  __device__ __forceinline__ int refresh_refine_body(const Geom g, const double* A,
                                                     const double* b, const double* c,
                                                     const double opt_tol, const double ptol) {
    const int m = g.m, n = g.n;
    const int tid = threadIdx.x, nt = blockDim.x;
    const int lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
    if (CLUSTER) csync();
    int ok = 0;
    if (rank == 0) {
      double* part = reinterpret_cast<double*>(redP);  // 192 doubles of partial sums
      // Structural basics as a list of rows in row order (flags[], its
      // warm-start use is over by now); nonbasic slacks as a list of slack
      // indices k in increasing order (rhsx, free until the next pivot).
      // Slack k sits in slot vpos[n + k] when nonbasic; when basic, in row
      // -1 - vpos[n + k].
      int* slist = flags;
      int* nlist = reinterpret_cast<int*>(rhsx);
      int* wcount = reinterpret_cast<int*>(redH);  // chunk offsets: [0,33) rows, [64,97) slacks
      const int nch = ceil_div(m, 32);
      for (int ch = warp; ch < 2 * nch; ch += nw) {
        const bool rows = ch < nch;
        const int i = (rows ? ch : ch - nch) * 32 + lane;
        const bool st = i < m && (rows ? basis[i] < n : vpos[n + i] >= 0);
        const unsigned bal = __ballot_sync(0xffffffffu, st);
        if (lane == 0) wcount[rows ? ch : 64 + ch - nch] = __popc(bal);
      }
      __syncthreads();
      if (tid < 2) {
        int acc = 0;
        for (int ch = 0; ch < nch; ++ch) {
          const int v = wcount[64 * tid + ch];
          wcount[64 * tid + ch] = acc;
          acc += v;
        }
        wcount[64 * tid + nch] = acc;
      }
      __syncthreads();
      for (int ch = warp; ch < 2 * nch; ch += nw) {
        const bool rows = ch < nch;
        const int i = (rows ? ch : ch - nch) * 32 + lane;
        const bool st = i < m && (rows ? basis[i] < n : vpos[n + i] >= 0);
        const unsigned bal = __ballot_sync(0xffffffffu, st);
        const int pos = __popc(bal & ((1u << lane) - 1u));
        if (st) {
          if (rows)
            slist[wcount[ch] + pos] = i;
          else
            nlist[wcount[64 + ch - nch] + pos] = i;
        }
      }
      __syncthreads();
      const int ns = wcount[nch], nn = wcount[64 + nch];
      // x_B and the duals are refined side by side, pass for pass (they are
      // independent: x_B from b, y from c), so that each pass's residuals
      // and corrections of both are in flight together; each stops at its
      // own convergence, and every element is computed exactly as it would
      // be alone.  Residuals rounded to FP32: rfx (rf) for x_B, rfy (col0)
      // for y.  Largest |correction| and |value| of a step: positive floats
      // order like their bit patterns, so a shared atomicMax works.
      float* rfx = rf;
      float* rfy = reinterpret_cast<float*>(col0);
      unsigned* mx = &sh->aux.w2;                          // x: [0] |correction|, [1] |value|
      unsigned* my = reinterpret_cast<unsigned*>(&sh->pad0);  // y: the same
      for (int i = tid; i < m; i += nt) xr[i] = (double)tab[(size_t)i * g.ldw + g.cw];
      // initial duals: y_k = d of slack k (0 when the slack is basic)
      for (int k = tid; k < m; k += nt) {
        const int sv = vpos[n + k];
        yr[k] = sv >= 0 ? (double)*elem(g, m, sv) : 0.0;
      }
      // y_k is exactly 0 for every basic slack k (it starts at 0 and its
      // correction is its own residual, -y_k), so the sums over k below run
      // over the nonbasic slacks (nlist, nn of them) only.  The range of each
      // structural basic's column sum is split in P parts (partial sums in
      // `part`, 192 doubles), combined in a fixed order; P = 1 above 96
      // basics
      const int P = (ns > 0 && ns <= 96) ? min(4, 192 / ns) : 1;
      const int kc = ceil_div(nn, P);
      bool xconv = false, yconv = false;
      for (int it = 0; it < kRefineIters; ++it) {
        if (tid == 0) mx[0] = mx[1] = my[0] = my[1] = 0u;
        __syncthreads();
        // r_k = b_k - sum_t A_k,col_t x_t - x_(slack k, when basic): one
        // thread per row, four interleaved partial sums over the basics
        for (int k = tid; k < m && !xconv; k += nt) {
          const double* Ak = A + (size_t)k * n;
          double p0 = 0.0, p1 = 0.0, p2 = 0.0, p3 = 0.0;
          int t = 0;
          for (; t + 4 <= ns; t += 4) {
            const int i0 = slist[t], i1 = slist[t + 1], i2 = slist[t + 2], i3 = slist[t + 3];
            p0 = fma(__ldg(Ak + basis[i0]), xr[i0], p0);
            p1 = fma(__ldg(Ak + basis[i1]), xr[i1], p1);
            p2 = fma(__ldg(Ak + basis[i2]), xr[i2], p2);
            p3 = fma(__ldg(Ak + basis[i3]), xr[i3], p3);
          }
          for (; t < ns; ++t) {
            const int i0 = slist[t];
            p0 = fma(__ldg(Ak + basis[i0]), xr[i0], p0);
          }
          double r = b[k] - ((p0 + p1) + (p2 + p3));
          const int sv = vpos[n + k];
          if (sv < 0) r = r - xr[-1 - sv];
          rfx[k] = (float)r;
        }
        // s_i = cB_i - (B^T y)_i: structural basic in row i with column col:
        // c_col - sum_k A_k,col y_k; basic slack k: -y_k
        for (int w = tid; w < ns * P && !yconv; w += nt) {
          const int t = w % ns, pp = w / ns;
          const int col = basis[slist[t]];
          const int u0 = pp * kc, u1 = min(nn, u0 + kc);
          double p0 = 0.0, p1 = 0.0;
          int u = u0;
          for (; u + 2 <= u1; u += 2) {
            const int k = nlist[u], k2 = nlist[u + 1];
            p0 = fma(__ldg(A + (size_t)k * n + col), yr[k], p0);
            p1 = fma(__ldg(A + (size_t)k2 * n + col), yr[k2], p1);
          }
          if (u < u1) p0 = fma(__ldg(A + (size_t)nlist[u] * n + col), yr[nlist[u]], p0);
          if (P == 1)
            rfy[slist[t]] = (float)(c[col] - (p0 + p1));
          else
            part[pp * ns + t] = p0 + p1;
        }
        for (int i = tid; i < m && !yconv; i += nt) {
          const int bi = basis[i];
          if (bi >= n) rfy[i] = (float)(bi < n + m ? -yr[bi - n] : 0.0);
        }
        __syncthreads();
        if (!yconv && P > 1) {
          for (int t = tid; t < ns; t += nt) {
            double sum = part[t];
            for (int pp = 1; pp < P; ++pp) sum += part[pp * ns + t];
            const int i = slist[t];
            rfy[i] = (float)(c[basis[i]] - sum);
          }
          __syncthreads();
        }
        // dx_i = sum_k Binv_ik r_k in FP32: one thread per row i over the
        // nonbasic slacks' columns, plus r_k when row i holds basic slack k
        for (int ib = tid & ~31; ib < m && !xconv; ib += nt) {  // warp-uniform trip count
          const int i = ib + lane;
          float acc = 0.f;
          if (i < m) {
            float q0 = 0.f, q1 = 0.f;
            int u = 0;
            for (; u + 2 <= nn; u += 2) {
              const int k0 = nlist[u], k1 = nlist[u + 1];
              q0 = fmaf((float)*elem(g, i, vpos[n + k0]), rfx[k0], q0);
              q1 = fmaf((float)*elem(g, i, vpos[n + k1]), rfx[k1], q1);
            }
            if (u < nn) {
              const int k0 = nlist[u];
              q0 = fmaf((float)*elem(g, i, vpos[n + k0]), rfx[k0], q0);
            }
            acc = q0 + q1;
            const int bi = basis[i];
            if (bi >= n && bi < n + m) acc = acc + rfx[bi - n];
            xr[i] += (double)acc;
          }
          const unsigned c0m = __reduce_max_sync(0xffffffffu, __float_as_uint(fabsf(acc)));
          const unsigned c1m =
              __reduce_max_sync(0xffffffffu, i < m ? __float_as_uint(fabsf((float)xr[i])) : 0u);
          if (lane == 0) {
            atomicMax(&mx[0], c0m);
            atomicMax(&mx[1], c1m);
          }
        }
        // dy_k = sum_i s_i Binv_ik in FP32: a basic slack k in row i takes
        // s_i, a nonbasic one sums its stored column over the structural
        // basics' rows (one thread per slack)
        for (int kb = tid & ~31; kb < m && !yconv; kb += nt) {  // warp-uniform trip count
          const int k = kb + lane;
          float acc = 0.f;
          if (k < m) {
            const int sv = vpos[n + k];
            if (sv < 0) {
              acc = rfy[-1 - sv];
            } else {
              // s_i is 0 on the rows of basic slacks (-y_k, and y_k is 0
              // there), so the sum runs over the structural basics' rows
              float q0 = 0.f, q1 = 0.f, q2 = 0.f, q3 = 0.f;
              int t = 0;
              for (; t + 4 <= ns; t += 4) {
                const int i0 = slist[t], i1 = slist[t + 1], i2 = slist[t + 2], i3 = slist[t + 3];
                q0 = fmaf(rfy[i0], (float)*elem(g, i0, sv), q0);
                q1 = fmaf(rfy[i1], (float)*elem(g, i1, sv), q1);
                q2 = fmaf(rfy[i2], (float)*elem(g, i2, sv), q2);
                q3 = fmaf(rfy[i3], (float)*elem(g, i3, sv), q3);
              }
              for (; t < ns; ++t) {
                const int i0 = slist[t];
                q0 = fmaf(rfy[i0], (float)*elem(g, i0, sv), q0);
              }
              acc = (q0 + q1) + (q2 + q3);
            }
            yr[k] += (double)acc;
          }
          const unsigned c0m = __reduce_max_sync(0xffffffffu, __float_as_uint(fabsf(acc)));
          const unsigned c1m =
              __reduce_max_sync(0xffffffffu, k < m ? __float_as_uint(fabsf((float)yr[k])) : 0u);
          if (lane == 0) {
            atomicMax(&my[0], c0m);
            atomicMax(&my[1], c1m);
          }
        }
        __syncthreads();
        if (!xconv && __uint_as_float(mx[0]) <= 1e-10f * fmaxf(1.f, __uint_as_float(mx[1])))
          xconv = true;
        if (!yconv && __uint_as_float(my[0]) <= 1e-10f * fmaxf(1.f, __uint_as_float(my[1])))
          yconv = true;
        if (xconv && yconv) break;
        __syncthreads();
      }
      // Reduced costs d_j = y^T a_j - c_j of the nonbasic structural
      // columns: one thread per column over coalesced rows of A (the rows of
      // the nonbasic slacks: y is 0 on the others), four interleaved partial
      // sums.  Nonbasic slack k: d = y_k.
      bool badd = false, badp = false;
      for (int j = tid; j < n; j += nt) {
        const int sv = vpos[j];
        if (sv < 0) continue;
        double p0 = 0.0, p1 = 0.0, p2 = 0.0, p3 = 0.0;
        int u = 0;
        for (; u + 4 <= nn; u += 4) {
          const int k0 = nlist[u], k1 = nlist[u + 1], k2 = nlist[u + 2], k3 = nlist[u + 3];
          p0 = fma(__ldg(A + (size_t)k0 * n + j), yr[k0], p0);
          p1 = fma(__ldg(A + (size_t)k1 * n + j), yr[k1], p1);
          p2 = fma(__ldg(A + (size_t)k2 * n + j), yr[k2], p2);
          p3 = fma(__ldg(A + (size_t)k3 * n + j), yr[k3], p3);
        }
        for (; u < nn; ++u) p0 = fma(__ldg(A + (size_t)nlist[u] * n + j), yr[nlist[u]], p0);
        const double d = ((p0 + p1) + (p2 + p3)) - c[j];
        *elem(g, m, sv) = (T)d;
        badd = badd || d < -opt_tol;
      }
      for (int k = tid; k < m; k += nt) {
        const int sv = vpos[n + k];
        if (sv < 0) continue;
        const double d = yr[k];
        *elem(g, m, sv) = (T)d;
        badd = badd || d < -opt_tol;
      }
      for (int i = tid; i < m; i += nt) {
        const T xv = (T)xr[i];
        for (int o = 0; o < K; ++o) {
          T* p = tab + (size_t)i * g.ldw + g.cw;
          *(o == rank ? p : remote(p, o)) = xv;
        }
        badp = badp || xr[i] < -ptol;
      }
      // z = c_B^T x_B: warp 0, lane-strided partial sums over the structural
      // basics combined by a butterfly (a fixed order)
      if (warp == 0) {
        double z = 0.0;
        for (int t = lane; t < ns; t += 32) {
          const int i = slist[t];
          z = fma(c[basis[i]], xr[i], z);
        }
        for (int o = 16; o > 0; o >>= 1) z += __shfl_xor_sync(0xffffffffu, z, o);
        if (lane == 0) {
          sh->z = z;
          for (int o = 0; o < K; ++o) {
            T* p = tab + (size_t)m * g.ldw + g.cw;
            *(o == rank ? p : remote(p, o)) = (T)z;
          }
        }
      }
      badd = __syncthreads_or(badd ? 1 : 0) != 0;
      badp = __syncthreads_or(badp ? 1 : 0) != 0;
      ok = (badp ? 0 : 1) | (badd ? 0 : 2) | (xconv && yconv ? 4 : 0);
      if (tid == 0) sh->aux.w1 = (unsigned)ok;
    }
    if (CLUSTER) {
      csync();
      ok = (int)remote(&sh->aux, 0)->w1;
      csync();
    }
    return ok;
  }

  // The structural block of the tableau from rows of A (Ac = A's column
  // c0 of row 0, cc = c + c0): a warp takes two rows at a time, each lane
  // eight coalesced columns of each, so that sixteen loads per lane are in
  // flight before the first conversion waits on one.  Out of line with plain
  // arguments, so that its registers do not add to the kernel's.
  static __device__ __noinline__ void load_block(T* __restrict__ const tb,
                                                 const double* __restrict__ const Ac,
                                                 const double* __restrict__ const cc,
                                                 const int* __restrict__ const flags,
                                                 const int m, const int n, const int nA,
                                                 const int ldw, const int na) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    constexpr int kR = 2, kQ = 8;
    for (int i0 = warp * kR; i0 <= m; i0 += nw * kR) {
      for (int j0 = 0; j0 < nA; j0 += 32 * kQ) {
        double v[kR][kQ];
#pragma unroll
        for (int r = 0; r < kR; ++r) {
          const int i = i0 + r;
          const double* src = i < m ? Ac + (size_t)i * n : cc;
          const bool live = i < m || (i == m && na == 0);
#pragma unroll
          for (int q = 0; q < kQ; ++q) {
            const int j = j0 + q * 32 + lane;
            v[r][q] = live && j < nA ? __ldg(src + j) : 0.0;
          }
        }
#pragma unroll
        for (int r = 0; r < kR; ++r) {
          const int i = i0 + r;
          if (i > m) continue;
          // -c in the objective row, or a negated constraint row
          const bool neg = i == m ? na == 0 : (na > 0 && flags[i] >= 0);
#pragma unroll
          for (int q = 0; q < kQ; ++q) {
            const int j = j0 + q * 32 + lane;
            if (j < nA) {
              const T x = to_tab(v[r][q], T(0));
              tb[(size_t)i * ldw + j] = neg ? -x : x;
            }
          }
        }
      }
    }
  }

  // The same block from A already rounded to FP32 (A32, rows `pitch` apart):
  // rows 0..m-1 are plain copies (half the bytes of the FP64 rows, nothing
  // to convert); row m (-c in a single-phase LP, 0 before phase I) is
  // converted separately, so that no conversion sits in the row loop.
  static __device__ __noinline__ void load_block32(float* __restrict__ const tb,
                                                   const float* __restrict__ const Ac,
                                                   const double* __restrict__ const cc,
                                                   const int* __restrict__ const flags,
                                                   const int m, const int pitch, const int nA,
                                                   const int ldw, const int na) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    constexpr int kR = 2, kQ = 8;
    for (int i0 = warp * kR; i0 < m; i0 += nw * kR) {
      for (int j0 = 0; j0 < nA; j0 += 32 * kQ) {
        float v[kR][kQ];
#pragma unroll
        for (int r = 0; r < kR; ++r) {
          const int i = min(i0 + r, m - 1);  // a row past m - 1 is loaded, not stored
#pragma unroll
          for (int q = 0; q < kQ; ++q) {
            const int j = j0 + q * 32 + lane;
            v[r][q] = j < nA ? __ldg(Ac + (size_t)i * pitch + j) : 0.f;
          }
        }
#pragma unroll
        for (int r = 0; r < kR; ++r) {
          const int i = i0 + r;
          if (i >= m) continue;
          const bool neg = na > 0 && flags[i] >= 0;  // a negated constraint row
#pragma unroll
          for (int q = 0; q < kQ; ++q) {
            const int j = j0 + q * 32 + lane;
            if (j < nA) tb[(size_t)i * ldw + j] = neg ? -v[r][q] : v[r][q];
          }
        }
      }
    }
    for (int j = threadIdx.x; j < nA; j += blockDim.x)
      tb[(size_t)m * ldw + j] = na == 0 ? -f64_to_f32_rn(__ldg(cc + j)) : 0.f;
  }

  // FP32 tableau of a single-CTA phase-II LP from the padded FP32 copy of A,
  // whose rows are exactly as long as the tableau's (a32_pitch(n) = ldw):
  // the whole block, rows 0..m-1, is one bulk (TMA) copy issued by one
  // thread and completing on the CTA's mbarrier (the rows' padding lands in
  // slots [n, ldw), which load() fills afterwards); the objective row -c is
  // converted meanwhile.  False when the copy did not complete within the
  // wait limit.
  __device__ bool load_block_bulk32(const Geom& g, const float* A32, const double* c) {
    const int m = g.m, n = g.n, ldw = g.ldw;
    const int tid = threadIdx.x, nt = blockDim.x;
    float* tb = reinterpret_cast<float*>(tab);
    unsigned long long* bar = &sh->bar;
    fence_proxy_async_smem();  // the previous LP's accesses to these rows come first
    if (tid == 0) mbar_init(bar, 1);
    __syncthreads();
    const unsigned bytes = (unsigned)m * (unsigned)ldw * 4u;
    if (tid == 0) {
      mbar_arrive_expect_tx(bar, bytes);
      if (bytes > 0) bulk_g2s(tb, A32, bytes, bar);
    }
    for (int j = tid; j < n; j += nt) tb[(size_t)m * ldw + j] = -f64_to_f32_rn(__ldg(c + j));
    bool ok = mbar_wait(bar, 0);
    if (!ok) mbar_wait(bar, 0);  // let a copy still in flight land before giving up
    __syncthreads();
    if (tid == 0) mbar_inval(bar);
    return ok;
  }

  // FP64 tableau: the structural block copied straight from rows of A (and
  // c for row m of a single-phase LP), no registers involved.  A row whose
  // source starts on a 16-byte boundary goes by one bulk (TMA) copy of its
  // whole 16-byte pairs, issued by the first warp and completing on the
  // CTA's mbarrier; the other rows, and an odd last element, by 8-byte
  // asynchronous copies.  Then the rows to negate are negated in place.
  // False when the bulk copies did not complete within the wait limit.
  __device__ bool load_rows_async(const Geom& g, int c0, int nA, const double* A,
                                  const double* c) {
    const int m = g.m, n = g.n, na = g.na, ldw = g.ldw;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
    const unsigned pair_bytes = (unsigned)(nA >> 1) * 16u;
    const int npair = (nA >> 1) << 1;  // elements the bulk copy of a row covers
    unsigned long long* bar = &sh->bar;
    const bool tab16 = (smem_addr(tab) & 15u) == 0 && (ldw & 1) == 0;
    auto src_of = [&](int i) { return i < m ? A + (size_t)i * n + c0 : c + c0; };
    auto bulk_row = [&](int i) {
      return tab16 && pair_bytes > 0 && (i < m || na == 0) &&
             (reinterpret_cast<uintptr_t>(src_of(i)) & 15u) == 0;
    };
    fence_proxy_async_smem();  // the previous LP's accesses to these rows come first
    if (tid == 0) mbar_init(bar, 1);
    __syncthreads();
    if (warp == 0) {
      int rows = 0;
      for (int i = lane; i <= m; i += 32) rows += bulk_row(i) ? 1 : 0;
      rows = __reduce_add_sync(0xffffffffu, rows);
      if (lane == 0) mbar_arrive_expect_tx(bar, (unsigned)rows * pair_bytes);
      __syncwarp();
      for (int i = lane; i <= m; i += 32)
        if (bulk_row(i)) bulk_g2s(tab + (size_t)i * ldw, src_of(i), pair_bytes, bar);
    }
    for (int i = warp; i <= m; i += nw) {
      T* dst = tab + (size_t)i * ldw;
      if (i == m && na > 0) {  // phase I starts from a zero objective row
        for (int j = lane; j < nA; j += 32) dst[j] = T(0);
        continue;
      }
      const double* src = src_of(i);
      for (int j = (bulk_row(i) ? npair : 0) + lane; j < nA; j += 32) {
        const unsigned sa = smem_addr(dst + j);
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(sa), "l"(src + j)
                     : "memory");
      }
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    bool ok = mbar_wait(bar, 0);
    if (!ok) mbar_wait(bar, 0);  // let copies still in flight land before giving up
    __syncthreads();
    if (tid == 0) mbar_inval(bar);
    // -c in the objective row of a single-phase LP; the rows with b_i < 0
    for (int i = warp; i <= m; i += nw) {
      const bool neg = i == m ? na == 0 : (na > 0 && flags[i] >= 0);
      if (!neg) continue;
      T* row = tab + (size_t)i * ldw;
      for (int j = lane; j < nA; j += 32) row[j] = -row[j];
    }
    return ok;
  }

  // Build the slack-basis tableau of LP lp: rows with b_i < 0 are negated
  // and get an artificial variable each (the a-th such row's artificial is
  // basic there and its slack takes column slot n + a); structural j sits in
  // slot j.  Coalesced along rows of A.
  // Out of line, on a copy of the solver (load changes no member), so that
  // the loaders' registers do not add to the pivot loop's.  When the bulk
  // copies of the load do not complete within the wait limit, LP lp is given
  // up (abandon) and the CTA -- every CTA of its cluster, which decide
  // together -- exits; the kernel's other CTAs go on.
  static __device__ __noinline__ void load_call(Solver self, const Geom g, int c0, int lc,
                                                const double* A, const double* b,
                                                const double* c, const float* A32,
                                                const LpArgs& a, int lp) {
    if (!self.load_body(g, c0, lc, A, b, c, A32)) {
      self.abandon(a, lp);
      asm volatile("exit;" ::: "memory");
    }
  }
  __device__ void load(const Geom& g, int c0, int lc, const double* A, const double* b,
                       const double* c, const float* A32, const LpArgs& a, int lp) {
    load_call(*this, g, c0, lc, A, b, c, A32, a, lp);
  }
  __device__ bool load_body(const Geom& g, int c0, int lc, const double* A, const double* b,
                            const double* c, const float* A32) {
    const int tid = threadIdx.x, nt = blockDim.x;
    const int m = g.m, n = g.n, na = g.na;
    const int warp = tid >> 5, lane = tid & 31, nw = nt >> 5;
    if (na > 0) {
      // flags[i] = index a of negated row i among the negated rows, else -1
      // (ballot per 32-row chunk, then a prefix sum over the chunks)
      int* wcount = reinterpret_cast<int*>(redH);
      const int nchunks = ceil_div(m, 32);
      for (int ch = warp; ch < nchunks; ch += nw) {
        const int i = ch * 32 + lane;
        const unsigned bal = __ballot_sync(0xffffffffu, i < m && b[i] < 0.0);
        if (lane == 0) wcount[ch] = __popc(bal);
      }
      __syncthreads();
      if (tid == 0) {
        int acc = 0;
        for (int ch = 0; ch < nchunks; ++ch) {
          const int v = wcount[ch];
          wcount[ch] = acc;
          acc += v;
        }
      }
      __syncthreads();
      for (int ch = warp; ch < nchunks; ch += nw) {
        const int i = ch * 32 + lane;
        const bool neg = i < m && b[i] < 0.0;
        const unsigned bal = __ballot_sync(0xffffffffu, neg);
        if (i < m) flags[i] = neg ? wcount[ch] + __popc(bal & ((1u << lane) - 1u)) : -1;
      }
      __syncthreads();
    }
    // labels
    for (int v = tid; v < n + m; v += nt) {
      if (v < n) {
        cvar[v] = v;
        vpos[v] = v;
      } else {
        const int i = v - n;
        const int ai = na > 0 ? flags[i] : -1;
        if (ai >= 0) {
          cvar[n + ai] = v;
          vpos[v] = n + ai;
          vpos[n + m + ai] = -1 - i;
          basis[i] = n + m + ai;
        } else {
          vpos[v] = -1 - i;
          basis[i] = v;
        }
      }
    }
    __syncthreads();
    const int ldw = g.ldw;
    // Structural block (slots [0, nA) of this CTA); row m is the objective
    // row (-c in a single-phase LP, 0 before phase I)
    const int nA = max(0, min(n - c0, lc));
    bool ok = true;
    if constexpr (sizeof(T) == 8) {
      ok = load_rows_async(g, c0, nA, A, c);
    } else if (A32) {
      const int pitch = a32_pitch(n);
      // one bulk copy when the copy's rows are the tableau's: a single-CTA
      // LP without phase-I columns, both addresses 16-byte aligned, and the
      // block within the mbarrier's transaction count
      const bool whole = c0 == 0 && na == 0 && ldw == pitch &&
                         ((smem_addr(tab) | (unsigned)reinterpret_cast<uintptr_t>(A32)) & 15u) == 0 &&
                         (size_t)m * ldw * 4 < (size_t(1) << 20);
      if (whole)
        ok = load_block_bulk32(g, A32, c);
      else
        load_block32(reinterpret_cast<float*>(tab), A32 + c0, c + c0, flags, m, pitch, nA, ldw,
                     na);
    } else {
      load_block(tab, A + c0, c + c0, flags, m, n, nA, ldw, na);
    }
    if (cluster_any(!ok)) return false;  // the cluster gives the LP up together
    // The rest of every row: slack slots of negated rows (-1 in their own
    // row), zero padding, and the RHS (|b_i|; 0 in the objective row).
    const int wr = ldw - nA;
    for (int e = tid; e < (m + 1) * wr; e += nt) {
      const int i = e / wr, lj = nA + (e - i * wr);
      T x = T(0);
      if (i < m) {
        if (lj < lc) {
          if (cvar[c0 + lj] - n == i) x = T(-1);  // the negated row's slack
        } else if (lj == g.cw) {
          const T bv = (T)__ldg(b + i);
          x = (na > 0 && flags[i] >= 0) ? -bv : bv;
        }
      }
      tab[(size_t)i * ldw + lj] = x;
    }
    __syncthreads();
    return true;
  }

  // The bulk copies of a tableau load did not complete within the wait
  // limit: the LP is reported undefined with kInfoLoad.
  __device__ void abandon(const LpArgs& a, int lp) {
    if (rank == 0 && threadIdx.x == 0) {
      a.status[lp] = kUndef;
      a.obj[lp] = 0.0;
      if (a.pivots) a.pivots[lp] = -1;
      if (a.info) a.info[lp] = kInfoLoad | a.info_or;
    }
    __syncthreads();
  }

  // Verify an optimal basis in FP64 and repair it if needed: a refresh,
  // then, while it finds a violation, dual simplex (x_B < 0) and primal
  // simplex pivots, each round verified by another refresh (at most four
  // repairs).  Returns kOpt once verified, kUnverified when a refresh cannot
  // judge the basis (or four repairs do not settle it), or the status a
  // repair ended on.
  __device__ int verify_basis(const Geom& g, int c0, int lc, const double* A, const double* b,
                              const double* c, const LpArgs& a, const float* w, int budget,
                              int& pivots, bool& bland, int& degen, int& cur, int& piv_fresh,
                              int& info) {
    const T ptol = (T)a.ptol;
    int st = kOpt;
    bool verified = false;
    for (int round = 0; round <= 4; ++round) {
      if (CLUSTER) csync();
      int fl = refresh(g, A, b, c, a);
      piv_fresh = pivots;
      info |= kInfoRefresh | ((fl & 8) ? kInfoFactor : 0);
      if ((fl & 7) == 7) {
        verified = true;
        break;
      }
      if (!(fl & 4)) break;  // no refresh could judge the basis
      if (round == 4) break;
      info |= kInfoRepair;
      if (lu && (round > 0 || (fl & 8))) {
        // the first repair on the tableau as it is did not settle the basis,
        // or its B^-1 could not even be refined: repairs on a tableau rebuilt
        // from the basis's FP64 factorisation
        if (!(fl & 8)) fl = refresh_lu(g, A, b, c, a.opt_tol, a.ptol) | 8;
        info |= kInfoFactor;
        if (!(fl & 4)) break;
        if ((fl & 3) == 3) {
          verified = true;
          break;
        }
        reinvert(g, A);
        info |= kInfoReinvert;
      }
      if (!(fl & 1)) {
        info |= kInfoDual;
        st = dual_loop(g, c0, lc, a, budget, pivots, cur, ptol);
        if (st != kOpt) break;
      }
      st = primal(g, c0, lc, a, w, budget, pivots, bland, degen, cur);
      if (st != kOpt) break;
    }
    if (st == kOpt && !verified) st = kUnverified;
    return st;
  }

  // Per-LP regions of the shared-memory layout.
  __device__ void place(const Layout& L, int m) {
    tab = reinterpret_cast<T*>(smem + L.tab);
    col0 = reinterpret_cast<T*>(smem + L.colA);
    col1 = reinterpret_cast<T*>(smem + L.colB);
    rhsx = reinterpret_cast<T*>(smem + L.rhsx);
    basis = reinterpret_cast<int*>(smem + L.basis);
    flags = reinterpret_cast<int*>(smem + L.flags);
    cvar = reinterpret_cast<int*>(smem + L.cvar);
    vpos = reinterpret_cast<int*>(smem + L.vpos);
    xr = reinterpret_cast<double*>(smem + L.ext);
    yr = xr + round_up(m + 1, 4);
    rf = reinterpret_cast<float*>(yr + round_up(m + 1, 4));
    gam = L.gam >= 0 ? reinterpret_cast<uint2*>(smem + L.gam) : nullptr;
  }

  // PART: the class's layouts hold the FP32 steepest-edge norms as partial
  // sums of this CTA's row groups (the norm region grown to fit them)
  template <bool PART>
  __device__ void run(const LpArgs& a, const ClassArgs& ca) {
    const int tid = threadIdx.x, nt = blockDim.x;
    constexpr bool kFP32 = sizeof(T) == 4;
    const int count = ca.count_dev ? *ca.count_dev : ca.count;
    for (;;) {
      if (rank == 0 && tid == 0) sh->ticket = atomicAdd(ca.ticket, 1);
      csync();
      if (CLUSTER) {
        // rank 0 drew the ticket: one thread per CTA fetches it
        if (rank != 0 && tid == 0) sh->ticket = remote(sh, 0)->ticket;
        __syncthreads();
      }
      const int t = sh->ticket;
      if (t >= count) break;
      const int lp = ca.order[t];
      const int m = a.m[lp], n = a.n[lp];
      const double* A = a.A + a.offA[lp];
      const float* A32 = a.A32 ? a.A32 + a.off32[lp] : nullptr;
      const double* b = a.b + a.offb[lp];
      const double* c = a.c + a.offc[lp];
      // two-phase when any b_i < 0 (the reference's rem list, simplex.cu:574-583)
      int na = 0;
      for (int i = tid; i < m; i += nt) na += b[i] < 0.0 ? 1 : 0;
      na = block_sum(na);
      const Geom g(m, n, na, K, V);
      const int pbytes = PART ? min(nt / g.nl, kMaxNormGroups) * g.cw * 4 : 0;
      const Layout L(m, g.ldw, n + m + na, (int)sizeof(T), ca.se, pbytes);
      if (L.total > ca.smem || na > ca.max_na || g.nl > (int)blockDim.x) {
        // the LP does not fit the layout this plan was built for (e.g. a
        // plan made without b has no room for phase-I columns): refuse it
        if (rank == 0 && tid == 0) {
          a.status[lp] = kUndef;
          a.obj[lp] = 0.0;
          if (a.pivots) a.pivots[lp] = -1;
          if (a.info) a.info[lp] = a.info_or;
        }
        __syncthreads();
        continue;
      }
      place(L, m);
      // FP32 on one CTA: the norms as partial sums where they fit the region
      ngrp = 0;
      if (kFP32 && !CLUSTER && gam) {
        const int G = min(nt / g.nl, kMaxNormGroups);
        if ((size_t)G * g.cw * 4 <= (size_t)L.gbytes) ngrp = G;
      }
      const int c0 = rank * g.cw;
      const int lc = max(0, min(g.cw, g.Wc - c0));
      load(g, c0, lc, A, b, c, A32, a, lp);
      int pivots = 0, degen = 0, cur = 0, st, info = 0;
      const float* w = a.weight ? a.weight + a.offw[lp] : nullptr;
      // final bases verified (and reported) in FP64: the FP32 tableau, and the
      // FP64 one with steepest-edge pricing in plans (LU scratch); the FP64
      // Dantzig path is the reference's method, reported as the oracle does
      const bool verify = kFP32 || (ca.se && a.pricing == 1 && lu != nullptr);
      bool bland = false;
      // pivot count at the last FP64 refresh: its x_B and objective are
      // reported only if no pivot followed it (-1: none yet)
      int piv_fresh = -1;
      // FP32 plans with an FP64 pass stop an FP32 solve at 4 (m + n) + 200
      // pivots (several times what these solves take) and hand the LP over
      const int user_piv = a.max_pivots > 0 ? a.max_pivots : 50 * (m + n) + 1000;
      const int max_piv = (kFP32 && a.fb) ? min(user_piv, 4 * (m + n) + 200) : user_piv;
      const T ptol = (T)a.ptol, opt_tol = (T)a.opt_tol;
      // A solve whose final basis the FP64 check cannot verify is repeated
      // cold from the slack basis when it was warm-started, with a pivot
      // budget of its own; a cold one is reported BLPG_UNDEF.  Phase-I LPs
      // (hints ignored) are verified when the plan has LU scratch: the
      // refactorisation handles their negated rows.
      const bool check = verify && (na == 0 || lu != nullptr);
      int budget = max_piv;
      for (int attempt = 0; attempt < 2; ++attempt) {
        st = -1;
        const bool warm = attempt == 0 && a.hint && na == 0;
        if (attempt > 0) {
          info |= kInfoFallback;
          if (CLUSTER) csync();
          load(g, c0, lc, A, b, c, A32, a, lp);
          piv_fresh = -1;
          bland = false;
          degen = 0;
          budget = pivots + max_piv;
        }
        if (na > 0) {
          // phase I on the artificials' objective, drive-out, phase II
          objective_row(g, c0, lc, c, true);
          __syncthreads();
          st = primal(g, c0, lc, a, w, budget, pivots, bland, degen, cur);
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
            st = primal(g, c0, lc, a, w, budget, pivots, bland, degen, cur);
          }
        } else {
            if (warm) {
              info |= kInfoWarm;
              if (crash(g, c0, a.hint + a.offbasis[lp], a, pivots, cur, lc) > 0)
                info |= kInfoPartial;
              // feasibility of the crashed basis judged on the tableau itself
              // (the final FP64 refresh verifies whatever basis the finish ends on)
              const int fl = check_feasible(g, c0, lc, ptol, opt_tol);
              if (fl & 1) {
                st = primal(g, c0, lc, a, w, budget, pivots, bland, degen, cur);
              } else if (fl & 2) {
                info |= kInfoDual;
                st = dual_loop(g, c0, lc, a, budget, pivots, cur, ptol);
                if (st == kOpt) st = primal(g, c0, lc, a, w, budget, pivots, bland, degen, cur);
              } else if (a.warm_mode == 1) {
                // infeasible both ways: shift the costs of the columns with
                // d_j < -opt_tol to small distinct positive values (dual
                // feasible), dual simplex to a primal-feasible basis, restore
                // the true costs, primal simplex
                info |= kInfoDual | kInfoShift;
                T* drow = tab + (size_t)m * g.ldw;
                for (int lj = tid; lj < lc; lj += nt) {
                  const int j = cvar[c0 + lj];
                  if (j < n + m && drow[lj] < -opt_tol)
                    drow[lj] = (T)a.shift * (T(1) + (T)((j * 7919) % 1000) / T(1000));
                }
                __syncthreads();
                st = dual_loop(g, c0, lc, a, budget, pivots, cur, ptol);
                if (st == kOpt) {
                  objective_row(g, c0, lc, c, false);
                  __syncthreads();
                  st = primal(g, c0, lc, a, w, budget, pivots, bland, degen, cur);
                }
              }
              if (st < 0 || st == kNoFeas) {
                // infeasible both ways (or dual simplex stuck): cold solve
                info |= kInfoFallback;
                if (CLUSTER) csync();
                load(g, c0, lc, A, b, c, A32, a, lp);
                piv_fresh = -1;
                bland = false;
                degen = 0;
                st = -1;
              }
            }
          if (st < 0) {
            const int period = kFP32 ? a.refresh_period : 0;
            for (;;) {
              st = primal(g, c0, lc, a, w, budget, pivots, bland, degen, cur, period);
              if (st != kRefresh) break;
              if (CLUSTER) csync();
              if (refresh(g, A, b, c, a) & 8) info |= kInfoFactor;
              piv_fresh = pivots;
              info |= kInfoRefresh;
            }
          }
        }
        // verify the final basis in FP64 and repair it if needed
        if (check && st == kOpt)
          st = verify_basis(g, c0, lc, A, b, c, a, w, budget, pivots, bland, degen, cur,
                            piv_fresh, info);
        // a warm start that ends unverified or at the pivot cap: once more, cold
        if (check && warm && (st == kUnverified || st == kUndef)) {
          if (st == kUnverified) info |= kInfoRetry;
          continue;
        }
        break;
      }
      if (st == kUnverified) {
        st = kUndef;
        info |= kInfoUnverified;
      }
      // unbounded: x_B of the final basis (where unboundedness was found)
      // from the FP64 refresh too, not from the FP32 tableau
      if (check && st == kUnbnd && piv_fresh != pivots) {
        if (CLUSTER) csync();
        if (refresh(g, A, b, c, a) & 8) info |= kInfoFactor;
        piv_fresh = pivots;
        info |= kInfoRefresh;
      }
      // FP32 plans: an LP the FP32 tableau could not settle (unverified, at
      // the pivot cap, or "infeasible" although b >= 0 makes the origin
      // feasible) goes to the plan's FP64 pass, which overwrites its results
      if (kFP32 && a.fb && (st == kUndef || (na == 0 && st == kNoFeas)) && rank == 0 &&
          tid == 0) {
        const int k = atomicAdd(a.fb, 1);
        a.fb[1 + k] = lp;
      }
      const bool refreshed = piv_fresh == pivots;
      if (CLUSTER) csync();
      // outputs (rank 0 holds a replica of the RHS column; after an FP64
      // refresh the FP64 x_B and objective are reported)
      if (rank == 0) {
        if (tid == 0) {
          a.status[lp] = st;
          a.obj[lp] = refreshed ? sh->z : (double)tab[(size_t)m * g.ldw + g.cw];
          if (a.pivots) a.pivots[lp] = pivots;
          if (a.info) a.info[lp] = info | a.info_or;
        }
        if (a.basis)
          for (int i = tid; i < m; i += nt) a.basis[a.offbasis[lp] + i] = basis[i];
        if (a.x) {
          double* x = a.x + a.offx[lp];
          for (int j = tid; j < n; j += nt) x[j] = 0.0;
          __syncthreads();
          for (int i = tid; i < m; i += nt)
            if (basis[i] < n)
              x[basis[i]] = refreshed ? xr[i] : (double)tab[(size_t)i * g.ldw + g.cw];
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

template <typename T, bool CLUSTER, bool PART = false>
__global__ void __launch_bounds__(512, 1) solve_kernel(const __grid_constant__ LpArgs a,
                                                        const __grid_constant__ ClassArgs ca) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Solver<T, CLUSTER> s;
  const Layout L(0, 0, 0, (int)sizeof(T), ca.se);  // the fixed header
  s.smem = smem_raw;
  s.redP = reinterpret_cast<Key*>(smem_raw + L.red);
  s.redR = s.redP + 32;
  s.redH = s.redP + 64;
  s.sh = reinterpret_cast<SharedState*>(smem_raw + L.state);
  s.K = ca.K;
  s.rank = CLUSTER ? (int)cg::this_cluster().block_rank() : 0;
  s.lu = ca.lu ? ca.lu + (size_t)(blockIdx.x / ca.K) * (size_t)ca.lu_stride : nullptr;
  s.template run<PART>(a, ca);
}

}  // namespace dev
}  // namespace blpg
