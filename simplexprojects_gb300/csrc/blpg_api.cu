// Host side of libblpg.so: plans (size classes + device work queues + CUDA
// graph), the C ABI entry points and the synchronous host-buffer solve.
//
// Reference host path: Simplex::ComputeLP (BLPG-Solver/src/simplex.cu:552-977)
// builds every tableau on the host with OpenMP, copies the whole tableau
// batch to the device on N user streams, launches one block per LP with
// blockDim = 32*(N/32)+32 and copies one objective per LP back, allocating
// and freeing device memory on every call.  Here the host only uploads
// A, b, c (tableaux are built in shared memory by the kernel), LPs are
// grouped into size classes that fix CTAs per LP, threads and shared memory,
// every class runs as one persistent launch fed by a device ticket queue, and
// a plan's launches are captured once into a CUDA graph and replayed.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <tuple>
#include <memory>
#include <atomic>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>

#include "blpg_internal.h"
#include "blpg_solver.cuh"

namespace blpg {
// solve_kernel<float, false, true> (partial-sum norm layouts), in blpg_part.cu
cudaError_t part_set_attrs(int max_smem);
cudaError_t part_occupancy(int* ctas_per_sm, int nt, int smem);
cudaError_t part_launch(int grid, int nt, int smem, cudaStream_t s, const dev::LpArgs& a,
                        const dev::ClassArgs& ca);
}  // namespace blpg

namespace blpg {

static thread_local std::string g_err;

int32_t fail(int32_t code, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

#define CK(call)                                                                  \
  do {                                                                            \
    cudaError_t e_ = (call);                                                      \
    if (e_ != cudaSuccess)                                                        \
      return fail(e_ == cudaErrorMemoryAllocation ? BLPG_ENOMEM : BLPG_ECUDA,     \
                  "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, \
                  __LINE__);                                                      \
  } while (0)

using dev::ClassArgs;
using dev::Geom;
using dev::Layout;
using dev::LpArgs;

// Tuning table (autotuner JSON).  Keys per precision p (fp64 | fp32):
//   "p_kK"        threads per CTA of cluster classes of K CTAs (K = 1: the
//                 default of every single-CTA class)
//   "p_cC"        threads per CTA of size class C (C = the CTAs per SM its
//                 layout admits for a single-CTA class, 100 + K for a cluster
//                 class); "p_cC_ctas" the CTAs per SM it runs with (at most C)
//   "p_smem"      the per-CTA shared-memory budget that picks cluster sizes
//   "p_ctas"      the cap on CTAs per SM of every single-CTA class
// The library starts from the table tuned on GB300 that the build compiles
// in (tuning/gb300.json); blpg_set_tuning replaces it, and a null table
// restores it.
struct Tuning {
  std::mutex mu;
  std::map<std::pair<int, int>, int> threads;  // (precision*16 + field, class or bucket)
  int generation = 0;  // bumped by every blpg_set_tuning: cached plans are rebuilt
  bool loaded = false;
};
static Tuning g_tuning;
#include "blpg_tuning_default.inc"  // kDefaultTuning: the compiled-in table (JSON text)
static void parse_tuning_locked(const char* json);

static int device_check(int device, cudaDeviceProp* prop) {
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0)
    return fail(BLPG_ENODEV, "no CUDA device (%s)", cudaGetErrorString(e));
  if (device < 0 || device >= ndev)
    return fail(BLPG_ENODEV, "device %d out of range (%d devices)", device, ndev);
  CK(cudaGetDeviceProperties(prop, device));
  if (prop->major != 10 || prop->minor != 3)
    return fail(BLPG_ENODEV, "device %d is sm_%d%d; libblpg is built for sm_103a only",
                device, prop->major, prop->minor);
  return BLPG_OK;
}

struct ClassPlan {
  int K = 1, nt = 128, max_m = 0, max_na = 0, smem = 0;
  int key = 1;  // tuning key: CTAs per SM the layout admits (single CTA), 100 + K (clusters)
  int max_ns = 0;  // most structural basics any member can have: min(m, n)
  long long lu_off = 0, lu_stride = 0;  // the class's LU refresh scratch (doubles)
  int ctas_per_sm = 1;
  int part = 0;  // FP32 steepest edge on one CTA: launched with the partial-sum norm layout
  int count = 0, grid = 0, order_off = 0;
  double work = 0;
};

}  // namespace blpg

struct blpg_plan {
  int device = 0;
  blpg_options opt{};
  int count = 0;
  int precision = BLPG_FP64;
  std::vector<int32_t> m, n, na;
  std::vector<int64_t> offA, offb, offc, offx, offbasis;
  int64_t extA = 0, extb = 0, extc = 0, extx = 0, extbasis = 0, extw = 0;
  int64_t minA = 0;  // smallest offset into A
  std::vector<blpg::ClassPlan> classes;
  std::vector<int32_t> order;
  // device arrays
  int32_t *d_m = nullptr, *d_n = nullptr, *d_order = nullptr, *d_tickets = nullptr;
  int64_t *d_off = nullptr;  // offA | offb | offc | offx | offbasis | offw | off32
  // FP32 plans whose LPs share A: every distinct block of A (offset, m, n)
  // rounded to FP32 once per execute, rows padded to the single-CTA tableau
  // row (a32_pitch) so that the loader takes a block in one bulk copy;
  // d_blk holds offA, off32, m, n per block
  float* d_A32 = nullptr;
  int64_t* d_blk = nullptr;
  int nblk = 0;
  int max_blk_rows = 0;
  double* d_lu = nullptr;    // LU refresh scratch of every class (FP32, FP64 steepest edge)
  size_t lu_doubles = 0;
  // FP32 plans: the FP64 pass, one persistent FP64 launch over the LPs the
  // FP32 pass hands over (d_fb: [0] count, [1..] LP ids), usually none
  bool has_fb = false;
  blpg::ClassPlan fb_class;
  int32_t* d_fb = nullptr;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev_in = nullptr, ev_out = nullptr, ev_fork = nullptr;
  std::vector<cudaStream_t> aux;      // one per class after the first
  std::vector<cudaEvent_t> ev_join;
  cudaGraphExec_t gexec = nullptr;
  blpg::LpArgs graph_args{};
  int launches = 0;
  int sm_count = 0;
  int smem_per_sm = 0, smem_reserved = 0, regs_per_sm = 0, threads_per_sm = 0;
};

namespace blpg {

static void release(blpg_plan* p) {
  if (!p) return;
  if (p->gexec) cudaGraphExecDestroy(p->gexec);
  cudaFree(p->d_m);
  cudaFree(p->d_n);
  cudaFree(p->d_order);
  cudaFree(p->d_tickets);
  cudaFree(p->d_off);
  cudaFree(p->d_A32);
  cudaFree(p->d_blk);
  cudaFree(p->d_lu);
  cudaFree(p->d_fb);
  if (p->ev_in) cudaEventDestroy(p->ev_in);
  if (p->ev_out) cudaEventDestroy(p->ev_out);
  if (p->ev_fork) cudaEventDestroy(p->ev_fork);
  for (auto e : p->ev_join) cudaEventDestroy(e);
  for (auto st : p->aux) cudaStreamDestroy(st);
  if (p->stream) cudaStreamDestroy(p->stream);
}

template <typename T, bool CL>
static int set_kernel_attrs(int max_smem) {
  cudaError_t e = cudaFuncSetAttribute(dev::solve_kernel<T, CL>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem);
  if (e != cudaSuccess)
    return fail(BLPG_ECUDA, "cudaFuncSetAttribute: %s", cudaGetErrorString(e));
  if (CL) {
    e = cudaFuncSetAttribute(dev::solve_kernel<T, CL>,
                             cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess)
      return fail(BLPG_ECUDA, "cluster attribute: %s", cudaGetErrorString(e));
  }
  return BLPG_OK;
}

template <typename T>
static int occupancy(const ClassPlan& c, int* ctas_per_sm, int* clusters) {
  *ctas_per_sm = 0;
  *clusters = 0;
  if (c.K == 1) {
    if (sizeof(T) == 4 && c.part) {
      CK(part_occupancy(ctas_per_sm, c.nt, c.smem));
    } else {
      CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas_per_sm,
                                                       dev::solve_kernel<T, false>, c.nt,
                                                       c.smem));
    }
  } else {
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = c.K;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(c.K, 1, 1);
    cfg.blockDim = dim3(c.nt, 1, 1);
    cfg.dynamicSmemBytes = c.smem;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    CK(cudaOccupancyMaxActiveClusters(clusters, dev::solve_kernel<T, true>, &cfg));
  }
  return BLPG_OK;
}

constexpr int kMaxThreads = 512;  // __launch_bounds__ of solve_kernel

template <typename T>
static int kernel_regs(bool cluster) {
  cudaFuncAttributes fa{};
  cudaError_t e = cluster ? cudaFuncGetAttributes(&fa, dev::solve_kernel<T, true>)
                          : cudaFuncGetAttributes(&fa, dev::solve_kernel<T, false>);
  return e == cudaSuccess && fa.numRegs > 0 ? fa.numRegs : 128;
}

static int tuning_value(int key0, int key1, int dflt) {
  std::lock_guard<std::mutex> lk(g_tuning.mu);
  if (!g_tuning.loaded) {
    parse_tuning_locked(kDefaultTuning);
    g_tuning.loaded = true;
  }
  auto it = g_tuning.threads.find({key0, key1});
  return it != g_tuning.threads.end() ? it->second : dflt;
}

// Threads per CTA for a class whose widest member has nl vector lanes per
// row and whose layout takes smem bytes: first the CTAs per SM (as many as
// shared memory admits, or the tuning table's "fpXX_ctas" target), then the
// most threads -- whole rows of lanes, at most the tuning table's threads
// per CTA (default 512) -- whose registers keep that many CTAs resident.
// Fewer CTAs per SM when a row of lanes does not fit otherwise.
static int pick_threads(const blpg_plan* p, int nl, int smem, int regs, int K, int key,
                        int override_nt, int* ctas_out) {
  const int by_smem = std::max(1, p->smem_per_sm / (smem + p->smem_reserved));
  int target = tuning_value(p->precision * 16 + 12, 1000 + key, 0);  // this class's
  if (target <= 0) target = tuning_value(p->precision * 16 + 14, 2, 0);  // every class's
  target = target > 0 ? std::min(target, by_smem) : by_smem;
  const int regs_alloc = dev::round_up(std::max(regs, 1), 8);
  if (override_nt > 0) {  // explicit threads per CTA: residency follows from it
    *ctas_out = 0;
    return std::min(dev::round_up(std::max(override_nt, nl), 32), kMaxThreads);
  }
  int want = tuning_value(p->precision * 16 + 13, 1000 + key, 0);  // this class's
  if (want <= 0) want = tuning_value(p->precision * 16 + K, 0, 512);
  for (int ctas = target; ctas >= 1; --ctas) {
    int cap = std::min(kMaxThreads, (p->regs_per_sm / ctas) / (regs_alloc * 32) * 32);
    cap = std::min(cap, p->threads_per_sm / ctas / 32 * 32);
    if (cap < nl && ctas > 1) continue;
    cap = std::max(cap, dev::round_up(nl, 32));
    int G = std::max(1, std::min(want, cap) / nl);
    int nt = dev::round_up(G * nl, 32);
    while (nt > cap && G > 1) nt = dev::round_up(--G * nl, 32);
    *ctas_out = ctas;
    return std::min(nt, kMaxThreads);
  }
  *ctas_out = 1;
  return std::min(dev::round_up(nl, 32), kMaxThreads);
}

// Size classes.  Every LP gets the smallest cluster size K whose layout fits
// the CTA shared-memory budget (default: the whole per-CTA shared memory,
// i.e. the fewest CTAs per LP).  LPs that need a cluster form one class per
// K; single-CTA LPs are grouped by how many CTAs of their own layout fit an
// SM (1..16, capped by the tuning table's "fpXX_ctas"), so small LPs run
// many per SM.  A CTA lays out each LP it takes in its own allocation, so a
// class needs only its largest member's layout and never splits.  Every
// class is launched with a full-residency grid, heaviest LPs first: the
// classes overlap on the GPU as earlier classes' persistent CTAs run out of
// work, which balances them without a work estimate.
template <typename T>
static int build_classes(blpg_plan* p, int max_smem, int max_cluster) {
  constexpr int V = dev::VecT<T>::V;
  const int elem = (int)sizeof(T);
  int budget = p->opt.cta_smem_budget;
  if (budget <= 0) budget = tuning_value(p->precision * 16 + 15, 1, max_smem);
  budget = std::min(budget, max_smem);
  const int se = p->opt.pricing == BLPG_PRICE_STEEPEST ? 1 : 0;
  const int min_cluster = std::max(1, std::min(p->opt.min_cluster, max_cluster));
  constexpr int kMaxCtasPerSm = 16;
  // default cap, from the autotuner on the uneven workload (GB300): FP64 small
  // LPs are bound by the FP64 pipe, so more than 4 CTAs per SM only lengthen
  // each LP (4 is 5 % faster than 16); FP32 gains up to 16
  const int cps_default = p->precision == BLPG_FP64 ? 4 : kMaxCtasPerSm;
  const int cps_cap =
      std::max(1, std::min(kMaxCtasPerSm, tuning_value(p->precision * 16 + 14, 2, cps_default)));
  auto cta_limit = [&](int cps) {  // per-CTA shared memory for cps CTAs per SM
    return std::min(max_smem, p->smem_per_sm / cps - p->smem_reserved);
  };
  struct Item {
    int K, nl, bytes;
    double work;
  };
  std::vector<Item> items(p->count);
  for (int k = 0; k < p->count; ++k) {
    const int m = p->m[k], n = p->n[k], na = p->na[k];
    int chosen = 0;
    for (int pass = 0; pass < 2 && !chosen; ++pass) {
      const int lim = pass == 0 ? budget : max_smem;
      for (int K = min_cluster; K <= max_cluster; K *= 2) {
        Geom g(m, n, na, K, V);
        const int bytes = Layout(m, g.ldw, n + m + na, elem, se).total;
        if (bytes <= lim && g.nl <= kMaxThreads) {
          chosen = K;
          items[k] = {K, g.nl, bytes, (double)(m + 1) * (double)(n + na + 1) * (double)(m + n)};
          break;
        }
      }
    }
    if (!chosen)
      return fail(BLPG_ETOOBIG,
                  "LP %d (m=%d, n=%d) needs more than %d CTAs of shared memory", k, m,
                  n, max_cluster);
  }
  std::map<int, std::vector<int>> groups;  // key: 100 + K for clusters, else CTAs per SM
  for (int k = 0; k < p->count; ++k) {
    int key = 100 + items[k].K;
    if (items[k].K == 1) {
      int cps = std::max(1, std::min(cps_cap, p->smem_per_sm / (items[k].bytes + p->smem_reserved)));
      while (cps > 1 && items[k].bytes > cta_limit(cps)) --cps;
      key = cps;
    }
    groups[key].push_back(k);
  }
  p->classes.clear();
  p->order.clear();
  std::vector<std::pair<ClassPlan, std::vector<int>>> built;
  for (auto& kv : groups) {
    auto& lps = kv.second;
    std::stable_sort(lps.begin(), lps.end(),
                     [&](int a, int b) { return items[a].work > items[b].work; });
    ClassPlan c;
    c.K = kv.first < 100 ? 1 : kv.first - 100;
    c.key = kv.first;
    int nl = 1;
    for (int lp : lps) {
      c.smem = std::max(c.smem, items[lp].bytes);
      c.max_m = std::max(c.max_m, p->m[lp]);
      c.max_na = std::max(c.max_na, p->na[lp]);
      c.max_ns = std::max(c.max_ns, std::min(p->m[lp], p->n[lp]));
      c.work += items[lp].work;
      nl = std::max(nl, items[lp].nl);
    }
    // threads: every member's row of vector lanes at least once
    c.nt = pick_threads(p, nl, c.smem, kernel_regs<T>(c.K > 1), c.K, c.key,
                        p->opt.threads_per_cta, &c.ctas_per_sm);
    c.count = (int)lps.size();
    int per_sm = 0, clusters = 0;
    int rc = occupancy<T>(c, &per_sm, &clusters);
    if (rc) return rc;
    // FP32 steepest edge on one CTA: when some member's norm partial sums (a
    // row per row group of this class's thread count) do not fit the region
    // its layout has, the class takes the kernel whose layouts grow that
    // region, if that costs no residency
    if (elem == 4 && se && c.K == 1) {
      ClassPlan cp = c;
      cp.part = 1;
      for (int lp : lps) {
        const int m = p->m[lp], n = p->n[lp], na = p->na[lp];
        const Geom g(m, n, na, 1, V);
        const int pb = std::min(c.nt / g.nl, dev::kMaxNormGroups) * g.cw * 4;
        cp.smem = std::max(cp.smem, Layout(m, g.ldw, n + m + na, elem, se, pb).total);
      }
      int per_sm2 = 0, clusters2 = 0;
      if (cp.smem > c.smem && cp.smem <= max_smem &&
          occupancy<T>(cp, &per_sm2, &clusters2) == BLPG_OK && per_sm2 >= per_sm) {
        c.smem = cp.smem;
        c.part = 1;
      }
    }
    const int slots = c.K == 1 ? per_sm * p->sm_count : clusters;
    if (slots <= 0)
      return fail(BLPG_ETOOBIG, "class K=%d nt=%d smem=%d cannot be resident", c.K, c.nt,
                  c.smem);
    if (c.K == 1) c.ctas_per_sm = per_sm;
    c.grid = std::min(slots, c.count) * c.K;  // full residency (persistent CTAs)
    built.emplace_back(c, lps);
  }
  // heaviest LPs first: clusters by size, then single-CTA classes by layout
  std::stable_sort(built.begin(), built.end(), [](const auto& a, const auto& b) {
    if (a.first.K != b.first.K) return a.first.K > b.first.K;
    return a.first.smem > b.first.smem;
  });
  for (auto& cb : built) {
    ClassPlan c = cb.first;
    c.order_off = (int)p->order.size();
    p->order.insert(p->order.end(), cb.second.begin(), cb.second.end());
    p->classes.push_back(c);
  }
  return BLPG_OK;
}

template <typename T>
static int launch_one(blpg_plan* p, size_t ci, const LpArgs& args, cudaStream_t s) {
  const ClassPlan& c = p->classes[ci];
  ClassArgs ca{};
  ca.order = p->d_order + c.order_off;
  ca.count = c.count;
  ca.ticket = p->d_tickets + ci;
  ca.K = c.K;
  ca.max_na = c.max_na;
  ca.se = p->opt.pricing == BLPG_PRICE_STEEPEST ? 1 : 0;
  ca.smem = c.smem;
  ca.lu = p->d_lu ? p->d_lu + c.lu_off : nullptr;
  ca.lu_stride = c.lu_stride;
  if (c.K == 1) {
    if (sizeof(T) == 4 && c.part) {
      CK(part_launch(c.grid, c.nt, c.smem, s, args, ca));
    } else {
      dev::solve_kernel<T, false><<<c.grid, c.nt, c.smem, s>>>(args, ca);
    }
    CK(cudaGetLastError());
  } else {
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = c.K;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(c.grid, 1, 1);
    cfg.blockDim = dim3(c.nt, 1, 1);
    cfg.dynamicSmemBytes = c.smem;
    cfg.stream = s;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    CK(cudaLaunchKernelEx(&cfg, dev::solve_kernel<T, true>, args, ca));
  }
  return BLPG_OK;
}

// The FP64 pass of an FP32 plan: one class holding every LP of the plan in
// the FP64 Dantzig layout (the reference's method, no LU verification), at
// the smallest cluster size where the largest fits, launched after the FP32
// classes over the device list they fill.  Returns false (no FP64 pass) when
// some LP needs more than 8 CTAs in FP64.
static bool build_fallback(blpg_plan* p, int max_smem) {
  ClassPlan c;
  for (int K = 1; K <= 8 && !c.smem; K *= 2) {
    int smem = 0, nl = 1, max_na = 0;
    bool fits = true;
    for (int k = 0; k < p->count && fits; ++k) {
      const int m = p->m[k], n = p->n[k], na = p->na[k];
      Geom g(m, n, na, K, dev::VecT<double>::V);
      const int bytes = Layout(m, g.ldw, n + m + na, 8, 0).total;
      fits = bytes <= max_smem && g.nl <= kMaxThreads;
      smem = std::max(smem, bytes);
      nl = std::max(nl, g.nl);
      max_na = std::max(max_na, na);
    }
    if (!fits) continue;
    c.K = K;
    c.smem = smem;
    c.max_na = max_na;
    c.nt = std::min(kMaxThreads, dev::round_up(std::max(nl, 256), 32));
  }
  if (!c.smem) return false;
  int per_sm = 0, clusters = 0;
  if (occupancy<double>(c, &per_sm, &clusters) != BLPG_OK) return false;
  const int slots = c.K == 1 ? per_sm * p->sm_count : clusters;
  if (slots <= 0) return false;
  c.ctas_per_sm = c.K == 1 ? per_sm : 1;
  c.grid = std::min({slots, std::max(1, p->count), 2 * p->sm_count}) * c.K;
  p->fb_class = c;
  return true;
}

static int launch_fallback(blpg_plan* p, const LpArgs& args, cudaStream_t s) {
  const ClassPlan& c = p->fb_class;
  LpArgs fa = args;
  fa.opt_tol = 1e-9;
  fa.piv_tol = 1e-7;
  fa.feas_tol = 1e-9;
  fa.phase1_tol = 1e-7;
  fa.deg_tol = 1e-12;
  fa.ptol = 1e-9;
  fa.pricing = 0;
  fa.weight = nullptr;
  fa.A32 = nullptr;
  fa.hint = nullptr;
  fa.refresh_period = 0;
  fa.fb = nullptr;
  fa.info_or = dev::kInfoFp64;
  ClassArgs ca{};
  ca.order = p->d_fb + 1;
  ca.count = 0;
  ca.count_dev = p->d_fb;
  ca.ticket = p->d_tickets + p->classes.size();
  ca.K = c.K;
  ca.max_na = c.max_na;
  ca.se = 0;
  ca.smem = c.smem;
  ca.lu = nullptr;
  if (c.K == 1) {
    dev::solve_kernel<double, false><<<c.grid, c.nt, c.smem, s>>>(fa, ca);
    CK(cudaGetLastError());
  } else {
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = c.K;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(c.grid, 1, 1);
    cfg.blockDim = dim3(c.nt, 1, 1);
    cfg.dynamicSmemBytes = c.smem;
    cfg.stream = s;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    CK(cudaLaunchKernelEx(&cfg, dev::solve_kernel<double, true>, fa, ca));
  }
  return BLPG_OK;
}

// Queue reset, then every class on its own stream (fork/join through
// events, so a captured graph has one parallel branch per class).
// A rounded to FP32 for FP32 tableau loads: every distinct block of A (blk:
// offA, off32, m, n), the same rounding as the in-kernel loader's
// (f64_to_f32_rn), rows padded with zeros to a32_pitch(n) elements.  A
// warp per row (blocks along y, rows along x, grid-stride), reads and writes
// coalesced along the row: one pass at HBM speed.
__global__ void round_a32_kernel(const double* __restrict__ A, float* __restrict__ A32,
                                 const long long* __restrict__ blk, int nblk) {
  const int lane = threadIdx.x & 31;
  const int wpb = blockDim.x >> 5;
  for (int bk = blockIdx.y; bk < nblk; bk += gridDim.y) {
    const long long offA = blk[4 * bk], off32 = blk[4 * bk + 1];
    const int m = (int)blk[4 * bk + 2], n = (int)blk[4 * bk + 3], ld = dev::a32_pitch(n);
    for (int i = blockIdx.x * wpb + (threadIdx.x >> 5); i < m; i += gridDim.x * wpb) {
      const double* src = A + offA + (long long)i * n;
      float* dst = A32 + off32 + (long long)i * ld;
      for (int j = lane; j < ld; j += 32) dst[j] = j < n ? dev::f64_to_f32_rn(__ldg(src + j)) : 0.f;
    }
  }
}

// The same rounding over a plain array, or CUDA's conversion instruction
// (__double2float_rn) for comparison (blpg_round_f32).
__global__ void round_f32_kernel(const double* __restrict__ in, float* __restrict__ out,
                                 long long n, int cuda_rn) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += stride)
    out[e] = cuda_rn ? __double2float_rn(in[e]) : dev::f64_to_f32_rn(in[e]);
}

template <typename T>
static int launch_classes(blpg_plan* p, const LpArgs& args, cudaStream_t s) {
  CK(cudaMemsetAsync(p->d_tickets, 0, sizeof(int32_t) * (p->classes.size() + 1), s));
  if (args.fb) CK(cudaMemsetAsync(args.fb, 0, sizeof(int32_t), s));
  const size_t nc = p->classes.size();
  if (nc == 0) return BLPG_OK;
  if (args.A32) {  // A rounded to FP32 before any class loads a tableau
    const int gx = std::max(1, std::min(dev::ceil_div(p->max_blk_rows, 8), 64));
    const int gy = std::max(1, std::min(p->nblk, 8 * std::max(1, p->sm_count) / gx + 1));
    round_a32_kernel<<<dim3(gx, gy), 256, 0, s>>>(args.A, const_cast<float*>(args.A32),
                                                  reinterpret_cast<const long long*>(p->d_blk),
                                                  p->nblk);
    CK(cudaGetLastError());
  }
  CK(cudaEventRecord(p->ev_fork, s));
  for (size_t ci = 1; ci < nc; ++ci) CK(cudaStreamWaitEvent(p->aux[ci - 1], p->ev_fork, 0));
  for (size_t ci = 0; ci < nc; ++ci) {
    int rc = launch_one<T>(p, ci, args, ci == 0 ? s : p->aux[ci - 1]);
    if (rc) return rc;
  }
  for (size_t ci = 1; ci < nc; ++ci) {
    CK(cudaEventRecord(p->ev_join[ci - 1], p->aux[ci - 1]));
    CK(cudaStreamWaitEvent(s, p->ev_join[ci - 1], 0));
  }
  if (args.fb) return launch_fallback(p, args, s);  // after every FP32 class
  return BLPG_OK;
}

static int launch_all(blpg_plan* p, const LpArgs& args, cudaStream_t s) {
  return p->precision == BLPG_FP32 ? launch_classes<float>(p, args, s)
                                   : launch_classes<double>(p, args, s);
}

static bool same_args(const LpArgs& a, const LpArgs& b) {
  return std::memcmp(&a, &b, sizeof(LpArgs)) == 0;
}

}  // namespace blpg

using namespace blpg;

extern "C" void blpg_options_init(blpg_options* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->precision = BLPG_FP64;
  o->use_graph = 1;
  o->max_cluster = 8;
}

extern "C" const char* blpg_last_error(void) { return g_err.c_str(); }

extern "C" const char* blpg_version(void) {
  return "blpg-gb300 1.0 (sm_103a; abi 1)";
}

namespace blpg {
static void parse_tuning_locked(const char* json) {
  g_tuning.threads.clear();
  if (!json) return;
  const char* s = json;
  while ((s = std::strchr(s, '"'))) {
    const char* e = std::strchr(s + 1, '"');
    if (!e) break;
    std::string key(s + 1, e - s - 1);
    const char* colon = std::strchr(e, ':');
    if (!colon) break;
    const char* v = colon + 1;
    while (*v == ' ' || *v == '\n' || *v == '\t') ++v;
    if (*v == '{' || *v == '[') {  // nested data ("measured"): skip the key
      s = e + 1;
      continue;
    }
    const int val = std::atoi(v);
    int bits = 0, K = 0, cls = 0;
    char tail[16] = {0};
    int prec = -1;
    if (std::sscanf(key.c_str(), "fp%d_", &bits) == 1) prec = bits == 64 ? BLPG_FP64 : (bits == 32 ? BLPG_FP32 : -1);
    if (prec >= 0) {
      const char* rest = key.c_str() + 5;
      if (std::sscanf(rest, "k%d%15s", &K, tail) == 1 && val > 0 && val <= 1024)
        g_tuning.threads[{prec * 16 + K, 0}] = val;
      else if (std::sscanf(rest, "c%d%15s", &cls, tail) == 2 && std::strcmp(tail, "_ctas") == 0 &&
               val > 0)
        g_tuning.threads[{prec * 16 + 12, 1000 + cls}] = val;
      else if (std::sscanf(rest, "c%d%15s", &cls, tail) == 1 && val > 0 && val <= 1024)
        g_tuning.threads[{prec * 16 + 13, 1000 + cls}] = val;
      else if (std::strcmp(rest, "smem") == 0 && val > 0)
        g_tuning.threads[{prec * 16 + 15, 1}] = val;
      else if (std::strcmp(rest, "ctas") == 0 && val > 0)
        g_tuning.threads[{prec * 16 + 14, 2}] = val;
      else if (std::strcmp(rest, "refresh_period") == 0 && val >= 0)
        g_tuning.threads[{prec * 16 + 11, 3}] = val;
    } else if (key == "overlap_mb" && val > 0) {
      g_tuning.threads[{-1, 1}] = val;
    } else if (key == "device_budget_mb" && val > 0) {
      g_tuning.threads[{-1, 2}] = val;
    } else if (key == "overlap_chunks" && val > 1) {
      g_tuning.threads[{-1, 3}] = val;
    } else if (key == "overlap_order" && val >= 0 && val <= 2) {
      g_tuning.threads[{-1, 4}] = val;
    }
    s = colon + 1;
  }
}
}  // namespace blpg

extern "C" int32_t blpg_set_tuning(const char* json) {
  std::lock_guard<std::mutex> lk(g_tuning.mu);
  parse_tuning_locked(json ? json : kDefaultTuning);
  g_tuning.loaded = true;
  ++g_tuning.generation;
  return BLPG_OK;
}

extern "C" int32_t blpg_plan_create(const blpg_batch* bt, const blpg_options* opt_in,
                                    blpg_plan** out) {
  if (!bt || !out || bt->count < 0 || (bt->count > 0 && (!bt->m || !bt->n)))
    return fail(BLPG_EINVAL, "blpg_plan_create: null batch, shapes or output");
  *out = nullptr;
  blpg_options opt;
  if (opt_in)
    opt = *opt_in;
  else
    blpg_options_init(&opt);
  if (opt.precision != BLPG_FP64 && opt.precision != BLPG_FP32)
    return fail(BLPG_EINVAL, "unknown precision %d", opt.precision);
  if (opt.max_cluster <= 0) opt.max_cluster = 8;
  if (opt.max_cluster > 8) opt.max_cluster = 8;
  cudaDeviceProp prop;
  int rc = device_check(opt.device, &prop);
  if (rc) return rc;
  CK(cudaSetDevice(opt.device));
  std::unique_ptr<blpg_plan> p(new blpg_plan);
  p->device = opt.device;
  p->opt = opt;
  p->precision = opt.precision;
  p->count = bt->count;
  p->sm_count = prop.multiProcessorCount;
  p->smem_per_sm = (int)prop.sharedMemPerMultiprocessor;
  p->smem_reserved = (int)prop.reservedSharedMemPerBlock;
  p->regs_per_sm = prop.regsPerMultiprocessor;
  p->threads_per_sm = prop.maxThreadsPerMultiProcessor;
  const int N = bt->count;
  p->m.assign(bt->m, bt->m + N);
  p->n.assign(bt->n, bt->n + N);
  p->na.assign(N, 0);
  p->offA.resize(N);
  p->offb.resize(N);
  p->offc.resize(N);
  p->offx.resize(N);
  p->offbasis.resize(N);
  int64_t pa = 0, pb = 0, pc = 0, pbs = 0;
  for (int k = 0; k < N; ++k) {
    const int m = p->m[k], n = p->n[k];
    if (m < 1 || n < 1 || m > BLPG_MAX_ROWS || n + m + 1 > BLPG_MAX_COLS)
      return fail(BLPG_EINVAL, "LP %d: m=%d n=%d out of range", k, m, n);
    p->offA[k] = bt->off_A ? bt->off_A[k] : pa;
    p->offb[k] = bt->off_b ? bt->off_b[k] : pb;
    p->offc[k] = bt->off_c ? bt->off_c[k] : pc;
    p->offx[k] = p->offc[k];
    p->offbasis[k] = pbs;
    if (p->offA[k] < 0 || p->offb[k] < 0 || p->offc[k] < 0)
      return fail(BLPG_EINVAL, "LP %d: negative offset", k);
    pa += (int64_t)m * n;
    pb += m;
    pc += n;
    pbs += m;
    p->extA = std::max(p->extA, p->offA[k] + (int64_t)m * n);
    p->minA = k == 0 ? p->offA[k] : std::min(p->minA, p->offA[k]);
    p->extb = std::max(p->extb, p->offb[k] + m);
    p->extc = std::max(p->extc, p->offc[k] + n);
    if (bt->b) {
      int neg = 0;
      for (int i = 0; i < m; ++i) neg += bt->b[p->offb[k] + i] < 0.0 ? 1 : 0;
      p->na[k] = neg;
    }
  }
  p->extx = p->extc;
  p->extbasis = pbs;
  const int max_smem = (int)prop.sharedMemPerBlockOptin;
  if (p->precision == BLPG_FP32) {
    if ((rc = set_kernel_attrs<float, false>(max_smem))) return rc;
    {
      const cudaError_t e = part_set_attrs(max_smem);
      if (e != cudaSuccess)
        return fail(BLPG_ECUDA, "cudaFuncSetAttribute: %s", cudaGetErrorString(e));
    }
    if ((rc = set_kernel_attrs<float, true>(max_smem))) return rc;
    if ((rc = set_kernel_attrs<double, false>(max_smem))) return rc;  // the FP64 pass
    if ((rc = set_kernel_attrs<double, true>(max_smem))) return rc;
    rc = build_classes<float>(p.get(), max_smem, opt.max_cluster);
  } else {
    if ((rc = set_kernel_attrs<double, false>(max_smem))) return rc;
    if ((rc = set_kernel_attrs<double, true>(max_smem))) return rc;
    rc = build_classes<double>(p.get(), max_smem, opt.max_cluster);
  }
  if (rc) return rc;
  p->launches = (int)p->classes.size();
  // device copies of shapes, offsets and queues
  const size_t nc = std::max<size_t>(1, p->classes.size());
  auto fail_free = [&](int code) {
    release(p.get());
    return code;
  };
  cudaError_t e;
#define CKF(call)                                                                    \
  do {                                                                               \
    e = (call);                                                                      \
    if (e != cudaSuccess)                                                            \
      return fail_free(fail(e == cudaErrorMemoryAllocation ? BLPG_ENOMEM : BLPG_ECUDA, \
                            "%s: %s", #call, cudaGetErrorString(e)));                \
  } while (0)
  CKF(cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking));
  CKF(cudaEventCreateWithFlags(&p->ev_in, cudaEventDisableTiming));
  CKF(cudaEventCreateWithFlags(&p->ev_out, cudaEventDisableTiming));
  CKF(cudaEventCreateWithFlags(&p->ev_fork, cudaEventDisableTiming));
  for (size_t ci = 1; ci < p->classes.size(); ++ci) {
    cudaStream_t st;
    cudaEvent_t ev;
    CKF(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    p->aux.push_back(st);
    CKF(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    p->ev_join.push_back(ev);
  }
  const size_t Nn = std::max(1, N);
  CKF(cudaMalloc(&p->d_m, sizeof(int32_t) * Nn));
  CKF(cudaMalloc(&p->d_n, sizeof(int32_t) * Nn));
  CKF(cudaMalloc(&p->d_order, sizeof(int32_t) * Nn));
  CKF(cudaMalloc(&p->d_tickets, sizeof(int32_t) * (nc + 1)));  // + the FP64 pass's
  CKF(cudaMalloc(&p->d_off, sizeof(int64_t) * 7 * Nn));
  // FP32 tableaux load A from an FP32 copy rounded once per execute (one
  // bandwidth-bound pass) when LPs share A: every element of A's extent read
  // by two LPs or more on average.  With an A per LP the copy would be an
  // extra serial pass over all of A, and the loaders convert instead (their
  // conversion overlaps other CTAs' pivots).
  int64_t readA = 0;
  for (int k = 0; k < N; ++k) readA += (int64_t)p->m[k] * p->n[k];
  std::vector<int64_t> off32;
  if (p->precision == BLPG_FP32 && p->extA > p->minA && readA >= 2 * (p->extA - p->minA)) {
    std::map<std::tuple<int64_t, int, int>, int64_t> blocks;  // (offA, m, n) -> off32
    std::vector<int64_t> blk;
    off32.resize((size_t)N);
    int64_t acc = 0;
    for (int k = 0; k < N; ++k) {
      const auto key = std::make_tuple(p->offA[k], p->m[k], p->n[k]);
      auto it = blocks.find(key);
      if (it == blocks.end()) {
        it = blocks.emplace(key, acc).first;
        blk.insert(blk.end(), {p->offA[k], acc, (int64_t)p->m[k], (int64_t)p->n[k]});
        acc += (int64_t)p->m[k] * dev::a32_pitch(p->n[k]);
        p->max_blk_rows = std::max(p->max_blk_rows, p->m[k]);
      }
      off32[k] = it->second;
    }
    p->nblk = (int)blocks.size();
    CKF(cudaMalloc(&p->d_A32, sizeof(float) * (size_t)std::max<int64_t>(acc, 4)));
    CKF(cudaMalloc(&p->d_blk, sizeof(int64_t) * blk.size()));
    CKF(cudaMemcpy(p->d_blk, blk.data(), sizeof(int64_t) * blk.size(), cudaMemcpyHostToDevice));
    p->launches += 1;
  }
  if (p->precision == BLPG_FP32 && N > 0 && build_fallback(p.get(), max_smem)) {
    CKF(cudaMalloc(&p->d_fb, sizeof(int32_t) * (size_t)(N + 1)));
    p->has_fb = true;
    p->launches += 1;
  }
  // FP64 scratch of the LU refresh (FP32 plans, FP64 plans with steepest
  // edge): per persistent CTA (cluster) of a class, the kernel matrix of the
  // largest possible basis (min(m, n) structural basics), five vectors and
  // two per warp (the rebuild solves a column per warp), rounded to 32
  // doubles; plans whose scratch would pass 4 GiB refresh by iterative
  // refinement only
  if (p->precision == BLPG_FP32 || p->opt.pricing == BLPG_PRICE_STEEPEST) {
    size_t total = 0;
    for (auto& c : p->classes) {
      const long long ns = std::max(1, c.max_ns);
      c.lu_stride = (ns * ns + (5 + 2 * (kMaxThreads / 32)) * ns + 31) / 32 * 32;
      c.lu_off = (long long)total;
      total += (size_t)c.lu_stride * (size_t)(c.grid / std::max(1, c.K));
    }
    if (total > 0 && total * sizeof(double) <= (size_t(4) << 30)) {
      CKF(cudaMalloc(&p->d_lu, sizeof(double) * total));
      p->lu_doubles = total;
    }
  }
  if (N > 0) {
    std::vector<int64_t> off(7 * (size_t)N, 0);
    std::copy(p->offA.begin(), p->offA.end(), off.begin());
    std::copy(p->offb.begin(), p->offb.end(), off.begin() + N);
    std::copy(p->offc.begin(), p->offc.end(), off.begin() + 2 * N);
    std::copy(p->offx.begin(), p->offx.end(), off.begin() + 3 * N);
    std::copy(p->offbasis.begin(), p->offbasis.end(), off.begin() + 4 * N);
    int64_t acc = 0;  // steepest-edge weights: n + m per LP, packed
    for (int k = 0; k < N; ++k) {
      off[5 * (size_t)N + k] = acc;
      acc += p->n[k] + p->m[k];
    }
    p->extw = acc;
    CKF(cudaMemcpy(p->d_m, p->m.data(), sizeof(int32_t) * N, cudaMemcpyHostToDevice));
    CKF(cudaMemcpy(p->d_n, p->n.data(), sizeof(int32_t) * N, cudaMemcpyHostToDevice));
    CKF(cudaMemcpy(p->d_order, p->order.data(), sizeof(int32_t) * N,
                   cudaMemcpyHostToDevice));
    if (!off32.empty()) std::copy(off32.begin(), off32.end(), off.begin() + 6 * N);
    CKF(cudaMemcpy(p->d_off, off.data(), sizeof(int64_t) * 7 * N, cudaMemcpyHostToDevice));
  }
#undef CKF
  *out = p.release();
  return BLPG_OK;
}

extern "C" int32_t blpg_plan_execute(blpg_plan* p, const double* dA, const double* db,
                                     const double* dc, const int32_t* basis_hint,
                                     blpg_result* out, void* stream_v) {
  return blpg_plan_execute_weighted(p, dA, db, dc, basis_hint, nullptr, out, stream_v);
}

extern "C" int32_t blpg_plan_execute_weighted(blpg_plan* p, const double* dA, const double* db,
                                              const double* dc, const int32_t* basis_hint,
                                              const float* price_weight, blpg_result* out,
                                              void* stream_v) {
  if (!p || !out || !out->status || !out->objective)
    return fail(BLPG_EINVAL, "blpg_plan_execute: null plan or outputs");
  if (price_weight && p->opt.pricing != BLPG_PRICE_STEEPEST)
    return fail(BLPG_EINVAL, "blpg_plan_execute: pricing weights need steepest-edge pricing");
  if (p->count == 0) return BLPG_OK;
  if (!dA || !db || !dc) return fail(BLPG_EINVAL, "blpg_plan_execute: null A, b or c");
  CK(cudaSetDevice(p->device));
  cudaStream_t user = (cudaStream_t)stream_v;
  LpArgs a{};
  a.m = p->d_m;
  a.n = p->d_n;
  const int N = p->count;
  a.offA = p->d_off;
  a.offb = p->d_off + N;
  a.offc = p->d_off + 2 * N;
  a.offx = p->d_off + 3 * N;
  a.offbasis = p->d_off + 4 * N;
  a.offw = p->d_off + 5 * N;
  a.pricing = p->opt.pricing == BLPG_PRICE_STEEPEST ? 1 : 0;
  a.weight = price_weight;
  a.A = dA;
  a.A32 = p->d_A32;
  a.off32 = p->d_A32 ? p->d_off + 6 * N : nullptr;
  a.fb = p->has_fb ? p->d_fb : nullptr;
  a.b = db;
  a.c = dc;
  a.status = out->status;
  a.obj = out->objective;
  a.x = out->x;
  a.pivots = out->pivots;
  a.basis = out->basis;
  const bool fp32 = p->precision == BLPG_FP32;
  a.opt_tol = p->opt.opt_tol > 0 ? p->opt.opt_tol : (fp32 ? 1e-5 : 1e-9);
  a.piv_tol = p->opt.piv_tol > 0 ? p->opt.piv_tol : (fp32 ? 1e-5 : 1e-7);
  a.feas_tol = p->opt.feas_tol > 0 ? p->opt.feas_tol : (fp32 ? 1e-6 : 1e-9);
  a.phase1_tol = fp32 ? 1e-4 : 1e-7;
  a.deg_tol = fp32 ? 1e-7 : 1e-12;
  a.harris = p->opt.ratio_rule == 1 ? 0 : 1;
  a.ptol = fp32 ? 1e-7 : 1e-9;
  // 0: the tuning table's period ("fpXX_refresh_period", 0 = termination
  // only); negative: termination only
  a.refresh_period = p->opt.refactor_period > 0
                         ? p->opt.refactor_period
                         : (p->opt.refactor_period == 0 ? tuning_value(p->precision * 16 + 11, 3, 0)
                                                        : 0);
  a.hint = basis_hint;
  a.info = out->info;
  a.warm_mode = p->opt.warm_mode == 0 ? 1 : (p->opt.warm_mode == 2 ? 0 : 1);
  a.shift = 0.1;
  a.max_pivots = p->opt.max_pivots;
  a.bland_after = p->opt.bland_after > 0 ? p->opt.bland_after : 64;
  CK(cudaEventRecord(p->ev_in, user));
  CK(cudaStreamWaitEvent(p->stream, p->ev_in, 0));
  if (p->opt.use_graph) {
    if (!p->gexec || !same_args(a, p->graph_args)) {
      if (p->gexec) {
        cudaGraphExecDestroy(p->gexec);
        p->gexec = nullptr;
      }
      cudaGraph_t graph = nullptr;
      CK(cudaStreamBeginCapture(p->stream, cudaStreamCaptureModeThreadLocal));
      int rc = launch_all(p, a, p->stream);
      cudaError_t ec = cudaStreamEndCapture(p->stream, &graph);
      if (rc) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
      }
      if (ec != cudaSuccess)
        return fail(BLPG_ECUDA, "graph capture: %s", cudaGetErrorString(ec));
      cudaError_t ei = cudaGraphInstantiate(&p->gexec, graph, 0);
      cudaGraphDestroy(graph);
      if (ei != cudaSuccess)
        return fail(BLPG_ECUDA, "graph instantiate: %s", cudaGetErrorString(ei));
      p->graph_args = a;
    }
    CK(cudaGraphLaunch(p->gexec, p->stream));
  } else {
    int rc = launch_all(p, a, p->stream);
    if (rc) return rc;
  }
  CK(cudaEventRecord(p->ev_out, p->stream));
  CK(cudaStreamWaitEvent(user, p->ev_out, 0));
  return BLPG_OK;
}

extern "C" int32_t blpg_round_f32(const double* d_in, float* d_out, int64_t count, int32_t mode,
                                  void* stream) {
  if (count < 0 || (count > 0 && (!d_in || !d_out)) || (mode != 0 && mode != 1))
    return fail(BLPG_EINVAL, "blpg_round_f32: bad arguments");
  if (count == 0) return BLPG_OK;
  const int grid = (int)std::min<int64_t>((count + 255) / 256, 4096);
  round_f32_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(d_in, d_out, (long long)count, mode);
  CK(cudaGetLastError());
  return BLPG_OK;
}

extern "C" int32_t blpg_plan_num_classes(const blpg_plan* p) {
  return p ? (int32_t)p->classes.size() : fail(BLPG_EINVAL, "null plan");
}

extern "C" int32_t blpg_plan_class_info(const blpg_plan* p, int32_t cls, int32_t* cluster,
                                        int32_t* threads, int32_t* smem_bytes,
                                        int32_t* num_lps) {
  if (!p || cls < 0 || cls >= (int32_t)p->classes.size())
    return fail(BLPG_EINVAL, "blpg_plan_class_info: bad plan or class");
  const ClassPlan& c = p->classes[cls];
  if (cluster) *cluster = c.K;
  if (threads) *threads = c.nt;
  if (smem_bytes) *smem_bytes = c.smem;
  if (num_lps) *num_lps = c.count;
  return BLPG_OK;
}

extern "C" int32_t blpg_plan_class_residency(const blpg_plan* p, int32_t cls,
                                             int32_t* ctas_per_sm, int32_t* grid) {
  if (!p || cls < 0 || cls >= (int32_t)p->classes.size())
    return fail(BLPG_EINVAL, "blpg_plan_class_residency: bad plan or class");
  const ClassPlan& c = p->classes[cls];
  if (ctas_per_sm) *ctas_per_sm = c.ctas_per_sm;
  if (grid) *grid = c.grid;
  return BLPG_OK;
}

extern "C" int32_t blpg_plan_class_key(const blpg_plan* p, int32_t cls, int32_t* key,
                                       int32_t* lp_ids) {
  if (!p || cls < 0 || cls >= (int32_t)p->classes.size())
    return fail(BLPG_EINVAL, "blpg_plan_class_key: bad plan or class");
  const ClassPlan& c = p->classes[cls];
  if (key) *key = c.key;
  if (lp_ids) std::copy(p->order.begin() + c.order_off, p->order.begin() + c.order_off + c.count,
                        lp_ids);
  return BLPG_OK;
}

extern "C" int32_t blpg_plan_launches(const blpg_plan* p) {
  return p ? p->launches : fail(BLPG_EINVAL, "null plan");
}

extern "C" void blpg_plan_destroy(blpg_plan* p) {
  if (!p) return;
  cudaSetDevice(p->device);
  if (p->stream) cudaStreamSynchronize(p->stream);
  release(p);
  delete p;
}

// ---------------------------------------------------------------------------
// Synchronous host-buffer solve with a small plan cache and a grow-only
// device workspace (the reference allocated and freed device memory on every
// ComputeLP call, simplex.cu:589-596, :895, :958).
// ---------------------------------------------------------------------------
namespace blpg {
struct Workspace {
  std::mutex mu;
  int device = -1;
  void* buf = nullptr;
  size_t cap = 0;
  blpg_plan* plan = nullptr;
  std::vector<int32_t> key_shapes;  // m, n per LP
  std::vector<int32_t> key_negs;    // count of b_i < 0 per LP
  std::vector<int64_t> key_offs;
  blpg_options key_opt{};
  int key_tuning = -1;  // tuning generation the cached plan was built with
};

static int tuning_generation() {
  std::lock_guard<std::mutex> lk(g_tuning.mu);
  return g_tuning.generation;
}
static Workspace g_ws;

// The cached plan fits the batch's shapes, offsets and options (its
// negative-b counts are checked separately): its workspace layout then fits
// too, since that depends only on shapes and offsets.
// Options compared field by field (a memcmp would also compare the struct's
// padding, which a caller's copy need not preserve); the per-call data
// pointers basis_hint and price_weight are not part of the plan.
static bool same_plan_options(const blpg_options& a, const blpg_options& b) {
  return a.precision == b.precision && a.max_pivots == b.max_pivots &&
         a.bland_after == b.bland_after && a.refactor_period == b.refactor_period &&
         a.opt_tol == b.opt_tol && a.piv_tol == b.piv_tol && a.device == b.device &&
         a.use_graph == b.use_graph && a.threads_per_cta == b.threads_per_cta &&
         a.max_cluster == b.max_cluster && a.min_cluster == b.min_cluster &&
         a.cta_smem_budget == b.cta_smem_budget && a.ratio_rule == b.ratio_rule &&
         a.feas_tol == b.feas_tol && a.warm_mode == b.warm_mode && a.pricing == b.pricing;
}

static bool plan_layout_matches(const Workspace& w, const blpg_batch* bt, const blpg_options& o,
                                const std::vector<int32_t>& shapes,
                                const std::vector<int64_t>& offs) {
  return w.plan && same_plan_options(w.key_opt, o) && w.key_shapes == shapes &&
         w.key_offs == offs && w.plan->count == bt->count && w.key_tuning == tuning_generation();
}
}  // namespace blpg

// ---------------------------------------------------------------------------
// Chunked host-buffer solve.  A batch whose uploads are large is split into
// contiguous chunks of LPs with about equal A volume, each with its own plan
// and stream; the uploads run one chunk after another on one stream and each
// chunk starts solving as soon as its own data has landed, so that the
// uploads overlap the solves of the chunks before them (the reference
// overlaps its copies and kernels over N streams, simplex.cu:914-955).
//
// Two layouts on the device:
//  * mirror: one device copy of the caller's arrays, offsets as given; chunk
//    k uploads the part of A, b and c below the highest element its LPs read
//    that earlier chunks did not already upload (any offsets work: an LP
//    reading far ahead only makes its chunk wait longer);
//  * ring: a packed batch whose inputs and outputs exceed the device budget
//    takes turns in two regions sized for the largest chunk, each chunk
//    relocated to its region's start (a chunk waits until the one two before
//    it has downloaded its results), in place of the reference's host-side
//    split by device memory (GPU_Tester.cu:194-238, 284-354).
// ---------------------------------------------------------------------------
namespace blpg {

constexpr size_t kOverlapBytes = size_t(64) << 20;  // uploads above this are pipelined
constexpr int kOverlapChunks = 8;  // measured best of 3, 4 and 8 for FP32 on GB300
constexpr int kMaxChunks = 64;

struct ChunkCache {
  std::mutex mu;
  int device = -1;
  void* buf = nullptr;
  size_t cap = 0;
  std::vector<blpg_plan*> plans;
  std::vector<cudaEvent_t> done;    // per chunk: its downloads are enqueued
  std::vector<cudaEvent_t> landed;  // per chunk: its uploads are enqueued
  cudaStream_t up = nullptr;        // every chunk's uploads, in chunk order
  std::vector<int32_t> bounds;      // LP index of each chunk's start, then count
  std::vector<int32_t> key_shapes, key_negs;
  std::vector<int64_t> key_offs;
  blpg_options key_opt{};
  int key_tuning = -1, ring = -1;  // ring 0: mirror layout
  void clear() {
    for (auto* pl : plans) blpg_plan_destroy(pl);
    plans.clear();
    for (auto e : done) cudaEventDestroy(e);
    for (auto e : landed) cudaEventDestroy(e);
    done.clear();
    landed.clear();
  }
};
static ChunkCache g_chunks;
static std::atomic<int> g_last_chunks{0};  // chunks of the last blpg_solve_batch (1 = one plan)

// Chunk bounds with about equal A volume.
static std::vector<int32_t> chunk_bounds(const blpg_batch* bt, int chunks) {
  const int N = bt->count;
  int64_t total = 0;
  for (int k = 0; k < N; ++k) total += (int64_t)bt->m[k] * bt->n[k];
  std::vector<int32_t> bounds{0};
  int64_t acc = 0;
  for (int k = 0; k < N; ++k) {
    acc += (int64_t)bt->m[k] * bt->n[k];
    const int done_chunks = (int)bounds.size();
    if (done_chunks < chunks && acc * chunks >= total * done_chunks && k + 1 < N)
      bounds.push_back(k + 1);
  }
  bounds.push_back(N);
  return bounds;
}

// Returns BLPG_OK after solving, or 1 when the batch is not for this path.
static int32_t solve_chunked(const blpg_batch* bt, const blpg_options& opt, blpg_result* out,
                             const std::vector<int32_t>& shapes, const std::vector<int64_t>& offs) {
  const int N = bt->count;
  const bool packed = !bt->off_A && !bt->off_b && !bt->off_c;
  // absolute offsets (the packed prefix where an offset array is absent),
  // the packed prefixes of basis, hint and weights, and the highest element
  // of A, b and c that LPs 0..k-1 read
  std::vector<int64_t> oA(N), ob(N), oc(N), pB(N + 1, 0), pW(N + 1, 0);
  std::vector<int64_t> hA(N + 1, 0), hb(N + 1, 0), hc(N + 1, 0);
  {
    int64_t pa = 0, pbb = 0, pc = 0;
    for (int k = 0; k < N; ++k) {
      const int m = bt->m[k], n = bt->n[k];
      if (m < 0 || n < 0) return 1;
      oA[k] = bt->off_A ? bt->off_A[k] : pa;
      ob[k] = bt->off_b ? bt->off_b[k] : pbb;
      oc[k] = bt->off_c ? bt->off_c[k] : pc;
      if (oA[k] < 0 || ob[k] < 0 || oc[k] < 0) return 1;  // the one-plan path reports it
      pa += (int64_t)m * n;
      pbb += m;
      pc += n;
      pB[k + 1] = pB[k] + m;
      pW[k + 1] = pW[k] + m + n;
      hA[k + 1] = std::max(hA[k], oA[k] + (int64_t)m * n);
      hb[k + 1] = std::max(hb[k], ob[k] + m);
      hc[k + 1] = std::max(hc[k], oc[k] + n);
    }
  }
  const size_t h2d = sizeof(double) * (size_t)(hA[N] + hb[N] + hc[N]);
  size_t free_b = 0, total_b = 0;
  int ndev = 0;  // no usable device: the one-plan path reports it
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || opt.device < 0 || opt.device >= ndev) return 1;
  CK(cudaSetDevice(opt.device));
  std::lock_guard<std::mutex> lk(g_chunks.mu);
  ChunkCache& cc = g_chunks;
  CK(cudaMemGetInfo(&free_b, &total_b));
  if (cc.device == opt.device) free_b += cc.cap;  // this path's own buffer is reused
  // inputs and outputs may take half the free memory (the plans' own state
  // needs the rest); the tuning table's "device_budget_mb" lowers that and
  // "overlap_mb" sets the upload volume from which copies are pipelined
  size_t budget = free_b / 2;
  const int budget_mb = tuning_value(-1, 2, 0);
  if (budget_mb > 0) budget = std::min(budget, (size_t)budget_mb << 20);
  const size_t io = h2d * 5 / 4;
  const bool big = h2d >= ((size_t)tuning_value(-1, 1, (int)(kOverlapBytes >> 20)) << 20);
  const bool tight = packed && io > budget;  // only a packed batch can be relocated
  if (!big && !tight) return 1;
  int chunks = std::max(2, std::min(kMaxChunks, tuning_value(-1, 3, kOverlapChunks)));
  int ring = 0;
  if (tight) {  // two regions of at most half the budget each
    ring = 2;
    chunks = (int)std::min<size_t>(kMaxChunks, std::max<size_t>(chunks,
                                                                io / std::max<size_t>(1, budget / 2) + 1));
  }
  if (N < 2 * chunks) return 1;
  const bool hint = opt.basis_hint != nullptr, wt = opt.price_weight != nullptr;
  std::vector<int32_t> negs((size_t)N);
  for (int k = 0; k < N; ++k) {
    int neg = 0;
    for (int i = 0; i < bt->m[k]; ++i) neg += bt->b[ob[k] + i] < 0.0 ? 1 : 0;
    negs[k] = neg;
  }
  const bool reuse = !cc.plans.empty() && cc.key_shapes == shapes && cc.key_offs == offs &&
                     cc.key_negs == negs && same_plan_options(cc.key_opt, opt) &&
                     cc.key_tuning == tuning_generation() && cc.ring == ring &&
                     cc.device == opt.device;
  std::vector<int32_t> bounds = reuse ? cc.bounds : chunk_bounds(bt, chunks);
  chunks = (int)bounds.size() - 1;
  if (!reuse) {
    cc.clear();
    if (cc.device != opt.device && cc.buf) {  // the buffer is on another device
      cudaFree(cc.buf);
      cc.buf = nullptr;
      cc.cap = 0;
    }
    cc.ring = ring;
    for (int ch = 0; ch < chunks; ++ch) {
      const int lo = bounds[ch], hi = bounds[ch + 1];
      blpg_batch sub{hi - lo, bt->m + lo, bt->n + lo, nullptr, nullptr, nullptr,
                     bt->A, bt->b, bt->c};
      if (ring) {  // packed, from the chunk's first element
        sub.A = bt->A + oA[lo];
        sub.b = bt->b + ob[lo];
        sub.c = bt->c + oc[lo];
      } else {  // the caller's offsets into the mirror
        sub.off_A = oA.data() + lo;
        sub.off_b = ob.data() + lo;
        sub.off_c = oc.data() + lo;
      }
      blpg_plan* pl = nullptr;
      int32_t rc = blpg_plan_create(&sub, &opt, &pl);
      if (rc) {
        cc.clear();
        return rc;
      }
      cc.plans.push_back(pl);
    }
    for (int ch = 0; ch < chunks; ++ch) {
      cudaEvent_t e1, e2;
      CK(cudaEventCreateWithFlags(&e1, cudaEventDisableTiming));
      cc.done.push_back(e1);
      CK(cudaEventCreateWithFlags(&e2, cudaEventDisableTiming));
      cc.landed.push_back(e2);
    }
    if (cc.up) cudaStreamDestroy(cc.up);  // on the plans' device
    cc.up = nullptr;
    CK(cudaStreamCreateWithFlags(&cc.up, cudaStreamNonBlocking));
    cc.bounds = bounds;
    cc.key_shapes = shapes;
    cc.key_offs = offs;
    cc.key_negs = negs;
    cc.key_opt = opt;
    cc.key_tuning = tuning_generation();
    cc.device = opt.device;
  }
  // device regions: A | b | c | status | objective | x | pivots | info |
  // basis | hint | weights, 256-byte aligned; the mirror has one region for
  // the whole batch, the ring two sized for the largest chunk
  auto al = [](size_t v) { return (v + 255) & ~(size_t)255; };
  size_t sA = 0, sb = 0, sc = 0, sn = 0, sbs = 0, sw = 0;
  const int regions = ring ? ring : 1;
  if (ring) {
    for (int ch = 0; ch < chunks; ++ch) {
      const int lo = bounds[ch], hi = bounds[ch + 1];
      sA = std::max(sA, al(sizeof(double) * (size_t)(hA[hi] - oA[lo])));
      sb = std::max(sb, al(sizeof(double) * (size_t)(hb[hi] - ob[lo])));
      sc = std::max(sc, al(sizeof(double) * (size_t)(hc[hi] - oc[lo])));
      sn = std::max(sn, al(sizeof(double) * (size_t)(hi - lo)));
      sbs = std::max(sbs, al(sizeof(int32_t) * (size_t)(pB[hi] - pB[lo])));
      sw = std::max(sw, al(sizeof(float) * (size_t)(pW[hi] - pW[lo])));
    }
  } else {
    sA = al(sizeof(double) * (size_t)hA[N]);
    sb = al(sizeof(double) * (size_t)hb[N]);
    sc = al(sizeof(double) * (size_t)hc[N]);
    sn = al(sizeof(double) * (size_t)N);
    sbs = al(sizeof(int32_t) * (size_t)pB[N]);
    sw = al(sizeof(float) * (size_t)pW[N]);
  }
  const size_t region = sA + sb + sc + 4 * sn + sc + 2 * sbs + sw;
  const size_t need = region * (size_t)regions;
  if (cc.cap < need) {
    for (auto* pl : cc.plans) cudaStreamSynchronize(pl->stream);
    if (cc.buf) cudaFree(cc.buf);
    cc.buf = nullptr;
    cc.cap = 0;
    CK(cudaMalloc(&cc.buf, need));
    cc.cap = need;
  }
  struct Region {
    double *A, *b, *c, *obj, *x;
    int32_t *status, *pivots, *info, *basis, *hint;
    float* w;
  };
  auto region_at = [&](int r) {
    char* o = (char*)cc.buf + (size_t)r * region;
    Region g;
    g.A = (double*)o, o += sA;
    g.b = (double*)o, o += sb;
    g.c = (double*)o, o += sc;
    g.status = (int32_t*)o, o += sn;
    g.obj = (double*)o, o += sn;
    g.pivots = (int32_t*)o, o += sn;
    g.info = (int32_t*)o, o += sn;
    g.x = (double*)o, o += sc;
    g.basis = (int32_t*)o, o += sbs;
    g.hint = (int32_t*)o, o += sbs;
    g.w = (float*)o;
    return g;
  };
  // Per chunk: the device pointers its plan reads and writes, and the host
  // ranges its uploads and downloads cover (element offsets into the
  // caller's arrays, and into the region).
  std::vector<blpg_result> dres((size_t)chunks);
  int64_t upA = 0, upb = 0, upc = 0;  // mirror: elements uploaded so far
  auto download = [&](int ch) -> int32_t {
    blpg_plan* pl = cc.plans[ch];
    cudaStream_t s = pl->stream;
    const int lo = bounds[ch], hi = bounds[ch + 1], cn = hi - lo;
    const blpg_result& d = dres[ch];
    CK(cudaMemcpyAsync(out->status + lo, d.status, sizeof(int32_t) * cn, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(out->objective + lo, d.objective, sizeof(double) * cn,
                       cudaMemcpyDeviceToHost, s));
    if (out->pivots)
      CK(cudaMemcpyAsync(out->pivots + lo, d.pivots, sizeof(int32_t) * cn, cudaMemcpyDeviceToHost,
                         s));
    if (out->info)
      CK(cudaMemcpyAsync(out->info + lo, d.info, sizeof(int32_t) * cn, cudaMemcpyDeviceToHost, s));
    if (out->basis)
      CK(cudaMemcpyAsync(out->basis + pB[lo], d.basis,
                         sizeof(int32_t) * (size_t)(pB[hi] - pB[lo]), cudaMemcpyDeviceToHost, s));
    if (out->x) {  // x of LP k sits where its c does
      int64_t lo_c = oc[lo], hi_c = oc[lo];
      for (int k = lo; k < hi; ++k) {
        lo_c = std::min(lo_c, oc[k]);
        hi_c = std::max(hi_c, oc[k] + bt->n[k]);
      }
      const double* src = ring ? d.x + (lo_c - oc[lo]) : d.x + lo_c;
      CK(cudaMemcpyAsync(out->x + lo_c, src, sizeof(double) * (size_t)(hi_c - lo_c),
                         cudaMemcpyDeviceToHost, s));
    }
    CK(cudaEventRecord(cc.done[ch], s));
    return BLPG_OK;
  };
  // Downloads into pageable host memory block the calling thread until the
  // chunk is solved, so chunk j's downloads are enqueued only after the
  // uploads and solve of chunk j + lag have been (lag = ring - 1: the last
  // chunk that can start before chunk j's region is needed again; the
  // mirror enqueues every chunk first).
  std::vector<double*> dA((size_t)chunks), db((size_t)chunks), dc((size_t)chunks);
  std::vector<int32_t*> dhint((size_t)chunks, nullptr);
  std::vector<float*> dw((size_t)chunks, nullptr);
  auto upload = [&](int ch) -> int32_t {
    cudaStream_t u = cc.up;
    const int lo = bounds[ch], hi = bounds[ch + 1];
    const Region g = region_at(ring ? ch % ring : 0);
    if (ring && ch >= ring) CK(cudaStreamWaitEvent(u, cc.done[ch - ring], 0));
    blpg_result& d = dres[ch];
    d = blpg_result{};
    dA[ch] = g.A;
    db[ch] = g.b;
    dc[ch] = g.c;
    if (ring) {  // relocated to the region's start
      CK(cudaMemcpyAsync(g.A, bt->A + oA[lo], sizeof(double) * (size_t)(hA[hi] - oA[lo]),
                         cudaMemcpyHostToDevice, u));
      CK(cudaMemcpyAsync(g.b, bt->b + ob[lo], sizeof(double) * (size_t)(hb[hi] - ob[lo]),
                         cudaMemcpyHostToDevice, u));
      CK(cudaMemcpyAsync(g.c, bt->c + oc[lo], sizeof(double) * (size_t)(hc[hi] - oc[lo]),
                         cudaMemcpyHostToDevice, u));
      d.status = g.status;
      d.objective = g.obj;
      d.pivots = out->pivots ? g.pivots : nullptr;
      d.info = out->info ? g.info : nullptr;
      d.x = out->x ? g.x : nullptr;
      d.basis = out->basis ? g.basis : nullptr;
      dhint[ch] = hint ? g.hint : nullptr;
      dw[ch] = wt ? g.w : nullptr;
    } else {  // the mirror: whatever LPs lo..hi-1 read that is not there yet
      if (hA[hi] > upA)
        CK(cudaMemcpyAsync(g.A + upA, bt->A + upA, sizeof(double) * (size_t)(hA[hi] - upA),
                           cudaMemcpyHostToDevice, u));
      if (hb[hi] > upb)
        CK(cudaMemcpyAsync(g.b + upb, bt->b + upb, sizeof(double) * (size_t)(hb[hi] - upb),
                           cudaMemcpyHostToDevice, u));
      if (hc[hi] > upc)
        CK(cudaMemcpyAsync(g.c + upc, bt->c + upc, sizeof(double) * (size_t)(hc[hi] - upc),
                           cudaMemcpyHostToDevice, u));
      upA = std::max(upA, hA[hi]);
      upb = std::max(upb, hb[hi]);
      upc = std::max(upc, hc[hi]);
      d.status = g.status + lo;
      d.objective = g.obj + lo;
      d.pivots = out->pivots ? g.pivots + lo : nullptr;
      d.info = out->info ? g.info + lo : nullptr;
      d.x = out->x ? g.x : nullptr;  // written at the LPs' own c offsets
      d.basis = out->basis ? g.basis + pB[lo] : nullptr;
      dhint[ch] = hint ? g.hint + pB[lo] : nullptr;
      dw[ch] = wt ? g.w + pW[lo] : nullptr;
    }
    if (hint)
      CK(cudaMemcpyAsync(dhint[ch], opt.basis_hint + pB[lo],
                         sizeof(int32_t) * (size_t)(pB[hi] - pB[lo]), cudaMemcpyHostToDevice, u));
    if (wt)
      CK(cudaMemcpyAsync(dw[ch], opt.price_weight + pW[lo],
                         sizeof(float) * (size_t)(pW[hi] - pW[lo]), cudaMemcpyHostToDevice, u));
    CK(cudaEventRecord(cc.landed[ch], u));
    return BLPG_OK;
  };
  auto launch = [&](int ch) -> int32_t {
    cudaStream_t s = cc.plans[ch]->stream;
    CK(cudaStreamWaitEvent(s, cc.landed[ch], 0));
    return blpg_plan_execute_weighted(cc.plans[ch], dA[ch], db[ch], dc[ch], dhint[ch], dw[ch],
                                      &dres[ch], s);
  };
  // Enqueue order.  Uploads from pinned memory return at once: every upload
  // of the mirror is enqueued before any solve, so that no copy is queued in
  // a hardware channel behind a solve that waits for a later copy (with a
  // plan per chunk and a graph branch per size class, streams share the
  // device's few channels).  Uploads from pageable memory return only once
  // staged, so they alternate with the solves, each chunk's solve enqueued
  // as soon as its uploads are.  The ring alternates too: a region's next
  // upload waits for its previous chunk's downloads.
  cudaPointerAttributes pa{};
  const bool pinned = cudaPointerGetAttributes(&pa, bt->A) == cudaSuccess &&
                      pa.type == cudaMemoryTypeHost;
  cudaGetLastError();  // a pageable pointer may leave an error on older runtimes
  const int lag = ring ? ring - 1 : chunks - 1;
  int32_t rc = BLPG_OK;
  const int order = tuning_value(-1, 4, 0);  // 1: alternate, 2: uploads first, 0: by memory kind
  if (!ring && (order == 2 || (order == 0 && pinned))) {
    for (int ch = 0; ch < chunks; ++ch)
      if ((rc = upload(ch))) return rc;
    for (int ch = 0; ch < chunks; ++ch)
      if ((rc = launch(ch))) return rc;
    for (int ch = 0; ch < chunks; ++ch)
      if ((rc = download(ch))) return rc;
  } else {
    for (int ch = 0; ch < chunks; ++ch) {
      if ((rc = upload(ch)) || (rc = launch(ch))) return rc;
      if (ch - lag >= 0 && (rc = download(ch - lag))) return rc;
    }
    for (int ch = std::max(0, chunks - lag); ch < chunks; ++ch)
      if ((rc = download(ch))) return rc;
  }
  for (auto* pl : cc.plans) CK(cudaStreamSynchronize(pl->stream));
  CK(cudaStreamSynchronize(cc.up));
  CK(cudaGetLastError());
  g_last_chunks = chunks;
  return BLPG_OK;
}

}  // namespace blpg

extern "C" int32_t blpg_solve_batch_chunks(void) { return blpg::g_last_chunks.load(); }

extern "C" int32_t blpg_release_workspace(void) {
  using namespace blpg;
  {
    std::lock_guard<std::mutex> lk(g_ws.mu);
    if (g_ws.plan) blpg_plan_destroy(g_ws.plan);  // synchronises its stream
    g_ws.plan = nullptr;
    if (g_ws.buf) cudaFree(g_ws.buf);
    g_ws.buf = nullptr;
    g_ws.cap = 0;
    g_ws.key_shapes.clear();
    g_ws.key_negs.clear();
    g_ws.key_offs.clear();
  }
  {
    std::lock_guard<std::mutex> lk(g_chunks.mu);
    ChunkCache& cc = g_chunks;
    if (cc.up) cudaStreamSynchronize(cc.up);
    cc.clear();  // destroys the chunk plans (each synchronises its stream)
    if (cc.up) cudaStreamDestroy(cc.up);
    cc.up = nullptr;
    if (cc.buf) cudaFree(cc.buf);
    cc.buf = nullptr;
    cc.cap = 0;
    cc.ring = -1;
    cc.bounds.clear();
    cc.key_shapes.clear();
    cc.key_negs.clear();
    cc.key_offs.clear();
  }
  return BLPG_OK;
}

extern "C" int32_t blpg_solve_batch(const blpg_batch* bt, const blpg_options* opt_in,
                                    blpg_result* out) {
  if (!bt || !out || !out->status || !out->objective)
    return fail(BLPG_EINVAL, "blpg_solve_batch: null batch or outputs");
  if (bt->count < 0) return fail(BLPG_EINVAL, "blpg_solve_batch: negative count");
  if (bt->count == 0) return BLPG_OK;
  if (!bt->A || !bt->b || !bt->c || !bt->m || !bt->n)
    return fail(BLPG_EINVAL, "blpg_solve_batch: null A, b, c, m or n");
  blpg_options opt;
  if (opt_in)
    opt = *opt_in;
  else
    blpg_options_init(&opt);
  const int N = bt->count;
  // plan cache key: shapes, offsets and options, then the negative-b counts
  std::vector<int32_t> shapes(2 * (size_t)N);
  for (int k = 0; k < N; ++k) {
    shapes[2 * k] = bt->m[k];
    shapes[2 * k + 1] = bt->n[k];
  }
  std::vector<int64_t> offs;
  if (bt->off_A) offs.insert(offs.end(), bt->off_A, bt->off_A + N);
  if (bt->off_b) offs.insert(offs.end(), bt->off_b, bt->off_b + N);
  if (bt->off_c) offs.insert(offs.end(), bt->off_c, bt->off_c + N);
  offs.push_back(bt->off_A ? 1 : 0);
  offs.push_back(bt->off_b ? 2 : 0);
  offs.push_back(bt->off_c ? 4 : 0);
  auto count_negs = [&]() {
    std::vector<int32_t> negs((size_t)N);
    int64_t pb = 0;
    for (int k = 0; k < N; ++k) {
      const int64_t ob = bt->off_b ? bt->off_b[k] : pb;
      int neg = 0;
      for (int i = 0; i < bt->m[k]; ++i) neg += bt->b[ob + i] < 0.0 ? 1 : 0;
      negs[k] = neg;
      pb += bt->m[k] > 0 ? bt->m[k] : 0;
    }
    return negs;
  };

  const bool hint = opt.basis_hint != nullptr;
  const bool wt = opt.price_weight != nullptr;
  if (wt && opt.pricing != BLPG_PRICE_STEEPEST)
    return fail(BLPG_EINVAL, "blpg_solve_batch: pricing weights need steepest-edge pricing");
  {
    const int32_t rc0 = solve_chunked(bt, opt, out, shapes, offs);
    if (rc0 != 1) return rc0;  // solved in chunks (or failed there)
  }
  g_last_chunks = 1;
  std::lock_guard<std::mutex> lk(g_ws.mu);
  int rc;
  // workspace: A | b | c | status | obj | x | pivots | info | hint | weights
  // (256-byte aligned); its layout depends only on shapes and offsets
  auto al = [](size_t v) { return (v + 255) & ~(size_t)255; };
  struct Slots {
    double *A, *b, *c;
    blpg_result res;
    int32_t* hint;
    float* w;
  };
  auto carve = [&](blpg_plan* p, Slots& sl) -> int {
    const size_t sA = al(sizeof(double) * p->extA), sb = al(sizeof(double) * p->extb),
                 sc = al(sizeof(double) * p->extc), sst = al(sizeof(int32_t) * N),
                 sob = al(sizeof(double) * N), sx = al(sizeof(double) * p->extx),
                 spv = al(sizeof(int32_t) * N), sbs = al(sizeof(int32_t) * p->extbasis),
                 sw = al(sizeof(float) * p->extw);
    const size_t need = sA + sb + sc + sst + sob + (out->x ? sx : 0) +
                        (out->pivots ? spv : 0) + (out->basis ? sbs : 0) +
                        (out->info ? spv : 0) + (hint ? sbs : 0) + (wt ? sw : 0);
    if (g_ws.cap < need || g_ws.device != p->device) {
      if (g_ws.buf) cudaFree(g_ws.buf);
      g_ws.buf = nullptr;
      g_ws.cap = 0;
      CK(cudaMalloc(&g_ws.buf, need));
      g_ws.cap = need;
      g_ws.device = p->device;
    }
    char* o = (char*)g_ws.buf;
    sl = Slots{};
    sl.A = (double*)o;
    o += sA;
    sl.b = (double*)o;
    o += sb;
    sl.c = (double*)o;
    o += sc;
    sl.res.status = (int32_t*)o;
    o += sst;
    sl.res.objective = (double*)o;
    o += sob;
    if (out->x) sl.res.x = (double*)o, o += sx;
    if (out->pivots) sl.res.pivots = (int32_t*)o, o += spv;
    if (out->basis) sl.res.basis = (int32_t*)o, o += sbs;
    if (out->info) sl.res.info = (int32_t*)o, o += spv;
    if (hint) sl.hint = (int32_t*)o, o += sbs;
    if (wt) sl.w = (float*)o, o += sw;
    return BLPG_OK;
  };
  auto upload = [&](blpg_plan* p, const Slots& sl) -> int {
    cudaStream_t s = p->stream;
    if (hint)
      CK(cudaMemcpyAsync(sl.hint, opt.basis_hint, sizeof(int32_t) * p->extbasis,
                         cudaMemcpyHostToDevice, s));
    if (wt)
      CK(cudaMemcpyAsync(sl.w, opt.price_weight, sizeof(float) * p->extw,
                         cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(sl.A, bt->A, sizeof(double) * p->extA, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(sl.b, bt->b, sizeof(double) * p->extb, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(sl.c, bt->c, sizeof(double) * p->extc, cudaMemcpyHostToDevice, s));
    return BLPG_OK;
  };
  Slots sl{};
  bool uploaded = false;
  if (plan_layout_matches(g_ws, bt, opt, shapes, offs)) {
    // the cached plan's layout fits: the uploads start now and the host
    // counts negative b's while they run
    if ((rc = carve(g_ws.plan, sl)) || (rc = upload(g_ws.plan, sl))) return rc;
    uploaded = true;
  }
  std::vector<int32_t> negs = count_negs();
  if (!uploaded || negs != g_ws.key_negs) {
    if (g_ws.plan) {
      blpg_plan_destroy(g_ws.plan);  // synchronises its stream (the uploads land)
      g_ws.plan = nullptr;
    }
    if ((rc = blpg_plan_create(bt, &opt, &g_ws.plan))) return rc;
    g_ws.key_shapes = shapes;
    g_ws.key_negs = negs;
    g_ws.key_offs = offs;
    g_ws.key_opt = opt;
    g_ws.key_tuning = tuning_generation();
    if (!uploaded) {
      if ((rc = carve(g_ws.plan, sl)) || (rc = upload(g_ws.plan, sl))) return rc;
    }
  }
  blpg_plan* p = g_ws.plan;
  cudaStream_t s = p->stream;
  double* dA = sl.A;
  double* db = sl.b;
  double* dc = sl.c;
  blpg_result& dres = sl.res;
  int32_t* dhint = sl.hint;
  float* dw = sl.w;
  if ((rc = blpg_plan_execute_weighted(p, dA, db, dc, dhint, dw, &dres, s))) return rc;
  CK(cudaMemcpyAsync(out->status, dres.status, sizeof(int32_t) * N, cudaMemcpyDeviceToHost,
                     s));
  CK(cudaMemcpyAsync(out->objective, dres.objective, sizeof(double) * N,
                     cudaMemcpyDeviceToHost, s));
  if (out->x)
    CK(cudaMemcpyAsync(out->x, dres.x, sizeof(double) * p->extx, cudaMemcpyDeviceToHost, s));
  if (out->pivots)
    CK(cudaMemcpyAsync(out->pivots, dres.pivots, sizeof(int32_t) * N,
                       cudaMemcpyDeviceToHost, s));
  if (out->basis)
    CK(cudaMemcpyAsync(out->basis, dres.basis, sizeof(int32_t) * p->extbasis,
                       cudaMemcpyDeviceToHost, s));
  if (out->info)
    CK(cudaMemcpyAsync(out->info, dres.info, sizeof(int32_t) * N, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  CK(cudaGetLastError());
  return BLPG_OK;
}
