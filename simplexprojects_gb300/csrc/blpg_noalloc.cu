// blpg_solve_noalloc: a solve entry point that allocates no memory.
//
// Some callers cannot call cudaMalloc: code that runs inside a memory pool
// or arena it does not own, a host application that has handed all device
// memory to its own allocator, or a framework hook that is not allowed to
// allocate on its thread.  For them this entry point runs the same pivot
// kernel as blpg_plan_execute, but keeps the kernel's scratch (the work-queue
// ticket and the LP order it hands out) in a file-scope __device__ array
// instead of plan memory.  The caller still passes every input and output
// as device pointers.
//
// Limits and behaviour:
//  - at most kNoAllocMaxLps LPs per call; larger counts are rejected with
//    BLPG_EINVAL before any GPU work;
//  - the scratch array (about 1 MiB) lives in every GPU that loads the
//    library until the process exits;
//  - the first call on a device looks up the array's device address with
//    cudaGetSymbolAddress, reads the device's properties and sets the
//    kernels' shared-memory attribute, under a lock (two host threads making
//    their first call at once do the set-up once); make that first call
//    before any stream capture;
//  - every call reuses the same array: calls whose GPU work overlaps (two
//    streams, or two host threads) race on it and must be serialised by the
//    caller; each call resets the ticket and the order list before its solve;
//  - single-phase LPs only (b >= 0): an LP with b_i < 0, or larger than the
//    max_m / max_n bounds, is refused by the kernel (status BLPG_UNDEF,
//    pivots -1);
//  - no cudaMalloc, cudaFree, stream, event or graph is created.
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <cstring>
#include <mutex>

#include "blpg_internal.h"
#include "blpg_solver.cuh"

namespace {

constexpr int kNoAllocMaxLps = 1 << 18;  // 262,144 LPs per call
constexpr int kOrderOffset = 64;         // [0] ticket, [64..] LP order
constexpr int kMaxDevices = 64;

static __device__ __align__(256) int32_t g_noalloc_scratch[kOrderOffset + kNoAllocMaxLps];

// Zero the ticket and write the identity LP order for `count` LPs.
__global__ void noalloc_reset(int32_t* scratch, int32_t count) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid == 0) scratch[0] = 0;
  for (int i = tid; i < count; i += gridDim.x * blockDim.x) scratch[kOrderOffset + i] = i;
}

// Per-device set-up, done once with that device current.  No heap use.
// `ready` is published with release ordering after the other fields are
// written, so a caller that reads it as true (acquire) sees them.  The
// occupancy of the last launch shape per precision is cached as well, so a
// repeated call makes no device queries.
struct DevSetup {
  std::atomic<bool> ready;
  int32_t* scratch;
  int sm_count;
  int max_smem;
  std::mutex occ_mu;
  int occ_key[2][3];  // [precision] (K, threads, smem) of the cached entry
  int occ_val[2];     // CTAs per SM (K = 1) or clusters
};
static DevSetup g_setup[kMaxDevices];
static std::mutex g_setup_mu;

template <typename T>
int32_t setup_attrs(int max_smem) {
  using blpg::fail;
  cudaError_t e = cudaFuncSetAttribute(blpg::dev::solve_kernel<T, false>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(blpg::dev::solve_kernel<T, true>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem);
  if (e != cudaSuccess)
    return fail(BLPG_ECUDA, "blpg_solve_noalloc: cudaFuncSetAttribute: %s",
                cudaGetErrorString(e));
  return BLPG_OK;
}

// Occupancy of a launch shape (CTAs per SM for K = 1, else clusters),
// answered from the per-device cache when the shape repeats.
template <typename T>
cudaError_t occupancy(DevSetup& st, int K, int nt, int smem, int* out) {
  const int pi = sizeof(T) == 4 ? 1 : 0;
  {
    std::lock_guard<std::mutex> lk(st.occ_mu);
    if (st.occ_key[pi][0] == K && st.occ_key[pi][1] == nt && st.occ_key[pi][2] == smem) {
      *out = st.occ_val[pi];
      return cudaSuccess;
    }
  }
  using namespace blpg::dev;
  cudaError_t e;
  *out = 0;
  if (K == 1) {
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(out, solve_kernel<T, false>, nt, smem);
  } else {
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = K;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(K, 1, 1);
    cfg.blockDim = dim3(nt, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    e = cudaOccupancyMaxActiveClusters(out, solve_kernel<T, true>, &cfg);
  }
  if (e == cudaSuccess && *out > 0) {
    std::lock_guard<std::mutex> lk(st.occ_mu);
    st.occ_key[pi][0] = K;
    st.occ_key[pi][1] = nt;
    st.occ_key[pi][2] = smem;
    st.occ_val[pi] = *out;
  }
  return e;
}

template <typename T>
int32_t run(int32_t count, int32_t max_m, int32_t max_n, const blpg::dev::LpArgs& a,
            DevSetup& st, cudaStream_t s) {
  using blpg::fail;
  using namespace blpg::dev;
  constexpr int V = VecT<T>::V;
  int32_t* scratch = st.scratch;
  const int max_smem = st.max_smem;
  int K = 0, nt = 0, smem = 0;
  for (int k = 1; k <= 8; k *= 2) {
    Geom g(max_m, max_n, 0, k, V);
    Layout L(max_m, g.ldw, max_n + max_m, (int)sizeof(T));
    if (L.total <= max_smem && g.nl <= 512) {
      K = k;
      smem = L.total;
      int G = g.nl >= 256 ? 1 : 256 / g.nl;
      nt = round_up(G * g.nl, 32);
      if (nt > 512) nt = round_up(g.nl, 32);
      break;
    }
  }
  if (!K)
    return fail(BLPG_ETOOBIG, "blpg_solve_noalloc: m=%d n=%d exceeds an 8-CTA cluster", max_m,
                max_n);
  ClassArgs ca{};
  ca.order = scratch + kOrderOffset;
  ca.count = count;
  ca.ticket = scratch;
  ca.K = K;
  ca.max_na = 0;
  ca.se = 0;  // Dantzig pricing: no column norms
  ca.smem = smem;
  noalloc_reset<<<(count + 255) / 256 > 0 ? (count + 255) / 256 : 1, 256, 0, s>>>(scratch, count);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess)
    return fail(BLPG_ECUDA, "blpg_solve_noalloc: reset launch: %s", cudaGetErrorString(e));
  if (K == 1) {
    int per_sm = 0;
    e = occupancy<T>(st, 1, nt, smem, &per_sm);
    if (e != cudaSuccess || per_sm <= 0)
      return fail(BLPG_ECUDA, "blpg_solve_noalloc: occupancy query failed");
    int grid = per_sm * st.sm_count;
    if (grid > count) grid = count;
    solve_kernel<T, false><<<grid, nt, smem, s>>>(a, ca);
  } else {
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = K;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.blockDim = dim3(nt, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int clusters = 0;
    e = occupancy<T>(st, K, nt, smem, &clusters);
    if (e != cudaSuccess || clusters <= 0)
      return fail(BLPG_ECUDA, "blpg_solve_noalloc: cluster occupancy query failed");
    if (clusters > count) clusters = count;
    cfg.gridDim = dim3(clusters * K, 1, 1);
    cfg.stream = s;
    e = cudaLaunchKernelEx(&cfg, solve_kernel<T, true>, a, ca);
  }
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess)
    return fail(BLPG_ECUDA, "blpg_solve_noalloc: launch: %s", cudaGetErrorString(e));
  return BLPG_OK;
}

}  // namespace

extern "C" int32_t blpg_solve_noalloc(int32_t count, int32_t max_m, int32_t max_n,
                                      const int32_t* d_m, const int32_t* d_n,
                                      const int64_t* d_off_A, const int64_t* d_off_b,
                                      const int64_t* d_off_c, const double* dA,
                                      const double* db, const double* dc, int32_t precision,
                                      int32_t* d_status, double* d_objective, double* d_x,
                                      int32_t* d_pivots, void* stream) {
  using blpg::fail;
  if (count < 0 || count > kNoAllocMaxLps)
    return fail(BLPG_EINVAL, "blpg_solve_noalloc: count %d outside [0, %d]", count,
                kNoAllocMaxLps);
  if (count == 0) return BLPG_OK;
  if (max_m < 1 || max_n < 1 || max_m > BLPG_MAX_ROWS || max_n + max_m + 1 > BLPG_MAX_COLS)
    return fail(BLPG_EINVAL, "blpg_solve_noalloc: max_m=%d max_n=%d out of range", max_m,
                max_n);
  if (!d_m || !d_n || !d_off_A || !d_off_b || !d_off_c || !dA || !db || !dc || !d_status ||
      !d_objective)
    return fail(BLPG_EINVAL, "blpg_solve_noalloc: null input or output pointer");
  if (precision != BLPG_FP64 && precision != BLPG_FP32)
    return fail(BLPG_EINVAL, "blpg_solve_noalloc: unknown precision %d", precision);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(BLPG_ENODEV, "blpg_solve_noalloc: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices)
    return fail(BLPG_ENODEV, "blpg_solve_noalloc: device %d not supported", dev);
  DevSetup& st = g_setup[dev];
  if (!st.ready.load(std::memory_order_acquire)) {
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!st.ready.load(std::memory_order_relaxed)) {
      cudaDeviceProp prop;
      e = cudaGetDeviceProperties(&prop, dev);
      if (e != cudaSuccess || prop.major != 10 || prop.minor != 3)
        return fail(BLPG_ENODEV, "blpg_solve_noalloc: device %d is not sm_103", dev);
      void* ptr = nullptr;
      e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
      if (e != cudaSuccess || !ptr)
        return fail(BLPG_ECUDA, "blpg_solve_noalloc: cudaGetSymbolAddress: %s",
                    cudaGetErrorString(e));
      const int max_smem = (int)prop.sharedMemPerBlockOptin;
      int32_t rc = setup_attrs<double>(max_smem);
      if (rc == BLPG_OK) rc = setup_attrs<float>(max_smem);
      if (rc != BLPG_OK) return rc;
      st.scratch = static_cast<int32_t*>(ptr);
      st.sm_count = prop.multiProcessorCount;
      st.max_smem = max_smem;
      st.ready.store(true, std::memory_order_release);
    }
  }
  blpg::dev::LpArgs a;
  std::memset(&a, 0, sizeof(a));
  a.m = d_m;
  a.n = d_n;
  a.offA = d_off_A;
  a.offb = d_off_b;
  a.offc = d_off_c;
  a.offx = d_off_c;
  a.offbasis = nullptr;
  a.A = dA;
  a.b = db;
  a.c = dc;
  a.status = d_status;
  a.obj = d_objective;
  a.x = d_x;
  a.pivots = d_pivots;
  a.basis = nullptr;
  const bool fp32 = precision == BLPG_FP32;
  a.opt_tol = fp32 ? 1e-5 : 1e-9;
  a.piv_tol = fp32 ? 1e-5 : 1e-7;
  a.feas_tol = fp32 ? 1e-6 : 1e-9;
  a.phase1_tol = fp32 ? 1e-4 : 1e-7;
  a.deg_tol = fp32 ? 1e-7 : 1e-12;
  a.harris = 1;
  a.max_pivots = 0;
  a.bland_after = 64;
  a.hint = nullptr;
  a.info = nullptr;
  a.ptol = fp32 ? 1e-7 : 1e-9;
  a.refresh_period = 0;
  a.warm_mode = 1;
  a.shift = 0.1;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  return fp32 ? run<float>(count, max_m, max_n, a, st, s)
              : run<double>(count, max_m, max_n, a, st, s);
}
