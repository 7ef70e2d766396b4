// The learned warm start's network: a multilayer perceptron that reads an
// LP's normalised [c; b; family one-hot] and scores every column (n + m of
// them) for membership in the optimal basis.  Hand-written kernels:
//   - gemm_tc_nt: C = A B^T + bias (+ReLU) on the 5th-generation tensor
//     cores (tcgen05.mma, BF16 operands, FP32 accumulators in TMEM), A and B
//     K-contiguous;
//   - the BCE-with-sigmoid gradient, ReLU backward, bias gradient,
//     transposes with BF16 conversion, and Adam on FP32 master weights;
//   - feature building from device-resident b, c and the top-m selection
//     that turns scores into a basis hint for the solver.
// Training runs these kernels only; the host just sequences them.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "blpg_internal.h"

namespace {

using bf16 = __nv_bfloat16;

#define MCK(call)                                                                         \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess)                                                                \
      return blpg::fail(e_ == cudaErrorMemoryAllocation ? BLPG_ENOMEM : BLPG_ECUDA,       \
                        "%s: %s", #call, cudaGetErrorString(e_));                         \
  } while (0)

constexpr int kTile = 64;   // all padded dimensions are multiples of 64

// ---------------------------------------------------------------------------
// C[M x N] = A[M x K] . B[N x K]^T (+ bias[N]) (ReLU), FP32 and/or BF16 out,
// on the 5th-generation tensor cores: BF16 operands in shared memory, FP32
// accumulators in tensor memory (TMEM).
//
// One CTA of 128 threads per 128 x 128 tile of C (M and N multiples of 64:
// rows of A and B past the matrix load as zeros, and what they produce is
// not stored).  K runs in chunks of 64 through three shared-memory stages:
// all threads stage a chunk of A (128 x 64) and B (128 x 64) by 16-byte
// cp.async in the canonical K-major layout without swizzle (core matrices of
// 8 rows x 16 bytes, 128 contiguous bytes; the two core matrices of a
// 16-wide K step 128 B apart, 8-row groups 1024 B apart, so chunk c of 16
// bytes -- row group c >> 6, K column group (c >> 3) & 7, row c & 7 -- sits
// at byte 16 c, and a warp's loads read 8 rows x 64 contiguous bytes), two
// chunks ahead of the tensor cores.  Thread 0 issues four tcgen05.mma
// (M = 128, N = 128, K = 16) per chunk and commits them to the stage's
// mbarrier; a stage is refilled once the commit of the chunk before has
// arrived.  The accumulator (TMEM lanes 0..127 = rows, 128 columns) is read
// back by tcgen05.ld, each warp its 32 lanes, and written out through shared
// memory in row-contiguous pieces.  Every mbarrier wait is
// bounded; a wait that runs out counts in g_tc_timeouts (checked by the host
// calls that synchronise), and the CTA still frees its TMEM.
// ---------------------------------------------------------------------------
constexpr int kTcM = 128, kTcN = 128, kTcK = 64, kTcStages = 3;
constexpr int kTcABytes = kTcM * kTcK * 2;  // 16 KB per stage
constexpr int kTcBBytes = kTcN * kTcK * 2;  // 16 KB per stage
constexpr int kTcSmem = kTcStages * (kTcABytes + kTcBBytes) + 64;
constexpr uint32_t kTcCols = kTcN;          // TMEM columns (FP32 accumulators)
// kind::f16 instruction descriptor: FP32 accumulator (bits 4-5 = 1), BF16 A
// and B (bits 7-9 = 1, 10-12 = 1), both K-major, N >> 3 at bit 17, M >> 4 at
// bit 24.
constexpr uint32_t kTcIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kTcN >> 3) << 17) |
                              ((uint32_t)(kTcM >> 4) << 24);
constexpr int kTcWaitLimit = 1 << 22;
__device__ int g_tc_timeouts = 0;

__device__ __forceinline__ uint32_t tc_smem(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
// Shared-memory matrix descriptor: start address, leading-dimension byte
// offset 128 (the next core matrix along K), stride byte offset 1024 (the
// next 8-row group), all in 16-byte units; descriptor version 1 (bit 46),
// no swizzle (layout type 0 in bits 61-63), base offset 0.
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)(128u >> 4) << 16) |
         ((uint64_t)(1024u >> 4) << 32) | (1ull << 46);
}
__device__ __forceinline__ bool tc_wait(uint32_t bar, uint32_t parity) {
  for (int it = 0; it < kTcWaitLimit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__global__ void __launch_bounds__(128) gemm_tc_nt(const bf16* __restrict__ A,
                                                  const bf16* __restrict__ B,
                                                  const float* __restrict__ bias,
                                                  float* __restrict__ Cf, bf16* __restrict__ Cb,
                                                  int M, int N, int K, int relu) {
  extern __shared__ __align__(1024) unsigned char tc_sm[];
  unsigned char* sa = tc_sm;                          // A stages
  unsigned char* sb = tc_sm + kTcStages * kTcABytes;  // B stages
  unsigned long long* bar = reinterpret_cast<unsigned long long*>(sb + kTcStages * kTcBBytes);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + kTcStages);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.y * kTcM, n0 = blockIdx.x * kTcN;
  const int nk = K / kTcK;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     tc_smem(tslot)),
                 "r"(kTcCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int s = 0; s < kTcStages; ++s)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem(&bar[s])) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tslot;

  auto load = [&](int kc, int st) {
    const int k0 = kc * kTcK;
    unsigned char* a = sa + st * kTcABytes;
    unsigned char* b = sb + st * kTcBBytes;
    for (int c = tid; c < kTcM * 8; c += 128) {
      const int row = m0 + (c >> 6) * 8 + (c & 7);
      const int kq = (c >> 3) & 7;
      if (row < M)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(tc_smem(a + c * 16)),
                     "l"(A + (size_t)row * K + k0 + kq * 8)
                     : "memory");
      else
        *reinterpret_cast<uint4*>(a + c * 16) = make_uint4(0u, 0u, 0u, 0u);
    }
    for (int c = tid; c < kTcN * 8; c += 128) {
      const int row = n0 + (c >> 6) * 8 + (c & 7);
      const int kq = (c >> 3) & 7;
      if (row < N)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(tc_smem(b + c * 16)),
                     "l"(B + (size_t)row * K + k0 + kq * 8)
                     : "memory");
      else
        *reinterpret_cast<uint4*>(b + c * 16) = make_uint4(0u, 0u, 0u, 0u);
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  };

  // chunks kc and kc + 1 in flight ahead of the tensor cores
  load(0, 0);
  if (nk > 1) load(1, 1);
  uint32_t phases = 0;  // bit s: parity of stage s's next commit
  bool ok = true;
  for (int kc = 0; kc < nk; ++kc) {
    const int st = kc % kTcStages;
    if (kc + 1 < nk)
      asm volatile("cp.async.wait_group 1;" ::: "memory");
    else
      asm volatile("cp.async.wait_group 0;" ::: "memory");
    // the chunk's shared-memory writes, before the tensor cores read them
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t a0 = tc_smem(sa + st * kTcABytes), b0 = tc_smem(sb + st * kTcBBytes);
#pragma unroll
      for (int t = 0; t < kTcK / 16; ++t) {
        const uint64_t da = tc_desc(a0 + 256u * t), db = tc_desc(b0 + 256u * t);
        const uint32_t acc = (kc > 0 || t > 0) ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
            "l"(da), "l"(db), "r"(kTcIdesc), "r"(acc)
            : "memory");
      }
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
              tc_smem(&bar[st]))
          : "memory");
    }
    if (kc + 2 < nk) {
      // chunk kc + 2 goes into the stage chunk kc - 1 used: its MMAs first
      const int sn = (kc + 2) % kTcStages;
      if (kc >= 1) {
        ok &= tc_wait(tc_smem(&bar[sn]), (phases >> sn) & 1u);
        phases ^= 1u << sn;
      }
      load(kc + 2, sn);
    }
  }
  {  // the last commit covers every MMA issued before it
    const int st = (nk - 1) % kTcStages;
    const uint32_t ph = (phases >> st) & 1u;
    if (!tc_wait(tc_smem(&bar[st]), ph)) {
      ok = false;
      tc_wait(tc_smem(&bar[st]), ph);  // let MMAs still running finish before TMEM is freed
    }
  }
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  // Epilogue: each warp reads its 32 rows (TMEM lanes) 16 columns at a time,
  // adds the bias, applies the ReLU and stages the tile row-major in the
  // freed operand stages (rows padded by 16 bytes against bank conflicts);
  // then the CTA writes it out in full 16-byte pieces along rows, so that a
  // warp's stores cover contiguous bytes.
  float* tile = reinterpret_cast<float*>(tc_sm);  // 128 x 132 floats < the stages' 96 KB
  constexpr int ldt = kTcN + 4;
  const int lrow = warp * 32 + lane;
  const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
  for (int c0 = 0; c0 < kTcN; c0 += 16) {
    uint32_t v[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
        "%11, %12, %13, %14, %15}, [%16];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
          "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]),
          "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
        : "r"(taddr + (uint32_t)c0));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    const int col = n0 + c0;
    float f[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      float x = __uint_as_float(v[j]);
      if (bias && col < N) x += bias[col + j];  // N is a multiple of 16
      if (relu) x = fmaxf(x, 0.f);
      f[j] = x;
    }
    float4* d = reinterpret_cast<float4*>(tile + (size_t)lrow * ldt + c0);
#pragma unroll
    for (int j = 0; j < 4; ++j) d[j] = make_float4(f[4 * j], f[4 * j + 1], f[4 * j + 2], f[4 * j + 3]);
  }
  __syncthreads();
  if (Cf) {  // 32 pieces of 4 floats per row
    for (int idx = tid; idx < kTcM * (kTcN / 4); idx += 128) {
      const int r = idx / (kTcN / 4), q = idx % (kTcN / 4);
      const int grow = m0 + r, gcol = n0 + 4 * q;
      if (grow < M && gcol < N)
        *reinterpret_cast<float4*>(Cf + (size_t)grow * N + gcol) =
            *reinterpret_cast<const float4*>(tile + (size_t)r * ldt + 4 * q);
    }
  }
  if (Cb) {  // 16 pieces of 8 BF16 per row
    for (int idx = tid; idx < kTcM * (kTcN / 8); idx += 128) {
      const int r = idx / (kTcN / 8), q = idx % (kTcN / 8);
      const int grow = m0 + r, gcol = n0 + 8 * q;
      if (grow < M && gcol < N) {
        const float* t = tile + (size_t)r * ldt + 8 * q;
        __nv_bfloat162 h[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) h[j] = __floats2bfloat162_rn(t[2 * j], t[2 * j + 1]);
        *reinterpret_cast<uint4*>(Cb + (size_t)grow * N + gcol) = *reinterpret_cast<const uint4*>(h);
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcCols)
                 : "memory");
  if (!ok && tid == 0) atomicAdd(&g_tc_timeouts, 1);
}

// out[c][r] = bf16(in[r][c]) for an R x C row-major input (FP32 or BF16).
template <typename Tin>
__global__ void transpose_bf16(const Tin* __restrict__ in, bf16* __restrict__ out, int R, int C) {
  __shared__ float t[32][33];
  const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
  for (int y = threadIdx.y; y < 32; y += 8) {
    const int r = by + y, c = bx + threadIdx.x;
    if (r < R && c < C) t[y][threadIdx.x] = (float)in[(size_t)r * C + c];
  }
  __syncthreads();
  for (int y = threadIdx.y; y < 32; y += 8) {
    const int c = bx + y, r = by + threadIdx.x;
    if (r < R && c < C) out[(size_t)c * R + r] = __float2bfloat16_rn(t[threadIdx.x][y]);
  }
}

__global__ void to_bf16(const float* __restrict__ in, bf16* __restrict__ out, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    out[i] = __float2bfloat16_rn(in[i]);
}

// dZ = (sigmoid(z) - y) / B on the valid columns (else 0), and the summed
// binary cross-entropy in *loss (one atomic per block).
__global__ void bce_grad(const float* __restrict__ z, const float* __restrict__ y,
                         float* __restrict__ dz, int B, int Npad, int nvalid,
                         float* __restrict__ loss) {
  __shared__ float red[32];
  float l = 0.f;
  const size_t total = (size_t)B * Npad;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const int c = (int)(i % Npad);
    if (c >= nvalid) {
      dz[i] = 0.f;
      continue;
    }
    const float zi = z[i], yi = y[i];
    const float p = 1.f / (1.f + expf(-zi));
    dz[i] = (p - yi) / (float)B;
    // log(1 + exp(-|z|)) + max(z, 0) - y z, the stable form of BCE
    l += log1pf(expf(-fabsf(zi))) + fmaxf(zi, 0.f) - yi * zi;
  }
  for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = l;
  __syncthreads();
  if (threadIdx.x < 32) {
    float v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.f;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0 && loss) atomicAdd(loss, v);
  }
}

// dz = dh * (h > 0) (the ReLU of the layer that produced h)
__global__ void relu_back(const float* __restrict__ dh, const bf16* __restrict__ h,
                          float* __restrict__ dz, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    dz[i] = __bfloat162float(h[i]) > 0.f ? dh[i] : 0.f;
}

// db[c] = sum_r dz[r][c]
__global__ void col_sum(const float* __restrict__ dz, float* __restrict__ db, int R, int C) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= C) return;
  float s = 0.f;
  for (int r = 0; r < R; ++r) s += dz[(size_t)r * C + c];
  db[c] = s;
}

__global__ void adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                     float* __restrict__ v, size_t n, float lr, float b1, float b2, float eps,
                     float c1, float c2) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

// Features of LP k: [c / c_scale; b / b_scale; one-hot(family)], normalised
// per family and feature: (v - mean) / std from the training set.  Row k of
// X (width ldx, zero padded).
__global__ void build_features(int count, int m, int n, int F, const int64_t* __restrict__ offb,
                               const int64_t* __restrict__ offc, const double* __restrict__ b,
                               const double* __restrict__ c, const int32_t* __restrict__ family,
                               const float* __restrict__ mean, const float* __restrict__ stdv,
                               float* __restrict__ X, int ldx) {
  const int k = blockIdx.x;
  if (k >= count) return;
  const int f = family[k];
  const int nf = n + m;
  float* row = X + (size_t)k * ldx;
  for (int j = threadIdx.x; j < ldx; j += blockDim.x) {
    float v = 0.f;
    if (j < nf) {
      const double raw = j < n ? c[offc[k] + j] : b[offb[k] + (j - n)];
      const int s = (f >= 0 && f < F ? f : 0) * nf + j;
      v = ((float)raw - mean[s]) / stdv[s];
    } else if (j < nf + F) {
      v = (j - nf) == f ? 1.f : 0.f;
    }
    row[j] = v;
  }
}

// Top-m selection: the m highest-scoring of n + m columns of LP k, in
// decreasing score order (ties by lower column), written as its basis hint.
// Steepest-edge weights from scores: w_j = 1 + beta * sigmoid(score_j) for
// the n[k] + m[k] columns of LP k (one CTA per LP).
__global__ void price_weights(const float* __restrict__ scores, int lds, int count,
                              const int32_t* __restrict__ d_m, const int32_t* __restrict__ d_n,
                              const int64_t* __restrict__ offw, float beta,
                              float* __restrict__ w) {
  const int k = blockIdx.x;
  if (k >= count) return;
  const int cols = d_n[k] + d_m[k];
  const float* sk = scores + (size_t)k * lds;
  float* wk = w + offw[k];
  for (int j = threadIdx.x; j < cols; j += blockDim.x)
    wk[j] = 1.f + beta / (1.f + expf(-sk[j]));
}

__global__ void __launch_bounds__(512) topm(const float* __restrict__ scores, int lds, int count,
                                            const int32_t* __restrict__ mm,
                                            const int32_t* __restrict__ nn,
                                            const int64_t* __restrict__ offhint,
                                            int32_t* __restrict__ hint) {
  extern __shared__ unsigned long long keys[];  // pow2 >= n + m
  const int k = blockIdx.x;
  if (k >= count) return;
  const int m = mm[k], n = nn[k], nc = n + m;
  int P = 1;
  while (P < nc) P <<= 1;
  for (int j = threadIdx.x; j < P; j += blockDim.x) {
    unsigned long long key = ~0ull;
    if (j < nc) {
      // descending score: order key = ~orderable(score); ties by column
      unsigned u = __float_as_uint(scores[(size_t)k * lds + j]);
      u = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
      key = ((unsigned long long)(~u) << 32) | (unsigned)j;
    }
    keys[j] = key;
  }
  __syncthreads();
  for (int size = 2; size <= P; size <<= 1)
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int i = threadIdx.x; i < P; i += blockDim.x) {
        const int p = i ^ stride;
        if (p > i) {
          const bool up = (i & size) == 0;
          const unsigned long long a = keys[i], b2 = keys[p];
          if ((a > b2) == up) {
            keys[i] = b2;
            keys[p] = a;
          }
        }
      }
      __syncthreads();
    }
  for (int i = threadIdx.x; i < m; i += blockDim.x) hint[offhint[k] + i] = (int32_t)(keys[i] & 0xffffffffu);
}

int grid_for(size_t n) {
  size_t g = (n + 255) / 256;
  return (int)(g > 4096 ? 4096 : (g ? g : 1));
}

}  // namespace

struct blpg_mlp {
  int d_in = 0, d_in_pad = 0, hidden = 0, layers = 0, d_out = 0, d_out_pad = 0;
  int max_batch = 0;
  // FP32 master parameters, packed: W1 b1 W2 b2 ... (W_l: out x in_pad)
  float* params = nullptr;
  float* grads = nullptr;
  float* adam_m = nullptr;
  float* adam_v = nullptr;
  size_t nparams = 0;
  std::vector<size_t> w_off, b_off;
  std::vector<int> fan_in, fan_out;
  bf16* wb = nullptr;   // BF16 W_l (out x in) for the forward GEMMs
  bf16* wtb = nullptr;  // BF16 W_l^T (in x out) for the backward GEMMs
  std::vector<size_t> wb_off;
  // activations for max_batch rows
  bf16* xb = nullptr;               // input, BF16
  std::vector<bf16*> hb;            // post-ReLU activations, BF16
  float* zf = nullptr;              // logits
  float* g1 = nullptr;              // gradient scratch (max width)
  float* g2 = nullptr;
  bf16* gtb = nullptr;              // transposed gradient, BF16
  bf16* htb = nullptr;              // transposed activation, BF16
  bf16* gb = nullptr;               // gradient, BF16 (A operand of dX GEMM)
  float* loss = nullptr;
  int step = 0;
};

namespace {

int layer_in(const blpg_mlp* n, int l) { return l == 0 ? n->d_in_pad : n->hidden; }
int layer_out(const blpg_mlp* n, int l) { return l == n->layers ? n->d_out_pad : n->hidden; }

int32_t gemm(const bf16* A, const bf16* B, const float* bias, float* Cf, bf16* Cb, int M, int N,
             int K, int relu, cudaStream_t s) {
  if (M % kTile || N % kTile || K % kTcK || M <= 0 || N <= 0 || K <= 0)
    return blpg::fail(BLPG_EINVAL, "gemm: %d x %d x %d not tile-aligned", M, N, K);
  MCK(cudaFuncSetAttribute(gemm_tc_nt, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem));
  dim3 grid((N + kTcN - 1) / kTcN, (M + kTcM - 1) / kTcM);
  gemm_tc_nt<<<grid, 128, kTcSmem, s>>>(A, B, bias, Cf, Cb, M, N, K, relu);
  MCK(cudaGetLastError());
  return BLPG_OK;
}

// Bounded waits of the tensor-core GEMMs that ran out since the last check.
int32_t check_timeouts() {
  int t = 0;
  MCK(cudaMemcpyFromSymbol(&t, g_tc_timeouts, sizeof(int)));
  if (t) {
    const int zero = 0;
    MCK(cudaMemcpyToSymbol(g_tc_timeouts, &zero, sizeof(int)));
    return blpg::fail(BLPG_ECUDA, "mlp: %d tensor-core GEMM tile(s) timed out", t);
  }
  return BLPG_OK;
}

template <typename Tin>
int32_t transpose(const Tin* in, bf16* out, int R, int C, cudaStream_t s) {
  dim3 grid((C + 31) / 32, (R + 31) / 32), block(32, 8);
  transpose_bf16<Tin><<<grid, block, 0, s>>>(in, out, R, C);
  MCK(cudaGetLastError());
  return BLPG_OK;
}

// Refresh the BF16 weight copies from the FP32 masters.
int32_t sync_weights(blpg_mlp* n, cudaStream_t s) {
  for (int l = 0; l <= n->layers; ++l) {
    const int in = layer_in(n, l), out = layer_out(n, l);
    const float* W = n->params + n->w_off[l];
    to_bf16<<<grid_for((size_t)in * out), 256, 0, s>>>(W, n->wb + n->wb_off[l], (size_t)in * out);
    MCK(cudaGetLastError());
    int32_t rc = transpose<float>(W, n->wtb + n->wb_off[l], out, in, s);
    if (rc) return rc;
  }
  return BLPG_OK;
}

int32_t forward(blpg_mlp* n, const float* dX, int B, cudaStream_t s) {
  if (B > n->max_batch || B % kTile)
    return blpg::fail(BLPG_EINVAL, "mlp: batch %d must be a multiple of 64 and <= %d", B,
                      n->max_batch);
  to_bf16<<<grid_for((size_t)B * n->d_in_pad), 256, 0, s>>>(dX, n->xb, (size_t)B * n->d_in_pad);
  MCK(cudaGetLastError());
  const bf16* x = n->xb;
  for (int l = 0; l <= n->layers; ++l) {
    const int in = layer_in(n, l), out = layer_out(n, l);
    const bool last = l == n->layers;
    int32_t rc = gemm(x, n->wb + n->wb_off[l], n->params + n->b_off[l], last ? n->zf : nullptr,
                      last ? nullptr : n->hb[l], B, out, in, last ? 0 : 1, s);
    if (rc) return rc;
    if (!last) x = n->hb[l];
  }
  return BLPG_OK;
}

// Backward pass for the last forward(): gradients into n->grads (FP32).
int32_t backward(blpg_mlp* n, const float* dY, int B, cudaStream_t s) {
  const int Dp = n->d_out_pad;
  bce_grad<<<grid_for((size_t)B * Dp), 256, 0, s>>>(n->zf, dY, n->g1, B, Dp, n->d_out, n->loss);
  MCK(cudaGetLastError());
  float* dz = n->g1;  // gradient w.r.t. the pre-activation of layer l
  for (int l = n->layers; l >= 0; --l) {
    const int in = layer_in(n, l), out = layer_out(n, l);
    const bf16* xin = l == 0 ? n->xb : n->hb[l - 1];
    // dW_l [out x in] = dz^T [out x B] . xin [B x in]  -> NT with A = dz^T, B = xin^T
    int32_t rc = transpose<float>(dz, n->gtb, B, out, s);
    if (rc) return rc;
    rc = transpose<bf16>(xin, n->htb, B, in, s);
    if (rc) return rc;
    rc = gemm(n->gtb, n->htb, nullptr, n->grads + n->w_off[l], nullptr, out, in, B, 0, s);
    if (rc) return rc;
    col_sum<<<(out + 127) / 128, 128, 0, s>>>(dz, n->grads + n->b_off[l], B, out);
    MCK(cudaGetLastError());
    if (l == 0) break;
    // dh_{l-1} [B x in] = dz [B x out] . W_l [out x in] -> NT with B = W_l^T (in x out)
    to_bf16<<<grid_for((size_t)B * out), 256, 0, s>>>(dz, n->gb, (size_t)B * out);
    MCK(cudaGetLastError());
    float* dh = dz == n->g1 ? n->g2 : n->g1;
    rc = gemm(n->gb, n->wtb + n->wb_off[l], nullptr, dh, nullptr, B, in, out, 0, s);
    if (rc) return rc;
    relu_back<<<grid_for((size_t)B * in), 256, 0, s>>>(dh, n->hb[l - 1], dh, (size_t)B * in);
    MCK(cudaGetLastError());
    dz = dh;
  }
  return BLPG_OK;
}

int pad64(int v) { return (v + 63) / 64 * 64; }

}  // namespace

extern "C" int32_t blpg_mlp_create(int32_t d_in, int32_t hidden, int32_t layers, int32_t d_out,
                                   int32_t max_batch, uint64_t seed, blpg_mlp** out) {
  using blpg::fail;
  if (!out || d_in < 1 || hidden < 64 || hidden % 64 || layers < 1 || layers > 8 || d_out < 1 ||
      max_batch < 64 || max_batch % 64)
    return fail(BLPG_EINVAL, "blpg_mlp_create: bad sizes");
  *out = nullptr;
  blpg_mlp* n = new blpg_mlp;
  n->d_in = d_in;
  n->d_in_pad = pad64(d_in);
  n->hidden = hidden;
  n->layers = layers;
  n->d_out = d_out;
  n->d_out_pad = pad64(d_out);
  n->max_batch = max_batch;
  size_t off = 0, woff = 0;
  for (int l = 0; l <= layers; ++l) {
    const int in = layer_in(n, l), o = layer_out(n, l);
    n->fan_in.push_back(l == 0 ? d_in : in);
    n->fan_out.push_back(o);
    n->w_off.push_back(off);
    off += (size_t)in * o;
    n->b_off.push_back(off);
    off += (size_t)o;
    n->wb_off.push_back(woff);
    woff += (size_t)in * o;
  }
  n->nparams = off;
  // He-normal weights (deterministic, seeded), zero biases
  std::vector<float> h(off, 0.f);
  blpg::Rng rng(seed);
  for (int l = 0; l <= layers; ++l) {
    const int in = layer_in(n, l), o = layer_out(n, l);
    const double sd = std::sqrt(2.0 / (double)n->fan_in[l]) * (l == layers ? 0.5 : 1.0);
    for (int r = 0; r < o; ++r)
      for (int c = 0; c < in; ++c) {
        const bool live = (l == 0 ? c < d_in : true) && (l == layers ? r < d_out : true);
        h[n->w_off[l] + (size_t)r * in + c] = live ? (float)(sd * rng.normal()) : 0.f;
      }
  }
  const int wmax = std::max(std::max(n->d_in_pad, hidden), n->d_out_pad);
  auto fail_free = [&](int32_t code) {
    blpg_mlp_destroy(n);
    return code;
  };
#define MAL(p, bytes)                                                            \
  do {                                                                           \
    if (cudaMalloc(&(p), (bytes)) != cudaSuccess)                                \
      return fail_free(fail(BLPG_ENOMEM, "blpg_mlp_create: cudaMalloc failed")); \
  } while (0)
  MAL(n->params, off * 4);
  MAL(n->grads, off * 4);
  MAL(n->adam_m, off * 4);
  MAL(n->adam_v, off * 4);
  MAL(n->wb, woff * 2);
  MAL(n->wtb, woff * 2);
  MAL(n->xb, (size_t)max_batch * n->d_in_pad * 2);
  for (int l = 0; l < layers; ++l) {
    bf16* p = nullptr;
    MAL(p, (size_t)max_batch * hidden * 2);
    n->hb.push_back(p);
  }
  MAL(n->zf, (size_t)max_batch * n->d_out_pad * 4);
  MAL(n->g1, (size_t)max_batch * wmax * 4);
  MAL(n->g2, (size_t)max_batch * wmax * 4);
  MAL(n->gtb, (size_t)max_batch * wmax * 2);
  MAL(n->htb, (size_t)max_batch * wmax * 2);
  MAL(n->gb, (size_t)max_batch * wmax * 2);
  MAL(n->loss, 4);
#undef MAL
  if (cudaMemcpy(n->params, h.data(), off * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemset(n->adam_m, 0, off * 4) != cudaSuccess ||
      cudaMemset(n->adam_v, 0, off * 4) != cudaSuccess)
    return fail_free(fail(BLPG_ECUDA, "blpg_mlp_create: initialisation copy failed"));
  int32_t rc = sync_weights(n, nullptr);
  if (rc) return fail_free(rc);
  if (cudaDeviceSynchronize() != cudaSuccess)
    return fail_free(fail(BLPG_ECUDA, "blpg_mlp_create: %s", cudaGetErrorString(cudaGetLastError())));
  *out = n;
  return BLPG_OK;
}

extern "C" void blpg_mlp_destroy(blpg_mlp* n) {
  if (!n) return;
  cudaFree(n->params);
  cudaFree(n->grads);
  cudaFree(n->adam_m);
  cudaFree(n->adam_v);
  cudaFree(n->wb);
  cudaFree(n->wtb);
  cudaFree(n->xb);
  for (auto p : n->hb) cudaFree(p);
  cudaFree(n->zf);
  cudaFree(n->g1);
  cudaFree(n->g2);
  cudaFree(n->gtb);
  cudaFree(n->htb);
  cudaFree(n->gb);
  cudaFree(n->loss);
  delete n;
}

extern "C" int64_t blpg_mlp_num_params(const blpg_mlp* n) {
  return n ? (int64_t)n->nparams : (int64_t)blpg::fail(BLPG_EINVAL, "null mlp");
}

extern "C" int32_t blpg_mlp_get_params(const blpg_mlp* n, float* host) {
  if (!n || !host) return blpg::fail(BLPG_EINVAL, "blpg_mlp_get_params: null");
  MCK(cudaMemcpy(host, n->params, n->nparams * 4, cudaMemcpyDeviceToHost));
  return BLPG_OK;
}

extern "C" int32_t blpg_mlp_set_params(blpg_mlp* n, const float* host) {
  if (!n || !host) return blpg::fail(BLPG_EINVAL, "blpg_mlp_set_params: null");
  MCK(cudaMemcpy(n->params, host, n->nparams * 4, cudaMemcpyHostToDevice));
  int32_t rc = sync_weights(n, nullptr);
  if (rc) return rc;
  MCK(cudaDeviceSynchronize());
  return BLPG_OK;
}

extern "C" int32_t blpg_mlp_gradients(blpg_mlp* n, const float* dX, const float* dY, int32_t B,
                                      float* host_grads, float* host_loss) {
  if (!n || !dX || !dY) return blpg::fail(BLPG_EINVAL, "blpg_mlp_gradients: null");
  MCK(cudaMemset(n->loss, 0, 4));
  int32_t rc = forward(n, dX, B, nullptr);
  if (rc) return rc;
  if ((rc = backward(n, dY, B, nullptr))) return rc;
  MCK(cudaDeviceSynchronize());
  if ((rc = check_timeouts())) return rc;
  if (host_grads) MCK(cudaMemcpy(host_grads, n->grads, n->nparams * 4, cudaMemcpyDeviceToHost));
  if (host_loss) MCK(cudaMemcpy(host_loss, n->loss, 4, cudaMemcpyDeviceToHost));
  return BLPG_OK;
}

extern "C" int32_t blpg_mlp_train_step(blpg_mlp* n, const float* dX, const float* dY, int32_t B,
                                       float lr, float* host_loss, void* stream) {
  if (!n || !dX || !dY) return blpg::fail(BLPG_EINVAL, "blpg_mlp_train_step: null");
  cudaStream_t s = (cudaStream_t)stream;
  MCK(cudaMemsetAsync(n->loss, 0, 4, s));
  int32_t rc = forward(n, dX, B, s);
  if (rc) return rc;
  if ((rc = backward(n, dY, B, s))) return rc;
  n->step += 1;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - std::pow(b1, (float)n->step), c2 = 1.f - std::pow(b2, (float)n->step);
  adam<<<grid_for(n->nparams), 256, 0, s>>>(n->params, n->grads, n->adam_m, n->adam_v, n->nparams,
                                            lr, b1, b2, 1e-8f, c1, c2);
  MCK(cudaGetLastError());
  if ((rc = sync_weights(n, s))) return rc;
  if (host_loss) {
    MCK(cudaMemcpyAsync(host_loss, n->loss, 4, cudaMemcpyDeviceToHost, s));
    MCK(cudaStreamSynchronize(s));
    if ((rc = check_timeouts())) return rc;
  }
  return BLPG_OK;
}

extern "C" int32_t blpg_mlp_predict(blpg_mlp* n, const float* dX, int32_t B, float* dlogits,
                                    void* stream) {
  if (!n || !dX || !dlogits) return blpg::fail(BLPG_EINVAL, "blpg_mlp_predict: null");
  cudaStream_t s = (cudaStream_t)stream;
  for (int r0 = 0; r0 < B; r0 += n->max_batch) {
    const int rows = std::min(n->max_batch, B - r0);
    if (rows % kTile)
      return blpg::fail(BLPG_EINVAL, "blpg_mlp_predict: rows must be a multiple of 64");
    int32_t rc = forward(n, dX + (size_t)r0 * n->d_in_pad, rows, s);
    if (rc) return rc;
    MCK(cudaMemcpyAsync(dlogits + (size_t)r0 * n->d_out_pad, n->zf,
                        (size_t)rows * n->d_out_pad * 4, cudaMemcpyDeviceToDevice, s));
  }
  return BLPG_OK;
}

extern "C" int32_t blpg_mlp_dims(const blpg_mlp* n, int32_t* d_in_pad, int32_t* d_out_pad) {
  if (!n) return blpg::fail(BLPG_EINVAL, "null mlp");
  if (d_in_pad) *d_in_pad = n->d_in_pad;
  if (d_out_pad) *d_out_pad = n->d_out_pad;
  return BLPG_OK;
}

extern "C" int32_t blpg_features(int32_t count, int32_t m, int32_t n, int32_t families,
                                 const int64_t* d_offb, const int64_t* d_offc, const double* db,
                                 const double* dc, const int32_t* d_family, const float* d_mean,
                                 const float* d_std, float* dX, int32_t ldx, void* stream) {
  if (count <= 0) return BLPG_OK;
  if (!d_offb || !d_offc || !db || !dc || !d_family || !d_mean || !d_std || !dX ||
      ldx < n + m + families)
    return blpg::fail(BLPG_EINVAL, "blpg_features: bad arguments");
  build_features<<<count, 128, 0, (cudaStream_t)stream>>>(count, m, n, families, d_offb, d_offc,
                                                          db, dc, d_family, d_mean, d_std, dX, ldx);
  MCK(cudaGetLastError());
  return BLPG_OK;
}

extern "C" int32_t blpg_price_weights(const float* d_scores, int32_t lds, int32_t count,
                                      const int32_t* d_m, const int32_t* d_n, int32_t max_cols,
                                      const int64_t* d_offw, float beta, float* d_weight,
                                      void* stream) {
  if (count <= 0) return BLPG_OK;
  if (!d_scores || !d_m || !d_n || !d_offw || !d_weight || max_cols < 1 || lds < max_cols)
    return blpg::fail(BLPG_EINVAL, "blpg_price_weights: bad arguments");
  price_weights<<<count, 128, 0, (cudaStream_t)stream>>>(d_scores, lds, count, d_m, d_n, d_offw,
                                                         beta, d_weight);
  MCK(cudaGetLastError());
  return BLPG_OK;
}

extern "C" int32_t blpg_topm_hint(const float* d_scores, int32_t lds, int32_t count,
                                  const int32_t* d_m, const int32_t* d_n, int32_t max_cols,
                                  const int64_t* d_offhint, int32_t* d_hint, void* stream) {
  if (count <= 0) return BLPG_OK;
  if (!d_scores || !d_m || !d_n || !d_offhint || !d_hint || max_cols < 1 || max_cols > 8192)
    return blpg::fail(BLPG_EINVAL, "blpg_topm_hint: bad arguments");
  int P = 1;
  while (P < max_cols) P <<= 1;
  topm<<<count, 512, P * 8, (cudaStream_t)stream>>>(d_scores, lds, count, d_m, d_n, d_offhint,
                                                   d_hint);
  MCK(cudaGetLastError());
  return BLPG_OK;
}
