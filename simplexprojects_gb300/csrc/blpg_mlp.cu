// The learned warm start's network: a multilayer perceptron that reads an
// LP's normalised [c; b; family one-hot] and scores every column (n + m of
// them) for membership in the optimal basis.  Hand-written kernels:
//   - gemm_bf16_nt: C = A B^T + bias (+ReLU) on the BF16 tensor cores
//     (mma.sync m16n8k16, FP32 accumulation), A and B K-contiguous;
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
constexpr int kKStep = 32;
constexpr int kSPad = 8;    // smem row padding (bf16) against bank conflicts

// C[M x N] = A[M x K] . B[N x K]^T (+ bias[N]) (ReLU); writes FP32 and/or BF16.
// 128 threads: 4 warps, each a 32x32 sub-tile of the 64x64 block tile.
__global__ void __launch_bounds__(128) gemm_bf16_nt(const bf16* __restrict__ A,
                                                    const bf16* __restrict__ B,
                                                    const float* __restrict__ bias,
                                                    float* __restrict__ Cf,
                                                    bf16* __restrict__ Cb, int M, int N, int K,
                                                    int relu) {
  __shared__ __align__(16) bf16 As[kTile][kKStep + kSPad];
  __shared__ __align__(16) bf16 Bs[kTile][kKStep + kSPad];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int m0 = blockIdx.y * kTile, n0 = blockIdx.x * kTile;
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int e = 0; e < 4; ++e) acc[i][j][e] = 0.f;
  for (int k0 = 0; k0 < K; k0 += kKStep) {
    // 64 rows x 32 bf16 = 64 x 4 chunks of 16 bytes per operand
    for (int c = tid; c < kTile * 4; c += 128) {
      const int r = c >> 2, q = (c & 3) * 8;
      *reinterpret_cast<uint4*>(&As[r][q]) =
          *reinterpret_cast<const uint4*>(A + (size_t)(m0 + r) * K + k0 + q);
      *reinterpret_cast<uint4*>(&Bs[r][q]) =
          *reinterpret_cast<const uint4*>(B + (size_t)(n0 + r) * K + k0 + q);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kKStep; kk += 16) {
      uint32_t af[2][4], bfr[4][2];
      const int ar = lane >> 2, ac = (lane & 3) * 2;
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const int r = wm + i * 16 + ar;
        af[i][0] = *reinterpret_cast<const uint32_t*>(&As[r][kk + ac]);
        af[i][1] = *reinterpret_cast<const uint32_t*>(&As[r + 8][kk + ac]);
        af[i][2] = *reinterpret_cast<const uint32_t*>(&As[r][kk + ac + 8]);
        af[i][3] = *reinterpret_cast<const uint32_t*>(&As[r + 8][kk + ac + 8]);
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int nr = wn + j * 8 + ar;
        bfr[j][0] = *reinterpret_cast<const uint32_t*>(&Bs[nr][kk + ac]);
        bfr[j][1] = *reinterpret_cast<const uint32_t*>(&Bs[nr][kk + ac + 8]);
      }
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
          asm volatile(
              "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
              "{%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, {%0, %1, %2, %3};"
              : "+f"(acc[i][j][0]), "+f"(acc[i][j][1]), "+f"(acc[i][j][2]), "+f"(acc[i][j][3])
              : "r"(af[i][0]), "r"(af[i][1]), "r"(af[i][2]), "r"(af[i][3]), "r"(bfr[j][0]),
                "r"(bfr[j][1]));
    }
    __syncthreads();
  }
  const int ar = lane >> 2, ac = (lane & 3) * 2;
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int r = m0 + wm + i * 16 + ar + h * 8;
        const int c = n0 + wn + j * 8 + ac;
        float v0 = acc[i][j][2 * h], v1 = acc[i][j][2 * h + 1];
        if (bias) {
          v0 += bias[c];
          v1 += bias[c + 1];
        }
        if (relu) {
          v0 = fmaxf(v0, 0.f);
          v1 = fmaxf(v1, 0.f);
        }
        if (Cf) *reinterpret_cast<float2*>(Cf + (size_t)r * N + c) = make_float2(v0, v1);
        if (Cb)
          *reinterpret_cast<__nv_bfloat162*>(Cb + (size_t)r * N + c) =
              __floats2bfloat162_rn(v0, v1);
      }
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
  if (M % kTile || N % kTile || K % kKStep)
    return blpg::fail(BLPG_EINVAL, "gemm: %d x %d x %d not tile-aligned", M, N, K);
  dim3 grid(N / kTile, M / kTile);
  gemm_bf16_nt<<<grid, 128, 0, s>>>(A, B, bias, Cf, Cb, M, N, K, relu);
  MCK(cudaGetLastError());
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
