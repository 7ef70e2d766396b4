// The learned warm start behind the C ABI (blpg_learned_*): one call takes a
// host batch of LPs of one shape, uploads A, b, c and the family ids, forms
// the network's features, runs the network, turns its basis probabilities
// into steepest-edge score weights and solves the batch with an FP32 plan,
// then downloads the results.  No reference counterpart (the reference has
// no learned part); it replaces the steps a caller of the plan API would
// otherwise chain by hand (blpg_features, blpg_mlp_predict,
// blpg_price_weights, blpg_plan_execute_weighted).
//
// The uploads run on a copy stream in three pieces, b/c/family ids of the
// first half of the LPs, then of the second half, then A; the network of
// each half runs on the compute stream as soon as its piece has landed, so
// the second half's upload and A's overlap the first half's network, and
// the solve waits for A.  The results come back in one copy of a packed
// device block into pinned staging, then into the caller's arrays.  Host
// input arrays in pinned memory make the uploads asynchronous to the host.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "blpg_internal.h"

struct blpg_learned {
  blpg_mlp* mlp = nullptr;  // not owned
  blpg_plan* plan = nullptr;
  int count = 0, m = 0, n = 0, families = 0;
  float beta = 1.f;
  int d_in_pad = 0, d_out_pad = 0, rows = 0;
  int64_t extA = 0, extb = 0, extc = 0, extw = 0;
  // the LPs [0, half) form the first upload and network piece (half a
  // multiple of 64, so each piece's network rows are); its b and c lie in
  // [0, eb1) and [0, ec1); half == count: one piece
  int half = 0;
  int64_t eb1 = 0, ec1 = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t stream_a = nullptr;  // uploads, beside the network
  cudaEvent_t first_landed = nullptr, all_landed = nullptr, a_landed = nullptr;
  // device buffers; obj, st, piv, info are one block (res) so that the
  // results download in one copy, into pinned staging (hres)
  double *A = nullptr, *b = nullptr, *c = nullptr, *obj = nullptr, *x = nullptr;
  int32_t *fam = nullptr, *dm = nullptr, *dn = nullptr, *st = nullptr, *piv = nullptr,
          *info = nullptr;
  void* res = nullptr;
  unsigned char* hres = nullptr;
  int64_t *offb = nullptr, *offc = nullptr, *offw = nullptr;
  float *mean = nullptr, *std_ = nullptr, *X = nullptr, *logits = nullptr, *w = nullptr;
};

namespace {

#define LCK(call)                                                                           \
  do {                                                                                      \
    cudaError_t e_ = (call);                                                                \
    if (e_ != cudaSuccess)                                                                  \
      return blpg::fail(e_ == cudaErrorMemoryAllocation ? BLPG_ENOMEM : BLPG_ECUDA,         \
                        "blpg_learned: %s: %s", #call, cudaGetErrorString(e_));             \
  } while (0)

// objective (8 bytes), status, pivots and info (4 each) per LP
constexpr size_t kResBytesPerLp = 20;

void release(blpg_learned* L) {
  if (!L) return;
  if (L->plan) blpg_plan_destroy(L->plan);
  void* bufs[] = {L->A,    L->b,    L->c,    L->x,    L->fam,   L->dm, L->dn,     L->res,
                  L->offb, L->offc, L->offw, L->mean, L->std_, L->X,  L->logits, L->w};
  for (void* p : bufs) cudaFree(p);
  if (L->hres) cudaFreeHost(L->hres);
  for (cudaEvent_t ev : {L->first_landed, L->all_landed, L->a_landed})
    if (ev) cudaEventDestroy(ev);
  if (L->stream_a) cudaStreamDestroy(L->stream_a);
  if (L->stream) cudaStreamDestroy(L->stream);
}

}  // namespace

extern "C" int32_t blpg_learned_create(blpg_mlp* mlp, int32_t families, const float* host_mean,
                                       const float* host_std, float beta,
                                       const blpg_batch* shapes, const blpg_options* opt_in,
                                       blpg_learned** out) {
  using blpg::fail;
  if (!mlp || !host_mean || !host_std || !shapes || !out || families < 1 || shapes->count < 1 ||
      !shapes->m || !shapes->n)
    return fail(BLPG_EINVAL, "blpg_learned_create: null or empty argument");
  *out = nullptr;
  const int N = shapes->count, m = shapes->m[0], n = shapes->n[0];
  for (int k = 0; k < N; ++k)
    if (shapes->m[k] != m || shapes->n[k] != n)
      return fail(BLPG_EINVAL, "blpg_learned_create: LP %d is %dx%d, the batch's shape is %dx%d",
                  k, shapes->m[k], shapes->n[k], m, n);
  int32_t din = 0, dout = 0;
  int32_t rc = blpg_mlp_dims(mlp, &din, &dout);
  if (rc) return rc;
  if (din < n + m + families || dout < n + m)
    return fail(BLPG_EINVAL,
                "blpg_learned_create: the network reads %d features and scores %d columns; "
                "the batch needs %d and %d",
                din, dout, n + m + families, n + m);
  blpg_options opt;
  if (opt_in)
    opt = *opt_in;
  else
    blpg_options_init(&opt);
  opt.pricing = BLPG_PRICE_STEEPEST;  // the network's probabilities weight steepest edge
  opt.basis_hint = nullptr;
  opt.price_weight = nullptr;
  blpg_learned* L = new blpg_learned;
  L->mlp = mlp;
  L->count = N;
  L->m = m;
  L->n = n;
  L->families = families;
  L->beta = beta;
  L->d_in_pad = din;
  L->d_out_pad = dout;
  L->rows = (N + 63) / 64 * 64;
  auto bail = [&](int32_t code) {
    release(L);
    delete L;
    return code;
  };
  if ((rc = blpg_plan_create(shapes, &opt, &L->plan))) return bail(rc);
  // offsets as the plan reads them (packed when null), and the weights' packing
  std::vector<int64_t> ob(N), oc(N), ow(N);
  int64_t pa = 0, pb = 0, pc = 0;
  for (int k = 0; k < N; ++k) {
    const int64_t oa = shapes->off_A ? shapes->off_A[k] : pa;
    ob[k] = shapes->off_b ? shapes->off_b[k] : pb;
    oc[k] = shapes->off_c ? shapes->off_c[k] : pc;
    ow[k] = (int64_t)k * (n + m);
    L->extA = std::max(L->extA, oa + (int64_t)m * n);
    L->extb = std::max(L->extb, ob[k] + m);
    L->extc = std::max(L->extc, oc[k] + n);
    pa += (int64_t)m * n;
    pb += m;
    pc += n;
  }
  L->extw = (int64_t)N * (n + m);
  // two pieces from 512 LPs up (below that the second network launch costs
  // more than the upload it hides)
  L->half = N >= 512 ? (N / 2 + 63) / 64 * 64 : N;
  for (int k = 0; k < L->half; ++k) {
    L->eb1 = std::max(L->eb1, ob[k] + m);
    L->ec1 = std::max(L->ec1, oc[k] + n);
  }
  cudaError_t e = cudaStreamCreateWithFlags(&L->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&L->stream_a, cudaStreamNonBlocking);
  for (cudaEvent_t* ev : {&L->first_landed, &L->all_landed, &L->a_landed})
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
  if (e != cudaSuccess) return bail(fail(BLPG_ECUDA, "blpg_learned_create: stream"));
  const size_t F = (size_t)families * (n + m);
#define LMAL(p, bytes)                                                              \
  do {                                                                              \
    if (cudaMalloc(&(p), (bytes)) != cudaSuccess)                                   \
      return bail(fail(BLPG_ENOMEM, "blpg_learned_create: %zu bytes", (size_t)(bytes))); \
  } while (0)
  LMAL(L->A, sizeof(double) * (size_t)L->extA);
  LMAL(L->b, sizeof(double) * (size_t)L->extb);
  LMAL(L->c, sizeof(double) * (size_t)L->extc);
  LMAL(L->res, kResBytesPerLp * (size_t)N);
  if (cudaMallocHost(&L->hres, kResBytesPerLp * (size_t)N) != cudaSuccess)
    return bail(fail(BLPG_ENOMEM, "blpg_learned_create: %zu pinned bytes",
                     kResBytesPerLp * (size_t)N));
  L->obj = static_cast<double*>(L->res);  // [0, 8N) objectives
  L->st = reinterpret_cast<int32_t*>(L->obj + N);  // [8N, 12N) statuses
  L->piv = L->st + N;                              // [12N, 16N) pivots
  L->info = L->piv + N;                            // [16N, 20N) info bits
  LMAL(L->x, sizeof(double) * (size_t)L->extc);
  LMAL(L->fam, sizeof(int32_t) * N);
  LMAL(L->dm, sizeof(int32_t) * N);
  LMAL(L->dn, sizeof(int32_t) * N);
  LMAL(L->offb, sizeof(int64_t) * N);
  LMAL(L->offc, sizeof(int64_t) * N);
  LMAL(L->offw, sizeof(int64_t) * N);
  LMAL(L->mean, sizeof(float) * F);
  LMAL(L->std_, sizeof(float) * F);
  LMAL(L->X, sizeof(float) * (size_t)L->rows * din);
  LMAL(L->logits, sizeof(float) * (size_t)L->rows * dout);
  LMAL(L->w, sizeof(float) * (size_t)L->extw);
#undef LMAL
  std::vector<int32_t> mm(N, m), nn(N, n);
  cudaMemcpy(L->dm, mm.data(), sizeof(int32_t) * N, cudaMemcpyHostToDevice);
  cudaMemcpy(L->dn, nn.data(), sizeof(int32_t) * N, cudaMemcpyHostToDevice);
  cudaMemcpy(L->offb, ob.data(), sizeof(int64_t) * N, cudaMemcpyHostToDevice);
  cudaMemcpy(L->offc, oc.data(), sizeof(int64_t) * N, cudaMemcpyHostToDevice);
  cudaMemcpy(L->offw, ow.data(), sizeof(int64_t) * N, cudaMemcpyHostToDevice);
  cudaMemcpy(L->mean, host_mean, sizeof(float) * F, cudaMemcpyHostToDevice);
  cudaMemcpy(L->std_, host_std, sizeof(float) * F, cudaMemcpyHostToDevice);
  // feature rows past the batch stay zero
  cudaMemset(L->X, 0, sizeof(float) * (size_t)L->rows * din);
  e = cudaDeviceSynchronize();
  if (e != cudaSuccess)
    return bail(fail(BLPG_ECUDA, "blpg_learned_create: %s", cudaGetErrorString(e)));
  *out = L;
  return BLPG_OK;
}

namespace {

// The body of blpg_learned_solve, arguments checked.
int32_t learned_solve(blpg_learned* L, const blpg_batch* bt, const int32_t* host_family,
                      blpg_result* out) {
  const int N = L->count, H = L->half;
  cudaStream_t s = L->stream, u = L->stream_a;
  const size_t d8 = sizeof(double);
  // the first piece's b, c and family ids, then its features and network
  LCK(cudaMemcpyAsync(L->b, bt->b, d8 * (size_t)L->eb1, cudaMemcpyHostToDevice, u));
  LCK(cudaMemcpyAsync(L->c, bt->c, d8 * (size_t)L->ec1, cudaMemcpyHostToDevice, u));
  LCK(cudaMemcpyAsync(L->fam, host_family, sizeof(int32_t) * H, cudaMemcpyHostToDevice, u));
  LCK(cudaEventRecord(L->first_landed, u));
  LCK(cudaStreamWaitEvent(s, L->first_landed, 0));
  int32_t rc;
  if ((rc = blpg_features(H, L->m, L->n, L->families, L->offb, L->offc, L->b, L->c, L->fam,
                          L->mean, L->std_, L->X, L->d_in_pad, s)))
    return rc;
  const int rows1 = H < N ? H : L->rows;
  if ((rc = blpg_mlp_predict(L->mlp, L->X, rows1, L->logits, s))) return rc;
  // the rest: the second piece (what the first did not cover), its network
  if (H < N) {
    if (L->extb > L->eb1)
      LCK(cudaMemcpyAsync(L->b + L->eb1, bt->b + L->eb1, d8 * (size_t)(L->extb - L->eb1),
                          cudaMemcpyHostToDevice, u));
    if (L->extc > L->ec1)
      LCK(cudaMemcpyAsync(L->c + L->ec1, bt->c + L->ec1, d8 * (size_t)(L->extc - L->ec1),
                          cudaMemcpyHostToDevice, u));
    LCK(cudaMemcpyAsync(L->fam + H, host_family + H, sizeof(int32_t) * (N - H),
                        cudaMemcpyHostToDevice, u));
    LCK(cudaEventRecord(L->all_landed, u));
    LCK(cudaStreamWaitEvent(s, L->all_landed, 0));
    if ((rc = blpg_features(N - H, L->m, L->n, L->families, L->offb + H, L->offc + H, L->b, L->c,
                            L->fam + H, L->mean, L->std_, L->X + (size_t)H * L->d_in_pad,
                            L->d_in_pad, s)))
      return rc;
    if ((rc = blpg_mlp_predict(L->mlp, L->X + (size_t)H * L->d_in_pad, L->rows - H,
                               L->logits + (size_t)H * L->d_out_pad, s)))
      return rc;
  }
  // A last: only the solve reads it
  LCK(cudaMemcpyAsync(L->A, bt->A, d8 * (size_t)L->extA, cudaMemcpyHostToDevice, u));
  LCK(cudaEventRecord(L->a_landed, u));
  if ((rc = blpg_price_weights(L->logits, L->d_out_pad, N, L->dm, L->dn, L->n + L->m, L->offw,
                               L->beta, L->w, s)))
    return rc;
  blpg_result dres{L->st, L->obj, out->x ? L->x : nullptr, out->pivots ? L->piv : nullptr,
                   nullptr, out->info ? L->info : nullptr};
  LCK(cudaStreamWaitEvent(s, L->a_landed, 0));
  if ((rc = blpg_plan_execute_weighted(L->plan, L->A, L->b, L->c, nullptr, L->w, &dres, s)))
    return rc;
  // one download of the packed results (objectives and statuses, then the
  // pivots and info bits when asked for)
  const size_t nres = (size_t)N * (out->info ? 20 : out->pivots ? 16 : 12);
  LCK(cudaMemcpyAsync(L->hres, L->res, nres, cudaMemcpyDeviceToHost, s));
  if (out->x)
    LCK(cudaMemcpyAsync(out->x, L->x, d8 * (size_t)L->extc, cudaMemcpyDeviceToHost, s));
  LCK(cudaStreamSynchronize(s));
  const unsigned char* h = L->hres;
  std::memcpy(out->objective, h, d8 * N);
  std::memcpy(out->status, h + 8 * (size_t)N, sizeof(int32_t) * N);
  if (out->pivots) std::memcpy(out->pivots, h + 12 * (size_t)N, sizeof(int32_t) * N);
  if (out->info) std::memcpy(out->info, h + 16 * (size_t)N, sizeof(int32_t) * N);
  return BLPG_OK;
}

}  // namespace

extern "C" int32_t blpg_learned_solve(blpg_learned* L, const blpg_batch* bt,
                                      const int32_t* host_family, blpg_result* out) {
  using blpg::fail;
  if (!L || !bt || !host_family || !out || !out->status || !out->objective)
    return fail(BLPG_EINVAL, "blpg_learned_solve: null argument");
  if (bt->count != L->count || !bt->A || !bt->b || !bt->c)
    return fail(BLPG_EINVAL, "blpg_learned_solve: the batch is not the one the solver was made for");
  const int32_t rc = learned_solve(L, bt, host_family, out);
  if (rc != BLPG_OK) {
    // a step failed with copies or kernels of this call still queued: let
    // them finish before the next call overwrites their buffers
    cudaStreamSynchronize(L->stream_a);
    cudaStreamSynchronize(L->stream);
  }
  return rc;
}

extern "C" void blpg_learned_destroy(blpg_learned* L) {
  if (!L) return;
  if (L->stream) cudaStreamSynchronize(L->stream);
  if (L->stream_a) cudaStreamSynchronize(L->stream_a);
  release(L);
  delete L;
}
