// Synthetic LP workloads and the reference's dense A/B/C text format.
//
// The five workload kinds restate the benchmark configurations of the GB300
// build (see blpg.h).  They replace the reference's random generator
// (parseBenchmark.cpp:321-376, which seeds rand() with the wall clock and
// loops until GLPK reports a feasible LP) with a seeded counter-based stream:
// every LP is max c^T x, A x <= b, x >= 0 with b >= 0, so the origin is
// feasible and the slack basis is a valid start, as in the reference's
// single-phase path (simplex.cu:874-890).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "blpg_internal.h"

namespace blpg {

double det_log(double x) {
  int e = 0;
  double f = std::frexp(x, &e);  // x = f * 2^e, f in [0.5, 1): exact
  if (f < 0.70710678118654752) {
    f = f * 2.0;
    e -= 1;
  }
  // log f = 2 atanh(s), s = (f - 1) / (f + 1), |s| <= 0.1716
  double s = (f - 1.0) / (f + 1.0);
  double s2 = s * s;
  double term = s, sum = s;
  for (int k = 3; k <= 31; k += 2) {
    term = term * s2;
    sum = sum + term / (double)k;
  }
  return 2.0 * sum + (double)e * 0.69314718055994530942;
}

double det_exp(double x) {
  // exp(x) = 2^k exp(r), r = x - k ln 2, |r| <= ln2 / 2; Taylor series in r.
  double kf = std::floor(x / 0.69314718055994530942 + 0.5);
  double r = x - kf * 0.69314718055994530942;
  double term = 1.0, sum = 1.0;
  for (int i = 1; i <= 24; ++i) {
    term = term * r / (double)i;
    sum = sum + term;
  }
  return std::ldexp(sum, (int)kf);
}

double Rng::normal() {
  for (;;) {
    double u = 2.0 * u01() - 1.0;
    double v = 2.0 * u01() - 1.0;
    double s = u * u + v * v;
    if (s >= 1.0 || s == 0.0) continue;
    return u * std::sqrt(-2.0 * det_log(s) / s);
  }
}

namespace {

constexpr int kFamilies = 64;
constexpr int kFamM = 174, kFamN = 142;
constexpr double kFamDensity = 0.2;

uint64_t family_seed(uint64_t seed) { return Rng::mix(seed ^ 0x5EEDFA11CAFEull); }

struct Shape {
  int32_t m = 0, n = 0, family = -1;
  double density = 0.6;
  bool unbounded = false;  // kind 4: instance-level unbounded flag
  bool degenerate = false; // kind 4: instance-level degenerate-rows flag
};

// The draws that fix an LP's shape come first in its stream.
Shape draw_shape(int32_t kind, int64_t index, Rng& r) {
  Shape s;
  switch (kind) {
    case 0: s.m = 28; s.n = 32; s.density = 0.6; break;
    case 1: {
      static const int32_t ms[4] = {50, 56, 74, 105};
      s.m = ms[r.below(4)];
      int32_t hi = (int32_t)std::floor(1.8 * (double)s.m);
      s.n = s.m + r.below(hi - s.m + 1);
      s.density = 0.6;
      break;
    }
    case 2: s.m = 205; s.n = 203; s.density = 0.15; break;
    case 3:
      s.m = kFamM; s.n = kFamN; s.family = (int32_t)(index % kFamilies);
      s.density = kFamDensity;
      break;
    case 4: {
      double fam = r.u01();
      if (fam < 0.3) {
        s.m = kFamM; s.n = kFamN; s.family = r.below(kFamilies);
        s.density = kFamDensity;
        break;
      }
      double lm = r.uniform(det_log(16.0), det_log(257.0));
      s.m = (int32_t)std::floor(det_exp(lm));
      if (s.m < 16) s.m = 16;
      if (s.m > 256) s.m = 256;
      int32_t lo = (s.m + 1) / 2;
      s.n = lo + r.below(2 * s.m - lo + 1);
      s.density = r.uniform(0.1, 0.6);
      s.unbounded = r.u01() < 0.05;
      s.degenerate = r.u01() < 0.05;
      break;
    }
    default: break;
  }
  return s;
}

// A values, then the Bernoulli keep mask, then b, then c (the draw order is
// part of the workload definition).
void draw_dense(Rng& r, int32_t m, int32_t n, double density, double* A,
                double* b, double* c) {
  const int64_t mn = (int64_t)m * n;
  for (int64_t e = 0; e < mn; ++e) A[e] = r.u01();
  for (int64_t e = 0; e < mn; ++e)
    if (r.u01() >= density) A[e] = 0.0;
  for (int32_t i = 0; i < m; ++i) b[i] = r.uniform(1.0, 10.0);
  for (int32_t j = 0; j < n; ++j) c[j] = r.uniform(1.0, 5.0);
}

void make_unbounded(Rng& r, int32_t m, int32_t n, double* A, double* c) {
  int32_t j = r.below(n);
  c[j] = r.uniform(1.0, 5.0);
  for (int32_t i = 0; i < m; ++i) A[(int64_t)i * n + j] = -r.u01();
}

void zero_rows(Rng& r, int32_t m, double* b) {
  for (int32_t i = 0; i < m; ++i)
    if (r.u01() < 0.05) b[i] = 0.0;
}

struct Family {
  std::vector<double> A, b, c;
};

void perturb(Rng& r, const Family& f, double* A, double* b, double* c) {
  std::memcpy(A, f.A.data(), sizeof(double) * (size_t)kFamM * kFamN);
  for (int32_t j = 0; j < kFamN; ++j) {
    double g = 1.0 + 0.1 * r.normal();
    double v = f.c[j] * g;
    c[j] = v > 0.01 ? v : 0.01;
  }
  for (int32_t i = 0; i < kFamM; ++i) b[i] = f.b[i] * r.uniform(0.8, 1.2);
}

}  // namespace
}  // namespace blpg

using namespace blpg;

extern "C" int64_t blpg_gen_shapes(int32_t kind, int64_t first, int32_t count,
                                   uint64_t seed, int32_t* m, int32_t* n,
                                   int32_t* family) {
  if (kind < 0 || kind > 4 || count < 0 || !m || !n)
    return fail(BLPG_EINVAL, "blpg_gen_shapes: bad arguments");
  int64_t total = 0;
  for (int32_t k = 0; k < count; ++k) {
    Rng r(seed + (uint64_t)(first + k));
    Shape s = draw_shape(kind, first + k, r);
    m[k] = s.m;
    n[k] = s.n;
    if (family) family[k] = s.family;
    total += (int64_t)s.m * s.n;
  }
  return total;
}

extern "C" int32_t blpg_gen_fill(int32_t kind, int64_t first, int32_t count,
                                 uint64_t seed, const int32_t* m,
                                 const int32_t* n, double* A, double* b,
                                 double* c, int32_t threads) {
  if (kind < 0 || kind > 4 || count < 0 || !m || !n || !A || !b || !c)
    return fail(BLPG_EINVAL, "blpg_gen_fill: bad arguments");
  std::vector<int64_t> oA(count + 1, 0), ob(count + 1, 0), oc(count + 1, 0);
  for (int32_t k = 0; k < count; ++k) {
    oA[k + 1] = oA[k] + (int64_t)m[k] * n[k];
    ob[k + 1] = ob[k] + m[k];
    oc[k + 1] = oc[k] + n[k];
  }
  std::vector<Family> fams;
  if (kind == 3 || kind == 4) {
    fams.resize(kFamilies);
    uint64_t fs = family_seed(seed);
    for (int f = 0; f < kFamilies; ++f) {
      Rng r(fs + (uint64_t)f);
      fams[f].A.resize((size_t)kFamM * kFamN);
      fams[f].b.resize(kFamM);
      fams[f].c.resize(kFamN);
      draw_dense(r, kFamM, kFamN, kFamDensity, fams[f].A.data(),
                 fams[f].b.data(), fams[f].c.data());
    }
  }
  int32_t bad = -1;
  auto work = [&](int32_t k0, int32_t k1) {
    for (int32_t k = k0; k < k1; ++k) {
      Rng r(seed + (uint64_t)(first + k));
      Shape s = draw_shape(kind, first + k, r);
      if (s.m != m[k] || s.n != n[k]) {
        bad = k;
        return;
      }
      double* Ak = A + oA[k];
      double* bk = b + ob[k];
      double* ck = c + oc[k];
      if (s.family >= 0) {
        perturb(r, fams[s.family], Ak, bk, ck);
        continue;
      }
      draw_dense(r, s.m, s.n, s.density, Ak, bk, ck);
      if (kind == 1) {
        if (r.u01() < 0.1) make_unbounded(r, s.m, s.n, Ak, ck);
        zero_rows(r, s.m, bk);
      } else if (kind == 4) {
        if (s.unbounded) make_unbounded(r, s.m, s.n, Ak, ck);
        if (s.degenerate) zero_rows(r, s.m, bk);
      }
    }
  };
  int32_t nt = threads > 0 ? threads : (int32_t)std::thread::hardware_concurrency();
  if (nt < 1) nt = 1;
  if (nt > count) nt = count > 0 ? count : 1;
  if (nt == 1) {
    work(0, count);
  } else {
    std::vector<std::thread> pool;
    int32_t per = (count + nt - 1) / nt;
    for (int32_t t = 0; t < nt; ++t) {
      int32_t k0 = t * per, k1 = k0 + per < count ? k0 + per : count;
      if (k0 < k1) pool.emplace_back(work, k0, k1);
    }
    for (auto& th : pool) th.join();
  }
  if (bad >= 0)
    return fail(BLPG_EINVAL, "blpg_gen_fill: shape of LP %d does not match kind %d",
                bad, kind);
  return BLPG_OK;
}

namespace {

bool read_numbers(const char* path, std::vector<double>& out, bool first_per_line) {
  std::ifstream in(path);
  if (!in) return false;
  std::string line;
  while (std::getline(in, line)) {
    std::istringstream ls(line);
    double v;
    if (first_per_line) {
      if (ls >> v) out.push_back(v);
    } else {
      while (ls >> v) out.push_back(v);
    }
  }
  return true;
}

}  // namespace

// Reader for the reference's dense text files (parseBenchmark.cpp:59-126).
extern "C" int32_t blpg_read_abc(const char* path_A, const char* path_B,
                                 const char* path_C, int32_t* m, int32_t* n,
                                 double* A, double* b, double* c) {
  if (!path_A || !path_B || !path_C || !m || !n)
    return fail(BLPG_EINVAL, "blpg_read_abc: null argument");
  std::ifstream in(path_A);
  if (!in) return fail(BLPG_EIO, "blpg_read_abc: cannot open %s", path_A);
  std::string first;
  std::getline(in, first);
  std::istringstream hs(first);
  long rows = -1, cols = -1;
  if (!(hs >> rows >> cols) || rows <= 0 || cols <= 0 || rows > BLPG_MAX_ROWS ||
      cols > BLPG_MAX_COLS)
    return fail(BLPG_EIO, "blpg_read_abc: bad header in %s", path_A);
  *m = (int32_t)rows;
  *n = (int32_t)cols;
  if (!A && !b && !c) return BLPG_OK;
  if (!A || !b || !c) return fail(BLPG_EINVAL, "blpg_read_abc: partial buffers");
  std::vector<double> av;
  std::string line;
  while (std::getline(in, line)) {
    std::istringstream ls(line);
    double v;
    while (ls >> v) av.push_back(v);
  }
  if ((long)av.size() != rows * cols)
    return fail(BLPG_EIO, "blpg_read_abc: %s holds %zu values, expected %ld", path_A,
                av.size(), rows * cols);
  std::vector<double> bv, cv;
  if (!read_numbers(path_B, bv, true) || (long)bv.size() < rows)
    return fail(BLPG_EIO, "blpg_read_abc: %s: expected %ld values", path_B, rows);
  if (!read_numbers(path_C, cv, true) || (long)cv.size() < cols)
    return fail(BLPG_EIO, "blpg_read_abc: %s: expected %ld values", path_C, cols);
  for (long e = 0; e < rows * cols; ++e) A[e] = av[e] == 0.0 ? 0.0 : av[e];
  for (long i = 0; i < rows; ++i) b[i] = bv[i];
  for (long j = 0; j < cols; ++j) c[j] = cv[j];
  return BLPG_OK;
}

// ---------------------------------------------------------------------------
// Batch files: a whole batch (shapes, offsets, A, b, c) in one binary file,
// and the per-LP results as text, one line per LP.  No reference
// counterpart: the reference only reads one LP's A/B/C text files
// (parseBenchmark.cpp:59-126) and replicates it (GPU_Tester.cu:119-127).
//
// Layout (little-endian, the byte order of the hosts this library runs on):
//   char    magic[8] = "BLPGBAT1"
//   uint32  version = 1, uint32 reserved = 0
//   int64   count, nA, nb, nc      (elements of A, b, c stored)
//   int32   m[count], n[count]
//   int64   off_A[count], off_b[count], off_c[count]
//   double  A[nA], b[nb], c[nc]
// Offsets are always stored (packed ones when the batch had none), so LPs
// that share A keep sharing it in the file.
// ---------------------------------------------------------------------------
namespace {

const char kBatchMagic[8] = {'B', 'L', 'P', 'G', 'B', 'A', 'T', '1'};

struct FileCloser {
  std::FILE* f;
  ~FileCloser() {
    if (f) std::fclose(f);
  }
};

bool little_endian() {
  const uint32_t one = 1;
  unsigned char c0;
  std::memcpy(&c0, &one, 1);
  return c0 == 1;
}

}  // namespace

extern "C" int32_t blpg_write_batch(const char* path, const blpg_batch* bt) {
  using blpg::fail;
  if (!path || !bt || bt->count < 0 || (bt->count > 0 && (!bt->m || !bt->n || !bt->A || !bt->b || !bt->c)))
    return fail(BLPG_EINVAL, "blpg_write_batch: null or negative argument");
  if (!little_endian()) return fail(BLPG_EIO, "blpg_write_batch: big-endian host");
  const int64_t N = bt->count;
  std::vector<int64_t> oA(N), ob(N), oc(N);
  int64_t pa = 0, pb = 0, pc = 0, nA = 0, nb = 0, nc = 0;
  for (int64_t k = 0; k < N; ++k) {
    const int64_t m = bt->m[k], n = bt->n[k];
    if (m < 0 || n < 0) return fail(BLPG_EINVAL, "blpg_write_batch: LP %lld has a negative size", (long long)k);
    oA[k] = bt->off_A ? bt->off_A[k] : pa;
    ob[k] = bt->off_b ? bt->off_b[k] : pb;
    oc[k] = bt->off_c ? bt->off_c[k] : pc;
    if (oA[k] < 0 || ob[k] < 0 || oc[k] < 0)
      return fail(BLPG_EINVAL, "blpg_write_batch: LP %lld has a negative offset", (long long)k);
    pa += m * n;
    pb += m;
    pc += n;
    nA = std::max(nA, oA[k] + m * n);
    nb = std::max(nb, ob[k] + m);
    nc = std::max(nc, oc[k] + n);
  }
  std::FILE* f = std::fopen(path, "wb");
  if (!f) return fail(BLPG_EIO, "blpg_write_batch: cannot create %s", path);
  FileCloser fc{f};
  const uint32_t ver[2] = {1u, 0u};
  const int64_t sizes[4] = {N, nA, nb, nc};
  bool ok = std::fwrite(kBatchMagic, 1, 8, f) == 8 && std::fwrite(ver, 4, 2, f) == 2 &&
            std::fwrite(sizes, 8, 4, f) == 4;
  ok = ok && std::fwrite(bt->m, 4, (size_t)N, f) == (size_t)N &&
       std::fwrite(bt->n, 4, (size_t)N, f) == (size_t)N;
  ok = ok && std::fwrite(oA.data(), 8, (size_t)N, f) == (size_t)N &&
       std::fwrite(ob.data(), 8, (size_t)N, f) == (size_t)N &&
       std::fwrite(oc.data(), 8, (size_t)N, f) == (size_t)N;
  ok = ok && std::fwrite(bt->A, 8, (size_t)nA, f) == (size_t)nA &&
       std::fwrite(bt->b, 8, (size_t)nb, f) == (size_t)nb &&
       std::fwrite(bt->c, 8, (size_t)nc, f) == (size_t)nc;
  if (!ok) return fail(BLPG_EIO, "blpg_write_batch: write to %s failed", path);
  return BLPG_OK;
}

extern "C" int32_t blpg_read_batch(const char* path, int64_t* count, int64_t* nA, int64_t* nb,
                                   int64_t* nc, int32_t* m, int32_t* n, int64_t* off_A,
                                   int64_t* off_b, int64_t* off_c, double* A, double* b,
                                   double* c) {
  using blpg::fail;
  if (!path || !count || !nA || !nb || !nc) return fail(BLPG_EINVAL, "blpg_read_batch: null argument");
  if (!little_endian()) return fail(BLPG_EIO, "blpg_read_batch: big-endian host");
  std::FILE* f = std::fopen(path, "rb");
  if (!f) return fail(BLPG_EIO, "blpg_read_batch: cannot open %s", path);
  FileCloser fc{f};
  char magic[8];
  uint32_t ver[2];
  int64_t sizes[4];
  if (std::fread(magic, 1, 8, f) != 8 || std::memcmp(magic, kBatchMagic, 8) != 0)
    return fail(BLPG_EIO, "blpg_read_batch: %s is not a batch file", path);
  if (std::fread(ver, 4, 2, f) != 2 || ver[0] != 1u)
    return fail(BLPG_EIO, "blpg_read_batch: %s: unsupported version", path);
  if (std::fread(sizes, 8, 4, f) != 4 || sizes[0] < 0 || sizes[0] > INT32_MAX || sizes[1] < 0 ||
      sizes[2] < 0 || sizes[3] < 0)
    return fail(BLPG_EIO, "blpg_read_batch: %s: bad header", path);
  // the file must be exactly as long as its header says, so that a damaged
  // header cannot make a caller allocate for data that is not there
  {
    const uint64_t cnt = (uint64_t)sizes[0], big = (uint64_t)1 << 58;  // 8 x 3 x 2^58 < 2^63
    bool fits = (uint64_t)sizes[1] < big && (uint64_t)sizes[2] < big && (uint64_t)sizes[3] < big;
    const uint64_t want = 48 + cnt * 32 + 8 * ((uint64_t)sizes[1] + (uint64_t)sizes[2] +
                                              (uint64_t)sizes[3]);
    long here = std::ftell(f), end = -1;
    if (here >= 0 && std::fseek(f, 0, SEEK_END) == 0) end = std::ftell(f);
    if (end < 0 || std::fseek(f, here, SEEK_SET) != 0)
      return fail(BLPG_EIO, "blpg_read_batch: %s: cannot seek", path);
    if (!fits || (uint64_t)end != want)
      return fail(BLPG_EIO, "blpg_read_batch: %s is truncated or its header is damaged", path);
  }
  *count = sizes[0];
  *nA = sizes[1];
  *nb = sizes[2];
  *nc = sizes[3];
  const bool none = !m && !n && !off_A && !off_b && !off_c && !A && !b && !c;
  if (none) return BLPG_OK;
  if (!m || !n || !off_A || !off_b || !off_c || !A || !b || !c)
    return fail(BLPG_EINVAL, "blpg_read_batch: partial buffers");
  const size_t N = (size_t)sizes[0];
  bool ok = std::fread(m, 4, N, f) == N && std::fread(n, 4, N, f) == N &&
            std::fread(off_A, 8, N, f) == N && std::fread(off_b, 8, N, f) == N &&
            std::fread(off_c, 8, N, f) == N;
  ok = ok && std::fread(A, 8, (size_t)sizes[1], f) == (size_t)sizes[1] &&
       std::fread(b, 8, (size_t)sizes[2], f) == (size_t)sizes[2] &&
       std::fread(c, 8, (size_t)sizes[3], f) == (size_t)sizes[3];
  if (!ok) return fail(BLPG_EIO, "blpg_read_batch: %s is truncated", path);
  for (size_t k = 0; k < N; ++k) {
    const int64_t mk = m[k], nk = n[k];
    if (mk < 0 || nk < 0 || off_A[k] < 0 || off_b[k] < 0 || off_c[k] < 0 ||
        off_A[k] + mk * nk > sizes[1] || off_b[k] + mk > sizes[2] || off_c[k] + nk > sizes[3])
      return fail(BLPG_EIO, "blpg_read_batch: %s: LP %zu lies outside the stored arrays", path, k);
  }
  return BLPG_OK;
}

extern "C" int32_t blpg_write_results(const char* path, const blpg_batch* bt,
                                      const blpg_result* res) {
  using blpg::fail;
  if (!path || !bt || !res || (bt->count > 0 && (!bt->n || !res->status || !res->objective)))
    return fail(BLPG_EINVAL, "blpg_write_results: null argument");
  std::FILE* f = std::strcmp(path, "-") == 0 ? stdout : std::fopen(path, "w");
  if (!f) return fail(BLPG_EIO, "blpg_write_results: cannot create %s", path);
  FileCloser fc{f == stdout ? nullptr : f};
  int64_t pc = 0;
  for (int64_t k = 0; k < bt->count; ++k) {
    const int64_t oc = bt->off_c ? bt->off_c[k] : pc;
    pc += bt->n[k];
    std::fprintf(f, "%d %.17g", res->status[k], res->objective[k]);
    if (res->x)
      for (int32_t j = 0; j < bt->n[k]; ++j) std::fprintf(f, " %.17g", res->x[oc + j]);
    std::fputc('\n', f);
  }
  if (std::ferror(f)) return fail(BLPG_EIO, "blpg_write_results: write to %s failed", path);
  return BLPG_OK;
}
