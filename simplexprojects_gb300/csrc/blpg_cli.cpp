// blpg_cli — the reference's command line over libblpg.
//
//   blpg_cli <benchmark-no | dimension> <average> <batch-size> <streams> <1|2>
//   blpg_cli <batch-file> <average> <results-file | -> <64|32> 3
//
// Mirrors BLPGSolver (GPU_Tester.cu:31-393, ReadMe:10-20):
//   mode 1: Netlib benchmark 1..8 (parseBenchmark.cpp:29-57) read from
//           $BLPG_BENCH_DIR (default ./benchmarks) as <NAME>_{A,B,C}.txt;
//           the minimisation objective is negated into max form and copied
//           to every LP of the batch (GPU_Tester.cu:119-127);
//   mode 2: a random dense LP of the given dimension, A_ij ~ U{1..999},
//           b_i ~ U{1..999}, c_j ~ U{1..499} as parseBenchmark.cpp:321-376
//           (seeded here, so runs repeat; the reference only prints GLPK's
//           answer in this mode and exits, GPU_Tester.cu:67-79).
//   mode 3: a batch file (blpg_write_batch) solved as it stands, in FP64 or
//           FP32, with the per-LP results written by blpg_write_results
//           (status, objective, x; "-" writes them to stdout).
// The batch is solved `average`+1 times; the first run is warm-up and the
// rest are averaged (GPU_Tester.cu:242-262).  Batches larger than what fits
// the device's free memory are split by the library (GPU_Tester.cu:194-238).
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "../../include/blpg_simplex.hpp"

namespace {

const char* kNames[8] = {"ADLITTLE", "AFIRO", "BLEND", "ISRAEL", "SC105", "SC205", "SC50A", "SC50B"};

int usage() {
  std::printf(
      "usage: blpg_cli <benchmark-no|dimension> <average> <batch-size> <streams> <1|2>\n"
      "       blpg_cli <batch-file> <average> <results-file|-> <64|32> 3\n"
      "  1: Netlib benchmark 1..8 from $BLPG_BENCH_DIR (default ./benchmarks)\n"
      "  2: random dense LP of the given dimension\n"
      "  3: a batch file, results to a file (or stdout)\n");
  return 2;
}

int fail_with_last_error() {
  std::fprintf(stderr, "%s\n", blpg_last_error());
  return 1;
}

// mode 3: blpg_read_batch -> blpg_solve_batch (timed) -> blpg_write_results
int solve_batch_file(const char* in, int avg, const char* out, int bits) {
  int64_t count = 0, nA = 0, nb = 0, nc = 0;
  if (blpg_read_batch(in, &count, &nA, &nb, &nc, nullptr, nullptr, nullptr, nullptr, nullptr,
                      nullptr, nullptr, nullptr))
    return fail_with_last_error();
  std::vector<int32_t> m(count), n(count);
  std::vector<int64_t> oA(count), ob(count), oc(count);
  std::vector<double> A(nA), b(nb), c(nc);
  if (blpg_read_batch(in, &count, &nA, &nb, &nc, m.data(), n.data(), oA.data(), ob.data(),
                      oc.data(), A.data(), b.data(), c.data()))
    return fail_with_last_error();
  const blpg_batch bt{(int32_t)count, m.data(), n.data(), oA.data(), ob.data(), oc.data(),
                      A.data(), b.data(), c.data()};
  blpg_options opt;
  blpg_options_init(&opt);
  opt.precision = bits == 32 ? BLPG_FP32 : BLPG_FP64;
  std::vector<int32_t> status(count), pivots(count);
  std::vector<double> obj(count), x(nc);
  blpg_result res{status.data(), obj.data(), x.data(), pivots.data(), nullptr, nullptr};
  double sum = 0.0;
  for (int it = 0; it <= avg; ++it) {
    const auto t0 = std::chrono::steady_clock::now();
    if (blpg_solve_batch(&bt, &opt, &res)) return fail_with_last_error();
    const double sec =
        std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::fprintf(stderr, "Iter %d: Time = %.6f Seconds\n", it, sec);
    if (it > 0) sum += sec;
  }
  std::fprintf(stderr, "%lld LPs (FP%d): %.6f s, %.1f LPs/s\n", (long long)count, bits,
               sum / avg, count / (sum / avg));
  if (blpg_write_results(out, &bt, &res)) return fail_with_last_error();
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 6) return usage();
  if (std::atoi(argv[5]) == 3) {
    const int bits = std::atoi(argv[4]);
    if (bits != 32 && bits != 64) return usage();
    return solve_batch_file(argv[1], std::max(1, std::atoi(argv[2])), argv[3], bits);
  }
  const int which = std::atoi(argv[1]);
  const int avg = std::max(1, std::atoi(argv[2]));
  const int batch = std::max(1, std::atoi(argv[3]));
  const int streams = std::max(1, std::atoi(argv[4]));
  const int mode = std::atoi(argv[5]);
  blpg::matrix<double> A;
  std::vector<double> b, c;
  bool minimise = false;
  if (mode == 1) {
    if (which < 1 || which > 8) return usage();
    const char* dir = std::getenv("BLPG_BENCH_DIR");
    std::string base = std::string(dir ? dir : "benchmarks") + "/" + kNames[which - 1];
    std::string pa = base + "_A.txt", pb = base + "_B.txt", pc = base + "_C.txt";
    int32_t m = 0, n = 0;
    if (blpg_read_abc(pa.c_str(), pb.c_str(), pc.c_str(), &m, &n, nullptr, nullptr, nullptr)) {
      std::fprintf(stderr, "%s\n", blpg_last_error());
      return 1;
    }
    A.resize(m, n);
    b.resize(m);
    c.resize(n);
    if (blpg_read_abc(pa.c_str(), pb.c_str(), pc.c_str(), &m, &n, A.data(), b.data(), c.data())) {
      std::fprintf(stderr, "%s\n", blpg_last_error());
      return 1;
    }
    std::printf("Benchmark = %s\nTotal Constraints =%d   Total Variables =%d\n", kNames[which - 1],
                m, n);
    minimise = true;  // the Netlib files are minimisation problems
  } else if (mode == 2) {
    if (which < 1 || which > 1000) return usage();
    A.resize(which, which);
    b.resize(which);
    c.resize(which);
    uint64_t s = 0x9E3779B97F4A7C15ull * (uint64_t)which;
    auto next = [&s]() {
      s ^= s << 13;
      s ^= s >> 7;
      s ^= s << 17;
      return s;
    };
    for (int i = 0; i < which; ++i) {
      for (int j = 0; j < which; ++j) A(i, j) = (double)(next() % 999 + 1);
      b[i] = (double)(next() % 999 + 1);
    }
    for (int j = 0; j < which; ++j) c[j] = (double)(next() % 499 + 1);
  } else {
    return usage();
  }
  blpg::matrix<double> C(batch, A.size2());
  for (int i = 0; i < batch; ++i)
    for (size_t j = 0; j < A.size2(); ++j) C(i, j) = minimise ? -c[j] : c[j];
  // one call per run: blpg_solve_batch pipelines a large batch in chunks and
  // splits one that does not fit the device itself (the reference's
  // multiple-batch path, GPU_Tester.cu:194-238, 284-354)
  std::vector<double> result(batch);
  std::vector<int> status(batch);
  double sum = 0.0;
  for (int it = 0; it <= avg; ++it) {
    const auto t0 = std::chrono::steady_clock::now();
    blpg::Simplex s(batch, 0);
    s.setConstratint(A, b);
    try {
      s.ComputeLP(C, streams);
    } catch (const std::exception& e) {
      std::fprintf(stderr, "%s\n", e.what());
      return 1;
    }
    auto r = s.getResultAll();
    auto st = s.getStatusAll();
    for (int i = 0; i < batch; ++i) {
      result[i] = r[i];
      status[i] = st[i];
    }
    const double sec =
        std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::printf("Iter %d: Time = %.6f Seconds\n", it, sec);
    if (it > 0) sum += sec;
  }
  std::printf("\n*****GPU RESULT*****\n\nWall time (in Seconds):: GPU= %.6f  (%d LPs, %.1f LPs/s)\n",
              sum / avg, batch, batch / (sum / avg));
  std::printf("\nVERIFICATION FOR CORRECTNESS\n");
  for (int i = 0; i < std::min(batch, 10); ++i)
    std::printf("GPU: %.10f (status %d) || GPU: %.10f\n", minimise ? -result[i] : result[i],
                status[i], minimise ? -result[batch - 1 - i] : result[batch - 1 - i]);
  return 0;
}
