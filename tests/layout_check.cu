// Host-only check of the per-LP shared-memory layout (blpg::dev::Layout, the
// same code the plans and the solve kernel evaluate): for every shape and
// thread count swept, the norm region holds the FP32 steepest-edge partial
// sums when asked to, grows the layout by no more than that needs, and every
// region the kernel addresses with 16-byte accesses starts 16-byte aligned.
// Prints "ok <cases>" or the first failing case; exit status 0 on success.
#include <cstdio>

#include "../simplexprojects_gb300/csrc/blpg_solver.cuh"

using namespace blpg::dev;

int main() {
  long cases = 0;
  for (int m = 1; m <= 256; m += 5)
    for (int n = 1; n <= 512; n += 7)
      for (int na = 0; na <= 2; na += 2)
        for (int nt = 64; nt <= 512; nt += 32) {
          const Geom g(m, n, na, 1, 4);
          if (g.nl > nt) continue;  // a class always has a row of lanes per CTA
          const int G = nt / g.nl < kMaxNormGroups ? nt / g.nl : kMaxNormGroups;
          const int need = G * g.cw * 4;
          const Layout base(m, g.ldw, n + m + na, 4, 1);
          const Layout grown(m, g.ldw, n + m + na, 4, 1, need);
          ++cases;
          const int growth = grown.total - base.total;
          const int extra = need > base.gbytes ? need - base.gbytes : 0;
          bool ok = grown.gbytes >= need && grown.gbytes >= base.gbytes && growth >= 0 &&
                    growth <= extra + 15 && (extra > 0 || growth == 0) &&
                    grown.gam % 16 == 0 && base.gam % 16 == 0 && grown.tab % 16 == 0 &&
                    grown.ext % 16 == 0 && grown.gam == base.gam &&
                    grown.tab == base.tab && grown.vpos == base.vpos && grown.ext == base.ext;
          // the partial sums stay inside the allocation
          ok = ok && grown.gam + need <= grown.total;
          if (!ok) {
            std::printf("fail m=%d n=%d na=%d nt=%d: need %d, gbytes %d -> %d, total %d -> %d\n", m,
                        n, na, nt, need, base.gbytes, grown.gbytes, base.total, grown.total);
            return 1;
          }
        }
  std::printf("ok %ld\n", cases);
  return 0;
}
