// Host-only harness for the CPU tests: runs the library's .mmp reader and
// setup (no CUDA calls) and prints the scaled-pair lists and the lab-frame
// multipoles so that they can be compared with the oracle.
#include <cstdio>

#include "../../openmmpol_gb300/csrc/ommp_internal.h"

using namespace ommp;

int main(int argc, char **argv) {
  if (argc != 2) return 2;
  HostModel m;
  std::string err;
  if (!read_mmp(argv[1], m, err) || !prepare_model(m, err)) {
    printf("ERR %s\n", err.c_str());
    return 1;
  }
  ScaledPairs p, u;
  build_m2d_pairs(m, p);
  build_d2d_pairs(m, u);
  printf("SIZES %d %d %d\n", m.mm, m.npol, m.ld_cart);
  for (int j = 0; j < m.npol; ++j)
    for (int k = p.ri[j]; k < p.ri[j + 1]; ++k) printf("M %d %d %.17g %.17g\n", j, p.src[k], p.sP[k], p.sD[k]);
  for (int j = 0; j < m.npol; ++j)
    for (int k = u.ri[j]; k < u.ri[j + 1]; ++k) printf("U %d %d %.17g\n", j, u.src[k], u.sP[k]);
  for (int i = 0; i < m.mm; ++i) {
    printf("Q %d", i);
    for (int c = 0; c < m.ld_cart; ++c) printf(" %.17g", m.q[(size_t)i * m.ld_cart + c]);
    printf("\n");
  }
  for (int k = 0; k < m.npol; ++k) printf("P %d %d %.17g %.17g\n", k, m.polar_mm[k], m.pol[k], m.thole[m.polar_mm[k]]);
  return 0;
}
