// Host-only harness for the CPU tests: the inner preconditioner's runs and
// near-field couplings (build_block_jacobi, build_near_field) of a .mmp
// file, printed for comparison with a brute-force search.  No CUDA call.
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
  ScaledPairs u;
  build_d2d_pairs(m, u);
  std::vector<int> info, ri, ci;
  std::vector<float> minv, blk;
  build_block_jacobi(m, u, 50.0, kMaxBlock, kBlockLinkBohr, info, minv);
  build_near_field(m, u, 50.0, info, kNearBohr, ri, ci, blk);
  printf("N %d %.17g\n", m.npol, kNearBohr);
  for (int j = 0; j < m.npol; ++j) {
    const double *p = &m.cmm[3 * (size_t)m.polar_mm[j]];
    printf("S %d %d %.17g %.17g %.17g\n", j, info[4 * (size_t)j], p[0], p[1], p[2]);
  }
  for (int j = 0; j < m.npol; ++j)
    for (int k = u.ri[j]; k < u.ri[j + 1]; ++k)
      if (u.sP[k] == 0.0) printf("Z %d %d\n", j, u.src[k]);
  for (int j = 0; j < m.npol; ++j)
    for (int e = ri[j]; e < ri[j + 1]; ++e) {
      printf("E %d %d", j, ci[e]);
      for (int k = 0; k < 9; ++k) printf(" %.9g", blk[9 * (size_t)e + k]);
      printf("\n");
    }
  return 0;
}
