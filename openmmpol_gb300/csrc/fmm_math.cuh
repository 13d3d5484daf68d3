// Cartesian multipole algebra of the fast multipole method (fmm.cu).
//
// Potentials 1/r are expanded in Cartesian Taylor series.  Multi-indices
// g = (a, b, c) of order |g| = a + b + c <= P are numbered in graded order
// (order 0, then the three of order 1, ...; inside an order by decreasing a,
// then decreasing b); term(a, b, c) gives the number.
//
//   multipole of sources about c      M_g = sum_i w_i(g), with for a charge
//                                     w = q v^g / g! and for a dipole mu
//                                     w = sum_k mu_k v^(g - e_k) / (g - e_k)!
//                                     (v = y_i - c), so that the potential
//                                     far away is sum_g (-1)^|g| M_g D_g(x - c)
//   derivatives of 1/r                D_g(R) = d^g (1/|R|), from the
//                                     recurrence n r^2 D_g = -(2n - 1)
//                                     sum_k g_k R_k D_(g - e_k) - (n - 1)
//                                     sum_k g_k (g_k - 1) D_(g - 2 e_k)
//   local expansion about d           phi(x) = sum_h L_h (x - d)^h with
//                                     L_h = (1 / h!) sum_g (-1)^|g| M_g
//                                     D_(g + h)(d - c), |g| + |h| <= p (so
//                                     derivatives to order p)
//   translations                      M2M: M_g(c) = sum_(k <= g) M_k(c')
//                                     s^(g - k) / (g - k)!, s = c' - c;
//                                     L2L: L_k(d') = sum_(h >= k) L_h(d)
//                                     h! / (k! (h - k)!) t^(h - k), t = d' - d
//   field at a target                 E = -grad phi = -sum_h L_h grad (x - d)^h
// (the expansions of the fast multipole method of Greengard and Rokhlin,
// written with Cartesian tensors as in the Cartesian treecode / FMM
// literature; the recurrence is the standard one for derivatives of 1/r).
#pragma once

#include <cmath>

#if defined(__CUDACC__)
#define FMM_HD __host__ __device__ __forceinline__
#else
#define FMM_HD inline
#endif

namespace ommp {
namespace fmm {

constexpr int kMaxOrder = 12;            // expansion order p

// number of multi-indices of order <= n
FMM_HD constexpr int nterms(int n) { return (n + 1) * (n + 2) * (n + 3) / 6; }

// graded index of (a, b, c)
FMM_HD int term(int a, int b, int c) {
  const int n = a + b + c;
  // inside order n: decreasing a, then decreasing b
  const int before_a = (n - a) * (n - a + 1) / 2;  // entries with larger a
  return nterms(n - 1) + before_a + (n - a - b);
}

// exponents of the graded index t (host-side enumeration; device code uses
// tables built from it)
inline void exponents(int t, int &a, int &b, int &c) {
  int n = 0;
  while (nterms(n) <= t) ++n;
  int r = t - nterms(n - 1);
  for (a = n; a >= 0; --a) {
    const int cnt = n - a + 1;
    if (r < cnt) break;
    r -= cnt;
  }
  b = n - a - r;
  c = n - a - b;
}

// D_g(R) for all |g| <= nmax into D[nterms(nmax)]
FMM_HD void derivatives(double x, double y, double z, int nmax, double *D) {
  const double r2 = x * x + y * y + z * z;
  const double ir2 = 1.0 / r2;
  D[0] = sqrt(ir2);
  const double R[3] = {x, y, z};
  for (int n = 1; n <= nmax; ++n) {
    const double f1 = -(2.0 * n - 1.0) / n * ir2, f2 = -(n - 1.0) / n * ir2;
    for (int a = n; a >= 0; --a)
      for (int b = n - a; b >= 0; --b) {
        const int c = n - a - b;
        const int g[3] = {a, b, c};
        double s1 = 0.0, s2 = 0.0;
        for (int k = 0; k < 3; ++k) {
          if (g[k] < 1) continue;
          int h[3] = {a, b, c};
          h[k] -= 1;
          s1 += g[k] * R[k] * D[term(h[0], h[1], h[2])];
          if (g[k] >= 2) {
            h[k] -= 1;
            s2 += g[k] * (g[k] - 1.0) * D[term(h[0], h[1], h[2])];
          }
        }
        D[term(a, b, c)] = f1 * s1 + f2 * s2;
      }
  }
}

// powers v^k / k! for k = 0..n of one coordinate
FMM_HD void scaled_powers(double v, int n, double *p) {
  p[0] = 1.0;
  for (int k = 1; k <= n; ++k) p[k] = p[k - 1] * v / k;
}

}  // namespace fmm
}  // namespace ommp
