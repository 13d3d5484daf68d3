// Pair arithmetic shared by the FP64/FP32 pair kernels (kernels.cu) and
// the double-single kernels (ds_kernels.cu): FP64 reciprocal square root from an
// FP32 seed, the FP32 damping pre-tests, and the damped dipole-field factors
// (Thole damping of the reference, src/mod_electrostatics.F90:978-1095).
#pragma once

#include <type_traits>

#include <cuda_runtime.h>

#include "kernels.h"

namespace ommp {
namespace gpu {
namespace {

// 1/sqrt(r2) in FP64 from the FP32 hardware estimate and one Newton-Raphson
// step y <- y + y (1 - r2 y^2) / 2 (quadratic convergence: the ~2^-23
// relative error of the seed becomes ~2e-14).  GB300 runs FP64 at 1/64 of
// the FP32 rate, so the seed and the conversions cost less than a full-
// precision FP64 reciprocal square root.
__device__ __forceinline__ double rinv_f64(double r2, float r2f) {
  double y = (double)rsqrtf(r2f);
  double e = fma(-r2, y * y, 1.0);
  return fma(0.5 * y, e, y);
}

// Damping pre-test in FP32 for the FP64 kernels.  AMOEBA damps when
// a u^3 < thr with u = r / (thole_t thole_s); squared: a^2 q^3 < thr^2 with
// q = r^2 (1/thole_t)^2 (1/thole_s)^2.  The FP32 test carries a relative
// margin of 1e-5 (FP32 rounding of q is ~1e-7), so every pair that the exact
// FP64 test damps enters the branch, where the FP64 test decides.
__device__ __forceinline__ bool maybe_damped_amoeba(float r2f, float2 wat, float2 was, float thr2m) {
  float q = r2f * wat.x * was.x;
  return fminf(wat.y, was.y) * (q * q * q) < thr2m;
}
// Wang-AL damps when r < thole_t thole_s, i.e. q < 1.
__device__ __forceinline__ bool maybe_damped_wang(float r2f, float2 wat, float2 was) {
  return r2f * wat.x * was.x < 1.00001f;
}

// ---------------------------------------------------------------------------
// dipole-dipole field
// ---------------------------------------------------------------------------
template <typename T>
struct Vec4;
template <>
struct Vec4<double> {
  using type = Pos64;
};
template <>
struct Vec4<float> {
  using type = float4;
};

__device__ __forceinline__ double fast_rsqrt(double x) { return rsqrt(x); }
__device__ __forceinline__ float fast_rsqrt(float x) { return rsqrtf(x); }
__device__ __forceinline__ double fast_exp(double x) { return exp(x); }
__device__ __forceinline__ float fast_exp(float x) { return __expf(x); }

// Damped r^-3 and 3 r^-5 factors of the dipole field for one pair.
template <typename T, bool AMOEBA>
__device__ __forceinline__ void dd_kernel(T r2, T wt, T ws, T at, T as, T thr, T &k3, T &k5x3) {
  T rinv = fast_rsqrt(r2);
  T ir2 = rinv * rinv;
  k3 = rinv * ir2;
  T k5 = k3 * ir2;
  T u = r2 * rinv * (wt * ws);
  if (AMOEBA) {
    T au3 = fmin(at, as) * u * u * u;
    if (au3 < thr) {
      T e = fast_exp(-au3);
      k3 *= T(1) - e;
      k5 *= T(1) - (T(1) + au3) * e;
    }
  } else {
    if (u < T(1)) {
      T u3 = u * u * u;
      T u4 = u3 * u;
      k3 *= T(4) * u3 - T(3) * u4;
      k5 *= u4;
    }
  }
  k5x3 = T(3) * k5;
}

// The pair factors in the precision of the kernel.  FP64: reciprocal square
// root from the FP32 seed plus one Newton step and the FP32 damping
// pre-test, so that only the arithmetic that needs FP64 runs on GB300's
// FP64 pipe.  FP32: the plain formulas.
template <typename T, bool AMOEBA>
__device__ __forceinline__ void dd_pair(T r2, T wt, T ws, T at, T as, float2 wat, float2 was, T thr,
                                        float thr2m, T &k3, T &k5x3) {
  if constexpr (std::is_same<T, double>::value) {
    float r2f = (float)r2;
    double rinv = rinv_f64(r2, r2f);
    double ir2 = rinv * rinv;
    k3 = rinv * ir2;
    double k5 = k3 * ir2;
    if (AMOEBA) {
      if (maybe_damped_amoeba(r2f, wat, was, thr2m)) {
        double u = r2 * rinv * (wt * ws);
        double au3 = fmin(at, as) * u * u * u;
        if (au3 < thr) {
          double e = exp(-au3);
          k3 *= 1.0 - e;
          k5 *= 1.0 - (1.0 + au3) * e;
        }
      }
    } else {
      if (maybe_damped_wang(r2f, wat, was)) {
        double u = r2 * rinv * (wt * ws);
        if (u < 1.0) {
          double u3 = u * u * u;
          double u4 = u3 * u;
          k3 *= 4.0 * u3 - 3.0 * u4;
          k5 *= u4;
        }
      }
    }
    k5x3 = 3.0 * k5;
  } else {
    dd_kernel<T, AMOEBA>(r2, wt, ws, at, as, thr, k3, k5x3);
  }
}


}  // namespace
}  // namespace gpu
}  // namespace ommp
