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

// FP32 value of a non-negative FP64 r2 by integer operations (exponent
// rebias, mantissa rounded to nearest), so that the conversion does not
// take a slot of GB300's narrow FP64 pipe.  Values below the FP32 normal
// range (only coincident sites) become 0.
__device__ __forceinline__ float r2_f32(double r2) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(r2) + (1ull << 28);
  const unsigned hi = (unsigned)(b >> 32);
  // (b >> 29) holds sign | exponent | 23 mantissa bits; subtracting
  // (1023 - 127) << 23 modulo 2^32 (0xC0000000) rebiases the exponent
  const unsigned f = (unsigned)(b >> 29) - 0xC0000000u;
  return __uint_as_float(hi < 0x38100000u ? 0u : f);
}

// 1/sqrt(r2) in FP64 from the FP32 hardware estimate and one Newton-Raphson
// step y <- y + (y / 2) (1 - r2 y^2) (quadratic convergence: the ~2^-23
// relative error of the seed becomes ~2e-14).  GB300 runs FP64 at 1/64 of
// the FP32 rate, so the seed costs less than a full-precision FP64
// reciprocal square root.  The seed y and y / 2 are widened to FP64 by
// integer operations (exponent rebias; infinities and NaNs kept), so the
// step takes three FP64 operations.
__device__ __forceinline__ double rinv_f64(double r2, float r2f) {
  const unsigned u = __float_as_uint(rsqrtf(r2f));
  const bool special = (u & 0x7F800000u) == 0x7F800000u;
  const unsigned hi = special ? (0x7FF00000u | (u >> 3)) : (u >> 3) + 0x38000000u;
  const unsigned lo = u << 29;
  const double y = __hiloint2double((int)hi, (int)lo);
  const double hy = __hiloint2double((int)(special ? hi : hi - 0x00100000u), (int)lo);
  const double e = fma(-r2, y * y, 1.0);
  return fma(hy, e, y);
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

// Damped r^-3 and r^-5 factors of one pair in FP64: reciprocal square root
// from the FP32 seed plus one Newton step and the FP32 damping pre-test, so
// that only the arithmetic that needs FP64 runs on GB300's FP64 pipe.
template <bool AMOEBA>
__device__ __forceinline__ void dd_pair_f64(double r2, double wt, double ws, double at, double as, float2 wat,
                                            float2 was, double thr, float thr2m, double &k3, double &k5) {
  const float r2f = r2_f32(r2);
  const double rinv = rinv_f64(r2, r2f);
  const double ir2 = rinv * rinv;
  k3 = rinv * ir2;
  k5 = k3 * ir2;
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
}

// The pair factors k3 and 3 k5 in the precision of the kernel (FP64:
// dd_pair_f64; FP32: the plain formulas).
template <typename T, bool AMOEBA>
__device__ __forceinline__ void dd_pair(T r2, T wt, T ws, T at, T as, float2 wat, float2 was, T thr,
                                        float thr2m, T &k3, T &k5x3) {
  if constexpr (std::is_same<T, double>::value) {
    double k5;
    dd_pair_f64<AMOEBA>(r2, wt, ws, at, as, wat, was, thr, thr2m, k3, k5);
    k5x3 = 3.0 * k5;
  } else {
    dd_kernel<T, AMOEBA>(r2, wt, ws, at, as, thr, k3, k5x3);
  }
}

// Field of a static multipole (charge; + dipole and quadrupole for AMOEBA,
// q[0..9]) at a polarizable target, d = target - source, Thole-damped
// (elec_prop_M2D pair term, src/mod_electrostatics.F90:2579-2731).
template <bool AMOEBA>
__device__ __forceinline__ void m2d_pair_f64(double dx, double dy, double dz, double wt, double ws,
                                             double at, double as, float2 wat, float2 was,
                                             const double *q, double thr, float thr2m,
                                             double &ex, double &ey, double &ez) {
  double r2 = dx * dx + dy * dy + dz * dz;
  float r2f = r2_f32(r2);
  double rinv = rinv_f64(r2, r2f);
  double ir2 = rinv * rinv;
  double k3 = rinv * ir2;
  if (AMOEBA) {
    double k5 = k3 * ir2;
    double k7 = k5 * ir2;
    if (maybe_damped_amoeba(r2f, wat, was, thr2m)) {
      double u = r2 * rinv * (wt * ws);  // r / (thole_t thole_s)
      double au3 = fmin(at, as) * u * u * u;
      if (au3 < thr) {
        double e = exp(-au3);
        k3 *= 1.0 - e;
        k5 *= 1.0 - (1.0 + au3) * e;
        k7 *= 1.0 - (1.0 + au3 + 0.6 * au3 * au3) * e;
      }
    }
    double mdr = q[1] * dx + q[2] * dy + q[3] * dz;
    double qx = q[4] * dx + q[5] * dy + q[7] * dz;
    double qy = q[5] * dx + q[6] * dy + q[8] * dz;
    double qz = q[7] * dx + q[8] * dy + q[9] * dz;
    double qxr = qx * dx + qy * dy + qz * dz;
    double c = q[0] * k3 + 3.0 * mdr * k5 + 15.0 * qxr * k7;
    double k5x6 = 6.0 * k5;
    ex += c * dx - q[1] * k3 - k5x6 * qx;
    ey += c * dy - q[2] * k3 - k5x6 * qy;
    ez += c * dz - q[3] * k3 - k5x6 * qz;
  } else {
    if (maybe_damped_wang(r2f, wat, was)) {
      double u = r2 * rinv * (wt * ws);
      if (u < 1.0) {
        double u3 = u * u * u;
        k3 *= 4.0 * u3 - 3.0 * u3 * u;
      }
    }
    double c = q[0] * k3;
    ex += c * dx;
    ey += c * dy;
    ez += c * dz;
  }
}

// The all-pairs form of m2d_pair_f64: the source record is staged once per
// tile as m2d_stage writes it (q, mu, 3 mu, 15 Q: 13 values for AMOEBA, the
// charge alone otherwise) and the field is kept as three sums, a = sum c d,
// b = sum k3 mu, t = sum k5 (15 Q) d, so that E = a - b - 0.4 t (m2d_field)
// and every accumulation is one FMA: 40 FP64 operations per AMOEBA pair.
constexpr int M2D_SLD = 13;

template <bool AMOEBA>
__device__ __forceinline__ void m2d_stage(const double *q, double *o) {
  o[0] = q[0];
  if (!AMOEBA) return;
  for (int c = 0; c < 3; ++c) {
    o[1 + c] = q[1 + c];
    o[4 + c] = 3.0 * q[1 + c];
  }
  for (int c = 0; c < 6; ++c) o[7 + c] = 15.0 * q[4 + c];
}

template <bool AMOEBA>
__device__ __forceinline__ void m2d_pair_acc(double dx, double dy, double dz, double wt, double ws, double at,
                                             double as, float2 wat, float2 was, const double *q, double thr,
                                             float thr2m, double *acc) {
  const double r2 = dx * dx + dy * dy + dz * dz;
  const float r2f = r2_f32(r2);
  const double rinv = rinv_f64(r2, r2f);
  const double ir2 = rinv * rinv;
  double k3 = rinv * ir2;
  if (AMOEBA) {
    double k5 = k3 * ir2;
    double k7 = k5 * ir2;
    if (maybe_damped_amoeba(r2f, wat, was, thr2m)) {
      double u = r2 * rinv * (wt * ws);  // r / (thole_t thole_s)
      double au3 = fmin(at, as) * u * u * u;
      if (au3 < thr) {
        double e = exp(-au3);
        k3 *= 1.0 - e;
        k5 *= 1.0 - (1.0 + au3) * e;
        k7 *= 1.0 - (1.0 + au3 + 0.6 * au3 * au3) * e;
      }
    }
    const double mdr3 = q[4] * dx + q[5] * dy + q[6] * dz;
    const double tx = q[7] * dx + q[8] * dy + q[10] * dz;
    const double ty = q[8] * dx + q[9] * dy + q[11] * dz;
    const double tz = q[10] * dx + q[11] * dy + q[12] * dz;
    const double qxr = tx * dx + ty * dy + tz * dz;
    const double c = fma(qxr, k7, fma(mdr3, k5, q[0] * k3));
    acc[0] = fma(c, dx, acc[0]);
    acc[1] = fma(c, dy, acc[1]);
    acc[2] = fma(c, dz, acc[2]);
    acc[3] = fma(k3, q[1], acc[3]);
    acc[4] = fma(k3, q[2], acc[4]);
    acc[5] = fma(k3, q[3], acc[5]);
    acc[6] = fma(k5, tx, acc[6]);
    acc[7] = fma(k5, ty, acc[7]);
    acc[8] = fma(k5, tz, acc[8]);
  } else {
    if (maybe_damped_wang(r2f, wat, was)) {
      double u = r2 * rinv * (wt * ws);
      if (u < 1.0) {
        double u3 = u * u * u;
        k3 *= 4.0 * u3 - 3.0 * u3 * u;
      }
    }
    const double c = q[0] * k3;
    acc[0] = fma(c, dx, acc[0]);
    acc[1] = fma(c, dy, acc[1]);
    acc[2] = fma(c, dz, acc[2]);
  }
}

template <bool AMOEBA>
__device__ __forceinline__ void m2d_field(const double *acc, double &ex, double &ey, double &ez) {
  if (AMOEBA) {
    ex = acc[0] - acc[3] - 0.4 * acc[6];
    ey = acc[1] - acc[4] - 0.4 * acc[7];
    ez = acc[2] - acc[5] - 0.4 * acc[8];
  } else {
    ex = acc[0];
    ey = acc[1];
    ez = acc[2];
  }
}

// |r| below 100 machine epsilons, r2 < 4.9e-28 (coincident sites), tested on
// the high word of the non-negative r2 (integer compare, no FP64 instruction)
__device__ __forceinline__ bool coincident(double r2) { return __double2hiint(r2) < 0x3a436930; }

// Per-site 128-bit fixed-point accumulators of the symmetric products
// (kernels.cu, ds_kernels.cu): integer addition is exact and associative,
// so the sums do not depend on the order of the CTAs.
// v added exactly into the two-word fixed-point value hi * 2^-16 + lo * 2^-80
// (hi two's complement, lo unsigned).  A value that is not finite or not
// below 2^36 in magnitude sets *bad instead (the whole product is then NaN).
__device__ __forceinline__ void fixed_add(unsigned long long *lo, unsigned long long *hi, double v,
                                          unsigned long long *bad) {
  if (!(fabs(v) < 68719476736.0)) {
    atomicOr(bad, 1ull);
    return;
  }
  const double s = v * 65536.0;  // exact
  double fl = floor(s);
  double fr = s - fl;  // exact, in [0, 1]
  if (fr >= 1.0) {     // s - floor(s) rounded up to 1 for tiny negative s
    fr = 0.0;
    fl += 1.0;
  }
  const unsigned long long h = (unsigned long long)(long long)fl;
  const unsigned long long l = (unsigned long long)(fr * 18446744073709551616.0);
  const unsigned long long old = atomicAdd(lo, l);
  atomicAdd(hi, h + (old + l < old ? 1ull : 0ull));
}

__device__ __forceinline__ double fixed_value(unsigned long long lo, unsigned long long hi) {
  return ((double)(long long)hi + (double)lo * 5.421010862427522e-20) * 1.52587890625e-05;
}

}  // namespace
}  // namespace gpu
}  // namespace ommp
