// Potential and field of the system at arbitrary points (QM coupling).
//
// potential_M2E / potential_D2E / field_M2E / field_D2E of the reference
// (src/mod_electrostatics.F90:3067-3336) behind ommp_{potential,field}_
// {mmpol,mm,pol}2ext (src/mod_interface.F90:250-330): every static site's
// multipoles (charge, dipole, quadrupole for AMOEBA; charge for Wang-AL) and
// every induced dipole act on every point, with the undamped Coulomb kernel
// and no screening.  The induced dipoles seen from outside are the D set for
// the potential and (P + D) / 2 for the field (AMOEBA), the single set
// otherwise.  The results are ADDED into the caller's array, as the
// reference's routines do.
//
// One CTA of 128 threads owns 128 points; sources stream through shared
// memory in tiles of 128 records, split over blockIdx.y with the partials
// summed in a fixed order: FP64 throughout, deterministic.
#include <cmath>

#include "engine.h"
#include "log.h"
#include "pair_math.cuh"

namespace ommp {
namespace gpu {
namespace {

constexpr int EXT_TPB = 128;

// SRC 0: AMOEBA multipoles (10 per site), 1: charges, 2: dipoles (3 per site)
template <int SRC>
struct SrcWidth;
template <>
struct SrcWidth<0> {
  static constexpr int value = 10;
};
template <>
struct SrcWidth<1> {
  static constexpr int value = 1;
};
template <>
struct SrcWidth<2> {
  static constexpr int value = 3;
};

// partial[split][n][C] (C = 1 potential, 3 field)
template <bool FIELD, int SRC>
__global__ void __launch_bounds__(EXT_TPB) k_ext(int n, const double *__restrict__ cext, int m,
                                                 const Pos64 *__restrict__ spos, const double *__restrict__ sdata,
                                                 double *__restrict__ partial, int per_split, int *bad_flag) {
  constexpr int LD = SrcWidth<SRC>::value;
  constexpr int C = FIELD ? 3 : 1;
  __shared__ double s_x[EXT_TPB], s_y[EXT_TPB], s_z[EXT_TPB];
  __shared__ double s_d[EXT_TPB * LD];
  const int j = blockIdx.x * EXT_TPB + threadIdx.x;
  const bool valid = j < n;
  double px = 0, py = 0, pz = 0;
  if (valid) {
    px = cext[3 * (size_t)j];
    py = cext[3 * (size_t)j + 1];
    pz = cext[3 * (size_t)j + 2];
  }
  double acc[C];
#pragma unroll
  for (int c = 0; c < C; ++c) acc[c] = 0.0;
  int bad = 0;
  const int s0 = blockIdx.y * per_split;
  const int s1 = min(m, s0 + per_split);
  for (int t0 = s0; t0 < s1; t0 += EXT_TPB) {
    __syncthreads();
    {
      const int i = t0 + threadIdx.x;
      if (i < s1) {
        const Pos64 p = spos[i];
        s_x[threadIdx.x] = p.x;
        s_y[threadIdx.x] = p.y;
        s_z[threadIdx.x] = p.z;
      }
      for (int k = threadIdx.x; k < EXT_TPB * LD; k += EXT_TPB) {
        const size_t g = (size_t)t0 * LD + k;
        if (g < (size_t)s1 * LD) s_d[k] = sdata[g];
      }
    }
    __syncthreads();
    if (!valid) continue;
    const int cnt = min(EXT_TPB, s1 - t0);
    for (int k = 0; k < cnt; ++k) {
      const double dx = px - s_x[k], dy = py - s_y[k], dz = pz - s_z[k];
      const double r2 = fma(dx, dx, fma(dy, dy, dz * dz));
      if (r2 < 4.930380657631324e-28) {  // |r| < 100 eps: the reference stops here
        bad = 1;
        continue;
      }
      const double k1 = rinv_f64(r2, r2_f32(r2));
      const double ir2 = k1 * k1;
      const double k2 = k1 * ir2;  // r^-3
      const double *q = &s_d[k * LD];
      if (SRC == 2) {
        const double mdr = fma(q[0], dx, fma(q[1], dy, q[2] * dz));
        if (!FIELD) {
          acc[0] = fma(mdr, k2, acc[0]);
        } else {
          const double f = 3.0 * mdr * (k2 * ir2);
          acc[0] += fma(f, dx, -q[0] * k2);
          acc[C > 1 ? 1 : 0] += fma(f, dy, -q[1] * k2);
          acc[C > 2 ? 2 : 0] += fma(f, dz, -q[2] * k2);
        }
      } else if (SRC == 1) {
        if (!FIELD) {
          acc[0] = fma(q[0], k1, acc[0]);
        } else {
          const double c = q[0] * k2;
          acc[0] = fma(c, dx, acc[0]);
          acc[C > 1 ? 1 : 0] = fma(c, dy, acc[C > 1 ? 1 : 0]);
          acc[C > 2 ? 2 : 0] = fma(c, dz, acc[C > 2 ? 2 : 0]);
        }
      } else {
        const double k3 = k2 * ir2;  // r^-5
        const double mdr = fma(q[1], dx, fma(q[2], dy, q[3] * dz));
        const double qx = fma(q[4], dx, fma(q[5], dy, q[7] * dz));
        const double qy = fma(q[5], dx, fma(q[6], dy, q[8] * dz));
        const double qz = fma(q[7], dx, fma(q[8], dy, q[9] * dz));
        const double qxr = fma(qx, dx, fma(qy, dy, qz * dz));
        if (!FIELD) {
          acc[0] += q[0] * k1 + mdr * k2 + 3.0 * qxr * k3;
        } else {
          const double k4 = k3 * ir2;  // r^-7
          const double c = q[0] * k2 + 3.0 * mdr * k3 + 15.0 * qxr * k4;
          const double k3x6 = 6.0 * k3;
          acc[0] += c * dx - q[1] * k2 - k3x6 * qx;
          acc[C > 1 ? 1 : 0] += c * dy - q[2] * k2 - k3x6 * qy;
          acc[C > 2 ? 2 : 0] += c * dz - q[3] * k2 - k3x6 * qz;
        }
      }
    }
  }
  if (bad) atomicOr(bad_flag, 1);
  if (valid) {
#pragma unroll
    for (int c = 0; c < C; ++c) partial[((size_t)blockIdx.y * n + j) * C + c] = acc[c];
  }
}

// out[j][c] = sum over the nsplit partial blocks, in order
__global__ void k_ext_sum(size_t total, int nsplit, const double *__restrict__ partial, double *__restrict__ out) {
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < total; k += (size_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int p = 0; p < nsplit; ++p) s += partial[(size_t)p * total + k];
    out[k] = s;
  }
}

__global__ void k_half_sum(size_t n, const double *__restrict__ a, const double *__restrict__ b,
                           double *__restrict__ out) {
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
    out[k] = 0.5 * (a[k] + b[k]);
}

int blocks_for_ext(size_t n) {
  size_t b = (n + 255) / 256;
  if (b < 1) b = 1;
  if (b > 2432) b = 2432;
  return (int)b;
}

int ext_split(int n, int m, int sms) {
  const int blocks = (n + EXT_TPB - 1) / EXT_TPB;
  const int tiles = (m + EXT_TPB - 1) / EXT_TPB;
  int split = (4 * sms + blocks - 1) / blocks;
  if (split > tiles) split = tiles;
  return split < 1 ? 1 : split;
}

template <bool FIELD>
void launch_src(int src, int n, const double *cext, int m, const Pos64 *spos, const double *sdata, double *partial,
                int nsplit, int *bad, cudaStream_t st) {
  const int tiles = (m + EXT_TPB - 1) / EXT_TPB;
  const int per = ((tiles + nsplit - 1) / nsplit) * EXT_TPB;
  dim3 grid((n + EXT_TPB - 1) / EXT_TPB, nsplit);
  add_launch_count(1);
  if (src == 0)
    k_ext<FIELD, 0><<<grid, EXT_TPB, 0, st>>>(n, cext, m, spos, sdata, partial, per, bad);
  else if (src == 1)
    k_ext<FIELD, 1><<<grid, EXT_TPB, 0, st>>>(n, cext, m, spos, sdata, partial, per, bad);
  else
    k_ext<FIELD, 2><<<grid, EXT_TPB, 0, st>>>(n, cext, m, spos, sdata, partial, per, bad);
}

}  // namespace
}  // namespace gpu

int System::ext_props(int which, bool field, int n, const double *cext_h, double *out_h) {
  if (which < 0 || which > 2 || n < 0) {
    set_last_error("external points: 'which' must be 0 (all), 1 (static) or 2 (induced), n >= 0");
    return kErrBadArg;
  }
  const bool do_mm = which != 2 && d_.m > 0, do_pol = which != 1 && d_.n > 0;
  if (do_pol && !ipd_done_) {
    set_last_error(field ? "IPD should be computed before computing D2E field."
                         : "IPD should be computed before D2E potential.");
    return kErrInput;
  }
  if (n == 0 || (!do_mm && !do_pol)) return kOk;
  const int C = field ? 3 : 1;
  const int sms = gpu::sm_count();
  const int smm = do_mm ? gpu::ext_split(n, d_.m, sms) : 0;
  const int spol = do_pol ? gpu::ext_split(n, d_.n, sms) : 0;
  const size_t need = 3 * (size_t)n + (size_t)(smm + spol) * n * C + (size_t)n * C + 3 * (size_t)d_.n;
  if (need > ext_cap_) {
    if (ext_buf_) cudaFree(ext_buf_);
    ext_buf_ = nullptr;
    ext_cap_ = 0;
    if (cudaMalloc((void **)&ext_buf_, need * sizeof(double)) != cudaSuccess) {
      cudaGetLastError();
      set_last_error("out of device memory for the external points");
      return kErrMemory;
    }
    ext_cap_ = need;
  }
  double *cext = ext_buf_;
  double *partial = cext + 3 * (size_t)n;
  double *out = partial + (size_t)(smm + spol) * n * C;
  double *mu = out + (size_t)n * C;
  cudaMemcpyAsync(cext, cext_h, 3 * (size_t)n * sizeof(double), cudaMemcpyHostToDevice, st_);
  cudaMemsetAsync(flag_, 0, sizeof(int), st_);
  if (do_mm) {
    const int src = m_.amoeba ? 0 : 1;
    if (field)
      gpu::launch_src<true>(src, n, cext, d_.m, d_.mm_pos, d_.mm_q, partial, smm, flag_, st_);
    else
      gpu::launch_src<false>(src, n, cext, d_.m, d_.mm_pos, d_.mm_q, partial, smm, flag_, st_);
  }
  if (do_pol) {
    const size_t nv = 3 * (size_t)d_.n;
    const double *dip = ipd_;  // D set (AMOEBA) or the only set
    if (field && m_.amoeba) {
      gpu::k_half_sum<<<gpu::blocks_for_ext(nv), 256, 0, st_>>>(nv, ipd_ + nv, ipd_, mu);
      gpu::add_launch_count(1);
      dip = mu;
    }
    double *pp = partial + (size_t)smm * n * C;
    if (field)
      gpu::launch_src<true>(2, n, cext, d_.n, d_.pol_pos, dip, pp, spol, flag_, st_);
    else
      gpu::launch_src<false>(2, n, cext, d_.n, d_.pol_pos, dip, pp, spol, flag_, st_);
  }
  gpu::k_ext_sum<<<gpu::blocks_for_ext((size_t)n * C), 256, 0, st_>>>((size_t)n * C, smm + spol, partial, out);
  gpu::add_launch_count(1);
  std::vector<double> h((size_t)n * C);
  int flag = 0;
  cudaMemcpyAsync(h.data(), out, h.size() * sizeof(double), cudaMemcpyDeviceToHost, st_);
  cudaMemcpyAsync(&flag, flag_, sizeof(int), cudaMemcpyDeviceToHost, st_);
  int st = check(cudaStreamSynchronize(st_), "external points");
  if (st) return st;
  if (flag) {
    set_last_error(
        "Requesting Coulomb kernel for two atoms placed in the same point, this could be an internal bug or "
        "a problem in your input file, please check.");
    return kErrNumeric;
  }
  for (size_t k = 0; k < h.size(); ++k) out_h[k] += h[k];
  return kOk;
}

}  // namespace ommp
