// Double-single pair passes of the polarization-energy gradient.
//
// The FP64 all-pairs pass of grad.cu runs GB300's FP64 pipe at ~90% and is
// bound by it (~207 FP64 instructions per pair).  These kernels evaluate the
// same unscaled pair sums with every quantity carried in double-single
// (ds_math.cuh), on the FP32 pipes, split in two passes so that each keeps
// its accumulators in registers:
//   k_grad_ds_mp   polarizable targets x static sources: the field gradient
//                  of the static multipoles (g0)
//   k_grad_ds_dip  static targets x polarizable sources: the field gradients
//                  of the D and P dipoles (hd, hp), the field of the mean
//                  dipole (e) and the target's quadrupole contracted with its
//                  field Hessian (h)
// The tensor formulas are grad_math.cuh's, instantiated on the double-single
// type.  Source tiles whose bounding box stays beyond the Thole damping range
// of the CTA's targets skip the damping test; in the others each pair is
// pre-tested in FP32 and its Thole factors formed in FP64.  Per tile the
// double-single sums go into FP64 sums (registers for the first pass,
// per-thread shared-memory slots for the second), and the split partials use
// the layout that k_grad_finish reads: [split][component][static site].
//
// Built with --fmad=false and -ftz=true like ds_kernels.cu.
#include <algorithm>
#include <cmath>

#include "ds_math.cuh"
#include "grad_math.cuh"
#include "kernels.h"
#include "pair_math.cuh"

namespace ommp {
namespace gpu {

namespace {

constexpr int GD_TPB = 128;
constexpr int GD_TILE = 128;

// Thole factors l3, l5, l7, l9 at u = r / (thole_t thole_s) (the damping of
// damped_coulomb_kernel, src/mod_electrostatics.F90:1018-1095)
template <bool AMOEBA>
__device__ __forceinline__ void damp_factors(double u, double a, double thr, double &f3, double &f5, double &f7,
                                             double &f9) {
  f3 = f5 = f7 = f9 = 1.0;
  if (AMOEBA) {
    const double au3 = a * u * u * u;
    if (au3 < thr) {
      const double e = exp(-au3);
      const double au6 = au3 * au3;
      f3 = 1.0 - e;
      f5 = 1.0 - (1.0 + au3) * e;
      f7 = 1.0 - (1.0 + au3 + 0.6 * au6) * e;
      f9 = 1.0 - (1.0 + au3 + (18.0 / 35.0) * au6 + (9.0 / 35.0) * au6 * au3) * e;
    }
  } else if (u < 1.0) {
    const double u3 = u * u * u, u4 = u3 * u;
    f3 = 4.0 * u3 - 3.0 * u4;
    f5 = u4;
    f7 = 0.2 * u4;
  }
}

struct DsK {
  dsf dx, dy, dz, k3, k5, k7, k9;
};

// d = target - source and the (damped) inverse powers; false for coincident
// sites (NEAR only: far tiles hold none)
template <bool NEAR, bool AMOEBA>
__device__ __forceinline__ bool ds_grad_geom(const float4 &th, const float4 &tl, const float4 &sh, const float4 &sl,
                                             double wt, double ws, double at, double as, float2 wat, float2 was,
                                             double thr, float thr2m, DsK &g) {
  g.dx = ds_diff(th.x, tl.x, sh.x, sl.x);
  g.dy = ds_diff(th.y, tl.y, sh.y, sl.y);
  g.dz = ds_diff(th.z, tl.z, sh.z, sl.z);
  const dsf dx = g.dx, dy = g.dy, dz = g.dz;
  float px = dx.h * dx.h, py = dy.h * dy.h, pz = dz.h * dz.h;
  float ex = fmaf(dx.h + dx.h, dx.l, fmaf(dx.h, dx.h, -px));
  float ey = fmaf(dy.h + dy.h, dy.l, fmaf(dy.h, dy.h, -py));
  float ez = fmaf(dz.h + dz.h, dz.l, fmaf(dz.h, dz.h, -pz));
  const dsf sa = two_sum(px, py);
  const dsf sb = two_sum(sa.h, pz);
  const dsf r2 = fast_two_sum(sb.h, ((ex + ey) + ez) + (sa.l + sb.l));
  if (NEAR && r2.h < 4.9e-28f) return false;
  const dsf rinv = ds_rsqrt(r2);
  const dsf ir2 = ds_sqr(rinv);
  g.k3 = ds_mul(rinv, ir2);
  g.k5 = ds_mul(g.k3, ir2);
  g.k7 = ds_mul(g.k5, ir2);
  g.k9 = ds_mul(g.k7, ir2);
  if (NEAR) {
    const bool maybe = AMOEBA ? maybe_damped_amoeba(r2.h, wat, was, thr2m) : maybe_damped_wang(r2.h, wat, was);
    if (maybe) {
      const double u = sqrt((double)r2.h + (double)r2.l) * (wt * ws);
      double f3, f5, f7, f9;
      damp_factors<AMOEBA>(u, fmin(at, as), thr, f3, f5, f7, f9);
      g.k3 = ds_mul(g.k3, to_ds(f3));
      g.k5 = ds_mul(g.k5, to_ds(f5));
      g.k7 = ds_mul(g.k7, to_ds(f7));
      if (AMOEBA) g.k9 = ds_mul(g.k9, to_ds(f9));
    }
  }
  return true;
}

// the CTA's targets all lie in one 128-site tile: distance^2 between its box
// and the source tile's box
__device__ __forceinline__ float box_gap2(const float4 *tbox, int ttile, const float4 *sbox, int stile) {
  const float4 blo = tbox[2 * ttile], bhi = tbox[2 * ttile + 1];
  const float4 slo = sbox[2 * stile], shi = sbox[2 * stile + 1];
  const float gx = fmaxf(0.f, fmaxf(slo.x - bhi.x, blo.x - shi.x));
  const float gy = fmaxf(0.f, fmaxf(slo.y - bhi.y, blo.y - shi.y));
  const float gz = fmaxf(0.f, fmaxf(slo.z - bhi.z, blo.z - shi.z));
  return gx * gx + gy * gy + gz * gz;
}

// polarizable targets j x static sources: g0 -> partial[split][6][mm] at the
// target's static index
template <bool AMOEBA>
__global__ void __launch_bounds__(GD_TPB) k_grad_ds_mp(DevSites s, double *__restrict__ partial, int per_split,
                                                       float thr2m, int *err) {
  constexpr int LD = AMOEBA ? 10 : 1;
  __shared__ float4 s_ph[GD_TILE], s_pl[GD_TILE];
  __shared__ float s_qh[GD_TILE * LD], s_ql[GD_TILE * LD];
  __shared__ double s_w[GD_TILE], s_a[GD_TILE];
  __shared__ float2 s_wa[GD_TILE];
  const int j = blockIdx.x * GD_TPB + threadIdx.x;
  const bool valid = j < s.n;
  const float4 th = valid ? s.pol_pos32[j] : make_float4(0.f, 0.f, 0.f, 0.f);
  const float4 tl = valid ? s.pol_pos32lo[j] : make_float4(0.f, 0.f, 0.f, 0.f);
  const int tm = valid ? s.polar_mm[j] : -1;
  const double wt = valid ? s.pol_pos[j].w : 0.0, at = valid && AMOEBA ? s.pol_a[j] : 0.0;
  const float2 wat = valid ? s.pol_wa32[j] : make_float2(0.f, 0.f);
  double sum[6] = {0, 0, 0, 0, 0, 0};
  int bad = 0;
  const int s0 = blockIdx.y * per_split;
  const int s1 = min(s.m, s0 + per_split);
  for (int t0 = s0; t0 < s1; t0 += GD_TILE) {
    __syncthreads();
    {
      const int k = threadIdx.x, i = t0 + k;
      if (i < s1) {
        s_ph[k] = s.mm_pos32[i];
        s_pl[k] = s.mm_pos32lo[i];
        s_w[k] = s.mm_pos[i].w;
        s_a[k] = AMOEBA ? s.mm_a[i] : 0.0;
        s_wa[k] = s.mm_wa32[i];
#pragma unroll
        for (int c = 0; c < LD; ++c) {
          const double v = s.mm_q[(size_t)i * LD + c];
          const float h = (float)v;
          s_qh[k * LD + c] = h;
          s_ql[k * LD + c] = (float)(v - (double)h);
        }
      }
    }
    __syncthreads();
    const int cnt = min(GD_TILE, s1 - t0);
    const bool far_tile = box_gap2(s.tile_box32, blockIdx.x, s.mm_tile_box32, t0 / GD_TILE) > s.m2d_r2max32;
    dsf acc[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) acc[c] = dsf{0.f, 0.f};
    if (valid) {
#pragma unroll 1
      for (int k = 0; k < cnt; ++k) {
        DsK g;
        if (far_tile) {
          ds_grad_geom<false, AMOEBA>(th, tl, s_ph[k], s_pl[k], 0.0, 0.0, 0.0, 0.0, wat, wat, 0.0, 0.f, g);
        } else {
          if (t0 + k == tm) continue;
          if (!ds_grad_geom<true, AMOEBA>(th, tl, s_ph[k], s_pl[k], wt, s_w[k], at, s_a[k], wat, s_wa[k], s.damp_thr,
                                          thr2m, g)) {
            bad = 1;
            continue;
          }
        }
        dsf q[LD];
#pragma unroll
        for (int c = 0; c < LD; ++c) q[c] = dsf{s_qh[k * LD + c], s_ql[k * LD + c]};
        gradmath::multipole_grad<AMOEBA>(q, g.dx, g.dy, g.dz, g.k3, g.k5, g.k7, g.k9, gradmath::One{}, acc);
      }
    }
#pragma unroll
    for (int c = 0; c < 6; ++c) sum[c] += (double)acc[c].h + (double)acc[c].l;
  }
  if (bad) atomicOr(err, 1);
  if (valid) {
    double *o = partial + (size_t)blockIdx.y * 6 * s.m + tm;
#pragma unroll
    for (int c = 0; c < 6; ++c) o[(size_t)c * s.m] = sum[c];
  }
}

// static targets t x polarizable sources: hd (hp), e (h) -> partial[split][ND][mm]
template <bool AMOEBA>
__global__ void __launch_bounds__(GD_TPB) k_grad_ds_dip(DevSites s, const double *__restrict__ ipd,
                                                        double *__restrict__ partial, int per_split, float thr2m,
                                                        int *err) {
  constexpr int NS = AMOEBA ? 2 : 1;        // dipole sets
  constexpr int ND = AMOEBA ? 18 : 9;       // hd[6] (hp[6]) e[3] (h[3])
  __shared__ float4 s_ph[GD_TILE], s_pl[GD_TILE];
  __shared__ float s_mh[GD_TILE * 3 * NS], s_ml[GD_TILE * 3 * NS];
  __shared__ double s_w[GD_TILE], s_a[GD_TILE];
  __shared__ float2 s_wa[GD_TILE];
  __shared__ int s_pm[GD_TILE];
  __shared__ double s_sum[ND * GD_TPB];
  const int t = blockIdx.x * GD_TPB + threadIdx.x;
  const bool valid = t < s.m;
  const float4 th = valid ? s.mm_pos32[t] : make_float4(0.f, 0.f, 0.f, 0.f);
  const float4 tl = valid ? s.mm_pos32lo[t] : make_float4(0.f, 0.f, 0.f, 0.f);
  const double wt = valid ? s.mm_pos[t].w : 0.0, at = valid && AMOEBA ? s.mm_a[t] : 0.0;
  const float2 wat = valid ? s.mm_wa32[t] : make_float2(0.f, 0.f);
  dsf Q[6], trq{0.f, 0.f};
  if (AMOEBA) {
#pragma unroll
    for (int c = 0; c < 6; ++c) Q[c] = valid ? to_ds(s.mm_q[(size_t)t * 10 + 4 + c]) : dsf{0.f, 0.f};
    trq = Q[0] + Q[2] + Q[5];
  }
#pragma unroll
  for (int c = 0; c < ND; ++c) s_sum[c * GD_TPB + threadIdx.x] = 0.0;
  int bad = 0;
  const int s0 = blockIdx.y * per_split;
  const int s1 = min(s.n, s0 + per_split);
  for (int t0 = s0; t0 < s1; t0 += GD_TILE) {
    __syncthreads();
    {
      const int k = threadIdx.x, i = t0 + k;
      if (i < s1) {
        s_ph[k] = s.pol_pos32[i];
        s_pl[k] = s.pol_pos32lo[i];
        s_w[k] = s.pol_pos[i].w;
        s_a[k] = AMOEBA ? s.pol_a[i] : 0.0;
        s_wa[k] = s.pol_wa32[i];
        s_pm[k] = s.polar_mm[i];
#pragma unroll
        for (int set = 0; set < NS; ++set)
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            const double v = ipd[((size_t)set * s.n + i) * 3 + c];
            const float h = (float)v;
            s_mh[(k * NS + set) * 3 + c] = h;
            s_ml[(k * NS + set) * 3 + c] = (float)(v - (double)h);
          }
      }
    }
    __syncthreads();
    const int cnt = min(GD_TILE, s1 - t0);
    const bool far_tile = box_gap2(s.mm_tile_box32, blockIdx.x, s.tile_box32, t0 / GD_TILE) > s.m2d_r2max32;
    dsf acc[ND];
#pragma unroll
    for (int c = 0; c < ND; ++c) acc[c] = dsf{0.f, 0.f};
    dsf *hd = acc, *hp = acc + 6;
    dsf *e = AMOEBA ? acc + 12 : acc + 6;
    dsf *h = AMOEBA ? acc + 15 : acc;  // AMOEBA only
    if (valid) {
#pragma unroll 1
      for (int k = 0; k < cnt; ++k) {
        DsK g;
        if (far_tile) {
          ds_grad_geom<false, AMOEBA>(th, tl, s_ph[k], s_pl[k], 0.0, 0.0, 0.0, 0.0, wat, wat, 0.0, 0.f, g);
        } else {
          if (s_pm[k] == t) continue;
          if (!ds_grad_geom<true, AMOEBA>(th, tl, s_ph[k], s_pl[k], wt, s_w[k], at, s_a[k], wat, s_wa[k], s.damp_thr,
                                          thr2m, g)) {
            bad = 1;
            continue;
          }
        }
        const float *mh = &s_mh[k * NS * 3], *ml = &s_ml[k * NS * 3];
        const dsf mD[3] = {{mh[0], ml[0]}, {mh[1], ml[1]}, {mh[2], ml[2]}};
        const dsf mdD = mD[0] * g.dx + mD[1] * g.dy + mD[2] * g.dz;
        gradmath::dipole_grad(mD, mdD, g.dx, g.dy, g.dz, g.k5, g.k7, gradmath::One{}, hd);
        if (AMOEBA) {
          const dsf mP[3] = {{mh[3], ml[3]}, {mh[4], ml[4]}, {mh[5], ml[5]}};
          const dsf mdP = mP[0] * g.dx + mP[1] * g.dy + mP[2] * g.dz;
          gradmath::dipole_grad(mP, mdP, g.dx, g.dy, g.dz, g.k5, g.k7, gradmath::One{}, hp);
          const dsf mb[3] = {0.5f * (mD[0] + mP[0]), 0.5f * (mD[1] + mP[1]), 0.5f * (mD[2] + mP[2])};
          const dsf mdb = 0.5f * (mdD + mdP);
          gradmath::dipole_field(mb, mdb, g.dx, g.dy, g.dz, g.k3, g.k5, gradmath::One{}, e);
          gradmath::dipole_hess_q(mb, mdb, g.dx, g.dy, g.dz, Q, trq, g.k5, g.k7, g.k9, gradmath::One{}, h);
        } else {
          gradmath::dipole_field(mD, mdD, g.dx, g.dy, g.dz, g.k3, g.k5, gradmath::One{}, e);
        }
      }
    }
#pragma unroll
    for (int c = 0; c < ND; ++c) s_sum[c * GD_TPB + threadIdx.x] += (double)acc[c].h + (double)acc[c].l;
  }
  if (bad) atomicOr(err, 1);
  if (valid) {
    double *o = partial + (size_t)blockIdx.y * ND * s.m + t;
#pragma unroll
    for (int c = 0; c < ND; ++c) o[(size_t)c * s.m] = s_sum[c * GD_TPB + threadIdx.x];
  }
}

// source splits minimising whole waves x tiles per split
int pick_split(int targets, int sources, int resident) {
  const int tblocks = (targets + GD_TPB - 1) / GD_TPB, tiles = (sources + GD_TILE - 1) / GD_TILE;
  int best = 1;
  double best_t = 1e300;
  for (int sp = 1; sp <= std::min(tiles, 64); ++sp) {
    const double tm = std::ceil((double)tblocks * sp / resident) * std::ceil((double)tiles / sp);
    if (tm < best_t * 0.999) {
      best_t = tm;
      best = sp;
    }
  }
  return best;
}

}  // namespace

int grad_ds_pick_split(const DevSites &s, int which, int sm_count) {
  int per_sm = 1;
  if (which == 0)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, s.amoeba ? k_grad_ds_mp<true> : k_grad_ds_mp<false>,
                                                  GD_TPB, 0);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, s.amoeba ? k_grad_ds_dip<true> : k_grad_ds_dip<false>,
                                                  GD_TPB, 0);
  const int resident = std::max(1, per_sm) * sm_count;
  return which == 0 ? pick_split(s.n, s.m, resident) : pick_split(s.m, s.n, resident);
}

void launch_grad_ds_mp(const DevSites &s, double *partial, int nsplit, int *err, cudaStream_t st) {
  if (s.n == 0) return;
  const int tiles = (s.m + GD_TILE - 1) / GD_TILE;
  const int per = ((tiles + nsplit - 1) / nsplit) * GD_TILE;
  const dim3 grid((s.n + GD_TPB - 1) / GD_TPB, nsplit);
  const float thr2m = (float)(s.damp_thr * s.damp_thr * (1.0 + 1e-5));
  if (s.amoeba)
    k_grad_ds_mp<true><<<grid, GD_TPB, 0, st>>>(s, partial, per, thr2m, err);
  else
    k_grad_ds_mp<false><<<grid, GD_TPB, 0, st>>>(s, partial, per, thr2m, err);
  add_launch_count(1);
}

void launch_grad_ds_dip(const DevSites &s, const double *ipd, double *partial, int nsplit, int *err,
                        cudaStream_t st) {
  if (s.m == 0 || s.n == 0) return;
  const int tiles = (s.n + GD_TILE - 1) / GD_TILE;
  const int per = ((tiles + nsplit - 1) / nsplit) * GD_TILE;
  const dim3 grid((s.m + GD_TPB - 1) / GD_TPB, nsplit);
  const float thr2m = (float)(s.damp_thr * s.damp_thr * (1.0 + 1e-5));
  if (s.amoeba)
    k_grad_ds_dip<true><<<grid, GD_TPB, 0, st>>>(s, ipd, partial, per, thr2m, err);
  else
    k_grad_ds_dip<false><<<grid, GD_TPB, 0, st>>>(s, ipd, partial, per, thr2m, err);
  add_launch_count(1);
}

}  // namespace gpu
}  // namespace ommp
