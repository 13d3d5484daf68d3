// GB300 (sm_103a) kernels of the induced-point-dipole path.
//
// Pair kernels (all-pairs, CUDA cores; the pair tensor math is not a dense
// contraction, so no tensor cores):
//   k_m2d_allpairs   field of the permanent multipoles at the polarizable
//                    sites, unscaled, Thole-damped (AMOEBA exp / Wang linear).
//                    Restates elec_prop_M2D + damped_coulomb_kernel + the
//                    q/mu/quad field formulas (src/mod_electrostatics.F90:
//                    1018-1095, 1097-1405, 2579-2731).
//   k_m2d_finish     fixed-order reduction of the source-split partials plus
//                    the scaled-pair correction pass: for every listed pair
//                    (s - 1) * f_ij is added, which equals the reference's
//                    "skip when s == 0, multiply when s != 1" rule.
//   k_tmu<T,...>     dipole-dipole field T.mu, target-outer like field_extD2D
//                    (src/mod_electrostatics.F90:2068-2109); FP64 or FP32 with
//                    compensated (Kahan) cross-tile sums.
//   k_tmu_finish     partial reduction, u-scale correction, sign and the
//                    1/alpha diagonal of TMatVec_otf/TMatVec_diag
//                    (src/mod_polarization.F90:459-504).
// Source tiles are staged in shared memory by the whole CTA with coalesced
// loads and broadcast to all threads; each thread owns one target site.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <type_traits>

#include "kernels.h"
#include "pair_math.cuh"

namespace ommp {
namespace gpu {

namespace {
constexpr int TPB = 128;   // targets per CTA
constexpr int TILE = 128;  // sources per shared-memory tile

template <bool AMOEBA>
__global__ void __launch_bounds__(TPB) k_m2d_allpairs(int n, int m, const Pos64 *__restrict__ pol_pos,
                                                      const double *__restrict__ pol_a,
                                                      const int *__restrict__ polar_mm,
                                                      const Pos64 *__restrict__ mm_pos,
                                                      const double *__restrict__ mm_a,
                                                      const double *__restrict__ mm_q, int ld,
                                                      const float2 *__restrict__ pol_wa,
                                                      const float2 *__restrict__ mm_wa,
                                                      double *__restrict__ partial, int per_split,
                                                      double thr, float thr2m, int *err_flag) {
  constexpr int LD = AMOEBA ? 10 : 1;         // multipole record in memory
  constexpr int SLD = AMOEBA ? M2D_SLD : 1;    // staged record (m2d_stage)
  constexpr int NA = AMOEBA ? 9 : 3;          // field sums (m2d_pair_acc)
  __shared__ Pos64 s_pos[TILE];
  __shared__ double s_a[TILE];
  __shared__ float2 s_wa[TILE];
  __shared__ double s_q[TILE * SLD];
  const int j = blockIdx.x * TPB + threadIdx.x;
  const bool valid = j < n;
  Pos64 pt = valid ? pol_pos[j] : Pos64{0, 0, 0, 0};
  // the target's own mm index and its thole (pol_pos stores 1/thole)
  const int tm = valid ? polar_mm[j] : -1;
  const double at = valid && AMOEBA ? pol_a[j] : 0.0;
  const float2 wat = valid ? pol_wa[j] : make_float2(0.f, 0.f);
  double acc[NA];
#pragma unroll
  for (int c = 0; c < NA; ++c) acc[c] = 0.0;
  int bad = 0;
  const int s0 = blockIdx.y * per_split;
  const int s1 = min(m, s0 + per_split);
  for (int t0 = s0; t0 < s1; t0 += TILE) {
    __syncthreads();
    for (int k = threadIdx.x; k < TILE; k += TPB) {
      int i = t0 + k;
      if (i < s1) {
        s_pos[k] = mm_pos[i];
        s_a[k] = AMOEBA ? mm_a[i] : 0.0;
        s_wa[k] = mm_wa[i];
        m2d_stage<AMOEBA>(&mm_q[(size_t)i * LD], &s_q[k * SLD]);
      }
    }
    __syncthreads();
    const int cnt = min(TILE, s1 - t0);
    if (!valid) continue;
    for (int k = 0; k < cnt; ++k) {
      const int i = t0 + k;
      if (i == tm) continue;
      const Pos64 ps = s_pos[k];
      double dx = pt.x - ps.x, dy = pt.y - ps.y, dz = pt.z - ps.z;
      if (coincident(dx * dx + dy * dy + dz * dz)) {
        bad = 1;
        continue;
      }
      m2d_pair_acc<AMOEBA>(dx, dy, dz, pt.w, ps.w, at, s_a[k], wat, s_wa[k], &s_q[k * SLD], thr, thr2m, acc);
    }
  }
  if (bad) atomicOr(err_flag, 1);
  if (valid) {
    double *o = partial + ((size_t)blockIdx.y * n + j) * 3;
    m2d_field<AMOEBA>(acc, o[0], o[1], o[2]);
  }
}

// Reduce partials and apply the scaled-pair corrections; out [n_ipd][n][3]
// with set 0 = D (direct field, d-scale) and set 1 = P (p-scale) for AMOEBA.
template <bool AMOEBA>
__global__ void k_m2d_finish(int n, int nsplit, const double *__restrict__ partial,
                             const Pos64 *__restrict__ pol_pos, const double *__restrict__ pol_a,
                             const Pos64 *__restrict__ mm_pos, const double *__restrict__ mm_a,
                             const double *__restrict__ mm_q, const float2 *__restrict__ pol_wa,
                             const float2 *__restrict__ mm_wa, const int *__restrict__ ri,
                             const int *__restrict__ src, const double *__restrict__ sP,
                             const double *__restrict__ sD, double thr, float thr2m,
                             double *__restrict__ out) {
  constexpr int LD = AMOEBA ? 10 : 1;
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  double e[3] = {0, 0, 0};
  for (int s = 0; s < nsplit; ++s)
    for (int c = 0; c < 3; ++c) e[c] += partial[((size_t)s * n + j) * 3 + c];
  double eP[3] = {e[0], e[1], e[2]}, eD[3] = {e[0], e[1], e[2]};
  Pos64 pt = pol_pos[j];
  double at = AMOEBA ? pol_a[j] : 0.0;
  float2 wat = pol_wa[j];
  for (int k = ri[j]; k < ri[j + 1]; ++k) {
    int i = src[k];
    Pos64 ps = mm_pos[i];
    double q[LD];
    for (int c = 0; c < LD; ++c) q[c] = mm_q[(size_t)i * LD + c];
    double fx = 0, fy = 0, fz = 0;
    m2d_pair_f64<AMOEBA>(pt.x - ps.x, pt.y - ps.y, pt.z - ps.z, pt.w, ps.w, at,
                         AMOEBA ? mm_a[i] : 0.0, wat, mm_wa[i], q, thr, thr2m, fx, fy, fz);
    double cp = sP[k] - 1.0, cd = sD[k] - 1.0;
    eP[0] += cp * fx;
    eP[1] += cp * fy;
    eP[2] += cp * fz;
    eD[0] += cd * fx;
    eD[1] += cd * fy;
    eD[2] += cd * fz;
  }
  if (AMOEBA) {
    for (int c = 0; c < 3; ++c) {
      out[(size_t)j * 3 + c] = eD[c];
      out[((size_t)n + j) * 3 + c] = eP[c];
    }
  } else {
    for (int c = 0; c < 3; ++c) out[(size_t)j * 3 + c] = eP[c];
  }
}

// partial[split][rhs][j][3] = E_dd(x)_j over the split's source range.
template <typename T, int NRHS, bool AMOEBA, bool KAHAN>
__global__ void __launch_bounds__(TPB) k_tmu(int n, const typename Vec4<T>::type *__restrict__ pos,
                                             const T *__restrict__ damp, const float2 *__restrict__ wa,
                                             const T *__restrict__ x, T *__restrict__ partial,
                                             int per_split, T thr, float thr2m) {
  using V4 = typename Vec4<T>::type;
  constexpr bool F64 = std::is_same<T, double>::value;
  __shared__ V4 s_pos[TILE];
  __shared__ T s_a[TILE];
  __shared__ float2 s_wa[TILE];
  __shared__ T s_mu[NRHS * 3][TILE];
  const int j = blockIdx.x * TPB + threadIdx.x;
  const bool valid = j < n;
  V4 pt;
  if (valid) {
    pt = pos[j];
  } else {
    pt.x = pt.y = pt.z = pt.w = T(0);
  }
  const T at = (valid && AMOEBA) ? damp[j] : T(0);
  const float2 wat = (F64 && valid) ? wa[j] : make_float2(0.f, 0.f);
  T acc[NRHS * 3], sum[NRHS * 3], comp[NRHS * 3];
#pragma unroll
  for (int c = 0; c < NRHS * 3; ++c) sum[c] = comp[c] = T(0);
  const int s0 = blockIdx.y * per_split;
  const int s1 = min(n, s0 + per_split);
  for (int t0 = s0; t0 < s1; t0 += TILE) {
    __syncthreads();
    {
      int k = threadIdx.x;  // TILE == TPB
      int i = t0 + k;
      if (i < s1) {
        s_pos[k] = pos[i];
        s_a[k] = AMOEBA ? damp[i] : T(0);
        if (F64) s_wa[k] = wa[i];
#pragma unroll
        for (int r = 0; r < NRHS; ++r)
#pragma unroll
          for (int c = 0; c < 3; ++c) s_mu[r * 3 + c][k] = x[((size_t)r * n + i) * 3 + c];
      }
    }
    __syncthreads();
    const int cnt = min(TILE, s1 - t0);
#pragma unroll
    for (int c = 0; c < NRHS * 3; ++c) acc[c] = T(0);
    if (valid) {
#pragma unroll 2
      for (int k = 0; k < cnt; ++k) {
        if (t0 + k == j) continue;
        const V4 ps = s_pos[k];
        T dx = pt.x - ps.x, dy = pt.y - ps.y, dz = pt.z - ps.z;
        T r2 = dx * dx + dy * dy + dz * dz;
        T k3, k5x3;
        dd_pair<T, AMOEBA>(r2, pt.w, ps.w, at, s_a[k], wat, F64 ? s_wa[k] : wat, thr, thr2m, k3, k5x3);
#pragma unroll
        for (int r = 0; r < NRHS; ++r) {
          T mx = s_mu[r * 3 + 0][k], my = s_mu[r * 3 + 1][k], mz = s_mu[r * 3 + 2][k];
          T f = k5x3 * (mx * dx + my * dy + mz * dz);
          acc[r * 3 + 0] += f * dx - k3 * mx;
          acc[r * 3 + 1] += f * dy - k3 * my;
          acc[r * 3 + 2] += f * dz - k3 * mz;
        }
      }
    }
    // cross-tile accumulation: compensated (Kahan) for FP32
#pragma unroll
    for (int c = 0; c < NRHS * 3; ++c) {
      if (KAHAN) {
        T y = acc[c] - comp[c];
        T t = sum[c] + y;
        comp[c] = (t - sum[c]) - y;
        sum[c] = t;
      } else {
        sum[c] += acc[c];
      }
    }
  }
  if (valid) {
#pragma unroll
    for (int r = 0; r < NRHS; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c)
        partial[(((size_t)blockIdx.y * NRHS + r) * n + j) * 3 + c] = sum[r * 3 + c];
  }
}

// y[r][j] = -(sum_split partial + scaled-pair corrections) (+ x/alpha)
template <typename T, bool AMOEBA>
__global__ void k_tmu_finish(int n, int nrhs, int nsplit, const T *__restrict__ partial,
                             const typename Vec4<T>::type *__restrict__ pos,
                             const T *__restrict__ damp, const float2 *__restrict__ wa,
                             const T *__restrict__ x, const double *__restrict__ alpha, bool dodiag,
                             const int *__restrict__ ri, const int *__restrict__ src,
                             const double *__restrict__ scale, T thr, float thr2m, T *__restrict__ y) {
  constexpr bool F64 = std::is_same<T, double>::value;
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int r = blockIdx.y;
  if (j >= n) return;
  double e[3] = {0, 0, 0};
  for (int s = 0; s < nsplit; ++s)
    for (int c = 0; c < 3; ++c) e[c] += (double)partial[(((size_t)s * nrhs + r) * n + j) * 3 + c];
  if (ri) {
    auto pt = pos[j];
    T at = AMOEBA ? damp[j] : T(0);
    float2 wat = F64 ? wa[j] : make_float2(0.f, 0.f);
    for (int k = ri[j]; k < ri[j + 1]; ++k) {
      int i = src[k];
      auto ps = pos[i];
      T dx = pt.x - ps.x, dy = pt.y - ps.y, dz = pt.z - ps.z;
      T r2 = dx * dx + dy * dy + dz * dz;
      T k3, k5x3;
      dd_pair<T, AMOEBA>(r2, pt.w, ps.w, at, AMOEBA ? damp[i] : T(0), wat, F64 ? wa[i] : wat, thr, thr2m, k3,
                         k5x3);
      const T *mu = &x[((size_t)r * n + i) * 3];
      T f = k5x3 * (mu[0] * dx + mu[1] * dy + mu[2] * dz);
      double cs = scale[k] - 1.0;
      e[0] += cs * (double)(f * dx - k3 * mu[0]);
      e[1] += cs * (double)(f * dy - k3 * mu[1]);
      e[2] += cs * (double)(f * dz - k3 * mu[2]);
    }
  }
  const T *xj = &x[((size_t)r * n + j) * 3];
  T *yj = &y[((size_t)r * n + j) * 3];
  double ia = dodiag ? 1.0 / alpha[j] : 0.0;
  for (int c = 0; c < 3; ++c) yj[c] = (T)(-e[c] + (dodiag ? (double)xj[c] * ia : 0.0));
}

// ---------------------------------------------------------------------------
// Symmetric FP64 dipole field: every unordered pair is evaluated once and
// both directions are accumulated (T_ij = T_ji), halving the FP64 work of
// the geometry.  Sites are grouped in super-tiles of 128 (4 warps x 32
// lanes).  Super-tile I meets the slots k of its half shell
// J = (I + k) mod ntile, k = 0..K (K = ntile / 2); slot 0 is the diagonal
// block (target side only, all ordered pairs); for even ntile the slot
// k = ntile/2 is handled by the lower of the two tiles only.  The work items
// (I, a chunk of consecutive slots) are handed out by an atomic counter to a
// persistent grid of as many CTAs as fit on the GPU at once, so that every
// SM stays busy to the end (a static grid leaves 4 CTAs on some SMs and 5 on
// others).  Inside a slot a
// warp pairs its 32 targets with each 32-site sub-tile of J in 32 rotation
// steps: at step t lane l meets source (l + t) mod 32, read from shared
// memory, and the source-side accumulators travel one lane per step by
// shuffle, so no lane ever shares an accumulator.  Source sides are summed
// over the 4 warps in shared memory; they and the target sides are added to
// per-site 128-bit fixed-point accumulators (2^-80 resolution) with integer
// atomics.  Integer addition is exact and associative, so the product is
// deterministic whatever the order of the CTAs, and the accumulators take
// O(n) memory.
// ---------------------------------------------------------------------------
constexpr int SYM_TILE = 128;

// dynamic shared memory of k_tmu_sym: the staged dipoles s_mu[C][128] and
// the four warps' source-side sums s_accj[4][C][128] (C = 3 NRHS doubles)
constexpr size_t sym_smem_bytes(int nrhs) { return (size_t)5 * 3 * nrhs * SYM_TILE * sizeof(double); }

// A launch serves the products of several systems (same column count and
// damping kind): job j covers the items [item0, item0 + base[j+1] - base[j])
// of its system's product, whose item space is fixed per system, so that a
// product may also be spread over several launches (its fixed-point sums add
// up across them).  A one-job table is the single-system product.
struct Sym64Job {
  const Pos64 *pos;
  const double *damp;
  const float2 *wa;
  const double *x;
  unsigned long long *lo, *hi, *bad;
  int n, ntile, K, chunk, nchunk, item0;
  double thr;
  float thr2m;
};
struct Sym64Table {
  int njobs;
  int base[kMaxSymSlices + 1];
  Sym64Job job[kMaxSymSlices];
};

template <int NRHS, bool AMOEBA>
__global__ void __launch_bounds__(SYM_TILE) k_tmu_sym(const __grid_constant__ Sym64Table tab,
                                                       unsigned *__restrict__ next) {
  constexpr int C = 3 * NRHS;
  __shared__ double s_x[SYM_TILE], s_y[SYM_TILE], s_z[SYM_TILE], s_w[SYM_TILE], s_a[SYM_TILE];
  __shared__ float2 s_wa[SYM_TILE];
  extern __shared__ double sym_dyn[];
  double(*s_mu)[SYM_TILE] = reinterpret_cast<double(*)[SYM_TILE]>(sym_dyn);
  double(*s_accj)[C][SYM_TILE] = reinterpret_cast<double(*)[C][SYM_TILE]>(sym_dyn + C * SYM_TILE);
  __shared__ int s_item;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int total = tab.base[tab.njobs];
  for (;;) {
    __syncthreads();  // every thread has read the previous item
    if (tid == 0) s_item = (int)atomicAdd(next, 1u);
    __syncthreads();
    const int item = s_item;
    if (item >= total) break;
    int jx = 0;
    while (jx + 1 < tab.njobs && tab.base[jx + 1] <= item) ++jx;
    const Sym64Job &jb = tab.job[jx];
    const int n = jb.n, ntile = jb.ntile, K = jb.K, chunk = jb.chunk, nchunk = jb.nchunk;
    const Pos64 *__restrict__ pos = jb.pos;
    const double *__restrict__ damp = jb.damp;
    const float2 *__restrict__ wa = jb.wa;
    const double *__restrict__ x = jb.x;
    unsigned long long *acc_lo = jb.lo, *acc_hi = jb.hi, *bad = jb.bad;
    const double thr = jb.thr;
    const float thr2m = jb.thr2m;
    const int local = jb.item0 + (item - tab.base[jx]);
    const int I = local / nchunk;
    const int ti = I * SYM_TILE + tid;
    const bool vi = ti < n;
    const Pos64 pi = vi ? pos[ti] : Pos64{0, 0, 0, 0};
    const double ai = (AMOEBA && vi) ? damp[ti] : 0.0;
    const float2 wai = vi ? wa[ti] : make_float2(0.f, 0.f);
    // each side's field 3 sum f d - sum k3 mu (f = k5 mu.d) is accumulated
    // as its two sums, one FMA per component each
    double mui[C], afi[C], aki[C];
#pragma unroll
    for (int c = 0; c < C; ++c) {
      mui[c] = vi ? x[((size_t)(c / 3) * n + ti) * 3 + (c % 3)] : 0.0;
      afi[c] = 0.0;
      aki[c] = 0.0;
    }
    const int k0 = (local - I * nchunk) * chunk;
    const int k1 = min(K + 1, k0 + chunk);
    for (int k = k0; k < k1; ++k) {
      int J = I + k;
      if (J >= ntile) J -= ntile;
      if (k > 0 && 2 * k == ntile && I >= ntile / 2) continue;  // the other tile of the pair owns it
      const bool diag = (k == 0);
      __syncthreads();
      {
        int sj = J * SYM_TILE + tid;
        bool v = sj < n;
        Pos64 p = v ? pos[sj] : Pos64{0, 0, 0, 0};
        s_x[tid] = p.x;
        s_y[tid] = p.y;
        s_z[tid] = p.z;
        s_w[tid] = p.w;
        s_a[tid] = (AMOEBA && v) ? damp[sj] : 0.0;
        s_wa[tid] = v ? wa[sj] : make_float2(0.f, 0.f);
#pragma unroll
        for (int c = 0; c < C; ++c) s_mu[c][tid] = v ? x[((size_t)(c / 3) * n + sj) * 3 + (c % 3)] : 0.0;
      }
      __syncthreads();
      for (int js = 0; js < 4; ++js) {
        double afj[C], akj[C];
#pragma unroll
        for (int c = 0; c < C; ++c) afj[c] = akj[c] = 0.0;
        for (int t = 0; t < 32; ++t) {
          const int jl = js * 32 + ((lane + t) & 31);
          const int gj = J * SYM_TILE + jl;
          if (vi && gj < n && gj != ti) {
            double dx = pi.x - s_x[jl], dy = pi.y - s_y[jl], dz = pi.z - s_z[jl];
            double r2 = dx * dx + dy * dy + dz * dz;
            double k3, k5;
            dd_pair_f64<AMOEBA>(r2, pi.w, s_w[jl], ai, s_a[jl], wai, s_wa[jl], thr, thr2m, k3, k5);
#pragma unroll
            for (int r = 0; r < NRHS; ++r) {
              double mx = s_mu[3 * r][jl], my = s_mu[3 * r + 1][jl], mz = s_mu[3 * r + 2][jl];
              double f = k5 * (mx * dx + my * dy + mz * dz);
              afi[3 * r] = fma(f, dx, afi[3 * r]);
              afi[3 * r + 1] = fma(f, dy, afi[3 * r + 1]);
              afi[3 * r + 2] = fma(f, dz, afi[3 * r + 2]);
              aki[3 * r] = fma(k3, mx, aki[3 * r]);
              aki[3 * r + 1] = fma(k3, my, aki[3 * r + 1]);
              aki[3 * r + 2] = fma(k3, mz, aki[3 * r + 2]);
              if (!diag) {
                double g = k5 * (mui[3 * r] * dx + mui[3 * r + 1] * dy + mui[3 * r + 2] * dz);
                afj[3 * r] = fma(g, dx, afj[3 * r]);
                afj[3 * r + 1] = fma(g, dy, afj[3 * r + 1]);
                afj[3 * r + 2] = fma(g, dz, afj[3 * r + 2]);
                akj[3 * r] = fma(k3, mui[3 * r], akj[3 * r]);
                akj[3 * r + 1] = fma(k3, mui[3 * r + 1], akj[3 * r + 1]);
                akj[3 * r + 2] = fma(k3, mui[3 * r + 2], akj[3 * r + 2]);
              }
            }
          }
          if (!diag) {
            // the accumulators of source s move to the lane that meets s next
#pragma unroll
            for (int c = 0; c < C; ++c) {
              afj[c] = __shfl_sync(0xffffffffu, afj[c], (lane + 1) & 31);
              akj[c] = __shfl_sync(0xffffffffu, akj[c], (lane + 1) & 31);
            }
          }
        }
        if (!diag) {
          // after 32 steps lane l holds the accumulators of source js*32 + l
#pragma unroll
          for (int c = 0; c < C; ++c) s_accj[warp][c][js * 32 + lane] = fma(3.0, afj[c], -akj[c]);
        }
      }
      if (!diag) {
        __syncthreads();
        const int sj = J * SYM_TILE + tid;
        if (sj < n) {
#pragma unroll
          for (int c = 0; c < C; ++c) {
            const double v = ((s_accj[0][c][tid] + s_accj[1][c][tid]) + s_accj[2][c][tid]) + s_accj[3][c][tid];
            const size_t o = ((size_t)(c / 3) * n + sj) * 3 + (c % 3);
            fixed_add(acc_lo + o, acc_hi + o, v, bad);
          }
        }
      }
    }
    if (vi) {
#pragma unroll
      for (int c = 0; c < C; ++c) {
        const size_t o = ((size_t)(c / 3) * n + ti) * 3 + (c % 3);
        fixed_add(acc_lo + o, acc_hi + o, fma(3.0, afi[c], -aki[c]), bad);
      }
    }
  }
}

// out[k] = the fixed-point accumulator k as a double (NaN when flagged)
__global__ void k_fixed_to_double(size_t total, const unsigned long long *__restrict__ lo,
                                  const unsigned long long *__restrict__ hi, const unsigned long long *bad,
                                  double *__restrict__ out) {
  const bool nan = *bad != 0ull;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < total; k += (size_t)gridDim.x * blockDim.x)
    out[k] = nan ? __longlong_as_double(0x7ff8000000000000ll) : fixed_value(lo[k], hi[k]);
}

// ---------------------------------------------------------------------------
// dense T matrix (create_tmat / dipole_T, src/mod_polarization.F90:327-435)
// ---------------------------------------------------------------------------
template <bool AMOEBA>
__global__ void k_build_tmat(int n, const Pos64 *__restrict__ pos, const double *__restrict__ damp,
                             const double *__restrict__ alpha, double thr, double *__restrict__ T) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;  // row block (target)
  int i = blockIdx.y;                             // column block (source)
  if (j >= n) return;
  size_t nn = 3 * (size_t)n;
  double blk[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  if (i == j) {
    double ia = 1.0 / alpha[j];
    blk[0][0] = blk[1][1] = blk[2][2] = ia;
  } else {
    Pos64 pt = pos[j], ps = pos[i];
    double d[3] = {pt.x - ps.x, pt.y - ps.y, pt.z - ps.z};
    double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    double k3, k5x3;
    dd_kernel<double, AMOEBA>(r2, pt.w, ps.w, AMOEBA ? damp[j] : 0.0, AMOEBA ? damp[i] : 0.0, thr,
                              k3, k5x3);
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) blk[a][b] = (a == b ? k3 : 0.0) - k5x3 * d[a] * d[b];
  }
  for (int b = 0; b < 3; ++b)
    for (int a = 0; a < 3; ++a) T[(3 * (size_t)i + b) * nn + 3 * (size_t)j + a] = blk[a][b];
}

// multiply the listed off-diagonal blocks by their u-scale
__global__ void k_scale_tmat(int n, const int *__restrict__ ri, const int *__restrict__ src,
                             const double *__restrict__ scale, double *__restrict__ T) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  size_t nn = 3 * (size_t)n;
  for (int k = ri[j]; k < ri[j + 1]; ++k) {
    int i = src[k];
    double s = scale[k];
    for (int b = 0; b < 3; ++b)
      for (int a = 0; a < 3; ++a) T[(3 * (size_t)i + b) * nn + 3 * (size_t)j + a] *= s;
  }
}

// y = A x (- diag(A) x when !dodiag), column major, nrhs columns
__global__ void k_gemv(int nn, const double *__restrict__ A, const double *__restrict__ x,
                       double *__restrict__ y, bool dodiag, const double *__restrict__ alpha) {
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  int c0 = blockIdx.y;  // rhs
  if (r >= nn) return;
  const double *xv = x + (size_t)c0 * nn;
  double acc = 0.0;
  for (int c = 0; c < nn; ++c) acc += A[(size_t)c * nn + r] * xv[c];
  if (!dodiag) acc -= xv[r] / alpha[r / 3];
  y[(size_t)c0 * nn + r] = acc;
}

// LU: pivot search in column k (one block), swap, update, scale
__global__ void k_lu_pivot(int nn, int k, double *A, int *piv, int *info) {
  __shared__ double sv[1024];
  __shared__ int si[1024];
  double best = -1.0;
  int bi = k;
  for (int r = k + threadIdx.x; r < nn; r += blockDim.x) {
    double v = fabs(A[(size_t)k * nn + r]);
    if (v > best) {
      best = v;
      bi = r;
    }
  }
  sv[threadIdx.x] = best;
  si[threadIdx.x] = bi;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      double o = sv[threadIdx.x + s];
      int oi = si[threadIdx.x + s];
      if (o > sv[threadIdx.x] || (o == sv[threadIdx.x] && oi < si[threadIdx.x])) {
        sv[threadIdx.x] = o;
        si[threadIdx.x] = oi;
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    piv[k] = si[0];
    if (sv[0] == 0.0 && *info == 0) *info = k + 1;
  }
}

__global__ void k_lu_swap(int nn, int k, double *A, const int *piv) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  int p = piv[k];
  if (c >= nn || p == k) return;
  double t = A[(size_t)c * nn + k];
  A[(size_t)c * nn + k] = A[(size_t)c * nn + p];
  A[(size_t)c * nn + p] = t;
}

__global__ void k_lu_update(int nn, int k, double *A, const int *info) {
  if (*info) return;
  int r = k + 1 + blockIdx.x * blockDim.x + threadIdx.x;
  int c = k + 1 + blockIdx.y;
  if (r >= nn || c >= nn) return;
  double l = A[(size_t)k * nn + r] / A[(size_t)k * nn + k];
  A[(size_t)c * nn + r] -= l * A[(size_t)c * nn + k];
}

__global__ void k_lu_scale(int nn, int k, double *A, const int *info) {
  if (*info) return;
  int r = k + 1 + blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nn) return;
  A[(size_t)k * nn + r] /= A[(size_t)k * nn + k];
}

// forward/back substitution for one rhs (single block)
__global__ void k_lu_solve(int nn, const double *A, const int *piv, double *b) {
  for (int k = 0; k < nn; ++k) {  // apply the row interchanges in order
    if (threadIdx.x == 0) {
      int p = piv[k];
      if (p != k) {
        double t = b[k];
        b[k] = b[p];
        b[p] = t;
      }
    }
  }
  __syncthreads();
  for (int k = 0; k < nn; ++k) {
    double bk = b[k];
    for (int r = k + 1 + threadIdx.x; r < nn; r += blockDim.x) b[r] -= A[(size_t)k * nn + r] * bk;
    __syncthreads();
  }
  for (int k = nn - 1; k >= 0; --k) {
    if (threadIdx.x == 0) b[k] /= A[(size_t)k * nn + k];
    __syncthreads();
    double bk = b[k];
    for (int r = threadIdx.x; r < k; r += blockDim.x) b[r] -= A[(size_t)k * nn + r] * bk;
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// BLAS-1 with deterministic two-stage reductions
// ---------------------------------------------------------------------------
// Columns run side by side (blockIdx.y = column), not one after another
// inside a block, and each thread sums about 8 elements of its column with
// four independent loads in flight: a block-serial column loop with ~2
// elements per thread left the 64-column dots of a batch latency-bound (1.4
// TB/s).  gridDim.x blocks of a column write partial[b][k]; the rows from
// gridDim.x to kRedBlocks are zeroed so that the fixed-order reduction over
// kRedBlocks rows is unchanged.
template <typename T>
__global__ void __launch_bounds__(kRedThreads) k_dots(int ncol, size_t n, const T *__restrict__ a,
                                                      const T *__restrict__ b, size_t bstride,
                                                      double *__restrict__ partial) {
  __shared__ double sh[kRedThreads / 32];
  const int k = blockIdx.y;
  const T *ak = a + (size_t)k * n;
  const T *bk = b + (size_t)k * bstride;
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (; i + 3 * stride < n; i += 4 * stride) {
#pragma unroll
    for (int u = 0; u < 4; ++u) acc[u] += (double)ak[i + u * stride] * (double)bk[i + u * stride];
  }
  for (; i < n; i += stride) acc[0] += (double)ak[i] * (double)bk[i];
  double s0 = (acc[0] + acc[1]) + (acc[2] + acc[3]);
  for (int o = 16; o > 0; o >>= 1) s0 += __shfl_down_sync(0xffffffffu, s0, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s0;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < kRedThreads / 32; ++w) s += sh[w];
    partial[(size_t)blockIdx.x * ncol + k] = s;
  }
  if (blockIdx.x == 0)
    for (int r = gridDim.x + threadIdx.x; r < kRedBlocks; r += blockDim.x) partial[(size_t)r * ncol + k] = 0.0;
}

// blocks per column of k_dots: about 8 elements per thread
inline int dots_blocks(size_t n) {
  size_t b = (n + (size_t)kRedThreads * 8 - 1) / ((size_t)kRedThreads * 8);
  if (b < 1) b = 1;
  if (b > (size_t)kRedBlocks) b = kRedBlocks;
  return (int)b;
}

__global__ void k_reduce_partials(int ncol, int nb, const double *__restrict__ partial,
                                  double *__restrict__ result) {
  // one warp per column, fixed lane order then fixed tree
  int k = blockIdx.x;
  double acc = 0.0;
  for (int b = threadIdx.x; b < nb; b += 32) acc += partial[(size_t)b * ncol + k];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if (threadIdx.x == 0) result[k] = acc;
}

__global__ void k_axpby(size_t n, double a, const double *x, double b, double *y) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    y[i] = a * x[i] + b * y[i];
}
__global__ void k_add(size_t n, const double *a, const double *b, double *out) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = a[i] + b[i];
}
__global__ void k_scale_alpha(int nrhs, int n, const double *alpha, const double *x, double *y) {
  size_t tot = (size_t)nrhs * n * 3;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < tot; i += (size_t)gridDim.x * blockDim.x)
    y[i] = alpha[(i / 3) % n] * x[i];
}
__global__ void k_to_f32(size_t n, const double *x, const double *scale, float *y) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    y[i] = (float)(x[i] * (scale ? *scale : 1.0));
}
// ncol columns of nv values, column k scaled by scale[k], in one launch
__global__ void k_to_f32_cols(size_t nv, size_t tot, const double *x, const double *scale, float *y) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < tot; i += (size_t)gridDim.x * blockDim.x)
    y[i] = (float)(x[i] * scale[i / nv]);
}

// start of the inner PCG with the first r.z on the device (no host read)
__global__ void k_cg_init(int ncol, const double *dots, CgCol *cols, double tol) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= ncol) return;
  CgCol c{};
  c.gold = dots[k];
  c.tol = tol;
  c.active = dots[k] > 0.0 ? 1 : 0;
  cols[k] = c;
}

__global__ void k_cg_alpha(int ncol, const double *dots, CgCol *cols, double eps) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= ncol) return;
  CgCol c = cols[k];
  if (!c.active) return;
  c.gama = dots[k];
  if (fabs(c.gama) < eps) {
    c.quick = 1;
    c.active = 0;
    c.alpha = 0.0;
  } else {
    c.alpha = c.gold / c.gama;
  }
  cols[k] = c;
}

// one column per blockIdx.y (see k_dots)
template <typename T>
__global__ void k_cg_update(int ncol, int n, T *x, T *r, const T *p, const T *h, T *z,
                            const T *alpha_pol, const CgCol *cols, double *partial) {
  __shared__ double sh[kRedThreads / 32];
  size_t nv = 3 * (size_t)n;
  const int k = blockIdx.y;
  double acc = 0.0;
  if (cols[k].active) {
    double al = cols[k].alpha;
    T a = (T)al;
    size_t off = (size_t)k * nv;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += (size_t)gridDim.x * blockDim.x) {
      if (sizeof(T) == 8) {
        x[off + i] += a * p[off + i];
        r[off + i] -= a * h[off + i];
      } else {
        x[off + i] = (T)((double)x[off + i] + al * (double)p[off + i]);
        r[off + i] = (T)((double)r[off + i] - al * (double)h[off + i]);
      }
      T zi = alpha_pol[i / 3] * r[off + i];
      z[off + i] = zi;
      acc += (double)r[off + i] * (double)zi;
    }
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < kRedThreads / 32; ++w) s += sh[w];
    partial[(size_t)blockIdx.x * ncol + k] = s;
  }
}

__global__ void k_cg_gnew(int ncol, int n, const double *dots, CgCol *cols, double *hist, int hist_stride) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= ncol) return;
  CgCol c = cols[k];
  if (!c.active) return;
  c.gnew = dots[k];
  c.rms = sqrt(c.gnew / (3.0 * n));
  c.iters += 1;
  if (hist && c.iters <= hist_stride) hist[(size_t)k * hist_stride + c.iters - 1] = c.rms;
  if (c.rms < c.tol) {
    c.converged = 1;
    c.active = 0;
  } else {
    c.beta = c.gnew / c.gold;
    c.gama = c.beta;  // the reference reuses gama for the beta ratio
    c.gold = c.gnew;
  }
  cols[k] = c;
}

template <typename T>
__global__ void k_cg_pupdate(int ncol, int n, T *p, const T *z, const CgCol *cols) {
  size_t nv = 3 * (size_t)n;
  const int k = blockIdx.y;
  if (!cols[k].active) return;
  T b = (T)cols[k].beta;
  size_t off = (size_t)k * nv;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += (size_t)gridDim.x * blockDim.x)
    p[off + i] = b * p[off + i] + z[off + i];
}

__global__ void k_ir_accumulate(int ncol, int n, double *mu, const float *d32, const double *scale) {
  size_t nv = 3 * (size_t)n;
  size_t tot = nv * ncol;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < tot; i += (size_t)gridDim.x * blockDim.x)
    mu[i] += scale[i / nv] * (double)d32[i];
}

__global__ void k_residual_update(int ncol, int n, double *r, const float *t32, const double *scale) {
  size_t nv = 3 * (size_t)n;
  size_t tot = nv * ncol;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < tot; i += (size_t)gridDim.x * blockDim.x)
    r[i] -= scale[i / nv] * (double)t32[i];
}

__global__ void k_residual(size_t tot, const double *rhs, const double *tmu, double *r) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < tot; i += (size_t)gridDim.x * blockDim.x)
    r[i] = rhs[i] - tmu[i];
}

__global__ void k_lincomb(int nvec, size_t n, const double *X, size_t ldx, const double *c, double *out) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int v = 0; v < nvec; ++v) acc += c[v] * X[(size_t)v * ldx + i];
    out[i] = acc;
  }
}

__global__ void __launch_bounds__(kRedThreads) k_diff_norms(size_t n, const double *a, const double *b,
                                                            double *partial) {
  __shared__ double s1[kRedThreads / 32], s2[kRedThreads / 32];
  double sq = 0.0, mx = 0.0;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    double d = a[i] - b[i];
    sq += d * d;
    mx = fmax(mx, fabs(d));
  }
  for (int o = 16; o > 0; o >>= 1) {
    sq += __shfl_down_sync(0xffffffffu, sq, o);
    mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
  }
  if ((threadIdx.x & 31) == 0) {
    s1[threadIdx.x >> 5] = sq;
    s2[threadIdx.x >> 5] = mx;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a1 = 0.0, a2 = 0.0;
    for (int w = 0; w < kRedThreads / 32; ++w) {
      a1 += s1[w];
      a2 = fmax(a2, s2[w]);
    }
    partial[2 * blockIdx.x] = a1;
    partial[2 * blockIdx.x + 1] = a2;
  }
}

__global__ void k_reduce_norms(int nb, const double *partial, double *out) {
  double a1 = 0.0, a2 = 0.0;
  for (int b = threadIdx.x; b < nb; b += 32) {
    a1 += partial[2 * b];
    a2 = fmax(a2, partial[2 * b + 1]);
  }
  for (int o = 16; o > 0; o >>= 1) {
    a1 += __shfl_down_sync(0xffffffffu, a1, o);
    a2 = fmax(a2, __shfl_down_sync(0xffffffffu, a2, o));
  }
  if (threadIdx.x == 0) {
    out[0] = a1;
    out[1] = a2;
  }
}

__global__ void k_any_diff(size_t n, const double *a, const double *b, int *flag) {
  const unsigned long long *ua = reinterpret_cast<const unsigned long long *>(a);
  const unsigned long long *ub = reinterpret_cast<const unsigned long long *>(b);
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    if (ua[i] != ub[i]) {
      *flag = 1;
      return;
    }
}

__global__ void k_check_finite(size_t n, const double *x, int *flag) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    if (!isfinite(x[i])) {
      *flag = 1;
      return;
    }
}

// Pipe-throughput calibration: 8 independent FMA chains per thread.
template <typename T>
__global__ void __launch_bounds__(256) k_fma_peak(T *out, int iters, T a, T b) {
  T x0 = (T)threadIdx.x, x1 = x0 + T(1), x2 = x0 + T(2), x3 = x0 + T(3);
  T x4 = x0 + T(4), x5 = x0 + T(5), x6 = x0 + T(6), x7 = x0 + T(7);
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b);
    x1 = fma(x1, a, b);
    x2 = fma(x2, a, b);
    x3 = fma(x3, a, b);
    x4 = fma(x4, a, b);
    x5 = fma(x5, a, b);
    x6 = fma(x6, a, b);
    x7 = fma(x7, a, b);
  }
  T s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == T(-1.2345)) out[blockIdx.x] = s;  // keeps the chains alive
}

// thr^2 with the relative safety margin of the FP32 damping pre-test
inline float damp_thr2_margin(const DevSites &s) {
  return (float)(s.damp_thr * s.damp_thr * (1.0 + 1e-5));
}

inline int blocks_for(size_t n, int tpb, int cap = 4 * 152 * 4) {
  size_t b = (n + tpb - 1) / tpb;
  if (b < 1) b = 1;
  if (b > (size_t)cap) b = cap;
  return (int)b;
}

}  // namespace

// kernels launched by the library: process total, and per host thread (the
// server drives several systems from several threads; a graph capture
// subtracts the kernels its own thread recorded, not those of the others)
static std::atomic<long long> g_launches{0};
static thread_local long long t_launches = 0;
long long launch_count() { return g_launches.load(std::memory_order_relaxed); }
long long thread_launch_count() { return t_launches; }
void add_launch_count(long long k) {
  g_launches.fetch_add(k, std::memory_order_relaxed);
  t_launches += k;
}

double launch_fma_peak(bool fp64, int iters, void *out, cudaStream_t st) {
  int blocks = sm_count() * 8, threads = 256;
  add_launch_count(1);
  if (fp64)
    k_fma_peak<double><<<blocks, threads, 0, st>>>((double *)out, iters, 0.999999, 1e-7);
  else
    k_fma_peak<float><<<blocks, threads, 0, st>>>((float *)out, iters, 0.999999f, 1e-7f);
  return 2.0 * 8.0 * (double)iters * blocks * threads;  // flop
}

int sm_count() {
  static std::atomic<int> cached{0};  // read by several server threads
  int v = cached.load(std::memory_order_relaxed);
  if (!v) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    if (v <= 0) v = 152;
    cached.store(v, std::memory_order_relaxed);
  }
  return v;
}

// ---- M2D -----------------------------------------------------------------
// Source splits of the FP64 permanent field: about 16 waves of CTAs, so
// that the last, partly filled wave idles few SMs (one wave of ~4.6 CTAs
// per SM left the SMs with 4 idle while those with 5 finished), with the
// split partials kept below 64 MiB.
int m2d_pick_split(const DevSites &s, int sms) {
  static int resident = 0;
  if (!resident) {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, k_m2d_allpairs<true>, TPB, 0);
    if (resident < 1) resident = 1;
  }
  const long long tblocks = (s.n + TPB - 1) / TPB;
  const long long want = 16LL * resident * sms;
  long long split = (want + tblocks - 1) / tblocks;
  const long long maxsplit = (s.m + TILE - 1) / TILE;
  const long long maxmem = (64LL << 20) / (24LL * (s.n > 0 ? s.n : 1));
  if (split > maxmem) split = maxmem;
  if (split > maxsplit) split = maxsplit;
  if (split < 1) split = 1;
  return (int)split;
}

size_t m2d_scratch_doubles(const DevSites &s, int nsplit) { return (size_t)nsplit * s.n * 3; }

// split partials -> FP64 scaled-pair corrections -> D and P sets
static void m2d_finish(const DevSites &s, double *out, const double *scratch, int nsplit, cudaStream_t st) {
  int fb = (s.n + 127) / 128;
  if (s.amoeba)
    k_m2d_finish<true><<<fb, 128, 0, st>>>(s.n, nsplit, scratch, s.pol_pos, s.pol_a, s.mm_pos, s.mm_a, s.mm_q,
                                           s.pol_wa32, s.mm_wa32, s.m2d_ri, s.m2d_src, s.m2d_sP, s.m2d_sD,
                                           s.damp_thr, damp_thr2_margin(s), out);
  else
    k_m2d_finish<false><<<fb, 128, 0, st>>>(s.n, nsplit, scratch, s.pol_pos, s.pol_a, s.mm_pos, s.mm_a,
                                            s.mm_q, s.pol_wa32, s.mm_wa32, s.m2d_ri, s.m2d_src, s.m2d_sP,
                                            s.m2d_sD, s.damp_thr, damp_thr2_margin(s), out);
}

void launch_m2d_finish(const DevSites &s, double *out, const double *partial, int nsplit, cudaStream_t st) {
  add_launch_count(1);
  m2d_finish(s, out, partial, nsplit, st);
}

void launch_m2d(const DevSites &s, double *out, double *scratch, int nsplit, int *err_flag,
                cudaStream_t st) {
  if (s.n == 0) return;
  add_launch_count(2);
  int tiles = (s.m + TILE - 1) / TILE;
  int per = ((tiles + nsplit - 1) / nsplit) * TILE;
  dim3 grid((s.n + TPB - 1) / TPB, nsplit);
  if (s.amoeba)
    k_m2d_allpairs<true><<<grid, TPB, 0, st>>>(s.n, s.m, s.pol_pos, s.pol_a, s.polar_mm, s.mm_pos, s.mm_a,
                                               s.mm_q, s.ld, s.pol_wa32, s.mm_wa32, scratch, per, s.damp_thr,
                                               damp_thr2_margin(s), err_flag);
  else
    k_m2d_allpairs<false><<<grid, TPB, 0, st>>>(s.n, s.m, s.pol_pos, s.pol_a, s.polar_mm, s.mm_pos, s.mm_a,
                                                s.mm_q, s.ld, s.pol_wa32, s.mm_wa32, scratch, per, s.damp_thr,
                                                damp_thr2_margin(s), err_flag);
  m2d_finish(s, out, scratch, nsplit, st);
}

void launch_m2d_ds(const DevSites &s, double *out, double *scratch, int nsplit, int *err_flag, cudaStream_t st) {
  if (s.n == 0) return;
  add_launch_count(2);
  launch_m2d_ds_pairs(s, scratch, nsplit, err_flag, st);
  m2d_finish(s, out, scratch, nsplit, st);
}

// ---- T.mu -----------------------------------------------------------------
int tmu_pick_split(const DevSites &s, int nrhs, int sms, bool fp32) {
  (void)nrhs;
  (void)fp32;
  int tblocks = (s.n + TPB - 1) / TPB;
  int want = 4 * sms;
  int split = (want + tblocks - 1) / tblocks;
  int maxsplit = (s.n + TILE - 1) / TILE;
  if (split > maxsplit) split = maxsplit;
  if (split < 1) split = 1;
  return split;
}

int tmu32_max_split(const DevSites &s, int sms) {
  int a = tmu_pick_split(s, 2, sms, true), b = tmu32_pick_split(s, sms);
  int tiles = (s.n + TILE - 1) / TILE;
  int m = 2 * (a > b ? a : b);
  if (m > tiles) m = tiles;
  return m < 1 ? 1 : m;
}

size_t tmu_scratch_doubles(const DevSites &s, int nrhs, int nsplit) {
  return (size_t)nsplit * nrhs * s.n * 3;
}

template <typename T, int NRHS, bool KAHAN>
static void tmu_allpairs(const DevSites &s, const typename Vec4<T>::type *pos, const T *damp, const T *x,
                         T *partial, int nsplit, cudaStream_t st) {
  add_launch_count(1);
  int tiles = (s.n + TILE - 1) / TILE;
  int per = ((tiles + nsplit - 1) / nsplit) * TILE;
  dim3 grid((s.n + TPB - 1) / TPB, nsplit);
  T thr = (T)s.damp_thr;
  const float2 *wa = std::is_same<T, double>::value ? s.pol_wa32 : nullptr;
  float thr2m = damp_thr2_margin(s);
  if (s.amoeba)
    k_tmu<T, NRHS, true, KAHAN><<<grid, TPB, 0, st>>>(s.n, pos, damp, wa, x, partial, per, thr, thr2m);
  else
    k_tmu<T, NRHS, false, KAHAN><<<grid, TPB, 0, st>>>(s.n, pos, damp, wa, x, partial, per, thr, thr2m);
}

// Columns per launch: the widest of 8/4/2/1 not above what is left and gmax.
inline int column_group(int left, int gmax) {
  int g = left < gmax ? left : gmax;
  return g >= 8 ? 8 : (g >= 4 ? 4 : (g >= 2 ? 2 : 1));
}

template <typename T, bool KAHAN>
static void tmu_dispatch(const DevSites &s, int nrhs, const typename Vec4<T>::type *pos, const T *damp,
                         const T *x, T *partial, int nsplit, int gmax, cudaStream_t st, int kver = 1) {
  // process the columns in groups sharing the pair geometry; every group
  // has its own [split][g][n][3] block of partials, one after the other
  int done = 0;
  while (done < nrhs) {
    int g = column_group(nrhs - done, gmax);
    size_t xo = (size_t)done * s.n * 3;
    T *pg = partial + (size_t)nsplit * done * s.n * 3;
    if constexpr (std::is_same<T, float>::value) {
      if (kver == 2) {
        add_launch_count(1);
        launch_tmu32_pairs(s, g, x + xo, pg, nsplit, st);
        done += g;
        continue;
      }
    }
    switch (g) {
      case 8: tmu_allpairs<T, 8, KAHAN>(s, pos, damp, x + xo, pg, nsplit, st); break;
      case 4: tmu_allpairs<T, 4, KAHAN>(s, pos, damp, x + xo, pg, nsplit, st); break;
      case 2: tmu_allpairs<T, 2, KAHAN>(s, pos, damp, x + xo, pg, nsplit, st); break;
      default: tmu_allpairs<T, 1, KAHAN>(s, pos, damp, x + xo, pg, nsplit, st); break;
    }
    done += g;
  }
}

template <typename T>
static void tmu_finish(const DevSites &s, int nrhs, int nsplit, const T *partial,
                       const typename Vec4<T>::type *pos, const T *damp, const T *x, bool dodiag, T *y,
                       int gmax, cudaStream_t st) {
  // the same column groups as tmu_dispatch, each with its own block
  int done = 0;
  while (done < nrhs) {
    int g = column_group(nrhs - done, gmax);
    const T *pg = partial + (size_t)nsplit * done * s.n * 3;
    add_launch_count(1);
    dim3 grid((s.n + 127) / 128, g);
    size_t xo = (size_t)done * s.n * 3;
    const float2 *wa = std::is_same<T, double>::value ? s.pol_wa32 : nullptr;
    float thr2m = damp_thr2_margin(s);
    if (s.amoeba)
      k_tmu_finish<T, true><<<grid, 128, 0, st>>>(s.n, g, nsplit, pg, pos, damp, wa, x + xo, s.pol_alpha,
                                                  dodiag, s.d2d_nnz ? s.d2d_ri : nullptr, s.d2d_src, s.d2d_s,
                                                  (T)s.damp_thr, thr2m, y + xo);
    else
      k_tmu_finish<T, false><<<grid, 128, 0, st>>>(s.n, g, nsplit, pg, pos, damp, wa, x + xo, s.pol_alpha,
                                                   dodiag, s.d2d_nnz ? s.d2d_ri : nullptr, s.d2d_src, s.d2d_s,
                                                   (T)s.damp_thr, thr2m, y + xo);
    done += g;
  }
}

void launch_tmu_finish64(const DevSites &s, int nrhs, const double *partial, const double *x, bool dodiag,
                         double *y, cudaStream_t st) {
  tmu_finish<double>(s, nrhs, 1, partial, s.pol_pos, s.pol_a, x, dodiag, y, 2, st);
}

void launch_tmu_finish32(const DevSites &s, int nrhs, const float *partial, const float *x, float *y,
                         cudaStream_t st) {
  tmu_finish<float>(s, nrhs, 1, partial, s.pol_pos32, s.pol_a32, x, true, y, 2, st);
}

void launch_tmu_f64(const DevSites &s, int nrhs, const double *x, double *y, bool dodiag, double *scratch,
                    int nsplit, cudaStream_t st) {
  if (s.n == 0) return;
  tmu_dispatch<double, false>(s, nrhs, s.pol_pos, s.pol_a, x, scratch, nsplit, 4, st);
  tmu_finish<double>(s, nrhs, nsplit, scratch, s.pol_pos, s.pol_a, x, dodiag, y, 4, st);
}

void launch_tmu_ds(const DevSites &s, int nrhs, const double *x, double *y, bool dodiag, double *scratch,
                   int nsplit, double *sym_scratch, cudaStream_t st) {
  if (s.n == 0) return;
  const size_t nv = 3 * (size_t)s.n;
  const bool sym = sym_scratch && s.n >= 2048;
  for (int c = 0; c < nrhs;) {
    const int g = nrhs - c >= 2 ? 2 : 1;
    if (sym) {
      // fixed-point sums (layout of launch_tmu_f64_sym), read out to doubles
      const size_t C = 3 * (size_t)g;
      unsigned long long *lo = reinterpret_cast<unsigned long long *>(sym_scratch);
      unsigned long long *hi = lo + C * s.n;
      double *e = sym_scratch + 2 * C * s.n;
      unsigned long long *bad = reinterpret_cast<unsigned long long *>(sym_scratch + 3 * C * s.n);
      unsigned *next = reinterpret_cast<unsigned *>(bad + 1);
      cudaMemsetAsync(lo, 0, 2 * C * s.n * sizeof(unsigned long long), st);
      cudaMemsetAsync(bad, 0, sizeof(unsigned long long), st);
      launch_tmu_ds_sym_pairs(s, g, x + c * nv, lo, hi, bad, next, st);
      launch_fixed_to_double(C * s.n, lo, hi, bad, e, st);
      tmu_finish<double>(s, g, 1, e, s.pol_pos, s.pol_a, x + c * nv, dodiag, y + c * nv, 2, st);
    } else {
      add_launch_count(1);
      launch_tmu_ds_pairs(s, g, x + c * nv, scratch, nsplit, st);
      tmu_finish<double>(s, g, nsplit, scratch, s.pol_pos, s.pol_a, x + c * nv, dodiag, y + c * nv, 2, st);
    }
    c += g;
  }
}

namespace {
struct SymPlan {
  int ntile, K, chunk, nchunk, nitems, ctas;
};
template <int NRHS, bool AMOEBA>
struct SymLaunch {
  int resident = 0;
  SymLaunch() {
    const int smem = (int)sym_smem_bytes(NRHS);
    cudaFuncSetAttribute(k_tmu_sym<NRHS, AMOEBA>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, k_tmu_sym<NRHS, AMOEBA>, SYM_TILE, smem);
    if (resident < 1) resident = 1;
  }
};
template <int NRHS, bool AMOEBA>
int sym_resident() {
  static const SymLaunch<NRHS, AMOEBA> cfg;  // thread-safe one-time set-up
  return cfg.resident;
}

// work items: about 16 per resident CTA, each a tile and a chunk of its slots
// (round_pairs > 0: at most a quarter of a CTA's share of round_pairs)
SymPlan sym_plan(int n, int ctas, double round_pairs) {
  SymPlan p;
  p.ntile = (n + SYM_TILE - 1) / SYM_TILE;
  p.K = p.ntile / 2;
  const long long units = (long long)p.ntile * (p.K + 1);
  long long chunk = units / (16LL * ctas);
  if (round_pairs > 0.0) {
    const long long cap = (long long)(round_pairs / (4.0 * ctas * SYM_TILE * SYM_TILE));
    chunk = std::min(chunk, cap);
  }
  if (chunk < 1) chunk = 1;
  if (chunk > p.K + 1) chunk = p.K + 1;
  p.chunk = (int)chunk;
  p.nchunk = (p.K + 1 + p.chunk - 1) / p.chunk;
  p.nitems = p.ntile * p.nchunk;
  p.ctas = ctas < p.nitems ? ctas : p.nitems;
  return p;
}

int sym64_resident(int g, bool amoeba) {
  if (g == 4) return amoeba ? sym_resident<4, true>() : sym_resident<4, false>();
  if (g == 2) return amoeba ? sym_resident<2, true>() : sym_resident<2, false>();
  return amoeba ? sym_resident<1, true>() : sym_resident<1, false>();
}

template <int NRHS, bool AMOEBA>
void launch_sym64_table(const Sym64Table &tab, unsigned *next, cudaStream_t st) {
  const int total = tab.base[tab.njobs];
  if (total <= 0) return;
  const int ctas_max = sym_resident<NRHS, AMOEBA>() * sm_count();
  const int ctas = ctas_max < total ? ctas_max : total;
  cudaMemsetAsync(next, 0, sizeof(unsigned), st);
  k_tmu_sym<NRHS, AMOEBA><<<ctas, SYM_TILE, sym_smem_bytes(NRHS), st>>>(tab, next);
}
}  // namespace

int tmu_f64_sym_items(const DevSites &s, int g, double round_pairs) {
  if (s.n == 0) return 0;
  return sym_plan(s.n, sym64_resident(g, s.amoeba) * sm_count(), round_pairs).nitems;
}

void launch_tmu_f64_sym_multi(int g, bool amoeba, const SymSlice *sl, int nsl, unsigned *next, cudaStream_t st) {
  Sym64Table tab{};
  int total = 0;
  for (int k = 0; k < nsl && tab.njobs < kMaxSymSlices; ++k) {
    const DevSites &s = *sl[k].s;
    if (sl[k].count <= 0 || s.n == 0) continue;
    const SymPlan p = sym_plan(s.n, sym64_resident(g, amoeba) * sm_count(), sl[k].round_pairs);
    Sym64Job &j = tab.job[tab.njobs];
    j.pos = s.pol_pos, j.damp = s.pol_a, j.wa = s.pol_wa32, j.x = static_cast<const double *>(sl[k].x);
    j.lo = sl[k].lo, j.hi = sl[k].hi, j.bad = sl[k].bad;
    j.n = s.n, j.ntile = p.ntile, j.K = p.K, j.chunk = p.chunk, j.nchunk = p.nchunk, j.item0 = sl[k].item0;
    j.thr = s.damp_thr;
    j.thr2m = damp_thr2_margin(s);
    tab.base[tab.njobs] = total;
    total += sl[k].count;
    ++tab.njobs;
  }
  tab.base[tab.njobs] = total;
  if (!total) return;
  add_launch_count(1);
  if (g == 4)
    amoeba ? launch_sym64_table<4, true>(tab, next, st) : launch_sym64_table<4, false>(tab, next, st);
  else if (g == 2)
    amoeba ? launch_sym64_table<2, true>(tab, next, st) : launch_sym64_table<2, false>(tab, next, st);
  else
    amoeba ? launch_sym64_table<1, true>(tab, next, st) : launch_sym64_table<1, false>(tab, next, st);
}

void launch_fixed_to_double(size_t total, const unsigned long long *lo, const unsigned long long *hi,
                            const unsigned long long *bad, double *out, cudaStream_t st) {
  add_launch_count(1);
  k_fixed_to_double<<<blocks_for(total, 256), 256, 0, st>>>(total, lo, hi, bad, out);
}

size_t tmu_sym_scratch_doubles(const DevSites &s, int nrhs) {
  if (s.n == 0) return 0;
  // two 64-bit accumulator words and one double per value of a column group
  // (at most four columns), the error flag and the work counter
  size_t C = 3 * (size_t)(nrhs < 4 ? nrhs : 4);
  return 3 * C * (size_t)s.n + 2;
}

void launch_tmu_f64_sym(const DevSites &s, int nrhs, const double *x, double *y, bool dodiag, double *scratch,
                        cudaStream_t st, int gmax) {
  if (s.n == 0) return;
  // columns in groups of 4 or 2 (gmax, what the scratch holds) and a last
  // single one share the pair geometry
  int done = 0;
  while (done < nrhs) {
    const int left = nrhs - done;
    int g = (left >= 4 && gmax >= 4) ? 4 : (left >= 2 && gmax >= 2 ? 2 : 1);
    size_t C = 3 * (size_t)g;
    unsigned long long *lo = reinterpret_cast<unsigned long long *>(scratch);
    unsigned long long *hi = lo + C * s.n;
    double *e = scratch + 2 * C * s.n;
    unsigned long long *bad = reinterpret_cast<unsigned long long *>(scratch + 3 * C * s.n);
    unsigned *next = reinterpret_cast<unsigned *>(bad + 1);
    const double *xg = x + (size_t)done * s.n * 3;
    cudaMemsetAsync(lo, 0, 2 * C * s.n * sizeof(unsigned long long), st);
    cudaMemsetAsync(bad, 0, sizeof(unsigned long long), st);
    SymSlice one{&s, xg, lo, hi, bad, 0, tmu_f64_sym_items(s, g)};
    launch_tmu_f64_sym_multi(g, s.amoeba, &one, 1, next, st);
    launch_fixed_to_double(C * s.n, lo, hi, bad, e, st);
    launch_tmu_finish64(s, g, e, xg, dodiag, y + (size_t)done * s.n * 3, st);
    done += g;
  }
}

void launch_tmu_f32(const DevSites &s, int nrhs, const float *x, float *y, float *scratch, int nsplit,
                    cudaStream_t st, int gmax, int kver, double *sym_scratch) {
  if (s.n == 0) return;
  if (kver == 3 && sym_scratch) {
    // symmetric kernel: fixed-point sums read out as floats into the third
    // block of the symmetric scratch, then the shared finishing pass
    const size_t nv = 3 * (size_t)s.n;
    for (int c = 0; c < nrhs;) {
      const int g = (nrhs - c >= 2 && gmax >= 2) ? 2 : 1;
      const size_t C = 3 * (size_t)g;
      unsigned long long *lo = reinterpret_cast<unsigned long long *>(sym_scratch);
      unsigned long long *hi = lo + C * s.n;
      float *e = reinterpret_cast<float *>(sym_scratch + 2 * C * s.n);
      unsigned long long *bad = reinterpret_cast<unsigned long long *>(sym_scratch + 3 * C * s.n);
      unsigned *next = reinterpret_cast<unsigned *>(bad + 1);
      launch_tmu32_sym_pairs(s, g, x + c * nv, lo, hi, bad, next, e, st);
      tmu_finish<float>(s, g, 1, e, s.pol_pos32, s.pol_a32, x + c * nv, true, y + c * nv, 2, st);
      c += g;
    }
    return;
  }
  tmu_dispatch<float, true>(s, nrhs, s.pol_pos32, s.pol_a32, x, scratch, nsplit, gmax, st, kver);
  tmu_finish<float>(s, nrhs, nsplit, scratch, s.pol_pos32, s.pol_a32, x, true, y, gmax, st);
}

// z = M^-1 r, one thread per site and column: the three rows of the site's
// block times the run's slice of r
__global__ void k_block_apply(int n, const int4 *__restrict__ info, const float *__restrict__ minv,
                              const float *__restrict__ r, float *__restrict__ z) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const size_t co = (size_t)blockIdx.y * 3 * n;
  const int4 b = info[j];
  const int w = 3 * b.y;
  const float *rr = r + co + 3 * (size_t)b.x;
  const float *m0 = minv + b.z + (size_t)(3 * b.w) * w;
  const float *m1 = m0 + w, *m2 = m1 + w;
  float z0 = 0.f, z1 = 0.f, z2 = 0.f;
  for (int l = 0; l < w; ++l) {
    const float v = rr[l];
    z0 = fmaf(m0[l], v, z0);
    z1 = fmaf(m1[l], v, z1);
    z2 = fmaf(m2[l], v, z2);
  }
  float *zz = z + co + 3 * (size_t)j;
  zz[0] = z0;
  zz[1] = z1;
  zz[2] = z2;
}

// z -= B^-1 w, the second half of the Neumann step (w read over the run,
// z[j] read and written by its own thread, so z may hold z0 in place)
__global__ void k_block_apply_sub(int n, const int4 *__restrict__ info, const float *__restrict__ minv,
                                  const float *__restrict__ w, float *__restrict__ z) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const size_t co = (size_t)blockIdx.y * 3 * n;
  const int4 b = info[j];
  const int wd = 3 * b.y;
  const float *ww = w + co + 3 * (size_t)b.x;
  const float *m0 = minv + b.z + (size_t)(3 * b.w) * wd;
  const float *m1 = m0 + wd, *m2 = m1 + wd;
  float t0 = 0.f, t1 = 0.f, t2 = 0.f;
  for (int l = 0; l < wd; ++l) {
    const float v = ww[l];
    t0 = fmaf(m0[l], v, t0);
    t1 = fmaf(m1[l], v, t1);
    t2 = fmaf(m2[l], v, t2);
  }
  float *zz = z + co + 3 * (size_t)j;
  zz[0] -= t0;
  zz[1] -= t1;
  zz[2] -= t2;
}

// y[j] = sum over the near-field row j of N_ji x[i] (3x3 FP32 blocks)
__global__ void k_near_apply(int n, const int *__restrict__ ri, const int *__restrict__ ci,
                             const float *__restrict__ blk, const float *__restrict__ x, float *__restrict__ y) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const size_t co = (size_t)blockIdx.y * 3 * n;
  float y0 = 0.f, y1 = 0.f, y2 = 0.f;
  for (int e = ri[j]; e < ri[j + 1]; ++e) {
    const float *b = blk + 9 * (size_t)e;
    const float *xi = x + co + 3 * (size_t)ci[e];
    const float a = xi[0], c = xi[1], d = xi[2];
    y0 = fmaf(b[0], a, fmaf(b[1], c, fmaf(b[2], d, y0)));
    y1 = fmaf(b[3], a, fmaf(b[4], c, fmaf(b[5], d, y1)));
    y2 = fmaf(b[6], a, fmaf(b[7], c, fmaf(b[8], d, y2)));
  }
  float *yy = y + co + 3 * (size_t)j;
  yy[0] = y0;
  yy[1] = y1;
  yy[2] = y2;
}

void launch_near_correct(int ncol, int n, const int4 *info, const float *minv, const int *ri, const int *ci,
                         const float *blk, float *z, float *w, cudaStream_t st) {
  if (n == 0) return;
  add_launch_count(2);
  dim3 grid((n + 127) / 128, ncol);
  k_near_apply<<<grid, 128, 0, st>>>(n, ri, ci, blk, z, w);
  k_block_apply_sub<<<grid, 128, 0, st>>>(n, info, minv, w, z);
}

void launch_block_apply(int ncol, int n, const int4 *info, const float *minv, const float *r, float *z,
                        cudaStream_t st) {
  if (n == 0) return;
  add_launch_count(1);
  dim3 grid((n + 127) / 128, ncol);
  k_block_apply<<<grid, 128, 0, st>>>(n, info, minv, r, z);
}

// Batched right-hand sides, set-major columns: rhs[s*nf + f] = E_M2D[s] + field[f]
__global__ void k_batch_rhs(int n, int nf, int nset, const double *__restrict__ e_m2d,
                            const double *__restrict__ fields, double *__restrict__ rhs) {
  size_t nv = 3 * (size_t)n;
  size_t tot = nv * nf * nset;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < tot; i += (size_t)gridDim.x * blockDim.x) {
    size_t col = i / nv, e = i % nv;
    size_t set = col / nf, f = col % nf;
    rhs[i] = e_m2d[set * nv + e] + fields[f * nv + e];
  }
}

// out[f][s][n][3] from set-major solution columns; with nsolved == 1 the P
// set repeats the D column (identical systems)
__global__ void k_batch_scatter(int n, int nf, int nipd, int nsolved, const double *__restrict__ x,
                                double *__restrict__ out) {
  size_t nv = 3 * (size_t)n;
  size_t tot = nv * nf * nipd;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < tot; i += (size_t)gridDim.x * blockDim.x) {
    size_t e = i % nv, rest = i / nv;
    size_t set = rest % nipd, f = rest / nipd;
    size_t src_set = nsolved == 1 ? 0 : set;
    out[i] = x[(src_set * nf + f) * nv + e];
  }
}

void launch_batch_rhs(int n, int nf, int nset, const double *e_m2d, const double *fields, double *rhs,
                      cudaStream_t st) {
  add_launch_count(1);
  k_batch_rhs<<<blocks_for((size_t)3 * n * nf * nset, 256), 256, 0, st>>>(n, nf, nset, e_m2d, fields, rhs);
}

void launch_batch_scatter(int n, int nf, int nipd, int nsolved, const double *x, double *out, cudaStream_t st) {
  add_launch_count(1);
  k_batch_scatter<<<blocks_for((size_t)3 * n * nf * nipd, 256), 256, 0, st>>>(n, nf, nipd, nsolved, x, out);
}

// ---- dense T ------------------------------------------------------------------
void launch_build_tmat(const DevSites &s, double *tmat, cudaStream_t st) {
  add_launch_count(s.d2d_nnz ? 2 : 1);
  dim3 grid((s.n + 127) / 128, s.n);
  if (s.amoeba)
    k_build_tmat<true><<<grid, 128, 0, st>>>(s.n, s.pol_pos, s.pol_a, s.pol_alpha, s.damp_thr, tmat);
  else
    k_build_tmat<false><<<grid, 128, 0, st>>>(s.n, s.pol_pos, s.pol_a, s.pol_alpha, s.damp_thr, tmat);
  if (s.d2d_nnz) k_scale_tmat<<<(s.n + 127) / 128, 128, 0, st>>>(s.n, s.d2d_ri, s.d2d_src, s.d2d_s, tmat);
}

void launch_gemv(int nn, const double *A, const double *x, double *y, bool dodiag, const double *alpha,
                 int nrhs, cudaStream_t st) {
  add_launch_count(1);
  dim3 grid((nn + 127) / 128, nrhs);
  k_gemv<<<grid, 128, 0, st>>>(nn, A, x, y, dodiag, alpha);
}

void launch_lu_factor(int nn, double *A, int *piv, int *info, double *work, cudaStream_t st) {
  (void)work;
  cudaMemsetAsync(info, 0, sizeof(int), st);
  for (int k = 0; k < nn; ++k) {
    add_launch_count(nn - k - 1 > 0 ? 4 : 2);
    k_lu_pivot<<<1, 1024, 0, st>>>(nn, k, A, piv, info);
    k_lu_swap<<<(nn + 255) / 256, 256, 0, st>>>(nn, k, A, piv);
    int rows = nn - k - 1;
    if (rows > 0) {
      dim3 g((rows + 127) / 128, rows);
      k_lu_update<<<g, 128, 0, st>>>(nn, k, A, info);
      k_lu_scale<<<(rows + 127) / 128, 128, 0, st>>>(nn, k, A, info);
    }
  }
}

void launch_lu_solve(int nn, const double *A, const int *piv, double *b, cudaStream_t st) {
  add_launch_count(1);
  k_lu_solve<<<1, 1024, 0, st>>>(nn, A, piv, b);
}

// ---- BLAS-1 ---------------------------------------------------------------------
void launch_dots(int ncol, size_t n, const double *a, const double *b, double *partial, cudaStream_t st) {
  if (ncol < 1) return;
  add_launch_count(1);
  k_dots<double><<<dim3(dots_blocks(n), ncol), kRedThreads, 0, st>>>(ncol, n, a, b, n, partial);
}
void launch_dots_bcast(int ncol, size_t n, const double *a, const double *b, double *partial,
                       cudaStream_t st) {
  if (ncol < 1) return;
  add_launch_count(1);
  k_dots<double><<<dim3(dots_blocks(n), ncol), kRedThreads, 0, st>>>(ncol, n, a, b, 0, partial);
}
void launch_dots_f32(int ncol, size_t n, const float *a, const float *b, double *partial, cudaStream_t st) {
  if (ncol < 1) return;
  add_launch_count(1);
  k_dots<float><<<dim3(dots_blocks(n), ncol), kRedThreads, 0, st>>>(ncol, n, a, b, n, partial);
}
void launch_reduce_partials(int ncol, const double *partial, double *result, cudaStream_t st) {
  add_launch_count(1);
  k_reduce_partials<<<ncol, 32, 0, st>>>(ncol, kRedBlocks, partial, result);
}
void launch_axpby(size_t n, double a, const double *x, double b, double *y, cudaStream_t st) {
  add_launch_count(1);
  k_axpby<<<blocks_for(n, 256), 256, 0, st>>>(n, a, x, b, y);
}
void launch_add(size_t n, const double *a, const double *b, double *out, cudaStream_t st) {
  add_launch_count(1);
  k_add<<<blocks_for(n, 256), 256, 0, st>>>(n, a, b, out);
}
void launch_scale_by_alpha(int nrhs, int n, const double *alpha, const double *x, double *y, cudaStream_t st) {
  add_launch_count(1);
  k_scale_alpha<<<blocks_for((size_t)nrhs * n * 3, 256), 256, 0, st>>>(nrhs, n, alpha, x, y);
}
void launch_to_f32_cols(int ncol, size_t nv, const double *x, const double *scale, float *y, cudaStream_t st) {
  if (ncol < 1 || nv == 0) return;
  add_launch_count(1);
  const size_t tot = nv * (size_t)ncol;
  k_to_f32_cols<<<blocks_for(tot, 256), 256, 0, st>>>(nv, tot, x, scale, y);
}
void launch_to_f32(size_t n, const double *x, const double *scale, float *y, cudaStream_t st) {
  add_launch_count(1);
  k_to_f32<<<blocks_for(n, 256), 256, 0, st>>>(n, x, scale, y);
}
void launch_cg_init(int ncol, const double *dots, CgCol *cols, double tol, cudaStream_t st) {
  add_launch_count(1);
  k_cg_init<<<(ncol + 127) / 128, 128, 0, st>>>(ncol, dots, cols, tol);
}
void launch_cg_alpha(int ncol, const double *dots, CgCol *cols, double eps, cudaStream_t st) {
  add_launch_count(1);
  k_cg_alpha<<<(ncol + 127) / 128, 128, 0, st>>>(ncol, dots, cols, eps);
}
void launch_cg_update(int ncol, int n, double *x, double *r, const double *p, const double *h, double *z,
                      const double *alpha_pol, const CgCol *cols, double *partial, cudaStream_t st) {
  if (ncol < 1) return;
  add_launch_count(1);
  k_cg_update<double><<<dim3(kRedBlocks, ncol), kRedThreads, 0, st>>>(ncol, n, x, r, p, h, z, alpha_pol, cols,
                                                                      partial);
}
void launch_cg_update_f32(int ncol, int n, float *x, float *r, const float *p, const float *h, float *z,
                          const float *alpha_pol, const CgCol *cols, double *partial, cudaStream_t st) {
  if (ncol < 1) return;
  add_launch_count(1);
  k_cg_update<float><<<dim3(kRedBlocks, ncol), kRedThreads, 0, st>>>(ncol, n, x, r, p, h, z, alpha_pol, cols,
                                                                     partial);
}
void launch_cg_gnew(int ncol, int n, const double *dots, CgCol *cols, double *hist, int hist_stride,
                    cudaStream_t st) {
  add_launch_count(1);
  k_cg_gnew<<<(ncol + 127) / 128, 128, 0, st>>>(ncol, n, dots, cols, hist, hist_stride);
}
void launch_cg_pupdate(int ncol, int n, double *p, const double *z, const CgCol *cols, cudaStream_t st) {
  if (ncol < 1) return;
  add_launch_count(1);
  k_cg_pupdate<double><<<dim3(blocks_for(3 * (size_t)n, 256), ncol), 256, 0, st>>>(ncol, n, p, z, cols);
}
void launch_cg_pupdate_f32(int ncol, int n, float *p, const float *z, const CgCol *cols, cudaStream_t st) {
  if (ncol < 1) return;
  add_launch_count(1);
  k_cg_pupdate<float><<<dim3(blocks_for(3 * (size_t)n, 256), ncol), 256, 0, st>>>(ncol, n, p, z, cols);
}
void launch_ir_accumulate(int ncol, int n, double *mu, const float *d32, const double *scale, cudaStream_t st) {
  add_launch_count(1);
  k_ir_accumulate<<<blocks_for((size_t)ncol * n * 3, 256), 256, 0, st>>>(ncol, n, mu, d32, scale);
}
void launch_residual_update(int ncol, int n, double *r, const float *t32, const double *scale, cudaStream_t st) {
  add_launch_count(1);
  k_residual_update<<<blocks_for((size_t)ncol * n * 3, 256), 256, 0, st>>>(ncol, n, r, t32, scale);
}
void launch_residual(size_t total, const double *rhs, const double *tmu, double *r, cudaStream_t st) {
  add_launch_count(1);
  k_residual<<<blocks_for(total, 256), 256, 0, st>>>(total, rhs, tmu, r);
}
void launch_lincomb(int nvec, size_t n, const double *X, size_t ldx, const double *c, double *out,
                    cudaStream_t st) {
  add_launch_count(1);
  k_lincomb<<<blocks_for(n, 256), 256, 0, st>>>(nvec, n, X, ldx, c, out);
}
void launch_diff_norms(size_t n, const double *a, const double *b, double *partial, cudaStream_t st) {
  add_launch_count(1);
  k_diff_norms<<<kRedBlocks, kRedThreads, 0, st>>>(n, a, b, partial);
}
void launch_reduce_norms(const double *partial, double *out, cudaStream_t st) {
  add_launch_count(1);
  k_reduce_norms<<<1, 32, 0, st>>>(kRedBlocks, partial, out);
}
void launch_any_diff(size_t n, const double *a, const double *b, int *flag, cudaStream_t st) {
  add_launch_count(1);
  k_any_diff<<<blocks_for(n, 256), 256, 0, st>>>(n, a, b, flag);
}
void launch_check_finite(size_t n, const double *x, int *flag, cudaStream_t st) {
  add_launch_count(1);
  k_check_finite<<<blocks_for(n, 256), 256, 0, st>>>(n, x, flag);
}

}  // namespace gpu
}  // namespace ommp
