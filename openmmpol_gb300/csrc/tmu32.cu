// FP32 dipole-dipole operator of the mixed-precision inner solver.
//
// Same product as the target-outer FP32 kernel in kernels.cu (the reference's
// field_extD2D double loop, src/mod_electrostatics.F90:1954-2111, and TMatVec_otf,
// src/mod_polarization.F90:459-481, restated
// for one FP32 launch per column group), organised for GB300's FP32 pipes:
//
//  * two targets per thread for one or two columns, so every source record
//    read from shared memory (one 16-byte position record and one 16-byte
//    dipole record per column) feeds two pairs and two independent
//    dependency chains;
//  * a per-tile classification: each 128-site source tile is compared with
//    the bounding box of the CTA's targets, and when the boxes are farther
//    apart than the largest distance at which Thole damping can act, the
//    whole tile runs an undamped inner loop with no self-pair test (20 FP32
//    instructions and one MUFU per pair and column); only the few tiles
//    near the targets run the damped loop;
//  * compensated (Kahan) accumulation across tiles, as before, and the same
//    [split][column][n][3] partial layout, so the scaled-pair correction and
//    diagonal pass (k_tmu_finish) is shared.
//
// Compiled with -ftz=true: the reciprocal square root is the plain MUFU
// approximation (r^2 is never subnormal for distinct sites).
#include <cmath>

#include "kernels.h"

namespace ommp {
namespace gpu {

namespace {

constexpr int T32_TPB = 128;   // threads per CTA
constexpr int T32_TILE = 128;  // sources per shared-memory tile (= tile-box granularity)

template <bool AMOEBA>
__device__ __forceinline__ void damped_factors(float r2, float wt, float ws, float at, float as, float thr,
                                               float &k3, float &k5) {
  float rinv = rsqrtf(r2);
  float ir2 = rinv * rinv;
  k3 = rinv * ir2;
  k5 = k3 * ir2;
  float u = r2 * rinv * (wt * ws);
  if (AMOEBA) {
    float au3 = fminf(at, as) * u * u * u;
    if (au3 < thr) {
      float e = __expf(-au3);
      k3 *= 1.f - e;
      k5 *= 1.f - (1.f + au3) * e;
    }
  } else {
    if (u < 1.f) {
      float u3 = u * u * u;
      float u4 = u3 * u;
      k3 *= 4.f * u3 - 3.f * u4;
      k5 *= u4;
    }
  }
}

// partial[split][g][j][3] over the split's sources.  TPT targets per thread:
// target t of thread x is blockIdx.x * TPB * TPT + t * TPB + x.
template <int G, int TPT, bool AMOEBA>
__global__ void __launch_bounds__(T32_TPB) k_tmu32(int n, const float4 *__restrict__ pos,
                                                   const float *__restrict__ damp,
                                                   const float4 *__restrict__ boxes, const float *__restrict__ x,
                                                   float *__restrict__ partial, int per_split, float thr,
                                                   float r2max) {
  __shared__ float4 s_pos[T32_TILE];
  __shared__ float4 s_mu[G][T32_TILE];  // x, y, z of column c; w = damping a of the source
  const int jb = blockIdx.x * (T32_TPB * TPT);
  float4 pt[TPT];
  float at[TPT];
  bool valid[TPT];
#pragma unroll
  for (int t = 0; t < TPT; ++t) {
    int j = jb + t * T32_TPB + threadIdx.x;
    valid[t] = j < n;
    pt[t] = valid[t] ? pos[j] : make_float4(0.f, 0.f, 0.f, 0.f);
    at[t] = (valid[t] && AMOEBA) ? damp[j] : 0.f;
  }
  // bounding box of this CTA's targets (the tiles they span)
  const int ntile = (n + T32_TILE - 1) / T32_TILE;
  const int tb0 = jb / T32_TILE;
  const int tb1 = min(ntile - 1, (jb + T32_TPB * TPT - 1) / T32_TILE);
  float4 blo = boxes[2 * tb0], bhi = boxes[2 * tb0 + 1];
  for (int tb = tb0 + 1; tb <= tb1; ++tb) {
    float4 lo = boxes[2 * tb], hi = boxes[2 * tb + 1];
    blo.x = fminf(blo.x, lo.x), blo.y = fminf(blo.y, lo.y), blo.z = fminf(blo.z, lo.z);
    bhi.x = fmaxf(bhi.x, hi.x), bhi.y = fmaxf(bhi.y, hi.y), bhi.z = fmaxf(bhi.z, hi.z);
  }

  // per tile the field 3 sum f d - sum k3 mu (f = k5 mu.d) is kept as its
  // two sums (one FMA per component each), combined into the compensated
  // cross-tile sum
  float acc[TPT][G * 3], acb[TPT][G * 3], sum[TPT][G * 3], comp[TPT][G * 3];
#pragma unroll
  for (int t = 0; t < TPT; ++t)
#pragma unroll
    for (int c = 0; c < G * 3; ++c) sum[t][c] = comp[t][c] = 0.f;

  const int s0 = blockIdx.y * per_split;
  const int s1 = min(n, s0 + per_split);
  for (int t0 = s0; t0 < s1; t0 += T32_TILE) {
    __syncthreads();
    {
      const int k = threadIdx.x;  // T32_TILE == T32_TPB
      const int i = t0 + k;
      if (i < s1) {
        s_pos[k] = pos[i];
        const float a = AMOEBA ? damp[i] : 0.f;
#pragma unroll
        for (int c = 0; c < G; ++c) {
          const float *xi = x + ((size_t)c * n + i) * 3;
          s_mu[c][k] = make_float4(xi[0], xi[1], xi[2], a);
        }
      }
    }
    __syncthreads();
    const int cnt = min(T32_TILE, s1 - t0);
    // uniform over the CTA: is any pair of this tile within damping range?
    const float4 slo = boxes[2 * (t0 / T32_TILE)], shi = boxes[2 * (t0 / T32_TILE) + 1];
    const float gx = fmaxf(0.f, fmaxf(slo.x - bhi.x, blo.x - shi.x));
    const float gy = fmaxf(0.f, fmaxf(slo.y - bhi.y, blo.y - shi.y));
    const float gz = fmaxf(0.f, fmaxf(slo.z - bhi.z, blo.z - shi.z));
    const bool far_tile = gx * gx + gy * gy + gz * gz > r2max;
#pragma unroll
    for (int t = 0; t < TPT; ++t)
#pragma unroll
      for (int c = 0; c < G * 3; ++c) acc[t][c] = acb[t][c] = 0.f;
    if (far_tile) {
#pragma unroll 4
      for (int k = 0; k < cnt; ++k) {
        const float4 ps = s_pos[k];
#pragma unroll
        for (int t = 0; t < TPT; ++t) {
          const float dx = pt[t].x - ps.x, dy = pt[t].y - ps.y, dz = pt[t].z - ps.z;
          const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
          const float rinv = rsqrtf(r2);
          const float ir2 = rinv * rinv;
          const float k3 = rinv * ir2;
          const float k5 = k3 * ir2;
#pragma unroll
          for (int c = 0; c < G; ++c) {
            const float4 m = s_mu[c][k];
            const float f = k5 * fmaf(m.x, dx, fmaf(m.y, dy, m.z * dz));
            acc[t][c * 3 + 0] = fmaf(f, dx, acc[t][c * 3 + 0]);
            acc[t][c * 3 + 1] = fmaf(f, dy, acc[t][c * 3 + 1]);
            acc[t][c * 3 + 2] = fmaf(f, dz, acc[t][c * 3 + 2]);
            acb[t][c * 3 + 0] = fmaf(k3, m.x, acb[t][c * 3 + 0]);
            acb[t][c * 3 + 1] = fmaf(k3, m.y, acb[t][c * 3 + 1]);
            acb[t][c * 3 + 2] = fmaf(k3, m.z, acb[t][c * 3 + 2]);
          }
        }
      }
    } else {
#pragma unroll 2
      for (int k = 0; k < cnt; ++k) {
        const float4 ps = s_pos[k];
        const float as = s_mu[0][k].w;
#pragma unroll
        for (int t = 0; t < TPT; ++t) {
          if (!valid[t] || t0 + k == jb + t * T32_TPB + (int)threadIdx.x) continue;
          const float dx = pt[t].x - ps.x, dy = pt[t].y - ps.y, dz = pt[t].z - ps.z;
          const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
          float k3, k5;
          damped_factors<AMOEBA>(r2, pt[t].w, ps.w, at[t], as, thr, k3, k5);
#pragma unroll
          for (int c = 0; c < G; ++c) {
            const float4 m = s_mu[c][k];
            const float f = k5 * fmaf(m.x, dx, fmaf(m.y, dy, m.z * dz));
            acc[t][c * 3 + 0] = fmaf(f, dx, acc[t][c * 3 + 0]);
            acc[t][c * 3 + 1] = fmaf(f, dy, acc[t][c * 3 + 1]);
            acc[t][c * 3 + 2] = fmaf(f, dz, acc[t][c * 3 + 2]);
            acb[t][c * 3 + 0] = fmaf(k3, m.x, acb[t][c * 3 + 0]);
            acb[t][c * 3 + 1] = fmaf(k3, m.y, acb[t][c * 3 + 1]);
            acb[t][c * 3 + 2] = fmaf(k3, m.z, acb[t][c * 3 + 2]);
          }
        }
      }
    }
    // compensated cross-tile accumulation
#pragma unroll
    for (int t = 0; t < TPT; ++t)
#pragma unroll
      for (int c = 0; c < G * 3; ++c) {
        const float y = fmaf(3.f, acc[t][c], -acb[t][c]) - comp[t][c];
        const float s = sum[t][c] + y;
        comp[t][c] = (s - sum[t][c]) - y;
        sum[t][c] = s;
      }
  }
#pragma unroll
  for (int t = 0; t < TPT; ++t) {
    const int j = jb + t * T32_TPB + threadIdx.x;
    if (!valid[t]) continue;
#pragma unroll
    for (int c = 0; c < G; ++c)
#pragma unroll
      for (int e = 0; e < 3; ++e) partial[(((size_t)blockIdx.y * G + c) * n + j) * 3 + e] = sum[t][c * 3 + e];
  }
}

template <int G, int TPT>
void launch_g(const DevSites &s, const float *x, float *partial, int nsplit, cudaStream_t st) {
  const int tiles = (s.n + T32_TILE - 1) / T32_TILE;
  const int per = ((tiles + nsplit - 1) / nsplit) * T32_TILE;
  dim3 grid((s.n + T32_TPB * TPT - 1) / (T32_TPB * TPT), nsplit);
  if (s.amoeba)
    k_tmu32<G, TPT, true><<<grid, T32_TPB, 0, st>>>(s.n, s.pol_pos32, s.pol_a32, s.tile_box32, x, partial, per,
                                                    (float)s.damp_thr, s.damp_r2max32);
  else
    k_tmu32<G, TPT, false><<<grid, T32_TPB, 0, st>>>(s.n, s.pol_pos32, s.pol_a32, s.tile_box32, x, partial, per,
                                                     (float)s.damp_thr, s.damp_r2max32);
}

}  // namespace

// one column group through the v2 pair kernel (g = 1, 2, 4 or 8)
void launch_tmu32_pairs(const DevSites &s, int g, const float *x, float *partial, int nsplit, cudaStream_t st) {
  switch (g) {
    case 8: launch_g<8, 1>(s, x, partial, nsplit, st); break;
    case 4: launch_g<4, 1>(s, x, partial, nsplit, st); break;
    case 2: launch_g<2, 2>(s, x, partial, nsplit, st); break;
    default: launch_g<1, 2>(s, x, partial, nsplit, st); break;
  }
}

int tmu32_pick_split(const DevSites &s, int sms) {
  // about six CTAs per SM for the one-column shape (two targets per thread)
  const int tblocks = (s.n + 2 * T32_TPB - 1) / (2 * T32_TPB);
  const int tiles = (s.n + T32_TILE - 1) / T32_TILE;
  int split = (6 * sms + tblocks - 1) / tblocks;
  if (split > tiles) split = tiles;
  return split < 1 ? 1 : split;
}

void tile_boxes32(const float4 *p, int n, float4 *boxes) {
  const int ntile = (n + T32_TILE - 1) / T32_TILE;
  for (int t = 0; t < ntile; ++t) {
    float4 lo = make_float4(INFINITY, INFINITY, INFINITY, 0.f), hi = make_float4(-INFINITY, -INFINITY, -INFINITY, 0.f);
    for (int i = t * T32_TILE; i < n && i < (t + 1) * T32_TILE; ++i) {
      lo.x = std::fmin(lo.x, p[i].x), lo.y = std::fmin(lo.y, p[i].y), lo.z = std::fmin(lo.z, p[i].z);
      hi.x = std::fmax(hi.x, p[i].x), hi.y = std::fmax(hi.y, p[i].y), hi.z = std::fmax(hi.z, p[i].z);
    }
    boxes[2 * t] = lo;
    boxes[2 * t + 1] = hi;
  }
}

float damp_r2max32(bool amoeba, double damp_thr, const double *inv_thole, const double *a, int n) {
  // AMOEBA damps when min(a_i, a_j) (r w_i w_j)^3 < thr (w = 1/thole), Wang-AL
  // when r w_i w_j < 1; bound r by the smallest w and the smallest a
  double wmin = INFINITY, amin = INFINITY;
  for (int i = 0; i < n; ++i) {
    wmin = std::fmin(wmin, inv_thole[i]);
    if (amoeba) amin = std::fmin(amin, a[i]);
  }
  if (n == 0) return 0.f;
  if (!(wmin > 0.0) || (amoeba && !(amin > 0.0))) return INFINITY;  // damping at any distance
  double rmax = amoeba ? std::cbrt(damp_thr / amin) / (wmin * wmin) : 1.0 / (wmin * wmin);
  // margin for the FP32 rounding of positions, boxes and the bound itself
  rmax = rmax * 1.001 + 1e-3;
  return (float)(rmax * rmax);
}

float m2d_r2max32(bool amoeba, double damp_thr, const double *pol_w, const double *pol_a, int n, const double *mm_w,
                  const double *mm_a, int m) {
  // a pair (polarizable target t, static source s) is damped only if
  // min(a_t, a_s) (r w_t w_s)^3 < thr (AMOEBA) or r w_t w_s < 1 (Wang-AL);
  // sources with w = inf (no Thole factor) or a = 0 (AMOEBA) never are
  if (n == 0 || m == 0) return 0.f;
  double wt = INFINITY, ws = INFINITY, amin = INFINITY;
  for (int i = 0; i < n; ++i) {
    wt = std::fmin(wt, pol_w[i]);
    if (amoeba) amin = std::fmin(amin, pol_a[i]);
  }
  bool any = false;
  for (int i = 0; i < m; ++i) {
    if (!std::isfinite(mm_w[i])) continue;
    if (amoeba && !(mm_a[i] > 0.0)) continue;
    any = true;
    ws = std::fmin(ws, mm_w[i]);
    if (amoeba) amin = std::fmin(amin, mm_a[i]);
  }
  if (!any) return 0.f;  // no source can be damped
  if (!(wt > 0.0) || !(ws > 0.0) || (amoeba && !(amin > 0.0))) return INFINITY;
  double rmax = amoeba ? std::cbrt(damp_thr / amin) / (wt * ws) : 1.0 / (wt * ws);
  rmax = rmax * 1.001 + 1e-3;
  return (float)(rmax * rmax);
}

}  // namespace gpu
}  // namespace ommp
