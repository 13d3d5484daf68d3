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
//
// The symmetric form (k_tmu32_sym, further down) evaluates each unordered
// pair once and accumulates both directions, as the FP64 product does.
#include <algorithm>
#include <cmath>

#include "kernels.h"
#include "pair_math.cuh"

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

// ---------------------------------------------------------------------------
// Symmetric FP32 operator.  The ordered kernel above spends ~20 FP32
// instructions per ordered pair, half of them on the geometry (differences,
// r^2, powers), which T_ij = T_ji lets two directions share.  Here every
// unordered pair is evaluated once: 9 geometry operations and 10 per
// direction (mu.d, the field factor, six accumulations), 29 in all instead of
// 40, on the half-shell schedule of the symmetric FP64 product (super-tile I
// meets the slots k = 0..ntile/2 of J = I + k, handed out by an atomic
// counter to a persistent grid).
//
// The arithmetic runs on pairs of sources with the paired FP32 instructions
// of sm_100 and later (__fadd2_rn, __fmul2_rn, __ffma2_rn: two FP32 lanes
// per instruction), so that 30 paired operations (with -k3/3 below) serve
// two pairs.  With scalar instructions the kernel was bound by instruction
// issue (77 % issue activity, FMA pipe 65 %); paired, it issues ~40 % fewer
// instructions per pair and the FMA pipe bounds it (a paired instruction
// holds the pipe for two cycles: the lane rate is the same).  Only the
// reciprocal square root and the damping test of near pairs stay per lane.
//
// Per CTA 128 threads own a super-tile of 256 targets, two per thread (lanes
// l and l + 32 of a 64-target warp slice).  J is staged as four sub-tiles of
// 64 sources, each as 32 source pairs (sources p and p + 32 of the sub-tile)
// in float4 records of two fields each ({f_a, f_b, g_a, g_b}: x, y, z, then
// mx, my, mz per column), every record twice in a row.  A warp meets a
// sub-tile in 32 rotation steps: at step t lane l takes pair (l + t) mod 32
// from its base address plus t (an immediate offset, no wrap-around) and
// evaluates it against both its targets (four pairs per step); the pair's
// source-side sums travel one lane per step by shuffle (two per component,
// 1.5 per pair).  The target side keeps the field's two sums (f d and k3 mu,
// f = k5 mu.d, each as a pair of partial sums over the two halves) and
// applies the factor 3 once per slot; the source side accumulates
// g d - (k3/3) mu (one extra product for -k3/3 per target and pair, where
// a second set of target dipoles would cost 12 registers per column) and
// the factor 3 is applied when the four warps' sums are combined.  The
// targets' compensated cross-slot sums live in shared memory.  The
// differences are taken as source minus target: every term is even in d.
//
// Slots whose tile boxes are farther apart than the damping range run an
// undamped loop; near slots and the diagonal slot (target side only, all
// ordered pairs of the tile, self pairs skipped) run the damped one.  Absent
// sites of the last tile sit at +-1e15 with zero dipoles.  Slot sums
// (FP32, at most 256 terms) go into per-site 128-bit fixed-point
// accumulators with integer atomics (converted from FP32 by integer
// operations), so the product is deterministic in any CTA order.
// ---------------------------------------------------------------------------
constexpr int S32_TPB = 128;
constexpr int S32_TILE = 256;
constexpr int S32_SUB = 64;  // sources per sub-tile (32 pairs)
constexpr int S32_NSUB = S32_TILE / S32_SUB;
constexpr float S32_FAR = 1.0e15f;

// float4 records per source pair: fields x, y, z, then mx, my, mz of each
// column, two fields per record
template <int G>
__host__ __device__ constexpr int s32_records() {
  return (3 + 3 * G + 1) / 2;
}

template <int G>
struct S32Smem {
  float4 rec[s32_records<G>()][S32_NSUB][2 * 32];  // each pair twice in a row
  float4 thole[S32_NSUB][2 * 32];                  // {w_a, w_b, a_a, a_b}: Thole factor, damping a
  float accj[4][3 * G][S32_TILE];                  // source-side sums of the four warps
  float sum[2][3 * G][S32_TPB], cmp[2][3 * G][S32_TPB];  // targets' compensated sums over slots
};

// fixed_add (pair_math.cuh) for an FP32 value, with integer operations only:
// the same 128-bit accumulator (units of 2^-80, hi holding the bits from
// 2^-16 up), fed with |v| = m 2^(e - 150) shifted to m 2^(e - 70) units and
// negated in two's complement for negative v.  The FP64 conversion of
// fixed_add takes ~6 FP64 instructions per value at 1/64 of the FP32 rate.
// |v| >= 2^36 (or not finite) raises the flag; |v| < 2^-80 adds nothing.
__device__ __forceinline__ void fixed_add_f32(unsigned long long *lo, unsigned long long *hi, float v,
                                              unsigned long long *bad) {
  const unsigned b = __float_as_uint(v);
  const int e = (int)((b >> 23) & 0xffu);
  if (e >= 127 + 36) {
    atomicOr(bad, 1ull);
    return;
  }
  const int sh = e - 70;
  if (e == 0 || sh <= -24) return;
  const unsigned long long m = (unsigned long long)((b & 0x7fffffu) | 0x800000u);
  unsigned long long l, h;
  if (sh < 0) {
    l = m >> (-sh);
    h = 0ull;
  } else if (sh < 64) {
    l = m << sh;
    h = sh == 0 ? 0ull : m >> (64 - sh);
  } else {
    l = 0ull;
    h = m << (sh - 64);
  }
  if (b >> 31) {
    l = ~l + 1ull;
    h = ~h + (l == 0ull ? 1ull : 0ull);
  }
  const unsigned long long old = atomicAdd(lo, l);
  atomicAdd(hi, h + (old + l < old ? 1ull : 0ull));
}

__device__ __forceinline__ void box_of_supertile(const float4 *__restrict__ boxes, int nbox, int T, float4 &lo,
                                                 float4 &hi) {
  lo = boxes[4 * T];
  hi = boxes[4 * T + 1];
  if (2 * T + 1 < nbox) {
    const float4 l2 = boxes[4 * T + 2], h2 = boxes[4 * T + 3];
    lo.x = fminf(lo.x, l2.x), lo.y = fminf(lo.y, l2.y), lo.z = fminf(lo.z, l2.z);
    hi.x = fmaxf(hi.x, h2.x), hi.y = fmaxf(hi.y, h2.y), hi.z = fmaxf(hi.z, h2.z);
  }
}

// damped_factors for a pair of sources against one target: the powers of
// 1/r on paired instructions, the damping test per half (a half beyond the
// damping range keeps its factors exactly: e = 0, or the factor 1)
template <bool AMOEBA>
__device__ __forceinline__ void damped_factors2(float2 r2, float wt, float2 ws, float at, float2 as, float thr,
                                                float2 &k3, float2 &k5) {
  const float2 rinv = make_float2(rsqrtf(r2.x), rsqrtf(r2.y));
  const float2 ir2 = __fmul2_rn(rinv, rinv);
  k3 = __fmul2_rn(rinv, ir2);
  k5 = __fmul2_rn(k3, ir2);
  const float2 u = __fmul2_rn(__fmul2_rn(r2, rinv), __fmul2_rn(make_float2(wt, wt), ws));
  const float2 one = make_float2(1.f, 1.f);
  if (AMOEBA) {
    const float2 am = make_float2(fminf(at, as.x), fminf(at, as.y));
    const float2 au3 = __fmul2_rn(__fmul2_rn(__fmul2_rn(am, u), u), u);
    if (au3.x < thr || au3.y < thr) {
      const float2 e = make_float2(au3.x < thr ? __expf(-au3.x) : 0.f, au3.y < thr ? __expf(-au3.y) : 0.f);
      k3 = __fmul2_rn(k3, __ffma2_rn(make_float2(-1.f, -1.f), e, one));
      k5 = __fmul2_rn(k5, __ffma2_rn(make_float2(-1.f - au3.x, -1.f - au3.y), e, one));
    }
  } else if (u.x < 1.f || u.y < 1.f) {
    const float2 u3 = __fmul2_rn(__fmul2_rn(u, u), u);
    const float2 u4 = __fmul2_rn(u3, u);
    const float2 f3 = __ffma2_rn(make_float2(4.f, 4.f), u3, __fmul2_rn(make_float2(-3.f, -3.f), u4));
    k3 = __fmul2_rn(k3, make_float2(u.x < 1.f ? f3.x : 1.f, u.y < 1.f ? f3.y : 1.f));
    k5 = __fmul2_rn(k5, make_float2(u.x < 1.f ? u4.x : 1.f, u.y < 1.f ? u4.y : 1.f));
  }
}

// a target's values as lane pairs, the same value in both halves
struct S32Target {
  float2 nx, ny, nz;  // minus the position
  float w, a;         // Thole factor and damping a (near slots)
  int idx;            // index in the super-tile
};

// one slot: the warp's 64 targets against the 256 staged sources.  The far
// loop is unrolled by 8 and the near one not at all: fully unrolled, the two
// loops overflowed the instruction cache (ncu: issue stalled on instruction
// fetch, 44 % issue activity).
template <bool NEAR, bool AMOEBA, int G>
__device__ __forceinline__ void s32_slot(bool diag, S32Smem<G> &sm, int warp, int lane, const S32Target (&tg)[2],
                                         const float2 (&mt)[2][3 * G], float thr,
                                         float2 (&af)[2][3 * G], float2 (&ak)[2][3 * G]) {
  constexpr int C = 3 * G, R = s32_records<G>();
  const int src = (lane + 1) & 31;
  const bool source_side = !NEAR || !diag;
#pragma unroll 1
  for (int js = 0; js < S32_NSUB; ++js) {
    float2 aj[C];
#pragma unroll
    for (int c = 0; c < C; ++c) aj[c] = make_float2(0.f, 0.f);
    auto step = [&](int t) {
      float2 f[2 * R];  // x, y, z, mx, my, mz, ... of the pair
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const float4 v = sm.rec[r][js][lane + t];
        f[2 * r] = make_float2(v.x, v.y);
        f[2 * r + 1] = make_float2(v.z, v.w);
      }
      float4 th;
      if (NEAR) th = sm.thole[js][lane + t];
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const float2 dx = __fadd2_rn(f[0], tg[u].nx), dy = __fadd2_rn(f[1], tg[u].ny),
                     dz = __fadd2_rn(f[2], tg[u].nz);
        const float2 r2 = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __fmul2_rn(dz, dz)));
        float2 k3, k5;
        if (NEAR) {
          // the self pair of the diagonal slot contributes nothing
          const int p = (lane + t) & 31;
          const bool self_a = diag && js * S32_SUB + p == tg[u].idx;
          const bool self_b = diag && js * S32_SUB + 32 + p == tg[u].idx;
          damped_factors2<AMOEBA>(make_float2(self_a ? 1.f : r2.x, self_b ? 1.f : r2.y), tg[u].w,
                                  make_float2(th.x, th.y), tg[u].a, make_float2(th.z, th.w), thr, k3, k5);
          if (self_a) k3.x = k5.x = 0.f;
          if (self_b) k3.y = k5.y = 0.f;
        } else {
          const float2 rinv = make_float2(rsqrtf(r2.x), rsqrtf(r2.y));
          const float2 ir2 = __fmul2_rn(rinv, rinv);
          k3 = __fmul2_rn(rinv, ir2);
          k5 = __fmul2_rn(k3, ir2);
        }
        float2 k3n;
        if (source_side) k3n = __fmul2_rn(k3, make_float2(-1.f / 3.f, -1.f / 3.f));
#pragma unroll
        for (int col = 0; col < G; ++col) {
          const float2 mx = f[3 + 3 * col], my = f[4 + 3 * col], mz = f[5 + 3 * col];
          const float2 fs = __fmul2_rn(k5, __ffma2_rn(mx, dx, __ffma2_rn(my, dy, __fmul2_rn(mz, dz))));
          af[u][3 * col + 0] = __ffma2_rn(fs, dx, af[u][3 * col + 0]);
          af[u][3 * col + 1] = __ffma2_rn(fs, dy, af[u][3 * col + 1]);
          af[u][3 * col + 2] = __ffma2_rn(fs, dz, af[u][3 * col + 2]);
          ak[u][3 * col + 0] = __ffma2_rn(k3, mx, ak[u][3 * col + 0]);
          ak[u][3 * col + 1] = __ffma2_rn(k3, my, ak[u][3 * col + 1]);
          ak[u][3 * col + 2] = __ffma2_rn(k3, mz, ak[u][3 * col + 2]);
          if (source_side) {
            const float2 g = __fmul2_rn(
                k5, __ffma2_rn(mt[u][3 * col], dx,
                               __ffma2_rn(mt[u][3 * col + 1], dy, __fmul2_rn(mt[u][3 * col + 2], dz))));
            aj[3 * col + 0] = __ffma2_rn(g, dx, __ffma2_rn(k3n, mt[u][3 * col + 0], aj[3 * col + 0]));
            aj[3 * col + 1] = __ffma2_rn(g, dy, __ffma2_rn(k3n, mt[u][3 * col + 1], aj[3 * col + 1]));
            aj[3 * col + 2] = __ffma2_rn(g, dz, __ffma2_rn(k3n, mt[u][3 * col + 2], aj[3 * col + 2]));
          }
        }
      }
      if (source_side) {
        // the sums of pair p move to the lane that meets p next
#pragma unroll
        for (int c = 0; c < C; ++c) {
          aj[c].x = __shfl_sync(0xffffffffu, aj[c].x, src);
          aj[c].y = __shfl_sync(0xffffffffu, aj[c].y, src);
        }
      }
    };
    if (NEAR) {
#pragma unroll 1  // near steps
      for (int t = 0; t < 32; ++t) step(t);
    } else {
#pragma unroll 8  // far steps
      for (int t = 0; t < 32; ++t) step(t);
    }
    if (source_side) {
      // after 32 steps lane l holds the sums of pair l: sources l and l + 32
#pragma unroll
      for (int c = 0; c < C; ++c) {
        sm.accj[warp][c][js * S32_SUB + lane] = aj[c].x;
        sm.accj[warp][c][js * S32_SUB + 32 + lane] = aj[c].y;
      }
    }
  }
}

// One launch serves the products of several systems (a multi-system work
// queue): job j covers the items [item0, item0 + base[j+1] - base[j]) of
// its system's product, and the persistent CTAs take global items in order
// from one counter.  A product's item space is fixed per system (the super-
// tile I and a chunk of its slots), so a product may also be spread over
// several launches; its fixed-point sums add up across them.  A one-job
// table is the single-system product.
struct S32Job {
  const float4 *pos;
  const float *damp;
  const float4 *boxes;
  const float *x;
  unsigned long long *lo, *hi, *bad;
  int n, ntile, nbox, K, chunk, nchunk, item0, amoeba;
  float thr, r2max;
};
struct S32Table {
  int njobs;
  int base[kMaxSymSlices + 1];  // first global item of each job; base[njobs] = total
  S32Job job[kMaxSymSlices];
};

template <int G>
__global__ void __launch_bounds__(S32_TPB, G == 1 ? 4 : 3) k_tmu32_sym(const __grid_constant__ S32Table tab,
                                                                       unsigned *__restrict__ next) {
  constexpr int C = 3 * G, R = s32_records<G>();
  extern __shared__ float4 s32_dyn[];
  S32Smem<G> &sm = *reinterpret_cast<S32Smem<G> *>(s32_dyn);
  __shared__ int s_item;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int total = tab.base[tab.njobs];
  for (;;) {
    __syncthreads();  // every thread has read the previous item and its sums
    if (tid == 0) s_item = (int)atomicAdd(next, 1u);
    __syncthreads();
    const int item = s_item;
    if (item >= total) break;
    int jx = 0;
    while (jx + 1 < tab.njobs && tab.base[jx + 1] <= item) ++jx;
    const S32Job &jb = tab.job[jx];
    const int n = jb.n, ntile = jb.ntile, nchunk = jb.nchunk;
    const float4 *__restrict__ pos = jb.pos;
    const float *__restrict__ damp = jb.damp;
    const float *__restrict__ x = jb.x;
    const bool amoeba = jb.amoeba != 0;
    const int local = jb.item0 + (item - tab.base[jx]);
    const int I = local / nchunk;
    S32Target tg[2];
    float2 mt[2][C];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      tg[u].idx = warp * 64 + u * 32 + lane;
      const int ti = I * S32_TILE + tg[u].idx;
      const bool v = ti < n;
      const float4 p = v ? pos[ti] : make_float4(S32_FAR, S32_FAR, S32_FAR, 0.f);
      tg[u].nx = make_float2(-p.x, -p.x), tg[u].ny = make_float2(-p.y, -p.y), tg[u].nz = make_float2(-p.z, -p.z);
      tg[u].w = p.w;
      tg[u].a = (amoeba && v) ? damp[ti] : 0.f;
#pragma unroll
      for (int c = 0; c < C; ++c) {
        const float m = v ? x[((size_t)(c / 3) * n + ti) * 3 + (c % 3)] : 0.f;
        mt[u][c] = make_float2(m, m);
        sm.sum[u][c][tid] = sm.cmp[u][c][tid] = 0.f;
      }
    }
    float4 ilo, ihi;
    box_of_supertile(jb.boxes, jb.nbox, I, ilo, ihi);
    const int k0 = (local - I * nchunk) * jb.chunk;
    const int k1 = min(jb.K + 1, k0 + jb.chunk);
    for (int k = k0; k < k1; ++k) {
      int J = I + k;
      if (J >= ntile) J -= ntile;
      if (k > 0 && 2 * k == ntile && I >= ntile / 2) continue;  // the other tile of the pair owns it
      const bool diag = (k == 0);
      __syncthreads();  // the previous slot's staging and sums are read
      {
        // thread tid stages pair (tid mod 32) of sub-tile tid / 32
        const int sb = tid >> 5, p = tid & 31;
        const int sa = J * S32_TILE + sb * S32_SUB + p, sbb = sa + 32;
        const bool va = sa < n, vb = sbb < n;
        const float4 pa = va ? pos[sa] : make_float4(-S32_FAR, -S32_FAR, -S32_FAR, 0.f);
        const float4 pb = vb ? pos[sbb] : make_float4(-S32_FAR, -S32_FAR, -S32_FAR, 0.f);
        float fa[2 * R], fb[2 * R];
        fa[0] = pa.x, fa[1] = pa.y, fa[2] = pa.z;
        fb[0] = pb.x, fb[1] = pb.y, fb[2] = pb.z;
#pragma unroll
        for (int c = 0; c < C; ++c) {
          fa[3 + c] = va ? x[((size_t)(c / 3) * n + sa) * 3 + (c % 3)] : 0.f;
          fb[3 + c] = vb ? x[((size_t)(c / 3) * n + sbb) * 3 + (c % 3)] : 0.f;
        }
        if (2 * R > 3 + C) fa[2 * R - 1] = fb[2 * R - 1] = 0.f;
#pragma unroll
        for (int r = 0; r < R; ++r) {
          const float4 v = make_float4(fa[2 * r], fb[2 * r], fa[2 * r + 1], fb[2 * r + 1]);
          sm.rec[r][sb][p] = v;
          sm.rec[r][sb][p + 32] = v;
        }
        const float4 th = make_float4(pa.w, pb.w, (amoeba && va) ? damp[sa] : 0.f, (amoeba && vb) ? damp[sbb] : 0.f);
        sm.thole[sb][p] = th;
        sm.thole[sb][p + 32] = th;
      }
      __syncthreads();
      bool far = false;
      if (!diag) {
        float4 jlo, jhi;
        box_of_supertile(jb.boxes, jb.nbox, J, jlo, jhi);
        const float gx = fmaxf(0.f, fmaxf(jlo.x - ihi.x, ilo.x - jhi.x));
        const float gy = fmaxf(0.f, fmaxf(jlo.y - ihi.y, ilo.y - jhi.y));
        const float gz = fmaxf(0.f, fmaxf(jlo.z - ihi.z, ilo.z - jhi.z));
        far = gx * gx + gy * gy + gz * gz > jb.r2max;
      }
      float2 af[2][C], ak[2][C];
#pragma unroll
      for (int u = 0; u < 2; ++u)
#pragma unroll
        for (int c = 0; c < C; ++c) af[u][c] = ak[u][c] = make_float2(0.f, 0.f);
      if (far)
        s32_slot<false, false, G>(false, sm, warp, lane, tg, mt, jb.thr, af, ak);
      else if (amoeba)
        s32_slot<true, true, G>(diag, sm, warp, lane, tg, mt, jb.thr, af, ak);
      else
        s32_slot<true, false, G>(diag, sm, warp, lane, tg, mt, jb.thr, af, ak);
      // the slot's target sums, compensated across slots
#pragma unroll
      for (int u = 0; u < 2; ++u)
#pragma unroll
        for (int c = 0; c < C; ++c) {
          const float s0 = sm.sum[u][c][tid];
          const float y = fmaf(3.f, af[u][c].x + af[u][c].y, -(ak[u][c].x + ak[u][c].y)) - sm.cmp[u][c][tid];
          const float s = s0 + y;
          sm.cmp[u][c][tid] = (s - s0) - y;
          sm.sum[u][c][tid] = s;
        }
      if (!diag) {
        __syncthreads();
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int q = h * S32_TPB + tid;
          const int sj = J * S32_TILE + q;
          if (sj < n) {
#pragma unroll
            for (int c = 0; c < C; ++c) {
              const float v = ((sm.accj[0][c][q] + sm.accj[1][c][q]) + sm.accj[2][c][q]) + sm.accj[3][c][q];
              const size_t o = ((size_t)(c / 3) * n + sj) * 3 + (c % 3);
              fixed_add_f32(jb.lo + o, jb.hi + o, 3.f * v, jb.bad);
            }
          }
        }
      }
    }
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const int ti = I * S32_TILE + tg[u].idx;
      if (ti >= n) continue;
#pragma unroll
      for (int c = 0; c < C; ++c) {
        const size_t o = ((size_t)(c / 3) * n + ti) * 3 + (c % 3);
        fixed_add_f32(jb.lo + o, jb.hi + o, sm.sum[u][c][tid] - sm.cmp[u][c][tid], jb.bad);
      }
    }
  }
}

// fixed-point sums -> float (NaN when an accumulator overflowed)
__global__ void k_fixed_to_float(size_t total, const unsigned long long *__restrict__ lo,
                                 const unsigned long long *__restrict__ hi, const unsigned long long *bad,
                                 float *__restrict__ out) {
  const bool nan = *bad != 0ull;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < total; k += (size_t)gridDim.x * blockDim.x)
    out[k] = nan ? __int_as_float(0x7fc00000) : (float)fixed_value(lo[k], hi[k]);
}

template <int G>
struct S32Launch {
  int resident = 0;
  S32Launch() {
    const int smem = (int)sizeof(S32Smem<G>);
    cudaFuncSetAttribute(k_tmu32_sym<G>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, k_tmu32_sym<G>, S32_TPB, smem);
    if (resident < 1) resident = 1;
  }
};
template <int G>
int s32_resident() {
  static const S32Launch<G> cfg;  // thread-safe one-time set-up
  return cfg.resident;
}

// the item space of one system's product: super-tiles x chunks of slots,
// about 16 items per resident CTA of the whole GPU
void s32_schedule(int n, int g, double round_pairs, int &ntile, int &K, int &chunk, int &nchunk) {
  ntile = (n + S32_TILE - 1) / S32_TILE;
  K = ntile / 2;
  const int ctas_max = (g == 2 ? s32_resident<2>() : s32_resident<1>()) * sm_count();
  long long c = (long long)ntile * (K + 1) / (16LL * ctas_max);
  // round_pairs > 0: at most a quarter of a CTA's share of round_pairs
  if (round_pairs > 0.0) c = std::min(c, (long long)(round_pairs / (4.0 * ctas_max * S32_TILE * S32_TILE)));
  if (c < 1) c = 1;
  if (c > K + 1) c = K + 1;
  chunk = (int)c;
  nchunk = (K + 1 + chunk - 1) / chunk;
}

template <int G>
void launch_s32_table(const S32Table &tab, unsigned *next, cudaStream_t st) {
  const int total = tab.base[tab.njobs];
  if (total <= 0) return;
  const int ctas_max = s32_resident<G>() * sm_count();
  const int ctas = ctas_max < total ? ctas_max : total;
  cudaMemsetAsync(next, 0, sizeof(unsigned), st);
  k_tmu32_sym<G><<<ctas, S32_TPB, sizeof(S32Smem<G>), st>>>(tab, next);
}

void fill_s32_job(S32Job &j, const DevSites &s, int g, const float *x, unsigned long long *lo,
                  unsigned long long *hi, unsigned long long *bad, int item0, double round_pairs) {
  j.pos = s.pol_pos32;
  j.damp = s.pol_a32;
  j.boxes = s.tile_box32;
  j.x = x;
  j.lo = lo, j.hi = hi, j.bad = bad;
  j.n = s.n;
  j.nbox = s.ntile;
  s32_schedule(s.n, g, round_pairs, j.ntile, j.K, j.chunk, j.nchunk);
  j.item0 = item0;
  j.amoeba = s.amoeba ? 1 : 0;
  j.thr = (float)s.damp_thr;
  j.r2max = s.damp_r2max32;
}

}  // namespace

int tmu32_sym_resident(int g, bool) { return g == 2 ? s32_resident<2>() : s32_resident<1>(); }

int tmu32_sym_items(const DevSites &s, int g, double round_pairs) {
  if (s.n == 0) return 0;
  int ntile, K, chunk, nchunk;
  s32_schedule(s.n, g, round_pairs, ntile, K, chunk, nchunk);
  return ntile * nchunk;
}

void launch_tmu32_sym_multi(int g, const SymSlice *sl, int nsl, unsigned *next, cudaStream_t st) {
  S32Table tab{};
  int total = 0;
  for (int k = 0; k < nsl && tab.njobs < kMaxSymSlices; ++k) {
    if (sl[k].count <= 0 || sl[k].s->n == 0) continue;
    fill_s32_job(tab.job[tab.njobs], *sl[k].s, g, static_cast<const float *>(sl[k].x), sl[k].lo, sl[k].hi,
                 sl[k].bad, sl[k].item0, sl[k].round_pairs);
    tab.base[tab.njobs] = total;
    total += sl[k].count;
    ++tab.njobs;
  }
  tab.base[tab.njobs] = total;
  if (!total) return;
  add_launch_count(1);
  if (g == 2)
    launch_s32_table<2>(tab, next, st);
  else
    launch_s32_table<1>(tab, next, st);
}

void launch_fixed_to_float(size_t total, const unsigned long long *lo, const unsigned long long *hi,
                           const unsigned long long *bad, float *out, cudaStream_t st) {
  add_launch_count(1);
  int blocks = (int)((total + 255) / 256);
  if (blocks > 4 * 152 * 4) blocks = 4 * 152 * 4;
  k_fixed_to_float<<<blocks < 1 ? 1 : blocks, 256, 0, st>>>(total, lo, hi, bad, out);
}

void launch_tmu32_sym_pairs(const DevSites &s, int g, const float *x, unsigned long long *lo, unsigned long long *hi,
                            unsigned long long *bad, unsigned *next, float *out, cudaStream_t st) {
  const size_t C = 3 * (size_t)g;
  cudaMemsetAsync(lo, 0, 2 * C * s.n * sizeof(unsigned long long), st);
  cudaMemsetAsync(bad, 0, sizeof(unsigned long long), st);
  SymSlice one{&s, x, lo, hi, bad, 0, tmu32_sym_items(s, g)};
  launch_tmu32_sym_multi(g, &one, 1, next, st);
  launch_fixed_to_float(C * s.n, lo, hi, bad, out, st);
}

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
