// Double-single T.mu: FP64-accurate dipole field on GB300's FP32 pipes.
//
// The refinement residual E - T mu of the mixed-precision solver needs the
// product to ~1e-12 relative; GB300 executes FP64 at 1/64 of its FP32 rate.
// This kernel carries every quantity of an undamped pair as an unevaluated
// sum of two floats (hi + lo, ~48-bit significand) built from error-free
// transformations (Knuth's TwoSum, Dekker's FastTwoSum, FMA-based TwoProd;
// double-word algorithms as analysed by Joldes, Muller and Popescu, ACM TOMS
// 44(4), 2017), so each pair costs ~230 FP32 instructions instead of ~34 FP64
// ones (~2,200 FP32 issue slots).  The few source tiles whose bounding box
// comes within the Thole damping range of the CTA's targets test each pair in
// FP32 and form the Thole factors of the (few) damped ones in FP64, applied
// in double-single.  Per tile and target
// the double-single sum is added to an FP64 accumulator; the split partials
// [split][n][3] go through the same scaled-pair / diagonal pass
// (k_tmu_finish<double>) as the FP64 product.
//
// Same product as TMatVec_otf / field_extD2D (src/mod_polarization.F90:459-481,
// src/mod_electrostatics.F90:1954-2111).  Built with --fmad=false so that no
// product is fused into a later addition behind the error-free
// transformations' back (every intended FMA is an explicit fmaf), and with
// -ftz=true (the reciprocal-square-root seed is the plain MUFU estimate).
#include <algorithm>
#include <cmath>

#include "ds_math.cuh"
#include "kernels.h"
#include "pair_math.cuh"

namespace ommp {
namespace gpu {

namespace {

constexpr int DS_TPB = 128;
constexpr int DS_TILE = 128;
constexpr int DS_TPT = 2;  // targets per thread

// One ordered pair in double-single: acc += 3 r^-5 (mu.d) d - r^-3 mu.
// NEAR: the pair may be damped; an FP32 pre-test (1e-5 margin) selects the
// pairs whose Thole factors are then formed in FP64 (exp) and applied in
// double-single.  Far pairs (tile boxes beyond the damping range) skip it.
// Geometry of one ordered pair: d and the (damped) factors r^-3, 3 r^-5.
// NEAR: the pair may be damped; an FP32 pre-test (1e-5 margin) selects the
// pairs whose Thole factors are then formed in FP64 (exp) and applied in
// double-single.  Far pairs (tile boxes beyond the damping range) skip it.
struct DsGeom {
  dsf dx, dy, dz, k3, k5x3;
};

template <bool NEAR, bool AMOEBA>
__device__ __forceinline__ DsGeom ds_geometry(const float4 &th, const float4 &tl, const float4 &sh,
                                              const float4 &sl, double wt, double ws, double at, double as,
                                              float2 wat, float2 was, double thr, float thr2m) {
  DsGeom g;
  g.dx = ds_diff(th.x, tl.x, sh.x, sl.x);
  g.dy = ds_diff(th.y, tl.y, sh.y, sl.y);
  g.dz = ds_diff(th.z, tl.z, sh.z, sl.z);
  const dsf dx = g.dx, dy = g.dy, dz = g.dz;
  // r^2
  float px = dx.h * dx.h, py = dy.h * dy.h, pz = dz.h * dz.h;
  float ex = fmaf(dx.h + dx.h, dx.l, fmaf(dx.h, dx.h, -px));
  float ey = fmaf(dy.h + dy.h, dy.l, fmaf(dy.h, dy.h, -py));
  float ez = fmaf(dz.h + dz.h, dz.l, fmaf(dz.h, dz.h, -pz));
  const dsf sa = two_sum(px, py);
  const dsf sb = two_sum(sa.h, pz);
  const dsf r2 = fast_two_sum(sb.h, ((ex + ey) + ez) + (sa.l + sb.l));
  const dsf rinv = ds_rsqrt(r2);
  const dsf ir2 = ds_sqr(rinv);
  dsf k3 = ds_mul(rinv, ir2);
  dsf k5 = ds_mul(k3, ir2);
  if (NEAR) {
    const bool maybe = AMOEBA ? maybe_damped_amoeba(r2.h, wat, was, thr2m) : maybe_damped_wang(r2.h, wat, was);
    if (maybe) {
      const double u = sqrt((double)r2.h + (double)r2.l) * (wt * ws);  // r / (thole_t thole_s)
      double f3 = 1.0, f5 = 1.0;
      if (AMOEBA) {
        const double au3 = fmin(at, as) * u * u * u;
        if (au3 < thr) {
          const double e = exp(-au3);
          f3 = 1.0 - e;
          f5 = 1.0 - (1.0 + au3) * e;
        }
      } else if (u < 1.0) {
        const double u3 = u * u * u;
        const double u4 = u3 * u;
        f3 = 4.0 * u3 - 3.0 * u4;
        f5 = u4;
      }
      k3 = ds_mul(k3, to_ds(f3));
      k5 = ds_mul(k5, to_ds(f5));
    }
  }
  g.k3 = k3;
  g.k5x3 = ds_mulf(k5, 3.0f);
  return g;
}

// acc += 3 r^-5 (mu.d) d - r^-3 mu for one column (mu as hi / lo floats)
__device__ __forceinline__ void ds_column(const DsGeom &g, const float4 &mh, const float4 &ml, float (&ah)[3],
                                          float (&al)[3]) {
  const dsf dx = g.dx, dy = g.dy, dz = g.dz;
  float qx = mh.x * dx.h, qy = mh.y * dy.h, qz = mh.z * dz.h;
  float fx = fmaf(ml.x, dx.h, fmaf(mh.x, dx.l, fmaf(mh.x, dx.h, -qx)));
  float fy = fmaf(ml.y, dy.h, fmaf(mh.y, dy.l, fmaf(mh.y, dy.h, -qy)));
  float fz = fmaf(ml.z, dz.h, fmaf(mh.z, dz.l, fmaf(mh.z, dz.h, -qz)));
  const dsf u1 = two_sum(qx, qy);
  const dsf u2 = two_sum(u1.h, qz);
  const dsf dot = fast_two_sum(u2.h, ((fx + fy) + fz) + (u1.l + u2.l));
  const dsf f = ds_mul(g.k5x3, dot);
  const dsf nk3{-g.k3.h, -g.k3.l};
  acc_mul(ah[0], al[0], f, dx);
  acc_mul(ah[0], al[0], nk3, dsf{mh.x, ml.x});
  acc_mul(ah[1], al[1], f, dy);
  acc_mul(ah[1], al[1], nk3, dsf{mh.y, ml.y});
  acc_mul(ah[2], al[2], f, dz);
  acc_mul(ah[2], al[2], nk3, dsf{mh.z, ml.z});
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const dsf r = fast_two_sum(ah[c], al[c]);
    ah[c] = r.h;
    al[c] = r.l;
  }
}

// partial[split][g][n][3]: G columns sharing each pair's geometry, TPT
// targets per thread (target t of thread x is blockIdx.x * TPB * TPT + t *
// TPB + x)
template <bool AMOEBA, int G, int TPT>
__global__ void __launch_bounds__(DS_TPB, 5) k_tmu_ds(int n, const float4 *__restrict__ ph, const float4 *__restrict__ pl,
                                                   const Pos64 *__restrict__ p64, const double *__restrict__ damp,
                                                   const float2 *__restrict__ wa, const float4 *__restrict__ boxes,
                                                   const double *__restrict__ x, double *__restrict__ partial,
                                                   int per_split, double thr, float thr2m, float r2max) {
  __shared__ float4 s_ph[DS_TILE], s_pl[DS_TILE], s_mh[G][DS_TILE], s_ml[G][DS_TILE];
  __shared__ Pos64 s_p64[DS_TILE];
  __shared__ double s_a[DS_TILE];
  __shared__ float2 s_wa[DS_TILE];
  const int jb = blockIdx.x * (DS_TPB * TPT);
  float4 th[TPT], tl[TPT];
  bool valid[TPT];
  double sum[TPT][G][3];
#pragma unroll
  for (int t = 0; t < TPT; ++t) {
    const int j = jb + t * DS_TPB + threadIdx.x;
    valid[t] = j < n;
    th[t] = valid[t] ? ph[j] : make_float4(0.f, 0.f, 0.f, 0.f);
    tl[t] = valid[t] ? pl[j] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int c = 0; c < G; ++c) sum[t][c][0] = sum[t][c][1] = sum[t][c][2] = 0.0;
  }
  const int ntile = (n + DS_TILE - 1) / DS_TILE;
  const int tb0 = jb / DS_TILE;
  const int tb1 = min(ntile - 1, (jb + DS_TPB * TPT - 1) / DS_TILE);
  float4 blo = boxes[2 * tb0], bhi = boxes[2 * tb0 + 1];
  for (int tb = tb0 + 1; tb <= tb1; ++tb) {
    float4 lo = boxes[2 * tb], hi = boxes[2 * tb + 1];
    blo.x = fminf(blo.x, lo.x), blo.y = fminf(blo.y, lo.y), blo.z = fminf(blo.z, lo.z);
    bhi.x = fmaxf(bhi.x, hi.x), bhi.y = fmaxf(bhi.y, hi.y), bhi.z = fmaxf(bhi.z, hi.z);
  }

  const int s0 = blockIdx.y * per_split;
  const int s1 = min(n, s0 + per_split);
  for (int t0 = s0; t0 < s1; t0 += DS_TILE) {
    __syncthreads();
    {
      const int k = threadIdx.x;
      const int i = t0 + k;
      if (i < s1) {
        s_ph[k] = ph[i];
        s_pl[k] = pl[i];
        s_p64[k] = p64[i];
        s_a[k] = AMOEBA ? damp[i] : 0.0;
        s_wa[k] = wa[i];
#pragma unroll
        for (int col = 0; col < G; ++col) {
          float mh[3], ml[3];
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            const double m = x[((size_t)col * n + i) * 3 + c];
            mh[c] = (float)m;
            ml[c] = (float)(m - (double)mh[c]);
          }
          s_mh[col][k] = make_float4(mh[0], mh[1], mh[2], 0.f);
          s_ml[col][k] = make_float4(ml[0], ml[1], ml[2], 0.f);
        }
      }
    }
    __syncthreads();
    const int cnt = min(DS_TILE, s1 - t0);
    const float4 slo = boxes[2 * (t0 / DS_TILE)], shi = boxes[2 * (t0 / DS_TILE) + 1];
    const float gx = fmaxf(0.f, fmaxf(slo.x - bhi.x, blo.x - shi.x));
    const float gy = fmaxf(0.f, fmaxf(slo.y - bhi.y, blo.y - shi.y));
    const float gz = fmaxf(0.f, fmaxf(slo.z - bhi.z, blo.z - shi.z));
    const bool far_tile = gx * gx + gy * gy + gz * gz > r2max;
    float ah[TPT][G][3], al[TPT][G][3];
#pragma unroll
    for (int t = 0; t < TPT; ++t)
#pragma unroll
      for (int col = 0; col < G; ++col)
#pragma unroll
        for (int c = 0; c < 3; ++c) ah[t][col][c] = al[t][col][c] = 0.f;
    if (far_tile) {
#pragma unroll 1
      for (int k = 0; k < cnt; ++k) {
        const float4 sh = s_ph[k], sl = s_pl[k];
#pragma unroll
        for (int t = 0; t < TPT; ++t) {
          const DsGeom g = ds_geometry<false, AMOEBA>(th[t], tl[t], sh, sl, 0.0, 0.0, 0.0, 0.0,
                                                      make_float2(0.f, 0.f), make_float2(0.f, 0.f), thr, thr2m);
#pragma unroll
          for (int col = 0; col < G; ++col) ds_column(g, s_mh[col][k], s_ml[col][k], ah[t][col], al[t][col]);
        }
      }
    } else {
      // tiles within the damping range: per-pair pre-test, FP64 Thole factors
      double wt[TPT], at[TPT];
      float2 wat[TPT];
#pragma unroll
      for (int t = 0; t < TPT; ++t) {
        const int j = valid[t] ? jb + t * DS_TPB + threadIdx.x : 0;
        wt[t] = p64[j].w;
        at[t] = AMOEBA ? damp[j] : 0.0;
        wat[t] = wa[j];
      }
#pragma unroll 1
      for (int k = 0; k < cnt; ++k) {
        const float4 sh = s_ph[k], sl = s_pl[k];
        const double ws = s_p64[k].w, as = s_a[k];
        const float2 was = s_wa[k];
#pragma unroll
        for (int t = 0; t < TPT; ++t) {
          if (!valid[t] || t0 + k == jb + t * DS_TPB + (int)threadIdx.x) continue;
          const DsGeom g =
              ds_geometry<true, AMOEBA>(th[t], tl[t], sh, sl, wt[t], ws, at[t], as, wat[t], was, thr, thr2m);
#pragma unroll
          for (int col = 0; col < G; ++col) ds_column(g, s_mh[col][k], s_ml[col][k], ah[t][col], al[t][col]);
        }
      }
    }
#pragma unroll
    for (int t = 0; t < TPT; ++t)
#pragma unroll
      for (int col = 0; col < G; ++col)
#pragma unroll
        for (int c = 0; c < 3; ++c) sum[t][col][c] += (double)ah[t][col][c] + (double)al[t][col][c];
  }
#pragma unroll
  for (int t = 0; t < TPT; ++t) {
    const int j = jb + t * DS_TPB + threadIdx.x;
    if (!valid[t]) continue;
#pragma unroll
    for (int col = 0; col < G; ++col)
#pragma unroll
      for (int c = 0; c < 3; ++c) partial[(((size_t)blockIdx.y * G + col) * n + j) * 3 + c] = sum[t][col][c];
  }
}

// ---------------------------------------------------------------------------
// Symmetric double-single T.mu: each unordered pair's geometry (coordinate
// differences, r^2, the reciprocal square root and the r^-3 / 3 r^-5
// factors, about 106 of the 227 FP32 operations of an ordered pair) is
// formed once and serves both directions, as in the FP64 kernel k_tmu_sym
// (kernels.cu): 128-site super-tile I meets the slots k of its half shell
// J = (I + k) mod ntile, work items (I, a chunk of slots) are taken from an
// atomic counter by a persistent grid, a warp pairs its 32 targets with 32
// sources in 32 rotation steps with the source-side double-single
// accumulators moving one lane per step by shuffle, and both sides end in
// the per-site 128-bit fixed-point accumulators (deterministic).  A slot
// whose tile boxes are farther apart than the damping range runs the
// undamped pair form; the others test each pair in FP32 first.
// ---------------------------------------------------------------------------
template <bool NEAR, bool AMOEBA, int G>
__device__ __forceinline__ void ds_sym_slot(bool diag, bool vi, int ti, int gbase, int n, const float4 &th,
                                            const float4 &tl, double wt, double at, float2 wat,
                                            const float4 (&mih)[G], const float4 (&mil)[G], const float4 *s_ph,
                                            const float4 *s_pl, const double *s_w, const double *s_a,
                                            const float2 *s_wa, const float4 (*s_mh)[DS_TILE],
                                            const float4 (*s_ml)[DS_TILE], double (*s_accj)[3 * G][DS_TILE],
                                            int warp, int lane, double thr, float thr2m, float (&aih)[G][3],
                                            float (&ail)[G][3]) {
  for (int js = 0; js < 4; ++js) {
    float ajh[G][3], ajl[G][3];
#pragma unroll
    for (int col = 0; col < G; ++col)
#pragma unroll
      for (int c = 0; c < 3; ++c) ajh[col][c] = ajl[col][c] = 0.f;
#pragma unroll 1
    for (int t = 0; t < 32; ++t) {
      const int jl = js * 32 + ((lane + t) & 31);
      const int gj = gbase + jl;
      if (vi && gj < n && gj != ti) {
        const DsGeom g = ds_geometry<NEAR, AMOEBA>(th, tl, s_ph[jl], s_pl[jl], wt, s_w[jl], at, s_a[jl], wat,
                                                   s_wa[jl], thr, thr2m);
#pragma unroll
        for (int col = 0; col < G; ++col) {
          ds_column(g, s_mh[col][jl], s_ml[col][jl], aih[col], ail[col]);
          if (!diag) ds_column(g, mih[col], mil[col], ajh[col], ajl[col]);
        }
      }
      if (!diag) {
        // the accumulators of source s move to the lane that meets s next
#pragma unroll
        for (int col = 0; col < G; ++col)
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            ajh[col][c] = __shfl_sync(0xffffffffu, ajh[col][c], (lane + 1) & 31);
            ajl[col][c] = __shfl_sync(0xffffffffu, ajl[col][c], (lane + 1) & 31);
          }
      }
    }
    if (!diag) {
      // after 32 steps lane l holds the accumulators of source js*32 + l
#pragma unroll
      for (int col = 0; col < G; ++col)
#pragma unroll
        for (int c = 0; c < 3; ++c)
          s_accj[warp][3 * col + c][js * 32 + lane] = (double)ajh[col][c] + (double)ajl[col][c];
    }
  }
}

// A launch serves the products of several systems (same column count and
// damping kind): job j covers the items [item0, item0 + base[j+1] - base[j])
// of its system's product (item space fixed per system), so a product may
// also be spread over several launches.  A one-job table is the
// single-system product.
struct DsSymJob {
  const float4 *ph, *pl;
  const Pos64 *p64;
  const double *damp;
  const float2 *wa;
  const float4 *boxes;
  const double *x;
  unsigned long long *lo, *hi, *bad;
  int n, ntile, K, chunk, nchunk, item0;
  double thr;
  float thr2m, r2max;
};
struct DsSymTable {
  int njobs;
  int base[kMaxSymSlices + 1];
  DsSymJob job[kMaxSymSlices];
};

template <bool AMOEBA, int G>
__global__ void __launch_bounds__(DS_TPB) k_tmu_ds_sym(const __grid_constant__ DsSymTable tab,
                                                       unsigned *__restrict__ next) {
  constexpr int C = 3 * G;
  __shared__ float4 s_ph[DS_TILE], s_pl[DS_TILE], s_mh[G][DS_TILE], s_ml[G][DS_TILE];
  __shared__ double s_w[DS_TILE], s_a[DS_TILE];
  __shared__ float2 s_wa[DS_TILE];
  __shared__ double s_accj[4][C][DS_TILE];
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
    const DsSymJob &jb = tab.job[jx];
    const int n = jb.n, ntile = jb.ntile, K = jb.K, chunk = jb.chunk, nchunk = jb.nchunk;
    const float4 *__restrict__ ph = jb.ph;
    const float4 *__restrict__ pl = jb.pl;
    const Pos64 *__restrict__ p64 = jb.p64;
    const double *__restrict__ damp = jb.damp;
    const float2 *__restrict__ wa = jb.wa;
    const float4 *__restrict__ boxes = jb.boxes;
    const double *__restrict__ x = jb.x;
    unsigned long long *acc_lo = jb.lo, *acc_hi = jb.hi, *bad = jb.bad;
    const double thr = jb.thr;
    const float thr2m = jb.thr2m, r2max = jb.r2max;
    const int local = jb.item0 + (item - tab.base[jx]);
    const int I = local / nchunk;
    const int ti = I * DS_TILE + tid;
    const bool vi = ti < n;
    const float4 th = vi ? ph[ti] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 tl = vi ? pl[ti] : make_float4(0.f, 0.f, 0.f, 0.f);
    const double wt = vi ? p64[ti].w : 0.0;
    const double at = (AMOEBA && vi) ? damp[ti] : 0.0;
    const float2 wat = vi ? wa[ti] : make_float2(0.f, 0.f);
    float4 mih[G], mil[G];
#pragma unroll
    for (int col = 0; col < G; ++col) {
      float mh[3] = {0.f, 0.f, 0.f}, ml[3] = {0.f, 0.f, 0.f};
      if (vi)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const double m = x[((size_t)col * n + ti) * 3 + c];
          mh[c] = (float)m;
          ml[c] = (float)(m - (double)mh[c]);
        }
      mih[col] = make_float4(mh[0], mh[1], mh[2], 0.f);
      mil[col] = make_float4(ml[0], ml[1], ml[2], 0.f);
    }
    const float4 ilo = boxes[2 * I], ihi = boxes[2 * I + 1];
    double sumi[C];
#pragma unroll
    for (int c = 0; c < C; ++c) sumi[c] = 0.0;
    const int k0 = (local - I * nchunk) * chunk;
    const int k1 = min(K + 1, k0 + chunk);
    for (int k = k0; k < k1; ++k) {
      int J = I + k;
      if (J >= ntile) J -= ntile;
      if (k > 0 && 2 * k == ntile && I >= ntile / 2) continue;  // the other tile of the pair owns it
      const bool diag = (k == 0);
      __syncthreads();
      {
        const int sj = J * DS_TILE + tid;
        const bool v = sj < n;
        s_ph[tid] = v ? ph[sj] : make_float4(0.f, 0.f, 0.f, 0.f);
        s_pl[tid] = v ? pl[sj] : make_float4(0.f, 0.f, 0.f, 0.f);
        s_w[tid] = v ? p64[sj].w : 0.0;
        s_a[tid] = (AMOEBA && v) ? damp[sj] : 0.0;
        s_wa[tid] = v ? wa[sj] : make_float2(0.f, 0.f);
#pragma unroll
        for (int col = 0; col < G; ++col) {
          float mh[3] = {0.f, 0.f, 0.f}, ml[3] = {0.f, 0.f, 0.f};
          if (v)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
              const double m = x[((size_t)col * n + sj) * 3 + c];
              mh[c] = (float)m;
              ml[c] = (float)(m - (double)mh[c]);
            }
          s_mh[col][tid] = make_float4(mh[0], mh[1], mh[2], 0.f);
          s_ml[col][tid] = make_float4(ml[0], ml[1], ml[2], 0.f);
        }
      }
      __syncthreads();
      // uniform over the CTA: are the two tiles' boxes within damping range?
      const float4 jlo = boxes[2 * J], jhi = boxes[2 * J + 1];
      const float gx = fmaxf(0.f, fmaxf(jlo.x - ihi.x, ilo.x - jhi.x));
      const float gy = fmaxf(0.f, fmaxf(jlo.y - ihi.y, ilo.y - jhi.y));
      const float gz = fmaxf(0.f, fmaxf(jlo.z - ihi.z, ilo.z - jhi.z));
      const bool far_slot = !diag && gx * gx + gy * gy + gz * gz > r2max;
      float aih[G][3], ail[G][3];
#pragma unroll
      for (int col = 0; col < G; ++col)
#pragma unroll
        for (int c = 0; c < 3; ++c) aih[col][c] = ail[col][c] = 0.f;
      if (far_slot)
        ds_sym_slot<false, AMOEBA, G>(diag, vi, ti, J * DS_TILE, n, th, tl, wt, at, wat, mih, mil, s_ph, s_pl, s_w,
                                      s_a, s_wa, s_mh, s_ml, s_accj, warp, lane, thr, thr2m, aih, ail);
      else
        ds_sym_slot<true, AMOEBA, G>(diag, vi, ti, J * DS_TILE, n, th, tl, wt, at, wat, mih, mil, s_ph, s_pl, s_w,
                                     s_a, s_wa, s_mh, s_ml, s_accj, warp, lane, thr, thr2m, aih, ail);
#pragma unroll
      for (int col = 0; col < G; ++col)
#pragma unroll
        for (int c = 0; c < 3; ++c) sumi[3 * col + c] += (double)aih[col][c] + (double)ail[col][c];
      if (!diag) {
        __syncthreads();
        const int sj = J * DS_TILE + tid;
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
        fixed_add(acc_lo + o, acc_hi + o, sumi[c], bad);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// E_M2D in double-single: field of the static multipoles (charge, dipole,
// quadrupole for AMOEBA; charge for Wang-AL) at the polarizable sites, the
// all-pairs part of elec_prop_M2D (src/mod_electrostatics.F90:2579-2731) at
// scale 1; the scaled pairs are corrected in FP64 by k_m2d_finish.
// ---------------------------------------------------------------------------
constexpr int M2D_LD = 10;  // q, mu (3), theta xx xy yy xz yz zz

// One target-source pair; q hi/lo in smem rows of M2D_LD floats.
template <bool NEAR, bool AMOEBA>
__device__ __forceinline__ void ds_m2d_pair(const float4 &th, const float4 &tl, const float4 &sh, const float4 &sl,
                                            const float *qh, const float *ql, float (&ah)[3], float (&al)[3],
                                            double wt, double ws, double at, double as, float2 wat, float2 was,
                                            double thr, float thr2m, int &bad) {
  const dsf dx = ds_diff(th.x, tl.x, sh.x, sl.x);
  const dsf dy = ds_diff(th.y, tl.y, sh.y, sl.y);
  const dsf dz = ds_diff(th.z, tl.z, sh.z, sl.z);
  float px = dx.h * dx.h, py = dy.h * dy.h, pz = dz.h * dz.h;
  float ex = fmaf(dx.h + dx.h, dx.l, fmaf(dx.h, dx.h, -px));
  float ey = fmaf(dy.h + dy.h, dy.l, fmaf(dy.h, dy.h, -py));
  float ez = fmaf(dz.h + dz.h, dz.l, fmaf(dz.h, dz.h, -pz));
  const dsf sa = two_sum(px, py);
  const dsf sb = two_sum(sa.h, pz);
  const dsf r2 = fast_two_sum(sb.h, ((ex + ey) + ez) + (sa.l + sb.l));
  if (NEAR && r2.h < 4.9e-28f) {  // |r| < 100 eps: coincident sites
    bad = 1;
    return;
  }
  const dsf rinv = ds_rsqrt(r2);
  const dsf ir2 = ds_sqr(rinv);
  dsf k3 = ds_mul(rinv, ir2);
  dsf k5 = ds_mul(k3, ir2), k7 = ds_mul(k5, ir2);
  if (NEAR) {
    const bool maybe = AMOEBA ? maybe_damped_amoeba(r2.h, wat, was, thr2m) : maybe_damped_wang(r2.h, wat, was);
    if (maybe) {
      const double u = sqrt((double)r2.h + (double)r2.l) * (wt * ws);
      double f3 = 1.0, f5 = 1.0, f7 = 1.0;
      if (AMOEBA) {
        const double au3 = fmin(at, as) * u * u * u;
        if (au3 < thr) {
          const double e = exp(-au3);
          f3 = 1.0 - e;
          f5 = 1.0 - (1.0 + au3) * e;
          f7 = 1.0 - (1.0 + au3 + 0.6 * au3 * au3) * e;
        }
      } else if (u < 1.0) {
        const double u3 = u * u * u;
        f3 = 4.0 * u3 - 3.0 * u3 * u;
      }
      k3 = ds_mul(k3, to_ds(f3));
      if (AMOEBA) {
        k5 = ds_mul(k5, to_ds(f5));
        k7 = ds_mul(k7, to_ds(f7));
      }
    }
  }
  if (AMOEBA) {
    // mu.d, theta d, d.theta.d
    const dsf mdr = ds_dot3(qh[1], ql[1], qh[2], ql[2], qh[3], ql[3], dx, dy, dz);
    const dsf tx = ds_dot3(qh[4], ql[4], qh[5], ql[5], qh[7], ql[7], dx, dy, dz);
    const dsf ty = ds_dot3(qh[5], ql[5], qh[6], ql[6], qh[8], ql[8], dx, dy, dz);
    const dsf tz = ds_dot3(qh[7], ql[7], qh[8], ql[8], qh[9], ql[9], dx, dy, dz);
    const dsf txr = ds_add(ds_add(ds_mul(tx, dx), ds_mul(ty, dy)), ds_mul(tz, dz));
    // c = q k3 + 3 mu.d k5 + 15 d.theta.d k7
    const dsf c = ds_add(ds_add(ds_mul(k3, dsf{qh[0], ql[0]}), ds_mulf(ds_mul(mdr, k5), 3.0f)),
                         ds_mulf(ds_mul(txr, k7), 15.0f));
    const dsf nk3{-k3.h, -k3.l};
    const dsf k5x6 = ds_mulf(k5, -6.0f);
    acc_mul(ah[0], al[0], c, dx);
    acc_mul(ah[0], al[0], nk3, dsf{qh[1], ql[1]});
    acc_mul(ah[0], al[0], k5x6, tx);
    acc_mul(ah[1], al[1], c, dy);
    acc_mul(ah[1], al[1], nk3, dsf{qh[2], ql[2]});
    acc_mul(ah[1], al[1], k5x6, ty);
    acc_mul(ah[2], al[2], c, dz);
    acc_mul(ah[2], al[2], nk3, dsf{qh[3], ql[3]});
    acc_mul(ah[2], al[2], k5x6, tz);
  } else {
    const dsf c = ds_mul(k3, dsf{qh[0], ql[0]});
    acc_mul(ah[0], al[0], c, dx);
    acc_mul(ah[1], al[1], c, dy);
    acc_mul(ah[2], al[2], c, dz);
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const dsf r = fast_two_sum(ah[k], al[k]);
    ah[k] = r.h;
    al[k] = r.l;
  }
}

// partial[split][j][3] over the split's static sources (the target's own
// site excluded; coincident sites set *err_flag)
template <bool AMOEBA>
__global__ void __launch_bounds__(DS_TPB, 4) k_m2d_ds(int n, int m, const float4 *__restrict__ ph,
                                                      const float4 *__restrict__ pl, const Pos64 *__restrict__ p64,
                                                      const double *__restrict__ pol_a, const float2 *__restrict__ pol_wa,
                                                      const int *__restrict__ polar_mm, const float4 *__restrict__ pbox,
                                                      const float4 *__restrict__ mh, const float4 *__restrict__ ml,
                                                      const Pos64 *__restrict__ m64, const double *__restrict__ mm_a,
                                                      const float2 *__restrict__ mm_wa, const double *__restrict__ mm_q,
                                                      const float4 *__restrict__ mbox, double *__restrict__ partial,
                                                      int per_split, double thr, float thr2m, float r2max, int *err_flag) {
  constexpr int LD = AMOEBA ? M2D_LD : 1;
  __shared__ float4 s_ph[DS_TILE], s_pl[DS_TILE];
  __shared__ float s_qh[DS_TILE * LD], s_ql[DS_TILE * LD];
  __shared__ double s_w[DS_TILE], s_a[DS_TILE];
  __shared__ float2 s_wa[DS_TILE];
  const int jb = blockIdx.x * (DS_TPB * DS_TPT);
  float4 th[DS_TPT], tl[DS_TPT];
  bool valid[DS_TPT];
  double sum[DS_TPT][3];
#pragma unroll
  for (int t = 0; t < DS_TPT; ++t) {
    const int j = jb + t * DS_TPB + threadIdx.x;
    valid[t] = j < n;
    th[t] = valid[t] ? ph[j] : make_float4(0.f, 0.f, 0.f, 0.f);
    tl[t] = valid[t] ? pl[j] : make_float4(0.f, 0.f, 0.f, 0.f);
    sum[t][0] = sum[t][1] = sum[t][2] = 0.0;
  }
  const int ntile = (n + DS_TILE - 1) / DS_TILE;
  const int tb0 = jb / DS_TILE;
  const int tb1 = min(ntile - 1, (jb + DS_TPB * DS_TPT - 1) / DS_TILE);
  float4 blo = pbox[2 * tb0], bhi = pbox[2 * tb0 + 1];
  for (int tb = tb0 + 1; tb <= tb1; ++tb) {
    float4 lo = pbox[2 * tb], hi = pbox[2 * tb + 1];
    blo.x = fminf(blo.x, lo.x), blo.y = fminf(blo.y, lo.y), blo.z = fminf(blo.z, lo.z);
    bhi.x = fmaxf(bhi.x, hi.x), bhi.y = fmaxf(bhi.y, hi.y), bhi.z = fmaxf(bhi.z, hi.z);
  }
  int bad = 0;
  const int s0 = blockIdx.y * per_split;
  const int s1 = min(m, s0 + per_split);
  for (int t0 = s0; t0 < s1; t0 += DS_TILE) {
    __syncthreads();
    {
      const int k = threadIdx.x;
      const int i = t0 + k;
      if (i < s1) {
        s_ph[k] = mh[i];
        s_pl[k] = ml[i];
        s_w[k] = m64[i].w;
        s_a[k] = AMOEBA ? mm_a[i] : 0.0;
        s_wa[k] = mm_wa[i];
#pragma unroll
        for (int c = 0; c < LD; ++c) {
          const double v = mm_q[(size_t)i * LD + c];
          const float h = (float)v;
          s_qh[k * LD + c] = h;
          s_ql[k * LD + c] = (float)(v - (double)h);
        }
      }
    }
    __syncthreads();
    const int cnt = min(DS_TILE, s1 - t0);
    const float4 slo = mbox[2 * (t0 / DS_TILE)], shi = mbox[2 * (t0 / DS_TILE) + 1];
    const float gx = fmaxf(0.f, fmaxf(slo.x - bhi.x, blo.x - shi.x));
    const float gy = fmaxf(0.f, fmaxf(slo.y - bhi.y, blo.y - shi.y));
    const float gz = fmaxf(0.f, fmaxf(slo.z - bhi.z, blo.z - shi.z));
    const bool far_tile = gx * gx + gy * gy + gz * gz > r2max;
    float ah[DS_TPT][3], al[DS_TPT][3];
#pragma unroll
    for (int t = 0; t < DS_TPT; ++t)
#pragma unroll
      for (int c = 0; c < 3; ++c) ah[t][c] = al[t][c] = 0.f;
    if (far_tile) {
#pragma unroll 1
      for (int k = 0; k < cnt; ++k) {
        const float4 sh = s_ph[k], sl = s_pl[k];
#pragma unroll
        for (int t = 0; t < DS_TPT; ++t)
          ds_m2d_pair<false, AMOEBA>(th[t], tl[t], sh, sl, &s_qh[k * LD], &s_ql[k * LD], ah[t], al[t], 0.0, 0.0,
                                     0.0, 0.0, make_float2(0.f, 0.f), make_float2(0.f, 0.f), thr, thr2m, bad);
      }
    } else {
      double wt[DS_TPT], at[DS_TPT];
      float2 wat[DS_TPT];
      int tm[DS_TPT];
#pragma unroll
      for (int t = 0; t < DS_TPT; ++t) {
        const int j = valid[t] ? jb + t * DS_TPB + threadIdx.x : 0;
        wt[t] = p64[j].w;
        at[t] = AMOEBA ? pol_a[j] : 0.0;
        wat[t] = pol_wa[j];
        tm[t] = valid[t] ? polar_mm[j] : -1;
      }
#pragma unroll 1
      for (int k = 0; k < cnt; ++k) {
        const float4 sh = s_ph[k], sl = s_pl[k];
        const double ws = s_w[k], as = s_a[k];
        const float2 was = s_wa[k];
#pragma unroll
        for (int t = 0; t < DS_TPT; ++t) {
          if (!valid[t] || t0 + k == tm[t]) continue;
          ds_m2d_pair<true, AMOEBA>(th[t], tl[t], sh, sl, &s_qh[k * LD], &s_ql[k * LD], ah[t], al[t], wt[t], ws,
                                    at[t], as, wat[t], was, thr, thr2m, bad);
        }
      }
    }
#pragma unroll
    for (int t = 0; t < DS_TPT; ++t)
#pragma unroll
      for (int c = 0; c < 3; ++c) sum[t][c] += (double)ah[t][c] + (double)al[t][c];
  }
  if (bad) atomicOr(err_flag, 1);
#pragma unroll
  for (int t = 0; t < DS_TPT; ++t) {
    const int j = jb + t * DS_TPB + threadIdx.x;
    if (!valid[t]) continue;
#pragma unroll
    for (int c = 0; c < 3; ++c) partial[((size_t)blockIdx.y * n + j) * 3 + c] = sum[t][c];
  }
}

}  // namespace

int tmu_ds_pick_split(const DevSites &s, int sms) {
  const int tblocks = (s.n + DS_TPB * DS_TPT - 1) / (DS_TPB * DS_TPT);
  const int tiles = (s.n + DS_TILE - 1) / DS_TILE;
  int split = (4 * sms + tblocks - 1) / tblocks;
  if (split > tiles) split = tiles;
  return split < 1 ? 1 : split;
}

namespace {
template <bool AMOEBA, int G, int TPT>
void launch_ds_shape(const DevSites &s, const double *x, double *partial, int nsplit, cudaStream_t st) {
  const int tiles = (s.n + DS_TILE - 1) / DS_TILE;
  const int per = ((tiles + nsplit - 1) / nsplit) * DS_TILE;
  dim3 grid((s.n + DS_TPB * TPT - 1) / (DS_TPB * TPT), nsplit);
  const float thr2m = (float)(s.damp_thr * s.damp_thr * (1.0 + 1e-5));
  k_tmu_ds<AMOEBA, G, TPT><<<grid, DS_TPB, 0, st>>>(s.n, s.pol_pos32, s.pol_pos32lo, s.pol_pos, s.pol_a,
                                                    s.pol_wa32, s.tile_box32, x, partial, per, s.damp_thr, thr2m,
                                                    s.damp_r2max32);
}
}  // namespace

// g = 1: two targets per thread; g = 2: one target per thread, two columns
// sharing the pair geometry (the same split keeps the grid size)
void launch_tmu_ds_pairs(const DevSites &s, int g, const double *x, double *partial, int nsplit, cudaStream_t st) {
  if (g == 2) {
    if (s.amoeba)
      launch_ds_shape<true, 2, 1>(s, x, partial, nsplit, st);
    else
      launch_ds_shape<false, 2, 1>(s, x, partial, nsplit, st);
  } else {
    if (s.amoeba)
      launch_ds_shape<true, 1, DS_TPT>(s, x, partial, nsplit, st);
    else
      launch_ds_shape<false, 1, DS_TPT>(s, x, partial, nsplit, st);
  }
}

namespace {
template <bool AMOEBA, int G>
int ds_sym_resident() {
  static const int r = [] {
    int v = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_tmu_ds_sym<AMOEBA, G>, DS_TPB, 0);
    return v < 1 ? 1 : v;
  }();
  return r;
}

int ds_sym_res(int g, bool amoeba) {
  if (g == 2) return amoeba ? ds_sym_resident<true, 2>() : ds_sym_resident<false, 2>();
  return amoeba ? ds_sym_resident<true, 1>() : ds_sym_resident<false, 1>();
}

// the item space of one system's product: about 16 items per resident CTA
// (round_pairs > 0: at most a quarter of a CTA's share of round_pairs)
void ds_sym_schedule(int n, int g, bool amoeba, double round_pairs, int &ntile, int &K, int &chunk, int &nchunk) {
  ntile = (n + DS_TILE - 1) / DS_TILE;
  K = ntile / 2;
  const int ctas_max = ds_sym_res(g, amoeba) * sm_count();
  long long c = (long long)ntile * (K + 1) / (16LL * ctas_max);
  if (round_pairs > 0.0) c = std::min(c, (long long)(round_pairs / (4.0 * ctas_max * DS_TILE * DS_TILE)));
  if (c < 1) c = 1;
  if (c > K + 1) c = K + 1;
  chunk = (int)c;
  nchunk = (K + 1 + chunk - 1) / chunk;
}

template <bool AMOEBA, int G>
void launch_ds_sym_table(const DsSymTable &tab, unsigned *next, cudaStream_t st) {
  const int total = tab.base[tab.njobs];
  if (total <= 0) return;
  const int ctas_max = ds_sym_resident<AMOEBA, G>() * sm_count();
  const int ctas = ctas_max < total ? ctas_max : total;
  cudaMemsetAsync(next, 0, sizeof(unsigned), st);
  k_tmu_ds_sym<AMOEBA, G><<<ctas, DS_TPB, 0, st>>>(tab, next);
}
}  // namespace

int tmu_ds_sym_items(const DevSites &s, int g, double round_pairs) {
  if (s.n == 0) return 0;
  int ntile, K, chunk, nchunk;
  ds_sym_schedule(s.n, g, s.amoeba, round_pairs, ntile, K, chunk, nchunk);
  return ntile * nchunk;
}

void launch_tmu_ds_sym_multi(int g, bool amoeba, const SymSlice *sl, int nsl, unsigned *next, cudaStream_t st) {
  DsSymTable tab{};
  int total = 0;
  for (int k = 0; k < nsl && tab.njobs < kMaxSymSlices; ++k) {
    const DevSites &s = *sl[k].s;
    if (sl[k].count <= 0 || s.n == 0) continue;
    DsSymJob &j = tab.job[tab.njobs];
    j.ph = s.pol_pos32, j.pl = s.pol_pos32lo, j.p64 = s.pol_pos, j.damp = s.pol_a, j.wa = s.pol_wa32;
    j.boxes = s.tile_box32, j.x = static_cast<const double *>(sl[k].x);
    j.lo = sl[k].lo, j.hi = sl[k].hi, j.bad = sl[k].bad;
    j.n = s.n;
    ds_sym_schedule(s.n, g, amoeba, sl[k].round_pairs, j.ntile, j.K, j.chunk, j.nchunk);
    j.item0 = sl[k].item0;
    j.thr = s.damp_thr;
    j.thr2m = (float)(s.damp_thr * s.damp_thr * (1.0 + 1e-5));
    j.r2max = s.damp_r2max32;
    tab.base[tab.njobs] = total;
    total += sl[k].count;
    ++tab.njobs;
  }
  tab.base[tab.njobs] = total;
  if (!total) return;
  add_launch_count(1);
  if (g == 2)
    amoeba ? launch_ds_sym_table<true, 2>(tab, next, st) : launch_ds_sym_table<false, 2>(tab, next, st);
  else
    amoeba ? launch_ds_sym_table<true, 1>(tab, next, st) : launch_ds_sym_table<false, 1>(tab, next, st);
}

// symmetric double-single pair sums of g (1 or 2) columns into the
// fixed-point accumulators lo / hi [g][n][3] (zeroed by the caller)
void launch_tmu_ds_sym_pairs(const DevSites &s, int g, const double *x, unsigned long long *lo,
                             unsigned long long *hi, unsigned long long *bad, unsigned *next, cudaStream_t st) {
  SymSlice one{&s, x, lo, hi, bad, 0, tmu_ds_sym_items(s, g)};
  launch_tmu_ds_sym_multi(g, s.amoeba, &one, 1, next, st);
}

}  // namespace gpu
}  // namespace ommp

namespace ommp {
namespace gpu {

int m2d_ds_pick_split(const DevSites &s, int sms) {
  const int tblocks = (s.n + DS_TPB * DS_TPT - 1) / (DS_TPB * DS_TPT);
  const int tiles = (s.m + DS_TILE - 1) / DS_TILE;
  int split = (4 * sms + tblocks - 1) / tblocks;
  if (split > tiles) split = tiles;
  return split < 1 ? 1 : split;
}

void launch_m2d_ds_pairs(const DevSites &s, double *partial, int nsplit, int *err_flag, cudaStream_t st) {
  const int tiles = (s.m + DS_TILE - 1) / DS_TILE;
  const int per = ((tiles + nsplit - 1) / nsplit) * DS_TILE;
  dim3 grid((s.n + DS_TPB * DS_TPT - 1) / (DS_TPB * DS_TPT), nsplit);
  const float thr2m = (float)(s.damp_thr * s.damp_thr * (1.0 + 1e-5));
  if (s.amoeba)
    k_m2d_ds<true><<<grid, DS_TPB, 0, st>>>(s.n, s.m, s.pol_pos32, s.pol_pos32lo, s.pol_pos, s.pol_a, s.pol_wa32,
                                            s.polar_mm, s.tile_box32, s.mm_pos32, s.mm_pos32lo, s.mm_pos, s.mm_a,
                                            s.mm_wa32, s.mm_q, s.mm_tile_box32, partial, per, s.damp_thr, thr2m,
                                            s.m2d_r2max32, err_flag);
  else
    k_m2d_ds<false><<<grid, DS_TPB, 0, st>>>(s.n, s.m, s.pol_pos32, s.pol_pos32lo, s.pol_pos, s.pol_a, s.pol_wa32,
                                             s.polar_mm, s.tile_box32, s.mm_pos32, s.mm_pos32lo, s.mm_pos, s.mm_a,
                                             s.mm_wa32, s.mm_q, s.mm_tile_box32, partial, per, s.damp_thr, thr2m,
                                             s.m2d_r2max32, err_flag);
}

}  // namespace gpu
}  // namespace ommp
