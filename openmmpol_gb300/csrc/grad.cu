// Geometric gradient of the polarization energy on the GPU
// (polelec_geomgrad, src/mod_geomgrad.F90:113-277).
//
// The reference builds, with the converged induced dipoles, the field
// gradient of the static multipoles and of the induced dipoles at the
// polarizable sites (Egrd_M2D, Egrd_D2D) and the field, field gradient and
// Hessian of the induced dipoles at the static sites (E/Egrd/EHes_D2M), then
// contracts them with the multipoles and adds the torque of the frame
// rotation.  Here the same quantities come from one all-pairs FP64 pass over
// every (static target, static source) pair of sites, so that the damped
// kernel of a pair is computed once for all of them:
//   k_grad_mu      the induced dipoles scattered to static-site order
//   k_grad_pairs   per target site t, unscaled sums over all sources s != t:
//                    g0  field gradient of the static multipoles of s
//                    hd  field gradient of the D dipole of s (hp: P dipole)
//                    e   field of the mean dipole (mu_D + mu_P) / 2
//                    h   the target's quadrupole contracted with the field
//                        Hessian of the mean dipole (AMOEBA)
//                  split over source ranges, partials in fixed order
//   k_grad_finish  per target: partials summed, the scaled pairs corrected
//                  by (s - 1) times their term (M2D p/d scales, D2D u
//                  scales, and for D2M the M2D lists read the other way),
//                  the gradient assembled, and the frame torque of the site
//                  evaluated (grad_math.cuh: frame_pullback)
//   k_grad_gather  the frame terms added to the atoms they act on through a
//                  fixed reverse list (deterministic; no atomics)
// AMOEBA uses both dipole sets: E/Egrd/EHes_D2M average the P dipoles with
// the d scales and the D dipoles with the p scales; Wang-AL has one set and
// only the charge terms.
#include <algorithm>
#include <cstdio>
#include <limits>
#include <vector>

#include "engine.h"
#include "grad_math.cuh"
#include "pair_math.cuh"

namespace ommp {

// device data of the gradient (built on the first call; topology only, the
// positions and lab-frame multipoles are the system's)
struct GradState {
  int mm = 0, nsplit = 1, ld = 1;
  double *q0 = nullptr;        // [mm][10] local-frame multipoles (AMOEBA)
  int4 *frame = nullptr;       // frame kind, z, x, y atoms (self when absent)
  int *mm_polar = nullptr;     // [mm] polarizable index or -1
  int *t_ri = nullptr, *t_src = nullptr;  // M2D lists read by static site
  double *t_sP = nullptr, *t_sD = nullptr;
  int *r_ri = nullptr, *r_src = nullptr;  // frame atom -> (site, slot) entries
  double *mu = nullptr;        // [mm][2*3] dipoles per static site
  double *partial = nullptr;   // [nsplit][nacc][mm] (FP64 pass)
  int ns_mp = 0, ns_dip = 0;   // double-single passes: splits and partials
  double *part_mp = nullptr, *part_dip = nullptr;
  double *base = nullptr;      // [mm][3]
  double *rot = nullptr;       // [mm][4][3]
  double *grad = nullptr;      // [mm][3]
};

void free_grad_state(GradState *g) {
  if (!g) return;
  void *bufs[] = {g->q0, g->frame, g->mm_polar, g->t_ri, g->t_src, g->t_sP, g->t_sD, g->r_ri, g->r_src,
                  g->mu, g->partial, g->base, g->rot, g->grad, g->part_mp, g->part_dip};
  for (void *b : bufs)
    if (b) cudaFree(b);
  delete g;
}

namespace gpu {
namespace {

constexpr int GTPB = 128;   // targets per CTA
constexpr int GTILE = 128;  // sources per shared-memory tile

template <bool AMOEBA>
struct Acc {
  static constexpr int N = AMOEBA ? 24 : 15;  // g0[6] hd[6] (hp[6]) e[3] (h[3])
};

struct GradArgs {
  int mm, n, nsplit;
  const Pos64 *mm_pos;
  const double *mm_a, *mm_q;
  const float2 *mm_wa;
  const int *mm_polar, *polar_mm;
  const double *ipd;  // [n_ipd][n][3]
  const double *mu;   // [mm][6] or [mm][3]
  const int *m2d_ri, *m2d_src;
  const double *m2d_sP, *m2d_sD;
  const int *d2d_ri, *d2d_src;
  const double *d2d_s;
  const int *t_ri, *t_src;
  const double *t_sP, *t_sD;
  const double *q0;
  const int4 *frame;
  const int *r_ri, *r_src;
  double *partial, *base, *rot, *grad;
  // partial sums read by k_grad_finish: components [0, 6) from pa (splits
  // na, component stride sa), components [6, nacc) from pb (nb, sb)
  const double *pa, *pb;
  int na, sa, nb, sb;
  double thr;
  float thr2m;
  int *err;
};

__global__ void k_grad_mu(int mm, int n, int nset, const int *__restrict__ mm_polar, const double *__restrict__ ipd,
                          double *__restrict__ mu) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= mm) return;
  const int p = mm_polar[i];
  for (int s = 0; s < nset; ++s)
    for (int c = 0; c < 3; ++c) mu[(size_t)i * 3 * nset + 3 * s + c] = p >= 0 ? ipd[((size_t)s * n + p) * 3 + c] : 0.0;
}

template <bool AMOEBA>
__global__ void __launch_bounds__(GTPB) k_grad_pairs(GradArgs g, int per_split) {
  constexpr int LD = AMOEBA ? 10 : 1;
  constexpr int NM = AMOEBA ? 6 : 3;
  constexpr int NA = Acc<AMOEBA>::N;
  __shared__ Pos64 s_pos[GTILE];
  __shared__ double s_a[GTILE];
  __shared__ float2 s_wa[GTILE];
  __shared__ int s_pol[GTILE];
  __shared__ double s_q[GTILE * LD];
  __shared__ double s_mu[GTILE * NM];
  const int t = blockIdx.x * GTPB + threadIdx.x;
  const bool valid = t < g.mm;
  const Pos64 pt = valid ? g.mm_pos[t] : Pos64{0, 0, 0, 0};
  const double at = valid && AMOEBA ? g.mm_a[t] : 0.0;
  const float2 wat = valid ? g.mm_wa[t] : make_float2(0.f, 0.f);
  const bool tpol = valid && g.mm_polar[t] >= 0;
  double Qt[6] = {0, 0, 0, 0, 0, 0};
  if (AMOEBA && valid)
    for (int c = 0; c < 6; ++c) Qt[c] = g.mm_q[(size_t)t * 10 + 4 + c];
  const double trq = Qt[0] + Qt[2] + Qt[5];
  double acc[NA];
#pragma unroll
  for (int c = 0; c < NA; ++c) acc[c] = 0.0;
  double *g0 = acc, *hd = acc + 6, *hp = acc + 12;
  double *e = AMOEBA ? acc + 18 : acc + 12;
  double *h = AMOEBA ? acc + 21 : acc;  // AMOEBA only
  int bad = 0;
  const int s0 = blockIdx.y * per_split;
  const int s1 = min(g.mm, s0 + per_split);
  for (int t0 = s0; t0 < s1; t0 += GTILE) {
    __syncthreads();
    for (int k = threadIdx.x; k < GTILE; k += GTPB) {
      const int i = t0 + k;
      if (i < s1) {
        s_pos[k] = g.mm_pos[i];
        s_a[k] = AMOEBA ? g.mm_a[i] : 0.0;
        s_wa[k] = g.mm_wa[i];
        s_pol[k] = g.mm_polar[i] >= 0;
      }
    }
    for (int k = threadIdx.x; k < GTILE * LD; k += GTPB) {
      const size_t q = (size_t)t0 * LD + k;
      if (q < (size_t)s1 * LD) s_q[k] = g.mm_q[q];
    }
    for (int k = threadIdx.x; k < GTILE * NM; k += GTPB) {
      const size_t q = (size_t)t0 * NM + k;
      if (q < (size_t)s1 * NM) s_mu[k] = g.mu[q];
    }
    __syncthreads();
    const int cnt = min(GTILE, s1 - t0);
    if (!valid) continue;
    for (int k = 0; k < cnt; ++k) {
      if (t0 + k == t) continue;
      const Pos64 ps = s_pos[k];
      const double dx = pt.x - ps.x, dy = pt.y - ps.y, dz = pt.z - ps.z;
      const double r2 = dx * dx + dy * dy + dz * dz;
      const int spol = s_pol[k];
      if (coincident(r2)) {
        if (tpol || spol) bad = 1;
        continue;
      }
      const float r2f = r2_f32(r2);
      const double rinv = rinv_f64(r2, r2f);
      const bool test = AMOEBA ? maybe_damped_amoeba(r2f, wat, s_wa[k], g.thr2m) : maybe_damped_wang(r2f, wat, s_wa[k]);
      double k3, k5, k7, k9;
      gradmath::damped_k<AMOEBA>(r2, rinv, pt.w * ps.w, fmin(at, s_a[k]), g.thr, test, k3, k5, k7, k9);
      gradmath::multipole_grad<AMOEBA>(&s_q[k * LD], dx, dy, dz, k3, k5, k7, k9, 1.0, g0);
      if (!spol) continue;
      const double *mD = &s_mu[k * NM];
      const double mdD = mD[0] * dx + mD[1] * dy + mD[2] * dz;
      gradmath::dipole_grad(mD, mdD, dx, dy, dz, k5, k7, 1.0, hd);
      if (AMOEBA) {
        const double *mP = mD + 3;
        const double mdP = mP[0] * dx + mP[1] * dy + mP[2] * dz;
        gradmath::dipole_grad(mP, mdP, dx, dy, dz, k5, k7, 1.0, hp);
        const double mb[3] = {0.5 * (mD[0] + mP[0]), 0.5 * (mD[1] + mP[1]), 0.5 * (mD[2] + mP[2])};
        const double mdb = 0.5 * (mdD + mdP);
        gradmath::dipole_field(mb, mdb, dx, dy, dz, k3, k5, 1.0, e);
        gradmath::dipole_hess_q(mb, mdb, dx, dy, dz, Qt, trq, k5, k7, k9, 1.0, h);
      } else {
        gradmath::dipole_field(mD, mdD, dx, dy, dz, k3, k5, 1.0, e);
      }
    }
  }
  if (bad) atomicOr(g.err, 1);
  if (valid) {
    double *o = g.partial + (size_t)blockIdx.y * NA * g.mm + t;
#pragma unroll
    for (int c = 0; c < NA; ++c) o[(size_t)c * g.mm] = acc[c];
  }
}

// exact damped factors of the pair (target t, source i) for the list passes
template <bool AMOEBA>
__device__ __forceinline__ bool pair_k(const GradArgs &g, const Pos64 &pt, double at, int i, double *d, double *k) {
  const Pos64 ps = g.mm_pos[i];
  d[0] = pt.x - ps.x;
  d[1] = pt.y - ps.y;
  d[2] = pt.z - ps.z;
  const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
  if (r2 < 4.9e-28) return false;
  const double rinv = 1.0 / sqrt(r2);
  gradmath::damped_k<AMOEBA>(r2, rinv, pt.w * ps.w, fmin(at, AMOEBA ? g.mm_a[i] : 0.0), g.thr, true, k[0], k[1],
                             k[2], k[3]);
  return true;
}

template <bool AMOEBA>
__global__ void k_grad_finish(GradArgs g) {
  constexpr int LD = AMOEBA ? 10 : 1;
  constexpr int NA = Acc<AMOEBA>::N;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= g.mm) return;
  double acc[NA];
  for (int c = 0; c < 6; ++c) {
    double s = 0.0;
    for (int p = 0; p < g.na; ++p) s += g.pa[((size_t)p * g.sa + c) * g.mm + t];
    acc[c] = s;
  }
  for (int c = 6; c < NA; ++c) {
    double s = 0.0;
    for (int p = 0; p < g.nb; ++p) s += g.pb[((size_t)p * g.sb + c - 6) * g.mm + t];
    acc[c] = s;
  }
  double *g0 = acc, *hd = acc + 6, *hp = acc + 12;
  double *e = AMOEBA ? acc + 18 : acc + 12;
  double *h = AMOEBA ? acc + 21 : acc;  // AMOEBA only
  const Pos64 pt = g.mm_pos[t];
  const double at = AMOEBA ? g.mm_a[t] : 0.0;
  const double *q = &g.mm_q[(size_t)t * LD];
  double Qt[6] = {0, 0, 0, 0, 0, 0};
  if (AMOEBA)
    for (int c = 0; c < 6; ++c) Qt[c] = q[4 + c];
  const double trq = Qt[0] + Qt[2] + Qt[5];
  // field gradient of the mean dipole at t (unscaled part)
  double gm[6];
  for (int c = 0; c < 6; ++c) gm[c] = AMOEBA ? 0.5 * (hd[c] + hp[c]) : 0.0;
  const double *ipdP = g.ipd + (AMOEBA ? (size_t)3 * g.n : 0);
  int bad = 0;
  double dP[6] = {0, 0, 0, 0, 0, 0}, dD[6] = {0, 0, 0, 0, 0, 0};
  const int j = g.mm_polar[t];
  if (j >= 0) {
    // static multipoles, p / d scales
    for (int kk = g.m2d_ri[j]; kk < g.m2d_ri[j + 1]; ++kk) {
      const int i = g.m2d_src[kk];
      double d[3], k[4];
      if (!pair_k<AMOEBA>(g, pt, at, i, d, k)) {
        bad = 1;
        continue;
      }
      double gg[6] = {0, 0, 0, 0, 0, 0};
      gradmath::multipole_grad<AMOEBA>(&g.mm_q[(size_t)i * LD], d[0], d[1], d[2], k[0], k[1], k[2], k[3], 1.0, gg);
      const double cp = g.m2d_sP[kk] - 1.0, cd = AMOEBA ? g.m2d_sD[kk] - 1.0 : 0.0;
      for (int c = 0; c < 6; ++c) {
        dP[c] += cp * gg[c];
        dD[c] += cd * gg[c];
      }
    }
    // induced dipoles, u scales
    for (int kk = g.d2d_ri[j]; kk < g.d2d_ri[j + 1]; ++kk) {
      const int p = g.d2d_src[kk];
      double d[3], k[4];
      if (!pair_k<AMOEBA>(g, pt, at, g.polar_mm[p], d, k)) {
        bad = 1;
        continue;
      }
      const double c = g.d2d_s[kk] - 1.0;
      const double *mD = &g.ipd[3 * (size_t)p];
      gradmath::dipole_grad(mD, gradmath::dot3(mD, d), d[0], d[1], d[2], k[1], k[2], c, hd);
      if (AMOEBA) {
        const double *mP = &ipdP[3 * (size_t)p];
        gradmath::dipole_grad(mP, gradmath::dot3(mP, d), d[0], d[1], d[2], k[1], k[2], c, hp);
      }
    }
  }
  // induced dipoles at the static site: the M2D lists read by static site
  for (int kk = g.t_ri[t]; kk < g.t_ri[t + 1]; ++kk) {
    const int p = g.t_src[kk];
    double d[3], k[4];
    if (!pair_k<AMOEBA>(g, pt, at, g.polar_mm[p], d, k)) {
      bad = 1;
      continue;
    }
    const double *mD = &g.ipd[3 * (size_t)p], *mP = &ipdP[3 * (size_t)p];
    const double cp = g.t_sP[kk] - 1.0, cd = AMOEBA ? g.t_sD[kk] - 1.0 : 0.0;
    double mc[3];
    for (int c = 0; c < 3; ++c) mc[c] = AMOEBA ? 0.5 * (cp * mD[c] + cd * mP[c]) : cp * mD[c];
    const double md = gradmath::dot3(mc, d);
    gradmath::dipole_field(mc, md, d[0], d[1], d[2], k[0], k[1], 1.0, e);
    if (AMOEBA) {
      gradmath::dipole_grad(mc, md, d[0], d[1], d[2], k[1], k[2], 1.0, gm);
      gradmath::dipole_hess_q(mc, md, d[0], d[1], d[2], Qt, trq, k[1], k[2], k[3], 1.0, h);
    }
  }
  if (bad) atomicOr(g.err, 1);
  // assembly (src/mod_geomgrad.F90:132-271)
  double b[3];
  for (int c = 0; c < 3; ++c) b[c] = -q[0] * e[c];
  if (AMOEBA) {
    double x[3];
    gradmath::sym_apply(gm, &q[1], x);
    for (int c = 0; c < 3; ++c) b[c] += x[c] - h[c];
  }
  if (j >= 0) {
    const double *mD = &g.ipd[3 * (size_t)j];
    if (AMOEBA) {
      const double *mP = &ipdP[3 * (size_t)j];
      double GP[6], GD[6], x[3], y[3];
      for (int c = 0; c < 6; ++c) {
        GP[c] = g0[c] + dP[c] + hp[c];
        GD[c] = g0[c] + dD[c] + hd[c];
      }
      gradmath::sym_apply(GP, mD, x);
      gradmath::sym_apply(GD, mP, y);
      for (int c = 0; c < 3; ++c) b[c] += 0.5 * (x[c] + y[c]);
    } else {
      double GM[6], x[3];
      for (int c = 0; c < 6; ++c) GM[c] = g0[c] + dP[c] + hd[c];
      gradmath::sym_apply(GM, mD, x);
      for (int c = 0; c < 3; ++c) b[c] += x[c];
    }
  }
  for (int c = 0; c < 3; ++c) g.base[3 * (size_t)t + c] = b[c];
  if (AMOEBA) {
    // torque of the frame rotation of the site's dipole and quadrupole
    const int4 f = g.frame[t];
    double out[4][3];
    const Pos64 pz = g.mm_pos[f.y], px = g.mm_pos[f.z], py = g.mm_pos[f.w];
    const double c0[3] = {pt.x, pt.y, pt.z}, cz[3] = {pz.x, pz.y, pz.z}, cx[3] = {px.x, px.y, px.z},
                 cy[3] = {py.x, py.y, py.z};
    if (!gradmath::frame_pullback(f.x, c0, cz, cx, cy, &g.q0[(size_t)t * 10], e, gm, out)) atomicOr(g.err, 2);
    double *r = &g.rot[12 * (size_t)t];
    for (int w = 0; w < 4; ++w)
      for (int c = 0; c < 3; ++c) r[3 * w + c] = out[w][c];
  }
}

// frame terms of every site for a given field E [mm][3] and field gradient
// G [mm][6] (rotation_geomgrad): rot [mm][4][3], error bit 2 on a degenerate frame
__global__ void k_rot_terms(int mm, const Pos64 *__restrict__ pos, const int4 *__restrict__ frame,
                            const double *__restrict__ q0, const double *__restrict__ E, const double *__restrict__ G,
                            double *__restrict__ rot, int *err) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= mm) return;
  const int4 f = frame[t];
  const Pos64 pt = pos[t], pz = pos[f.y], px = pos[f.z], py = pos[f.w];
  const double c0[3] = {pt.x, pt.y, pt.z}, cz[3] = {pz.x, pz.y, pz.z}, cx[3] = {px.x, px.y, px.z},
               cy[3] = {py.x, py.y, py.z};
  double out[4][3];
  if (!gradmath::frame_pullback(f.x, c0, cz, cx, cy, &q0[(size_t)t * 10], &E[3 * (size_t)t], &G[6 * (size_t)t], out))
    atomicOr(err, 2);
  double *r = &rot[12 * (size_t)t];
  for (int w = 0; w < 4; ++w)
    for (int c = 0; c < 3; ++c) r[3 * w + c] = out[w][c];
}

__global__ void k_grad_gather(int mm, bool amoeba, const double *__restrict__ base, const double *__restrict__ rot,
                              const int *__restrict__ r_ri, const int *__restrict__ r_src, double *__restrict__ grad) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= mm) return;
  double s[3] = {base[3 * (size_t)t], base[3 * (size_t)t + 1], base[3 * (size_t)t + 2]};
  if (amoeba)
    for (int k = r_ri[t]; k < r_ri[t + 1]; ++k) {
      const double *r = &rot[3 * (size_t)r_src[k]];
      for (int c = 0; c < 3; ++c) s[c] += r[c];
    }
  for (int c = 0; c < 3; ++c) grad[3 * (size_t)t + c] = s[c];
}

// source splits: the split count whose launch, in whole waves of the
// resident CTAs, finishes first (time ~ waves x tiles per split)
int grad_pick_split(int mm, int resident) {
  const int tblocks = (mm + GTPB - 1) / GTPB, tiles = (mm + GTILE - 1) / GTILE;
  int best = 1;
  double best_t = 1e300;
  for (int s = 1; s <= std::min(tiles, 64); ++s) {
    const double waves = std::ceil((double)tblocks * s / resident);
    const double tm = waves * std::ceil((double)tiles / s);
    if (tm < best_t * 0.999) {
      best_t = tm;
      best = s;
    }
  }
  return best;
}

}  // namespace
}  // namespace gpu

// device lists and buffers of the gradient (topology only): built once
int System::ensure_grad_state() {
  if (grad_) return kOk;
  const int mm = d_.m, n = d_.n;
  const bool amoeba = m_.amoeba;
  const int nset = amoeba ? 2 : 1;
  const int nacc = amoeba ? gpu::Acc<true>::N : gpu::Acc<false>::N;
  int st;
  GradState *gs = new GradState();
  gs->mm = mm;
  int resident = 0;
  if (amoeba)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, gpu::k_grad_pairs<true>, gpu::GTPB, 0);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, gpu::k_grad_pairs<false>, gpu::GTPB, 0);
  gs->nsplit = gpu::grad_pick_split(mm, std::max(1, resident) * gpu::sm_count());
  // M2D lists read by static site, and the frame reverse list
  std::vector<int> t_ri(mm + 1, 0), t_src(m2d_pairs_.src.size());
  std::vector<double> t_sP(t_src.size()), t_sD(t_src.size());
  for (size_t k = 0; k < m2d_pairs_.src.size(); ++k) t_ri[m2d_pairs_.src[k] + 1]++;
  for (int i = 0; i < mm; ++i) t_ri[i + 1] += t_ri[i];
  {
    std::vector<int> fill(t_ri.begin(), t_ri.end() - 1);
    for (int j = 0; j < n; ++j)
      for (int k = m2d_pairs_.ri[j]; k < m2d_pairs_.ri[j + 1]; ++k) {
        const int i = m2d_pairs_.src[k], at = fill[i]++;
        t_src[at] = j;
        t_sP[at] = m2d_pairs_.sP[k];
        t_sD[at] = amoeba ? m2d_pairs_.sD[k] : 1.0;
      }
  }
  std::vector<int4> fr(mm);
  std::vector<int> r_ri(mm + 1, 0), r_src;
  for (int i = 0; i < mm; ++i) {
    const int fk = amoeba ? m_.frame[i] : 0;
    fr[i] = make_int4(fk, m_.iz[i] >= 0 ? m_.iz[i] : i, m_.ix[i] >= 0 ? m_.ix[i] : i, m_.iy[i] >= 0 ? m_.iy[i] : i);
  }
  {
    std::vector<std::vector<int>> rev(mm);
    for (int i = 0; i < mm; ++i) {
      if (fr[i].x == 0) continue;
      const int atoms[4] = {i, fr[i].y, fr[i].z, fr[i].w};
      for (int w = 0; w < 4; ++w) rev[atoms[w]].push_back(4 * i + w);
    }
    for (int i = 0; i < mm; ++i) {
      r_ri[i + 1] = r_ri[i] + (int)rev[i].size();
      r_src.insert(r_src.end(), rev[i].begin(), rev[i].end());
    }
  }
  auto alloc = [&](auto *&p, size_t cnt) {
    return cudaMalloc((void **)&p, std::max<size_t>(cnt, 1) * sizeof(*p)) == cudaSuccess ? 0 : 1;
  };
  int bad = alloc(gs->q0, amoeba ? 10 * (size_t)mm : 1) | alloc(gs->frame, mm) | alloc(gs->mm_polar, mm) |
            alloc(gs->t_ri, mm + 1) | alloc(gs->t_src, t_src.size()) | alloc(gs->t_sP, t_src.size()) |
            alloc(gs->t_sD, t_src.size()) | alloc(gs->r_ri, mm + 1) | alloc(gs->r_src, r_src.size()) |
            alloc(gs->mu, 3 * (size_t)nset * mm) | alloc(gs->partial, (size_t)gs->nsplit * nacc * mm) |
            alloc(gs->base, 3 * (size_t)mm) | alloc(gs->rot, 12 * (size_t)mm) | alloc(gs->grad, 3 * (size_t)mm);
  if (bad) {
    cudaGetLastError();
    free_grad_state(gs);
    set_last_error("out of device memory for the polarization gradient");
    return kErrMemory;
  }
  auto up = [&](void *dst, const void *src, size_t bytes) {
    if (bytes) cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st_);
  };
  if (amoeba) up(gs->q0, m_.q0.data(), 10 * (size_t)mm * sizeof(double));
  up(gs->frame, fr.data(), mm * sizeof(int4));
  up(gs->mm_polar, m_.mm_polar.data(), mm * sizeof(int));
  up(gs->t_ri, t_ri.data(), t_ri.size() * sizeof(int));
  up(gs->t_src, t_src.data(), t_src.size() * sizeof(int));
  up(gs->t_sP, t_sP.data(), t_sP.size() * sizeof(double));
  up(gs->t_sD, t_sD.data(), t_sD.size() * sizeof(double));
  up(gs->r_ri, r_ri.data(), r_ri.size() * sizeof(int));
  up(gs->r_src, r_src.data(), r_src.size() * sizeof(int));
  st = check(cudaStreamSynchronize(st_), "gradient setup");  // host vectors die here
  if (st) {
    free_grad_state(gs);
    return st;
  }
  grad_ = gs;
  return kOk;
}

int System::polelec_geomgrad(double *grad_h) {
  const int mm = d_.m, n = d_.n;
  std::fill(grad_h, grad_h + 3 * (size_t)mm, 0.0);
  if (n == 0) return kOk;
  int st;
  if (!ipd_done_) {
    st = ensure_m2d();
    if (st) return st;
    st = polarization(e_m2d_, kSolverNone, kMatvNone, nullptr);
    if (st) return st;
  }
  const bool amoeba = m_.amoeba;
  const int nset = amoeba ? 2 : 1;
  const int nacc = amoeba ? gpu::Acc<true>::N : gpu::Acc<false>::N;
  st = ensure_grad_state();
  if (st) return st;
  GradState &gs = *grad_;
  gpu::GradArgs a{};
  a.mm = mm;
  a.n = n;
  a.nsplit = gs.nsplit;
  a.mm_pos = d_.mm_pos;
  a.mm_a = d_.mm_a;
  a.mm_q = d_.mm_q;
  a.mm_wa = d_.mm_wa32;
  a.mm_polar = gs.mm_polar;
  a.polar_mm = d_.polar_mm;
  a.ipd = ipd_;
  a.mu = gs.mu;
  a.m2d_ri = d_.m2d_ri;
  a.m2d_src = d_.m2d_src;
  a.m2d_sP = d_.m2d_sP;
  a.m2d_sD = d_.m2d_sD;
  a.d2d_ri = d_.d2d_ri;
  a.d2d_src = d_.d2d_src;
  a.d2d_s = d_.d2d_s;
  a.t_ri = gs.t_ri;
  a.t_src = gs.t_src;
  a.t_sP = gs.t_sP;
  a.t_sD = gs.t_sD;
  a.q0 = gs.q0;
  a.frame = gs.frame;
  a.r_ri = gs.r_ri;
  a.r_src = gs.r_src;
  a.partial = gs.partial;
  a.pa = gs.partial;
  a.pb = gs.partial + 6 * (size_t)mm;
  a.na = a.nb = gs.nsplit;
  a.sa = a.sb = nacc;
  a.base = gs.base;
  a.rot = gs.rot;
  a.grad = gs.grad;
  a.thr = d_.damp_thr;
  a.thr2m = (float)(d_.damp_thr * d_.damp_thr * (1.0 + 1e-5));
  a.err = flag_;
  cudaMemsetAsync(flag_, 0, sizeof(int), st_);
  const int tb = (mm + gpu::GTPB - 1) / gpu::GTPB;
  // the mixed modes evaluate the pair sums in double-single (FP32 pipes)
  const bool ds = precision_ != kPrecFP64;
  if (ds && !gs.part_mp) {
    const int sms = gpu::sm_count();
    gs.ns_mp = gpu::grad_ds_pick_split(d_, 0, sms);
    gs.ns_dip = gpu::grad_ds_pick_split(d_, 1, sms);
    if (cudaMalloc((void **)&gs.part_mp, (size_t)gs.ns_mp * 6 * mm * sizeof(double)) != cudaSuccess ||
        cudaMalloc((void **)&gs.part_dip, (size_t)gs.ns_dip * (nacc - 6) * mm * sizeof(double)) != cudaSuccess) {
      cudaGetLastError();
      if (gs.part_mp) cudaFree(gs.part_mp);
      gs.part_mp = nullptr;
      set_last_error("out of device memory for the polarization gradient");
      return kErrMemory;
    }
    // the first pass writes only the polarizable sites' rows
    cudaMemsetAsync(gs.part_mp, 0, (size_t)gs.ns_mp * 6 * mm * sizeof(double), st_);
  }
  KEv ev{};
  if (ktime_on_) ev = kt_begin(3, 1);
  if (ds) {
    gpu::launch_grad_ds_mp(d_, gs.part_mp, gs.ns_mp, flag_, st_);
    gpu::launch_grad_ds_dip(d_, ipd_, gs.part_dip, gs.ns_dip, flag_, st_);
    a.pa = gs.part_mp;
    a.na = gs.ns_mp;
    a.sa = 6;
    a.pb = gs.part_dip;
    a.nb = gs.ns_dip;
    a.sb = nacc - 6;
  } else {
    const int tiles = (mm + gpu::GTILE - 1) / gpu::GTILE;
    const int per = ((tiles + gs.nsplit - 1) / gs.nsplit) * gpu::GTILE;
    const dim3 grid(tb, gs.nsplit);
    gpu::k_grad_mu<<<(mm + 255) / 256, 256, 0, st_>>>(mm, n, nset, gs.mm_polar, ipd_, gs.mu);
    if (amoeba)
      gpu::k_grad_pairs<true><<<grid, gpu::GTPB, 0, st_>>>(a, per);
    else
      gpu::k_grad_pairs<false><<<grid, gpu::GTPB, 0, st_>>>(a, per);
    gpu::add_launch_count(2);
  }
  if (ktime_on_) kt_end(ev);
  if (amoeba)
    gpu::k_grad_finish<true><<<tb, gpu::GTPB, 0, st_>>>(a);
  else
    gpu::k_grad_finish<false><<<tb, gpu::GTPB, 0, st_>>>(a);
  gpu::k_grad_gather<<<(mm + 255) / 256, 256, 0, st_>>>(mm, amoeba, gs.base, gs.rot, gs.r_ri, gs.r_src, gs.grad);
  gpu::add_launch_count(2);
  int flag = 0;
  cudaMemcpyAsync(grad_h, gs.grad, 3 * (size_t)mm * sizeof(double), cudaMemcpyDeviceToHost, st_);
  cudaMemcpyAsync(&flag, flag_, sizeof(int), cudaMemcpyDeviceToHost, st_);
  st = check(cudaStreamSynchronize(st_), "polarization gradient");
  if (st) return st;
  if (flag & 1) {
    std::fill(grad_h, grad_h + 3 * (size_t)mm, 0.0);
    set_last_error(
        "Requesting Coulomb kernel for two atoms placed in the same point, this could be an internal bug or "
        "a problem in your input file, please check.");
    return kErrNumeric;
  }
  if (flag & 2) {
    std::fill(grad_h, grad_h + 3 * (size_t)mm, 0.0);
    set_last_error("Ill defined rotation axis (either u or v vectors have 0 norm.");
    return kErrInput;
  }
  return kOk;
}

// gradient = base [mm][3] + the frame forces of the static multipoles in E
// [mm][3] and field gradient G [mm][6] (device arrays), copied to grad_h
int System::frame_forces(const double *E, const double *G, const double *base, double *grad_h) {
  const int mm = d_.m;
  int st = ensure_grad_state();
  if (st) return st;
  GradState &gs = *grad_;
  const bool amoeba = m_.amoeba;
  cudaMemsetAsync(flag_, 0, sizeof(int), st_);
  if (amoeba) gpu::k_rot_terms<<<(mm + 127) / 128, 128, 0, st_>>>(mm, d_.mm_pos, gs.frame, gs.q0, E, G, gs.rot, flag_);
  gpu::k_grad_gather<<<(mm + 255) / 256, 256, 0, st_>>>(mm, amoeba, base, gs.rot, gs.r_ri, gs.r_src, gs.grad);
  gpu::add_launch_count(amoeba ? 2 : 1);
  int flag = 0;
  cudaMemcpyAsync(grad_h, gs.grad, 3 * (size_t)mm * sizeof(double), cudaMemcpyDeviceToHost, st_);
  cudaMemcpyAsync(&flag, flag_, sizeof(int), cudaMemcpyDeviceToHost, st_);
  st = check(cudaStreamSynchronize(st_), "frame forces");
  if (st) return st;
  if (flag & 2) {
    std::fill(grad_h, grad_h + 3 * (size_t)mm, 0.0);
    set_last_error("Ill defined rotation axis (either u or v vectors have 0 norm.");
    return kErrInput;
  }
  return kOk;
}

int System::rotation_geomgrad(const double *E_h, const double *G_h, double *grad_h) {
  const int mm = d_.m;
  std::fill(grad_h, grad_h + 3 * (size_t)mm, 0.0);
  if (mm == 0 || !m_.amoeba) return kOk;  // point charges have no frame
  int st = ensure_grad_state();
  if (st) return st;
  GradState &gs = *grad_;
  // E, G staged in the partial buffer (at least 24 mm doubles), zero base
  double *E = gs.partial, *G = gs.partial + 3 * (size_t)mm;
  cudaMemcpyAsync(E, E_h, 3 * (size_t)mm * sizeof(double), cudaMemcpyHostToDevice, st_);
  cudaMemcpyAsync(G, G_h, 6 * (size_t)mm * sizeof(double), cudaMemcpyHostToDevice, st_);
  cudaMemsetAsync(gs.base, 0, 3 * (size_t)mm * sizeof(double), st_);
  return frame_forces(E, G, gs.base, grad_h);
}

}  // namespace ommp
