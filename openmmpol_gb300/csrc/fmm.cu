// Fast multipole method for the FP64 dipole-field product T.mu (the
// reference's FMM path of TMatVec / field_extD2D, src/mod_electrostatics.F90:
// 1954-2065 with src/fast_multipoles/), enabled by ommp_enable_fmm.
//
// GB300 design: a uniform octree over the polarizable sites whose leaf side
// is at least the Thole damping range (every damped pair is a near pair), of
// the depth that minimises near-field pairs plus M2L work; Cartesian Taylor
// expansions of order p (fmm_math.cuh); all passes in FP64:
//   k_fmm_p2m     leaf multipoles of the dipoles (one CTA per leaf)
//   k_fmm_m2m     parent multipoles from the 8 children, level by level
//   k_fmm_m2l     local expansions from the well-separated cells of each
//                 level (children of the parent's neighbours that are not
//                 neighbours).  The derivatives of 1/r depend only on the
//                 integer offset of the two cells, so they are tabulated
//                 once per order for the 7^3 offsets at unit cell size and
//                 scaled per level (1/r^(n+1) is homogeneous): the M2L is a
//                 gather of products, its (target term, source term) pairs
//                 spread evenly over the threads, each pair with its own
//                 shared-memory accumulator summed per target term in a
//                 fixed order (deterministic)
//   k_fmm_l2l     children's local expansions from the parent's
//   k_fmm_l2p     far field of the leaf's local expansion at each site plus
//                 the near field of the 27 neighbouring leaves, direct, with
//                 the Thole damping of the direct kernels
// then the finishing pass of the direct product (scaled-pair corrections
// with exact pair terms, sign, 1/alpha diagonal).  Sites are kept in leaf
// order on the device (a counting sort per geometry).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <vector>

#include "engine.h"
#include "fmm_math.cuh"
#include "log.h"
#include "pair_math.cuh"

namespace ommp {

struct FmmState {
  int p = 0, K = 0, KD = 0, npairs = 0;
  int L = -1, ncell = 0, nalloc_cell = 0;
  double h0 = 0.0, ox = 0.0, oy = 0.0, oz = 0.0;
  std::vector<int> off;        // first cell of each level
  bool built = false;
  // device
  int *cnt = nullptr;          // sites per cell, every level
  int *leaf_start = nullptr;   // [nleaf + 1] in sorted order
  int *perm = nullptr;         // sorted -> polarizable index
  gpu::Pos64 *spos = nullptr;  // sorted positions, w = 1/thole
  double *sa = nullptr;        // sorted Thole damping a
  float2 *swa = nullptr;       // sorted FP32 damping pre-test data
  short4 *terms = nullptr;     // exponents (a, b, c) and order of each term
  int4 *pairs = nullptr;       // M2L pairs: g, index of g + h in the 2p table, h, (-1)^|g|
  int *hoff = nullptr;         // [K + 1] first pair of each target term h
  double *dunit = nullptr;     // [343][KD] derivatives of 1/r to order p at unit cell offsets
  // translation lists (M2M, L2L), grouped by target term: source term and
  // packed |m| (bits 0-7) with the parities of m (bits 8-10), coefficient
  int2 *mm_e = nullptr, *ll_e = nullptr;
  double *mm_c = nullptr, *ll_c = nullptr;
  int *mm_off = nullptr, *ll_off = nullptr;
  double *M = nullptr, *Lc = nullptr;  // [2][ncell][K]
  double *field = nullptr;     // [2][n][3]
  size_t field_n = 0;
};

void free_fmm_state(FmmState *f) {
  if (!f) return;
  void *b[] = {f->cnt, f->leaf_start, f->perm, f->spos, f->sa, f->swa, f->terms, f->pairs, f->hoff, f->dunit,
               f->M, f->Lc, f->field, f->mm_e, f->ll_e, f->mm_c, f->ll_c, f->mm_off, f->ll_off};
  for (void *p : b)
    if (p) cudaFree(p);
  delete f;
}

namespace gpu {
namespace {

constexpr int FT = 128;  // threads per CTA
constexpr int FCH = 32;  // sites staged per chunk in the P2M
constexpr int kMaxTermsPerThread = (fmm::nterms(fmm::kMaxOrder) + FT - 1) / FT;

struct FmmArgs {
  int p, K, L, ncell, ncol;
  double h0, ox, oy, oz;
  const int *cnt, *leaf_start, *perm;
  const Pos64 *spos;
  const double *sa;
  const float2 *swa;
  const short4 *terms;
  const int4 *pairs;
  const int *hoff;
  const double *dunit;
  double *M, *Lc;
  int KD;
  const int2 *mm_e, *ll_e;
  const double *mm_c, *ll_c;
  const int *mm_off, *ll_off;
};

// sign of s^m for the child offset s = (b - 1/2) h_c per axis (bit b = 0:
// negative component) and the parities packed in e.y bits 8-10
__device__ __forceinline__ double child_sign(int packed, int bx, int by, int bz) {
  const int neg = (((packed >> 8) & 1) & (bx ^ 1)) ^ (((packed >> 9) & 1) & (by ^ 1)) ^ (((packed >> 10) & 1) & (bz ^ 1));
  return neg ? -1.0 : 1.0;
}

__device__ __forceinline__ void cell_xyz(int idx, int l, int &x, int &y, int &z) {
  const int n = 1 << l;
  z = idx % n;
  y = (idx / n) % n;
  x = idx / (n * n);
}
__device__ __forceinline__ int cell_idx(int l, int x, int y, int z) {
  const int n = 1 << l;
  return (x * n + y) * n + z;
}
__device__ __forceinline__ int level_off(int l) { return ((1 << (3 * l)) - 1) / 7; }

// leaf multipoles of the dipoles x [col][n][3]
__global__ void __launch_bounds__(FT) k_fmm_p2m(FmmArgs a, const double *__restrict__ x, int n) {
  __shared__ double s_p[3][fmm::kMaxOrder + 1][FCH];
  __shared__ double s_mu[3][FCH];
  const int c = blockIdx.x, col = blockIdx.y;
  const int s0 = a.leaf_start[c], s1 = a.leaf_start[c + 1];
  if (s0 == s1) return;
  int cx, cy, cz;
  cell_xyz(c, a.L, cx, cy, cz);
  const double h = a.h0 / (1 << a.L);
  const double ctr[3] = {a.ox + (cx + 0.5) * h, a.oy + (cy + 0.5) * h, a.oz + (cz + 0.5) * h};
  double acc[kMaxTermsPerThread];
  for (int j = 0; j < kMaxTermsPerThread; ++j) acc[j] = 0.0;
  for (int b0 = s0; b0 < s1; b0 += FCH) {
    __syncthreads();
    const int k = threadIdx.x;
    if (k < FCH && b0 + k < s1) {
      const Pos64 ps = a.spos[b0 + k];
      const int pi = a.perm[b0 + k];
      const double v[3] = {ps.x - ctr[0], ps.y - ctr[1], ps.z - ctr[2]};
      for (int d = 0; d < 3; ++d) {
        double pw = 1.0;
        s_p[d][0][k] = 1.0;
        for (int m = 1; m <= a.p; ++m) {
          pw = pw * v[d] / m;
          s_p[d][m][k] = pw;
        }
        s_mu[d][k] = x[((size_t)col * n + pi) * 3 + d];
      }
    }
    __syncthreads();
    const int cnt = min(FCH, s1 - b0);
    for (int j = 0; j < kMaxTermsPerThread; ++j) {
      const int t = threadIdx.x + j * FT;
      if (t >= a.K) break;
      const short4 e = a.terms[t];
      double w = 0.0;
      for (int q = 0; q < cnt; ++q) {
        if (e.x) w += s_mu[0][q] * s_p[0][e.x - 1][q] * s_p[1][e.y][q] * s_p[2][e.z][q];
        if (e.y) w += s_mu[1][q] * s_p[0][e.x][q] * s_p[1][e.y - 1][q] * s_p[2][e.z][q];
        if (e.z) w += s_mu[2][q] * s_p[0][e.x][q] * s_p[1][e.y][q] * s_p[2][e.z - 1][q];
      }
      acc[j] += w;
    }
  }
  double *Mc = a.M + ((size_t)col * a.ncell + level_off(a.L) + c) * a.K;
  for (int j = 0; j < kMaxTermsPerThread; ++j) {
    const int t = threadIdx.x + j * FT;
    if (t < a.K) Mc[t] = acc[j];
  }
}

// parents at level l - 1 from their children at level l:
// M_g(parent) = sum_children sum_(k <= g) M_k(child) s^(g - k) / (g - k)!
__global__ void __launch_bounds__(FT) k_fmm_m2m(FmmArgs a, int l) {
  const int pc = blockIdx.x, col = blockIdx.y;
  if (a.cnt[level_off(l - 1) + pc] == 0) return;
  int px, py, pz;
  cell_xyz(pc, l - 1, px, py, pz);
  double hp[fmm::kMaxOrder + 1];  // (h_c / 2)^k
  hp[0] = 1.0;
  for (int k = 1; k <= a.p; ++k) hp[k] = hp[k - 1] * 0.5 * a.h0 / (1 << l);
  double acc[kMaxTermsPerThread];
  for (int j = 0; j < kMaxTermsPerThread; ++j) acc[j] = 0.0;
  for (int ch = 0; ch < 8; ++ch) {
    const int bx = ch >> 2, by = (ch >> 1) & 1, bz = ch & 1;
    const int cc = cell_idx(l, 2 * px + bx, 2 * py + by, 2 * pz + bz);
    if (a.cnt[level_off(l) + cc] == 0) continue;
    const double *Mc = a.M + ((size_t)col * a.ncell + level_off(l) + cc) * a.K;
    for (int j = 0; j < kMaxTermsPerThread; ++j) {
      const int t = threadIdx.x + j * FT;
      if (t >= a.K) break;
      double w = 0.0;
      for (int e = a.mm_off[t]; e < a.mm_off[t + 1]; ++e) {
        const int2 ent = a.mm_e[e];
        w += Mc[ent.x] * a.mm_c[e] * hp[ent.y & 255] * child_sign(ent.y, bx, by, bz);
      }
      acc[j] += w;
    }
  }
  double *Mp = a.M + ((size_t)col * a.ncell + level_off(l - 1) + pc) * a.K;
  for (int j = 0; j < kMaxTermsPerThread; ++j) {
    const int t = threadIdx.x + j * FT;
    if (t < a.K) Mp[t] = acc[j];
  }
}

// local expansions at level l from the well-separated cells of the level
__global__ void __launch_bounds__(FT) k_fmm_m2l(FmmArgs a, int l) {
  extern __shared__ double sh[];
  double *s_m = sh;               // [K] source multipole scaled by h^-|g|
  double *s_acc = sh + a.K;       // [npairs] per-pair accumulators
  const int npairs = a.hoff[a.K];
  const int tc = blockIdx.x, col = blockIdx.y;
  if (a.cnt[level_off(l) + tc] == 0) return;
  int tx, ty, tz;
  cell_xyz(tc, l, tx, ty, tz);
  const int n = 1 << l;
  const double hinv = (1 << l) / a.h0;
  for (int q = threadIdx.x; q < npairs; q += FT) s_acc[q] = 0.0;
  for (int ox = -1; ox <= 1; ++ox)
    for (int oy = -1; oy <= 1; ++oy)
      for (int oz = -1; oz <= 1; ++oz) {
        const int PX = (tx >> 1) + ox, PY = (ty >> 1) + oy, PZ = (tz >> 1) + oz;
        if (PX < 0 || PY < 0 || PZ < 0 || 2 * PX >= n || 2 * PY >= n || 2 * PZ >= n) continue;
        for (int ch = 0; ch < 8; ++ch) {
          const int sx = 2 * PX + (ch >> 2), sy = 2 * PY + ((ch >> 1) & 1), sz = 2 * PZ + (ch & 1);
          const int dx = tx - sx, dy = ty - sy, dz = tz - sz;
          if (abs(dx) <= 1 && abs(dy) <= 1 && abs(dz) <= 1) continue;
          const int sc = cell_idx(l, sx, sy, sz);
          if (a.cnt[level_off(l) + sc] == 0) continue;  // uniform over the CTA
          __syncthreads();
          const double *Ms = a.M + ((size_t)col * a.ncell + level_off(l) + sc) * a.K;
          for (int g = threadIdx.x; g < a.K; g += FT) {
            const int ng = a.terms[g].w;
            double f = 1.0;
            for (int i = 0; i < ng; ++i) f *= hinv;
            s_m[g] = Ms[g] * f;
          }
          __syncthreads();
          const double *D = a.dunit + (size_t)(((dx + 3) * 7 + (dy + 3)) * 7 + (dz + 3)) * a.KD;
          for (int q = threadIdx.x; q < npairs; q += FT) {
            const int4 pr = a.pairs[q];
            s_acc[q] += (pr.w ? -s_m[pr.x] : s_m[pr.x]) * D[pr.y];
          }
        }
      }
  __syncthreads();
  double *Lt = a.Lc + ((size_t)col * a.ncell + level_off(l) + tc) * a.K;
  for (int hh = threadIdx.x; hh < a.K; hh += FT) {
    double s = 0.0;
    for (int q = a.hoff[hh]; q < a.hoff[hh + 1]; ++q) s += s_acc[q];
    const short4 e = a.terms[hh];
    double f = hinv;  // h^-(|h| + 1) / h!
    for (int i = 0; i < e.w; ++i) f *= hinv;
    for (int i = 2; i <= e.x; ++i) f /= i;
    for (int i = 2; i <= e.y; ++i) f /= i;
    for (int i = 2; i <= e.z; ++i) f /= i;
    Lt[hh] += s * f;
  }
}

// The same M2L with the (target term, source term) pairs of each thread
// held in registers (orders up to 8: at most kRegPairs pairs per thread),
// both columns in one CTA sharing the derivative row staged in shared memory.
constexpr int kRegPairs = 24;
__global__ void __launch_bounds__(FT) k_fmm_m2l_reg(FmmArgs a, int l) {
  extern __shared__ double sh[];
  double *s_m = sh;                // [2][K]
  double *s_d = sh + 2 * a.K;      // [KD]
  double *s_acc = s_d + a.KD;      // [npairs]
  const int npairs = a.hoff[a.K];
  const int tc = blockIdx.x;
  if (a.cnt[level_off(l) + tc] == 0) return;
  int tx, ty, tz;
  cell_xyz(tc, l, tx, ty, tz);
  const int n = 1 << l;
  const double hinv = (1 << l) / a.h0;
  int pk[kRegPairs];
  double acc0[kRegPairs], acc1[kRegPairs];
#pragma unroll
  for (int j = 0; j < kRegPairs; ++j) {
    const int q = threadIdx.x + j * FT;
    pk[j] = -1;
    if (q < npairs) {
      const int4 pr = a.pairs[q];
      pk[j] = pr.x | (pr.y << 10) | (pr.w << 20);
    }
    acc0[j] = acc1[j] = 0.0;
  }
  for (int ox = -1; ox <= 1; ++ox)
    for (int oy = -1; oy <= 1; ++oy)
      for (int oz = -1; oz <= 1; ++oz) {
        const int PX = (tx >> 1) + ox, PY = (ty >> 1) + oy, PZ = (tz >> 1) + oz;
        if (PX < 0 || PY < 0 || PZ < 0 || 2 * PX >= n || 2 * PY >= n || 2 * PZ >= n) continue;
        for (int ch = 0; ch < 8; ++ch) {
          const int sx = 2 * PX + (ch >> 2), sy = 2 * PY + ((ch >> 1) & 1), sz = 2 * PZ + (ch & 1);
          const int dx = tx - sx, dy = ty - sy, dz = tz - sz;
          if (abs(dx) <= 1 && abs(dy) <= 1 && abs(dz) <= 1) continue;
          const int sc = cell_idx(l, sx, sy, sz);
          if (a.cnt[level_off(l) + sc] == 0) continue;  // uniform over the CTA
          __syncthreads();
          for (int i = threadIdx.x; i < a.ncol * a.K; i += FT) {
            const int col = i / a.K, g = i - col * a.K;
            const int ng = a.terms[g].w;
            double f = 1.0;
            for (int r = 0; r < ng; ++r) f *= hinv;
            s_m[i] = a.M[((size_t)col * a.ncell + level_off(l) + sc) * a.K + g] * f;
          }
          const double *D = a.dunit + (size_t)(((dx + 3) * 7 + (dy + 3)) * 7 + (dz + 3)) * a.KD;
          for (int i = threadIdx.x; i < a.KD; i += FT) s_d[i] = D[i];
          __syncthreads();
#pragma unroll
          for (int j = 0; j < kRegPairs; ++j) {
            if (pk[j] < 0) continue;
            const int g = pk[j] & 1023;
            const double d = (pk[j] >> 20) ? -s_d[(pk[j] >> 10) & 1023] : s_d[(pk[j] >> 10) & 1023];
            acc0[j] += s_m[g] * d;
            acc1[j] += s_m[a.K + g] * d;
          }
        }
      }
  for (int col = 0; col < a.ncol; ++col) {
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kRegPairs; ++j) {
      const int q = threadIdx.x + j * FT;
      if (q < npairs) s_acc[q] = col ? acc1[j] : acc0[j];
    }
    __syncthreads();
    double *Lt = a.Lc + ((size_t)col * a.ncell + level_off(l) + tc) * a.K;
    for (int hh = threadIdx.x; hh < a.K; hh += FT) {
      double s = 0.0;
      for (int q = a.hoff[hh]; q < a.hoff[hh + 1]; ++q) s += s_acc[q];
      const short4 e = a.terms[hh];
      double f = hinv;  // h^-(|h| + 1) / h!
      for (int i = 0; i < e.w; ++i) f *= hinv;
      for (int i = 2; i <= e.x; ++i) f /= i;
      for (int i = 2; i <= e.y; ++i) f /= i;
      for (int i = 2; i <= e.z; ++i) f /= i;
      Lt[hh] += s * f;
    }
  }
}

// children at level l + 1 from their parent at level l:
// L_k(child) += sum_(h >= k) L_h(parent) h! / (k! (h - k)!) t^(h - k)
__global__ void __launch_bounds__(FT) k_fmm_l2l(FmmArgs a, int l) {
  const int cc = blockIdx.x, col = blockIdx.y;
  if (a.cnt[level_off(l + 1) + cc] == 0) return;
  int cx, cy, cz;
  cell_xyz(cc, l + 1, cx, cy, cz);
  double hp[fmm::kMaxOrder + 1];  // (h_c / 2)^k
  hp[0] = 1.0;
  for (int k = 1; k <= a.p; ++k) hp[k] = hp[k - 1] * 0.5 * a.h0 / (1 << (l + 1));
  const int bx = cx & 1, by = cy & 1, bz = cz & 1;
  const double *Lp = a.Lc + ((size_t)col * a.ncell + level_off(l) + cell_idx(l, cx >> 1, cy >> 1, cz >> 1)) * a.K;
  double *Lch = a.Lc + ((size_t)col * a.ncell + level_off(l + 1) + cc) * a.K;
  for (int k = threadIdx.x; k < a.K; k += FT) {
    double w = 0.0;
    for (int e = a.ll_off[k]; e < a.ll_off[k + 1]; ++e) {
      const int2 ent = a.ll_e[e];
      w += Lp[ent.x] * a.ll_c[e] * hp[ent.y & 255] * child_sign(ent.y, bx, by, bz);
    }
    Lch[k] += w;
  }
}

// far field of the leaf's local expansion plus the direct near field of the
// 27 neighbouring leaves at each site of the leaf; field [col][n][3]
template <bool AMOEBA>
__global__ void __launch_bounds__(FT) k_fmm_l2p(FmmArgs a, const double *__restrict__ x, int n, double thr,
                                                 float thr2m, double *__restrict__ field) {
  __shared__ Pos64 s_pos[FT];
  __shared__ double s_a[FT];
  __shared__ float2 s_wa[FT];
  __shared__ double s_mu[FT * 3];
  __shared__ double s_L[fmm::nterms(fmm::kMaxOrder)];
  const int c = blockIdx.x, col = blockIdx.y;
  const int s0 = a.leaf_start[c], s1 = a.leaf_start[c + 1];
  if (s0 == s1) return;
  int cx, cy, cz;
  cell_xyz(c, a.L, cx, cy, cz);
  const int nl = 1 << a.L;
  const double h = a.h0 / nl;
  const double ctr[3] = {a.ox + (cx + 0.5) * h, a.oy + (cy + 0.5) * h, a.oz + (cz + 0.5) * h};
  const double *Lt = a.Lc + ((size_t)col * a.ncell + level_off(a.L) + c) * a.K;
  for (int t = threadIdx.x; t < a.K; t += FT) s_L[t] = Lt[t];
  for (int b0 = s0; b0 < s1; b0 += FT) {
    const int si = b0 + threadIdx.x;
    const bool valid = si < s1;
    Pos64 pt = valid ? a.spos[si] : Pos64{0, 0, 0, 0};
    const double at = valid && AMOEBA ? a.sa[si] : 0.0;
    const float2 wat = valid ? a.swa[si] : make_float2(0.f, 0.f);
    double e[3] = {0.0, 0.0, 0.0};
    __syncthreads();
    if (valid) {
      const double u[3] = {pt.x - ctr[0], pt.y - ctr[1], pt.z - ctr[2]};
      double pu[3][fmm::kMaxOrder + 1];
      for (int d = 0; d < 3; ++d) {
        pu[d][0] = 1.0;
        for (int m = 1; m <= a.p; ++m) pu[d][m] = pu[d][m - 1] * u[d];
      }
      for (int t = 0; t < a.K; ++t) {
        const short4 ex = a.terms[t];
        const double Lv = s_L[t];
        if (ex.x) e[0] -= Lv * ex.x * pu[0][ex.x - 1] * pu[1][ex.y] * pu[2][ex.z];
        if (ex.y) e[1] -= Lv * ex.y * pu[0][ex.x] * pu[1][ex.y - 1] * pu[2][ex.z];
        if (ex.z) e[2] -= Lv * ex.z * pu[0][ex.x] * pu[1][ex.y] * pu[2][ex.z - 1];
      }
    }
    for (int ox = -1; ox <= 1; ++ox)
      for (int oy = -1; oy <= 1; ++oy)
        for (int oz = -1; oz <= 1; ++oz) {
          const int X = cx + ox, Y = cy + oy, Z = cz + oz;
          if (X < 0 || Y < 0 || Z < 0 || X >= nl || Y >= nl || Z >= nl) continue;
          const int nc = cell_idx(a.L, X, Y, Z);
          const int r0 = a.leaf_start[nc], r1 = a.leaf_start[nc + 1];
          for (int t0 = r0; t0 < r1; t0 += FT) {
            __syncthreads();
            const int k = t0 + threadIdx.x;
            if (k < r1) {
              s_pos[threadIdx.x] = a.spos[k];
              s_a[threadIdx.x] = AMOEBA ? a.sa[k] : 0.0;
              s_wa[threadIdx.x] = a.swa[k];
              const int pi = a.perm[k];
              for (int d = 0; d < 3; ++d) s_mu[threadIdx.x * 3 + d] = x[((size_t)col * n + pi) * 3 + d];
            }
            __syncthreads();
            if (!valid) continue;
            const int cnt = min(FT, r1 - t0);
            for (int q = 0; q < cnt; ++q) {
              if (t0 + q == si) continue;
              const Pos64 ps = s_pos[q];
              const double dx = pt.x - ps.x, dy = pt.y - ps.y, dz = pt.z - ps.z;
              const double r2 = dx * dx + dy * dy + dz * dz;
              if (r2 < 4.9e-28) continue;
              double k3, k5x3;
              dd_pair<double, AMOEBA>(r2, pt.w, ps.w, at, s_a[q], wat, s_wa[q], thr, thr2m, k3, k5x3);
              const double *mu = &s_mu[q * 3];
              const double f = k5x3 * (mu[0] * dx + mu[1] * dy + mu[2] * dz);
              e[0] += f * dx - k3 * mu[0];
              e[1] += f * dy - k3 * mu[1];
              e[2] += f * dz - k3 * mu[2];
            }
          }
        }
    if (valid) {
      const int pi = a.perm[si];
      for (int d = 0; d < 3; ++d) field[((size_t)col * n + pi) * 3 + d] = e[d];
    }
  }
}

}  // namespace
}  // namespace gpu

int System::set_fmm(bool on, int order) {
  if (order < 2 || order > fmm::kMaxOrder) {
    set_last_error("FMM expansion order must be between 2 and 12");
    return kErrBadArg;
  }
  if (fmm_ && fmm_->p != order) {
    free_fmm_state(fmm_);
    fmm_ = nullptr;
  }
  fmm_on_ = on;
  fmm_order_ = order;
  return kOk;
}

void System::fmm_invalidate() {
  if (fmm_) fmm_->built = false;
}

int System::fmm_prepare() {
  if (fmm_ && fmm_->built) return kOk;
  const int n = d_.n;
  if (!fmm_) {
    fmm_ = new FmmState();
    FmmState &f = *fmm_;
    f.p = fmm_order_;
    f.K = fmm::nterms(f.p);
    f.KD = fmm::nterms(f.p);  // |g| + |h| <= p: derivatives to order p
    // terms, M2L pairs sorted by target term, unit-offset derivative tables
    std::vector<short4> terms(f.K);
    for (int t = 0; t < f.K; ++t) {
      int a, b, c;
      fmm::exponents(t, a, b, c);
      terms[t] = make_short4((short)a, (short)b, (short)c, (short)(a + b + c));
    }
    std::vector<int4> pairs;
    std::vector<int> hoff(f.K + 1, 0);
    for (int h = 0; h < f.K; ++h) {
      hoff[h] = (int)pairs.size();
      const int nh = terms[h].w;
      for (int g = 0; g < fmm::nterms(f.p - nh); ++g)
        pairs.push_back(make_int4(g, fmm::term(terms[g].x + terms[h].x, terms[g].y + terms[h].y, terms[g].z + terms[h].z),
                                  h, terms[g].w & 1));
    }
    hoff[f.K] = (int)pairs.size();
    f.npairs = (int)pairs.size();
    std::vector<double> dunit((size_t)343 * f.KD, 0.0);
    for (int i = -3; i <= 3; ++i)
      for (int j = -3; j <= 3; ++j)
        for (int k = -3; k <= 3; ++k) {
          if (std::abs(i) <= 1 && std::abs(j) <= 1 && std::abs(k) <= 1) continue;
          fmm::derivatives(i, j, k, f.p, &dunit[(size_t)(((i + 3) * 7 + (j + 3)) * 7 + (k + 3)) * f.KD]);
        }
    // translation lists: M2M (target g, source k <= g, 1 / (g - k)!) and L2L
    // (target k, source h >= k, h! / (k! (h - k)!)), grouped by target term
    std::vector<int2> mm_e, ll_e;
    std::vector<double> mm_c, ll_c;
    std::vector<int> mm_off(f.K + 1, 0), ll_off(f.K + 1, 0);
    auto fact = [](int k) {
      double r = 1.0;
      for (int i = 2; i <= k; ++i) r *= i;
      return r;
    };
    auto pack = [](int mx, int my, int mz) { return (mx + my + mz) | ((mx & 1) << 8) | ((my & 1) << 9) | ((mz & 1) << 10); };
    for (int t = 0; t < f.K; ++t) {
      const short4 e = terms[t];
      mm_off[t] = (int)mm_e.size();
      for (int k = 0; k < f.K; ++k) {
        const short4 q = terms[k];
        if (q.x > e.x || q.y > e.y || q.z > e.z) continue;
        const int mx = e.x - q.x, my = e.y - q.y, mz = e.z - q.z;
        mm_e.push_back(make_int2(k, pack(mx, my, mz)));
        mm_c.push_back(1.0 / (fact(mx) * fact(my) * fact(mz)));
      }
      ll_off[t] = (int)ll_e.size();
      for (int h = 0; h < f.K; ++h) {
        const short4 q = terms[h];
        if (q.x < e.x || q.y < e.y || q.z < e.z) continue;
        const int mx = q.x - e.x, my = q.y - e.y, mz = q.z - e.z;
        ll_e.push_back(make_int2(h, pack(mx, my, mz)));
        ll_c.push_back(fact(q.x) * fact(q.y) * fact(q.z) /
                       (fact(e.x) * fact(e.y) * fact(e.z) * fact(mx) * fact(my) * fact(mz)));
      }
    }
    mm_off[f.K] = (int)mm_e.size();
    ll_off[f.K] = (int)ll_e.size();
    bool bad = cudaMalloc((void **)&f.mm_e, mm_e.size() * sizeof(int2)) != cudaSuccess ||
               cudaMalloc((void **)&f.ll_e, ll_e.size() * sizeof(int2)) != cudaSuccess ||
               cudaMalloc((void **)&f.mm_c, mm_c.size() * sizeof(double)) != cudaSuccess ||
               cudaMalloc((void **)&f.ll_c, ll_c.size() * sizeof(double)) != cudaSuccess ||
               cudaMalloc((void **)&f.mm_off, mm_off.size() * sizeof(int)) != cudaSuccess ||
               cudaMalloc((void **)&f.ll_off, ll_off.size() * sizeof(int)) != cudaSuccess;
    bad = bad || cudaMalloc((void **)&f.terms, f.K * sizeof(short4)) != cudaSuccess ||
               cudaMalloc((void **)&f.pairs, pairs.size() * sizeof(int4)) != cudaSuccess ||
               cudaMalloc((void **)&f.hoff, hoff.size() * sizeof(int)) != cudaSuccess ||
               cudaMalloc((void **)&f.dunit, dunit.size() * sizeof(double)) != cudaSuccess;
    if (bad) {
      cudaGetLastError();
      set_last_error("out of device memory for the FMM tables");
      return kErrMemory;
    }
    cudaMemcpyAsync(f.terms, terms.data(), f.K * sizeof(short4), cudaMemcpyHostToDevice, st_);
    cudaMemcpyAsync(f.pairs, pairs.data(), pairs.size() * sizeof(int4), cudaMemcpyHostToDevice, st_);
    cudaMemcpyAsync(f.hoff, hoff.data(), hoff.size() * sizeof(int), cudaMemcpyHostToDevice, st_);
    cudaMemcpyAsync(f.dunit, dunit.data(), dunit.size() * sizeof(double), cudaMemcpyHostToDevice, st_);
    cudaMemcpyAsync(f.mm_e, mm_e.data(), mm_e.size() * sizeof(int2), cudaMemcpyHostToDevice, st_);
    cudaMemcpyAsync(f.ll_e, ll_e.data(), ll_e.size() * sizeof(int2), cudaMemcpyHostToDevice, st_);
    cudaMemcpyAsync(f.mm_c, mm_c.data(), mm_c.size() * sizeof(double), cudaMemcpyHostToDevice, st_);
    cudaMemcpyAsync(f.ll_c, ll_c.data(), ll_c.size() * sizeof(double), cudaMemcpyHostToDevice, st_);
    cudaMemcpyAsync(f.mm_off, mm_off.data(), mm_off.size() * sizeof(int), cudaMemcpyHostToDevice, st_);
    cudaMemcpyAsync(f.ll_off, ll_off.data(), ll_off.size() * sizeof(int), cudaMemcpyHostToDevice, st_);
    int st = check(cudaStreamSynchronize(st_), "FMM tables");
    if (st) return st;
    const size_t smem = (f.K + (size_t)f.npairs) * sizeof(double);
    if (smem > 48 * 1024)
      cudaFuncSetAttribute(gpu::k_fmm_m2l, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    const size_t smem_reg = (2 * (size_t)f.K + f.KD + f.npairs) * sizeof(double);
    if (f.npairs <= gpu::kRegPairs * gpu::FT && smem_reg > 48 * 1024)
      cudaFuncSetAttribute(gpu::k_fmm_m2l_reg, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_reg);
  }
  FmmState &f = *fmm_;
  // geometry: bounding cube of the polarizable sites, leaf level
  std::vector<double> px(n), py(n), pz(n);
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int j = 0; j < n; ++j) {
    const double *c = &m_.cmm[3 * (size_t)m_.polar_mm[j]];
    px[j] = c[0], py[j] = c[1], pz[j] = c[2];
    for (int d = 0; d < 3; ++d) lo[d] = std::min(lo[d], c[d]), hi[d] = std::max(hi[d], c[d]);
  }
  double side = std::max({hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]});
  side = side * (1.0 + 1e-9) + 1e-6;
  const double rdamp = std::sqrt((double)d_.damp_r2max32);
  if (!std::isfinite(rdamp)) {
    set_last_error("FMM: the Thole damping range is unbounded, the near field cannot hold every damped pair");
    return kErrInput;
  }
  // depth: leaf side >= damping range; minimise near pairs x 40 + M2L pairs
  int bestL = 0;
  double best = std::numeric_limits<double>::infinity();
  std::vector<int> leaf(n);
  for (int L = 2; L <= 7; ++L) {
    const int nl = 1 << L;
    const double h = side / nl;
    if (h < rdamp) break;
    std::vector<int> cnt((size_t)nl * nl * nl, 0);
    for (int j = 0; j < n; ++j) {
      const int x = std::min(nl - 1, (int)((px[j] - lo[0]) / h)), y = std::min(nl - 1, (int)((py[j] - lo[1]) / h)),
                z = std::min(nl - 1, (int)((pz[j] - lo[2]) / h));
      cnt[((size_t)x * nl + y) * nl + z]++;
    }
    double near = 0.0, cells = 0.0;
    for (int x = 0; x < nl; ++x)
      for (int y = 0; y < nl; ++y)
        for (int z = 0; z < nl; ++z) {
          const int c = cnt[((size_t)x * nl + y) * nl + z];
          if (!c) continue;
          cells += 1.0;
          int nb = 0;
          for (int i = std::max(0, x - 1); i <= std::min(nl - 1, x + 1); ++i)
            for (int j = std::max(0, y - 1); j <= std::min(nl - 1, y + 1); ++j)
              for (int k = std::max(0, z - 1); k <= std::min(nl - 1, z + 1); ++k) nb += cnt[((size_t)i * nl + j) * nl + k];
          near += (double)c * nb;
        }
    const double cost = 40.0 * near + 189.0 * cells * 8.0 / 7.0 * f.npairs;
    if (cost < best) {
      best = cost;
      bestL = L;
    }
  }
  if (bestL == 0) {  // fewer than four damping ranges across: the direct sums serve
    f.L = -1;
    f.built = true;
    log_msg(kVerbHigh, nullptr, "FMM: system too small for a tree with near field >= damping range; direct sums");
    return kOk;
  }
  const int L = bestL, nl = 1 << L;
  const double h = side / nl;
  f.L = L;
  f.h0 = side;
  f.ox = lo[0], f.oy = lo[1], f.oz = lo[2];
  f.off.assign(L + 2, 0);
  for (int l = 0; l <= L; ++l) f.off[l + 1] = f.off[l] + (1 << (3 * l));
  f.ncell = f.off[L + 1];
  const int nleaf = nl * nl * nl;
  std::vector<int> start(nleaf + 1, 0);
  for (int j = 0; j < n; ++j) {
    const int x = std::min(nl - 1, (int)((px[j] - lo[0]) / h)), y = std::min(nl - 1, (int)((py[j] - lo[1]) / h)),
              z = std::min(nl - 1, (int)((pz[j] - lo[2]) / h));
    leaf[j] = (x * nl + y) * nl + z;
    start[leaf[j] + 1]++;
  }
  for (int c = 0; c < nleaf; ++c) start[c + 1] += start[c];
  std::vector<int> perm(n), fill(start.begin(), start.end() - 1);
  for (int j = 0; j < n; ++j) perm[fill[leaf[j]]++] = j;
  std::vector<int> cnt(f.ncell, 0);
  for (int c = 0; c < nleaf; ++c) cnt[f.off[L] + c] = start[c + 1] - start[c];
  for (int l = L; l > 0; --l) {
    const int nc = 1 << l;
    for (int x = 0; x < nc; ++x)
      for (int y = 0; y < nc; ++y)
        for (int z = 0; z < nc; ++z) {
          const int pc = ((x >> 1) * (nc >> 1) + (y >> 1)) * (nc >> 1) + (z >> 1);
          cnt[f.off[l - 1] + pc] += cnt[f.off[l] + (x * nc + y) * nc + z];
        }
  }
  std::vector<gpu::Pos64> spos(n);
  std::vector<double> sa(n);
  std::vector<float2> swa(n);
  for (int s = 0; s < n; ++s) {
    const int j = perm[s];
    const double w = 1.0 / m_.thole[m_.polar_mm[j]];
    spos[s] = gpu::Pos64{px[j], py[j], pz[j], w};
    sa[s] = m_.damping[j];
    swa[s] = make_float2((float)(w * w), (float)(m_.damping[j] * m_.damping[j]));
  }
  auto renew = [&](auto *&ptr, size_t count) {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    return cudaMalloc((void **)&ptr, std::max<size_t>(count, 1) * sizeof(*ptr)) == cudaSuccess ? 0 : 1;
  };
  int bad = renew(f.cnt, f.ncell) | renew(f.leaf_start, nleaf + 1) | renew(f.perm, n) | renew(f.spos, n) |
            renew(f.sa, n) | renew(f.swa, n);
  if (f.nalloc_cell < f.ncell) {
    bad |= renew(f.M, 2 * (size_t)f.ncell * f.K) | renew(f.Lc, 2 * (size_t)f.ncell * f.K);
    f.nalloc_cell = f.ncell;
  }
  if (f.field_n < 6 * (size_t)n) {
    bad |= renew(f.field, 6 * (size_t)n);
    f.field_n = 6 * (size_t)n;
  }
  if (bad) {
    cudaGetLastError();
    set_last_error("out of device memory for the FMM tree");
    return kErrMemory;
  }
  cudaMemcpyAsync(f.cnt, cnt.data(), cnt.size() * sizeof(int), cudaMemcpyHostToDevice, st_);
  cudaMemcpyAsync(f.leaf_start, start.data(), start.size() * sizeof(int), cudaMemcpyHostToDevice, st_);
  cudaMemcpyAsync(f.perm, perm.data(), n * sizeof(int), cudaMemcpyHostToDevice, st_);
  cudaMemcpyAsync(f.spos, spos.data(), n * sizeof(gpu::Pos64), cudaMemcpyHostToDevice, st_);
  cudaMemcpyAsync(f.sa, sa.data(), n * sizeof(double), cudaMemcpyHostToDevice, st_);
  cudaMemcpyAsync(f.swa, swa.data(), n * sizeof(float2), cudaMemcpyHostToDevice, st_);
  int st = check(cudaStreamSynchronize(st_), "FMM tree upload");  // host vectors die here
  if (st) return st;
  log_msg(kVerbHigh, nullptr, "FMM: order %d, %d levels, leaf side %.2f bohr, %d sites", f.p, L, h, n);
  f.built = true;
  return kOk;
}

bool System::fmm_tree() const { return fmm_ && fmm_->built && fmm_->L >= 0; }

int System::fmm_tmu(int ncol, const double *x, double *y, bool dodiag) {
  int st = fmm_prepare();
  if (st) return st;
  FmmState &f = *fmm_;
  if (f.L < 0) {
    set_last_error("FMM: no tree for this system");
    return kErrInput;
  }
  const int n = d_.n;
  const size_t nv = 3 * (size_t)n;
  gpu::FmmArgs a{};
  a.p = f.p;
  a.K = f.K;
  a.KD = f.KD;
  a.L = f.L;
  a.ncell = f.ncell;
  a.h0 = f.h0;
  a.ox = f.ox, a.oy = f.oy, a.oz = f.oz;
  a.cnt = f.cnt;
  a.leaf_start = f.leaf_start;
  a.perm = f.perm;
  a.spos = f.spos;
  a.sa = f.sa;
  a.swa = f.swa;
  a.terms = f.terms;
  a.pairs = f.pairs;
  a.hoff = f.hoff;
  a.dunit = f.dunit;
  a.M = f.M;
  a.Lc = f.Lc;
  a.mm_e = f.mm_e;
  a.ll_e = f.ll_e;
  a.mm_c = f.mm_c;
  a.ll_c = f.ll_c;
  a.mm_off = f.mm_off;
  a.ll_off = f.ll_off;
  const float thr2m = (float)(d_.damp_thr * d_.damp_thr * (1.0 + 1e-5));
  const size_t smem = (f.K + (size_t)f.npairs) * sizeof(double);
  for (int c0 = 0; c0 < ncol; c0 += 2) {
    const int g = std::min(2, ncol - c0);
    a.ncol = g;
    const double *xg = x + c0 * nv;
    cudaMemsetAsync(f.M, 0, 2 * (size_t)f.ncell * f.K * sizeof(double), st_);
    cudaMemsetAsync(f.Lc, 0, 2 * (size_t)f.ncell * f.K * sizeof(double), st_);
    const int nleaf = 1 << (3 * f.L);
    gpu::k_fmm_p2m<<<dim3(nleaf, g), gpu::FT, 0, st_>>>(a, xg, n);
    for (int l = f.L; l >= 1; --l) gpu::k_fmm_m2m<<<dim3(1 << (3 * (l - 1)), g), gpu::FT, 0, st_>>>(a, l);
    if (f.npairs <= gpu::kRegPairs * gpu::FT) {
      const size_t smem_reg = (2 * (size_t)f.K + f.KD + f.npairs) * sizeof(double);
      for (int l = 2; l <= f.L; ++l) gpu::k_fmm_m2l_reg<<<dim3(1 << (3 * l), 1), gpu::FT, smem_reg, st_>>>(a, l);
    } else {
      for (int l = 2; l <= f.L; ++l) gpu::k_fmm_m2l<<<dim3(1 << (3 * l), g), gpu::FT, smem, st_>>>(a, l);
    }
    for (int l = 2; l < f.L; ++l) gpu::k_fmm_l2l<<<dim3(1 << (3 * (l + 1)), g), gpu::FT, 0, st_>>>(a, l);
    if (m_.amoeba)
      gpu::k_fmm_l2p<true><<<dim3(nleaf, g), gpu::FT, 0, st_>>>(a, xg, n, d_.damp_thr, thr2m, f.field);
    else
      gpu::k_fmm_l2p<false><<<dim3(nleaf, g), gpu::FT, 0, st_>>>(a, xg, n, d_.damp_thr, thr2m, f.field);
    gpu::add_launch_count(2 + f.L + (f.L - 1) + std::max(0, f.L - 2));
    gpu::launch_tmu_finish64(d_, g, f.field, xg, dodiag, y + c0 * nv, st_);
  }
  return check(cudaGetLastError(), "FMM T.mu launch");
}

}  // namespace ommp
