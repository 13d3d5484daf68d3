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
#include <atomic>
#include <cmath>
#include <cstring>
#include <limits>
#include <vector>

#include "engine.h"
#include "fmm_math.cuh"
#include "log.h"
#include "pair_math.cuh"

namespace ommp {

// one octree: its sources and targets sorted by leaf (for T.mu both are the
// polarizable sites and share the arrays)
struct FmmTree {
  int L = -1, ncell = 0, nalloc_cell = 0;
  double h0 = 0.0, ox = 0.0, oy = 0.0, oz = 0.0;
  std::vector<int> off;        // first cell of each level
  bool built = false;
  int *cnt = nullptr, *cnt_t = nullptr;                // sources / targets per cell, every level
  int *leaf_start = nullptr, *leaf_start_t = nullptr;  // [nleaf + 1]
  int *perm = nullptr, *perm_t = nullptr;              // sorted -> site index
  gpu::Pos64 *spos = nullptr, *spos_t = nullptr;       // w = 1/thole (inf without Thole factor)
  double *sa = nullptr, *sa_t = nullptr;               // Thole damping a
  float2 *swa = nullptr, *swa_t = nullptr;             // FP32 damping pre-test data
  double *sq = nullptr;                                // sorted multipoles [n][ld] (M2D sources)
  int *tmm = nullptr;                                  // targets' static index (M2D self pair)
  double *M = nullptr, *Lc = nullptr;                  // [2][ncell][K]
  float *M32 = nullptr;  // M scaled to the cell size, FP32 (the M2L input), after M in its block
  bool shared = false;                                 // targets are the sources
};

struct FmmState {
  int p = 0, K = 0, KD = 0, npairs = 0;
  short4 *terms = nullptr;     // exponents (a, b, c) and order of each term
  int4 *pairs = nullptr;       // M2L pairs: g, index of g + h in the derivative table, h, (-1)^|g|
  int *hoff = nullptr;         // [K + 1] first pair of each target term h
  double *dunit = nullptr;     // [343][KD] derivatives of 1/r to order p at unit cell offsets
  float *dunit32 = nullptr;    // the same in FP32 (the FP32 M2L)
  // translation lists (M2M, L2L), grouped by target term: source term and
  // packed |m| (bits 0-7) with the parities of m (bits 8-10), coefficient
  int2 *mm_e = nullptr, *ll_e = nullptr;
  double *mm_c = nullptr, *ll_c = nullptr;
  int *mm_off = nullptr, *ll_off = nullptr;
  FmmTree d2d, m2d;            // polarizable sites; static sources with polarizable targets
  double *field = nullptr;     // [2][n][3]
  size_t field_n = 0;
  bool built = false;          // d2d tree for the current geometry
};

void free_tree(FmmTree &t) {
  void *b[] = {t.cnt, t.leaf_start, t.perm, t.spos, t.sa, t.swa, t.sq, t.M, t.Lc};
  for (void *p : b)
    if (p) cudaFree(p);
  if (!t.shared) {
    void *c[] = {t.cnt_t, t.leaf_start_t, t.perm_t, t.spos_t, t.sa_t, t.swa_t, t.tmm};
    for (void *p : c)
      if (p) cudaFree(p);
  } else if (t.tmm) {
    cudaFree(t.tmm);
  }
  t = FmmTree();
}

void free_fmm_state(FmmState *f) {
  if (!f) return;
  void *b[] = {f->terms, f->pairs, f->hoff, f->dunit, f->dunit32, f->field, f->mm_e, f->ll_e, f->mm_c, f->ll_c, f->mm_off,
               f->ll_off};
  for (void *p : b)
    if (p) cudaFree(p);
  free_tree(f->d2d);
  free_tree(f->m2d);
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
  const int *cnt_t;  // targets per cell (M2L / L2L skip cells without targets)
  const Pos64 *spos;
  const double *sa;
  const float2 *swa;
  const short4 *terms;
  const int4 *pairs;
  const int *hoff;
  const double *dunit;
  const float *dunit32;
  double *M, *Lc;
  float *M32;
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
  if (a.cnt_t[level_off(l) + tc] == 0) return;
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

// The FP32 M2L input: the multipoles of the cells of levels 2..L scaled to
// the cell size, M_g h^-|g| (h the level's cell side), in FP32; one thread
// per (column, cell, term)
__global__ void k_fmm_m32(FmmArgs a, int first_cell, int ncells) {
  const size_t total = (size_t)a.ncol * ncells * a.K;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int g = (int)(i % a.K);
    const size_t cc = i / a.K;
    const int col = (int)(cc / ncells);
    const int c = first_cell + (int)(cc % ncells);
    int l = 0;
    while (l < a.L && level_off(l + 1) <= c) ++l;
    const double hinv = (1 << l) / a.h0;
    double f = 1.0;
    for (int r = 0; r < a.terms[g].w; ++r) f *= hinv;
    const size_t o = ((size_t)col * a.ncell + c) * a.K + g;
    a.M32[o] = (float)(a.M[o] * f);
  }
}

// the unit-offset derivative table of the arithmetic type
template <typename T>
__device__ __forceinline__ const T *tables(const FmmArgs &a);
template <>
__device__ __forceinline__ const double *tables<double>(const FmmArgs &a) {
  return a.dunit;
}
template <>
__device__ __forceinline__ const float *tables<float>(const FmmArgs &a) {
  return a.dunit32;
}

// The same M2L with the (target term, source term) pairs of each thread
// held in registers (PJ pairs per thread of NT), both columns in one CTA
// sharing the derivative row staged in shared memory.
// instantiations: 256 threads x 12 pairs (orders <= 8), 512 x 16 (<= 10).
// T = float: the multipoles (scaled to the cell size), the unit-offset
// derivatives and the pair sums in FP32, the sum over source terms of each
// local term and the local expansion in FP64.  The FP32 rounding (~1e-6
// of a local coefficient) is far below the expansion's own truncation
// error (~1e-4 at order 10), and GB300 issues FP32 at 64x its FP64 rate.
template <typename T, int NT, int PJ>
__global__ void __launch_bounds__(NT) k_fmm_m2l_reg(FmmArgs a, int l) {
  extern __shared__ __align__(16) unsigned char sh_raw[];
  T *sh = reinterpret_cast<T *>(sh_raw);
  T *s_m = sh;                // [2][K]
  T *s_d = sh + 2 * a.K;      // [KD]
  T *s_acc = s_d + a.KD;      // [npairs]
  const T *dunit = tables<T>(a);
  const int npairs = a.hoff[a.K];
  const int tc = blockIdx.x;
  if (a.cnt_t[level_off(l) + tc] == 0) return;
  int tx, ty, tz;
  cell_xyz(tc, l, tx, ty, tz);
  const int n = 1 << l;
  const double hinv = (1 << l) / a.h0;
  int pk[PJ];
  T acc0[PJ], acc1[PJ];
#pragma unroll
  for (int j = 0; j < PJ; ++j) {
    const int q = threadIdx.x + j * NT;
    pk[j] = -1;
    if (q < npairs) {
      const int4 pr = a.pairs[q];
      pk[j] = pr.x | (pr.y << 10) | (pr.w << 20);
    }
    acc0[j] = acc1[j] = T(0);
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
          for (int i = threadIdx.x; i < a.ncol * a.K; i += NT) {
            const int col = i / a.K, g = i - col * a.K;
            if constexpr (std::is_same<T, float>::value) {
              s_m[i] = a.M32[((size_t)col * a.ncell + level_off(l) + sc) * a.K + g];  // k_fmm_m32
            } else {
              const int ng = a.terms[g].w;
              double f = 1.0;
              for (int r = 0; r < ng; ++r) f *= hinv;
              s_m[i] = a.M[((size_t)col * a.ncell + level_off(l) + sc) * a.K + g] * f;
            }
          }
          const T *D = dunit + (size_t)(((dx + 3) * 7 + (dy + 3)) * 7 + (dz + 3)) * a.KD;
          for (int i = threadIdx.x; i < a.KD; i += NT) s_d[i] = D[i];
          __syncthreads();
#pragma unroll
          for (int j = 0; j < PJ; ++j) {
            if (pk[j] < 0) continue;
            const int g = pk[j] & 1023;
            const T d = (pk[j] >> 20) ? -s_d[(pk[j] >> 10) & 1023] : s_d[(pk[j] >> 10) & 1023];
            acc0[j] += s_m[g] * d;
            acc1[j] += s_m[a.K + g] * d;
          }
        }
      }
  for (int col = 0; col < a.ncol; ++col) {
    __syncthreads();
#pragma unroll
    for (int j = 0; j < PJ; ++j) {
      const int q = threadIdx.x + j * NT;
      if (q < npairs) s_acc[q] = col ? acc1[j] : acc0[j];
    }
    __syncthreads();
    double *Lt = a.Lc + ((size_t)col * a.ncell + level_off(l) + tc) * a.K;
    for (int hh = threadIdx.x; hh < a.K; hh += NT) {
      double s = 0.0;
      for (int q = a.hoff[hh]; q < a.hoff[hh + 1]; ++q) s += (double)s_acc[q];
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
  if (a.cnt_t[level_off(l + 1) + cc] == 0) return;
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
    // near field 3 sum f d - sum k3 mu (f = k5 mu.d) as its two sums
    double nf[3] = {0.0, 0.0, 0.0}, nk[3] = {0.0, 0.0, 0.0};
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
              if (coincident(r2)) continue;
              double k3, k5;
              dd_pair_f64<AMOEBA>(r2, pt.w, ps.w, at, s_a[q], wat, s_wa[q], thr, thr2m, k3, k5);
              const double *mu = &s_mu[q * 3];
              const double f = k5 * (mu[0] * dx + mu[1] * dy + mu[2] * dz);
              nf[0] = fma(f, dx, nf[0]);
              nf[1] = fma(f, dy, nf[1]);
              nf[2] = fma(f, dz, nf[2]);
              nk[0] = fma(k3, mu[0], nk[0]);
              nk[1] = fma(k3, mu[1], nk[1]);
              nk[2] = fma(k3, mu[2], nk[2]);
            }
          }
        }
    if (valid) {
      for (int d = 0; d < 3; ++d) e[d] += fma(3.0, nf[d], -nk[d]);
      const int pi = a.perm[si];
      for (int d = 0; d < 3; ++d) field[((size_t)col * n + pi) * 3 + d] = e[d];
    }
  }
}

// leaf multipoles of the static multipoles (charge; dipole and quadrupole
// for AMOEBA, the potential of a quadrupole being sum_kl Q_kl d_k d_l (1/r)
// of its traceless part); one column
template <bool AMOEBA>
__global__ void __launch_bounds__(FT) k_fmm_p2m_mp(FmmArgs a, const double *__restrict__ sq) {
  constexpr int LD = AMOEBA ? 10 : 1;
  __shared__ double s_p[3][fmm::kMaxOrder + 1][FCH];
  __shared__ double s_q[LD][FCH];
  const int c = blockIdx.x;
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
      const double v[3] = {ps.x - ctr[0], ps.y - ctr[1], ps.z - ctr[2]};
      for (int d = 0; d < 3; ++d) {
        double pw = 1.0;
        s_p[d][0][k] = 1.0;
        for (int m = 1; m <= a.p; ++m) {
          pw = pw * v[d] / m;
          s_p[d][m][k] = pw;
        }
      }
      for (int d = 0; d < LD; ++d) s_q[d][k] = sq[(size_t)(b0 + k) * LD + d];
      if (AMOEBA) {  // traceless part of the quadrupole
        const double t3 = (s_q[4][k] + s_q[6][k] + s_q[9][k]) / 3.0;
        s_q[4][k] -= t3;
        s_q[6][k] -= t3;
        s_q[9][k] -= t3;
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
        auto P = [&](int d, int m) { return s_p[d][m][q]; };
        w += s_q[0][q] * P(0, e.x) * P(1, e.y) * P(2, e.z);
        if (AMOEBA) {
          if (e.x) w += s_q[1][q] * P(0, e.x - 1) * P(1, e.y) * P(2, e.z);
          if (e.y) w += s_q[2][q] * P(0, e.x) * P(1, e.y - 1) * P(2, e.z);
          if (e.z) w += s_q[3][q] * P(0, e.x) * P(1, e.y) * P(2, e.z - 1);
          // sum_kl Q_kl v^(g - e_k - e_l) / (g - e_k - e_l)!; Q stored xx xy yy xz yz zz
          if (e.x >= 2) w += s_q[4][q] * P(0, e.x - 2) * P(1, e.y) * P(2, e.z);
          if (e.y >= 2) w += s_q[6][q] * P(0, e.x) * P(1, e.y - 2) * P(2, e.z);
          if (e.z >= 2) w += s_q[9][q] * P(0, e.x) * P(1, e.y) * P(2, e.z - 2);
          if (e.x && e.y) w += 2.0 * s_q[5][q] * P(0, e.x - 1) * P(1, e.y - 1) * P(2, e.z);
          if (e.x && e.z) w += 2.0 * s_q[7][q] * P(0, e.x - 1) * P(1, e.y) * P(2, e.z - 1);
          if (e.y && e.z) w += 2.0 * s_q[8][q] * P(0, e.x) * P(1, e.y - 1) * P(2, e.z - 1);
        }
      }
      acc[j] += w;
    }
  }
  double *Mc = a.M + ((size_t)level_off(a.L) + c) * a.K;
  for (int j = 0; j < kMaxTermsPerThread; ++j) {
    const int t = threadIdx.x + j * FT;
    if (t < a.K) Mc[t] = acc[j];
  }
}

// far field of the leaf's local expansion plus the direct damped near field
// of the static multipoles in the 27 neighbouring leaves at each polarizable
// target of the leaf; field [n][3] at the targets' polarizable index
template <bool AMOEBA>
__global__ void __launch_bounds__(FT) k_fmm_l2p_m2d(FmmArgs a, const int *__restrict__ leaf_start_t,
                                                     const int *__restrict__ perm_t, const Pos64 *__restrict__ spos_t,
                                                     const double *__restrict__ sa_t, const float2 *__restrict__ swa_t,
                                                     const int *__restrict__ tmm, const double *__restrict__ sq,
                                                     double thr, float thr2m, double *__restrict__ field, int *err) {
  constexpr int LD = AMOEBA ? 10 : 1;
  __shared__ Pos64 s_pos[FT];
  __shared__ double s_a[FT];
  __shared__ float2 s_wa[FT];
  __shared__ int s_mm[FT];
  __shared__ double s_q[FT * LD];
  __shared__ double s_L[fmm::nterms(fmm::kMaxOrder)];
  const int c = blockIdx.x;
  const int s0 = leaf_start_t[c], s1 = leaf_start_t[c + 1];
  if (s0 == s1) return;
  int cx, cy, cz;
  cell_xyz(c, a.L, cx, cy, cz);
  const int nl = 1 << a.L;
  const double h = a.h0 / nl;
  const double ctr[3] = {a.ox + (cx + 0.5) * h, a.oy + (cy + 0.5) * h, a.oz + (cz + 0.5) * h};
  const double *Lt = a.Lc + ((size_t)level_off(a.L) + c) * a.K;
  for (int t = threadIdx.x; t < a.K; t += FT) s_L[t] = Lt[t];
  int bad = 0;
  for (int b0 = s0; b0 < s1; b0 += FT) {
    const int si = b0 + threadIdx.x;
    const bool valid = si < s1;
    const Pos64 pt = valid ? spos_t[si] : Pos64{0, 0, 0, 0};
    const double at = valid && AMOEBA ? sa_t[si] : 0.0;
    const float2 wat = valid ? swa_t[si] : make_float2(0.f, 0.f);
    const int self = valid ? tmm[si] : -1;
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
              s_mm[threadIdx.x] = a.perm[k];
              for (int d = 0; d < LD; ++d) s_q[threadIdx.x * LD + d] = sq[(size_t)k * LD + d];
            }
            __syncthreads();
            if (!valid) continue;
            const int cnt = min(FT, r1 - t0);
            for (int q = 0; q < cnt; ++q) {
              if (s_mm[q] == self) continue;
              const Pos64 ps = s_pos[q];
              const double dx = pt.x - ps.x, dy = pt.y - ps.y, dz = pt.z - ps.z;
              if (coincident(dx * dx + dy * dy + dz * dz)) {
                bad = 1;
                continue;
              }
              m2d_pair_f64<AMOEBA>(dx, dy, dz, pt.w, ps.w, at, s_a[q], wat, s_wa[q], &s_q[q * LD], thr, thr2m, e[0],
                                   e[1], e[2]);
            }
          }
        }
    if (valid) {
      const int pi = perm_t[si];
      for (int d = 0; d < 3; ++d) field[(size_t)pi * 3 + d] = e[d];
    }
  }
  if (bad) atomicOr(err, 1);
}

}  // namespace
}  // namespace gpu

namespace {
std::atomic<bool> g_fmm_auto{false};
}  // namespace

void set_fmm_auto(bool on) { g_fmm_auto = on; }
bool fmm_auto() { return g_fmm_auto; }

int System::set_fmm(bool on, int order) {
  int st = set_fmm_order_pol(order);
  if (st) return st;
  st = set_fmm_order_static(order);
  if (st) return st;
  fmm_on_ = on;
  return kOk;
}

int System::set_fmm_order_pol(int order) {
  if (order < 2 || order > fmm::kMaxOrder) {
    set_last_error("FMM expansion order must be between 2 and 12");
    return kErrBadArg;
  }
  if (fmm_ && fmm_->p != order) {
    free_fmm_state(fmm_);
    fmm_ = nullptr;
  }
  fmm_order_ = order;
  return kOk;
}

void System::fmm_drop_static() {
  if (fmms_) fmms_->m2d.built = false;
  if (m2d_method_ == kM2dFMM) m2d_done_ = false;  // a field of the old settings
}

int System::set_fmm_order_static(int order) {
  if (order < 2 || order > fmm::kMaxOrder) {
    set_last_error("FMM expansion order must be between 2 and 12");
    return kErrBadArg;
  }
  if (order == fmm_order_static_) return kOk;
  if (fmms_) {
    free_fmm_state(fmms_);
    fmms_ = nullptr;
  }
  fmm_order_static_ = order;
  fmm_drop_static();
  return kOk;
}

// The reference treats two leaf cells as near when the gap between them is
// below fmm_distance and stops subdividing a cell whose half diagonal is below
// fmm_min_cell_size (src/fast_multipoles/mod_tree.F90:177,
// mod_octatree.F90:98).  Here the near field is the 27 neighbouring leaves of
// a uniform octree, so cells farther apart are separated by at least one leaf
// side: both settings become lower bounds of that side (the min cell size as
// a half diagonal, side = 2 d / sqrt 3), beside the damping range.
double System::fmm_min_leaf() const { return std::max(fmm_dfar_, 2.0 * fmm_mincell_ / std::sqrt(3.0)); }

int System::set_fmm_distance(double d) {
  if (!(d >= 0.0) || !std::isfinite(d)) {
    set_last_error("FMM distance must be a finite non-negative length (bohr)");
    return kErrBadArg;
  }
  fmm_dfar_ = d;
  fmm_invalidate();
  fmm_drop_static();
  return kOk;
}

int System::set_fmm_min_cell_size(double d) {
  if (!(d >= 0.0) || !std::isfinite(d)) {
    set_last_error("FMM minimum cell size must be a finite non-negative length (bohr)");
    return kErrBadArg;
  }
  fmm_mincell_ = d;
  fmm_invalidate();
  fmm_drop_static();
  return kOk;
}

void System::fmm_invalidate() {
  if (fmm_) {
    fmm_->built = false;
    fmm_->d2d.built = false;
  }
  if (fmms_) fmms_->m2d.built = false;
}

namespace {

// per-order tables: terms, M2L pairs sorted by target term, unit-offset
// derivative tensors, M2M / L2L translation lists
int build_tables(FmmState &f, int p, cudaStream_t st) {
  f.p = p;
  f.K = fmm::nterms(p);
  f.KD = fmm::nterms(p);  // |g| + |h| <= p: derivatives to order p
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
    for (int g = 0; g < fmm::nterms(p - nh); ++g)
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
        fmm::derivatives(i, j, k, p, &dunit[(size_t)(((i + 3) * 7 + (j + 3)) * 7 + (k + 3)) * f.KD]);
      }
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
      ll_c.push_back(fact(q.x) * fact(q.y) * fact(q.z) / (fact(e.x) * fact(e.y) * fact(e.z) * fact(mx) * fact(my) * fact(mz)));
    }
  }
  mm_off[f.K] = (int)mm_e.size();
  ll_off[f.K] = (int)ll_e.size();
  auto up = [&](auto *&dst, const auto &v) {
    if (cudaMalloc((void **)&dst, std::max<size_t>(v.size(), 1) * sizeof(v[0])) != cudaSuccess) return 1;
    cudaMemcpyAsync(dst, v.data(), v.size() * sizeof(v[0]), cudaMemcpyHostToDevice, st);
    return 0;
  };
  std::vector<float> dunit32(dunit.begin(), dunit.end());
  int bad = up(f.terms, terms) | up(f.pairs, pairs) | up(f.hoff, hoff) | up(f.dunit, dunit) |
            up(f.dunit32, dunit32) | up(f.mm_e, mm_e) |
            up(f.ll_e, ll_e) | up(f.mm_c, mm_c) | up(f.ll_c, ll_c) | up(f.mm_off, mm_off) | up(f.ll_off, ll_off);
  if (bad) {
    cudaGetLastError();
    set_last_error("out of device memory for the FMM tables");
    return kErrMemory;
  }
  const size_t smem = (f.K + (size_t)f.npairs) * sizeof(double);
  if (smem > 48 * 1024) cudaFuncSetAttribute(gpu::k_fmm_m2l, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  const size_t smem_reg = (2 * (size_t)f.K + f.KD + f.npairs) * sizeof(float);
  if (smem_reg > 48 * 1024) {
    cudaFuncSetAttribute(gpu::k_fmm_m2l_reg<float, 256, 12>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem_reg);
    cudaFuncSetAttribute(gpu::k_fmm_m2l_reg<float, 512, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem_reg);
  }
  return cudaStreamSynchronize(st) == cudaSuccess ? kOk : kErrCuda;  // host vectors die here
}

// geometry of one tree: sources xs [ns][3] and targets xt [nt][3] (targets
// the sources when xt is null) sorted by leaf, leaf side >= rdamp, depth
// minimising near pairs x 40 + M2L term pairs
struct TreeLayout {
  int L = -1, ncell = 0;
  double side = 0.0, lo[3] = {0, 0, 0};
  std::vector<int> off, start_s, perm_s, start_t, perm_t, cnt_s, cnt_t;
};

bool plan_tree(int ns, const double *xs, int nt, const double *xt, double rdamp, int npairs, TreeLayout &o) {
  const bool same = xt == nullptr;
  if (same) {
    xt = xs;
    nt = ns;
  }
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int pass = 0; pass < 2; ++pass) {
    const double *x = pass ? xt : xs;
    const int m = pass ? nt : ns;
    for (int j = 0; j < m; ++j)
      for (int d = 0; d < 3; ++d) lo[d] = std::min(lo[d], x[3 * (size_t)j + d]), hi[d] = std::max(hi[d], x[3 * (size_t)j + d]);
  }
  double side = std::max({hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]});
  side = side * (1.0 + 1e-9) + 1e-6;
  if (!std::isfinite(rdamp)) return false;
  auto leaf_of = [&](const double *c, int nl, double h) {
    const int x = std::min(nl - 1, (int)((c[0] - lo[0]) / h)), y = std::min(nl - 1, (int)((c[1] - lo[1]) / h)),
              z = std::min(nl - 1, (int)((c[2] - lo[2]) / h));
    return (x * nl + y) * nl + z;
  };
  int bestL = 0;
  double best = std::numeric_limits<double>::infinity();
  for (int L = 2; L <= 7; ++L) {
    const int nl = 1 << L;
    const double h = side / nl;
    if (h < rdamp) break;
    std::vector<int> cs((size_t)nl * nl * nl, 0), ct((size_t)nl * nl * nl, 0);
    for (int j = 0; j < ns; ++j) cs[leaf_of(&xs[3 * (size_t)j], nl, h)]++;
    for (int j = 0; j < nt; ++j) ct[leaf_of(&xt[3 * (size_t)j], nl, h)]++;
    double near = 0.0, cells = 0.0;
    for (int x = 0; x < nl; ++x)
      for (int y = 0; y < nl; ++y)
        for (int z = 0; z < nl; ++z) {
          const int c = ct[((size_t)x * nl + y) * nl + z];
          if (!c) continue;
          cells += 1.0;
          int nb = 0;
          for (int i = std::max(0, x - 1); i <= std::min(nl - 1, x + 1); ++i)
            for (int j = std::max(0, y - 1); j <= std::min(nl - 1, y + 1); ++j)
              for (int k = std::max(0, z - 1); k <= std::min(nl - 1, z + 1); ++k) nb += cs[((size_t)i * nl + j) * nl + k];
          near += (double)c * nb;
        }
    const double cost = 40.0 * near + 189.0 * cells * 8.0 / 7.0 * npairs;
    if (cost < best) {
      best = cost;
      bestL = L;
    }
  }
  if (bestL == 0) return false;
  const int L = bestL, nl = 1 << L, nleaf = nl * nl * nl;
  const double h = side / nl;
  o.L = L;
  o.side = side;
  for (int d = 0; d < 3; ++d) o.lo[d] = lo[d];
  o.off.assign(L + 2, 0);
  for (int l = 0; l <= L; ++l) o.off[l + 1] = o.off[l] + (1 << (3 * l));
  o.ncell = o.off[L + 1];
  auto sort = [&](int m, const double *x, std::vector<int> &start, std::vector<int> &perm, std::vector<int> &cnt) {
    std::vector<int> leaf(m);
    start.assign(nleaf + 1, 0);
    for (int j = 0; j < m; ++j) {
      leaf[j] = leaf_of(&x[3 * (size_t)j], nl, h);
      start[leaf[j] + 1]++;
    }
    for (int c = 0; c < nleaf; ++c) start[c + 1] += start[c];
    perm.resize(m);
    std::vector<int> fill(start.begin(), start.end() - 1);
    for (int j = 0; j < m; ++j) perm[fill[leaf[j]]++] = j;
    cnt.assign(o.ncell, 0);
    for (int c = 0; c < nleaf; ++c) cnt[o.off[L] + c] = start[c + 1] - start[c];
    for (int l = L; l > 0; --l) {
      const int nc = 1 << l;
      for (int x = 0; x < nc; ++x)
        for (int y = 0; y < nc; ++y)
          for (int z = 0; z < nc; ++z)
            cnt[o.off[l - 1] + ((x >> 1) * (nc >> 1) + (y >> 1)) * (nc >> 1) + (z >> 1)] +=
                cnt[o.off[l] + (x * nc + y) * nc + z];
    }
  };
  sort(ns, xs, o.start_s, o.perm_s, o.cnt_s);
  if (!same) sort(nt, xt, o.start_t, o.perm_t, o.cnt_t);
  return true;
}

template <typename T>
int upload(T *&dst, const std::vector<T> &v, cudaStream_t st) {
  if (dst) cudaFree(dst);
  dst = nullptr;
  if (cudaMalloc((void **)&dst, std::max<size_t>(v.size(), 1) * sizeof(T)) != cudaSuccess) return 1;
  if (!v.empty()) cudaMemcpyAsync(dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st);
  return 0;
}

void tree_args(const FmmState &f, const FmmTree &t, int ncol, gpu::FmmArgs &a) {
  a = gpu::FmmArgs{};
  a.p = f.p;
  a.K = f.K;
  a.KD = f.KD;
  a.L = t.L;
  a.ncell = t.ncell;
  a.ncol = ncol;
  a.h0 = t.h0;
  a.ox = t.ox, a.oy = t.oy, a.oz = t.oz;
  a.cnt = t.cnt;
  a.cnt_t = t.cnt_t;
  a.leaf_start = t.leaf_start;
  a.perm = t.perm;
  a.spos = t.spos;
  a.sa = t.sa;
  a.swa = t.swa;
  a.terms = f.terms;
  a.pairs = f.pairs;
  a.hoff = f.hoff;
  a.dunit = f.dunit;
  a.dunit32 = f.dunit32;
  a.M = t.M;
  a.M32 = t.M32;
  a.Lc = t.Lc;
  a.mm_e = f.mm_e;
  a.ll_e = f.ll_e;
  a.mm_c = f.mm_c;
  a.ll_c = f.ll_c;
  a.mm_off = f.mm_off;
  a.ll_off = f.ll_off;
}

// upward pass from the leaf multipoles, M2L, downward pass (columns of a)
void run_tree(const FmmState &f, const FmmTree &t, const gpu::FmmArgs &a, int ncol, cudaStream_t st) {
  const size_t smem = (f.K + (size_t)f.npairs) * sizeof(double);
  for (int l = t.L; l >= 1; --l) gpu::k_fmm_m2m<<<dim3(1 << (3 * (l - 1)), ncol), gpu::FT, 0, st>>>(a, l);
  const size_t smem_reg = (2 * (size_t)f.K + f.KD + f.npairs) * sizeof(float);
  const bool reg = f.npairs <= 16 * 512;
  if (reg && t.L >= 2) {
    const int c0 = ((1 << 6) - 1) / 7, nc = t.ncell - c0;  // the cells of levels 2..L
    gpu::k_fmm_m32<<<gpu::sm_count() * 8, 256, 0, st>>>(a, c0, nc);
    gpu::add_launch_count(1);
  }
  if (f.npairs <= 12 * 256) {
    for (int l = 2; l <= t.L; ++l)
      gpu::k_fmm_m2l_reg<float, 256, 12><<<dim3(1 << (3 * l), 1), 256, smem_reg, st>>>(a, l);
  } else if (f.npairs <= 16 * 512) {
    for (int l = 2; l <= t.L; ++l)
      gpu::k_fmm_m2l_reg<float, 512, 16><<<dim3(1 << (3 * l), 1), 512, smem_reg, st>>>(a, l);
  } else {
    for (int l = 2; l <= t.L; ++l) gpu::k_fmm_m2l<<<dim3(1 << (3 * l), ncol), gpu::FT, smem, st>>>(a, l);
  }
  for (int l = 2; l < t.L; ++l) gpu::k_fmm_l2l<<<dim3(1 << (3 * (l + 1)), ncol), gpu::FT, 0, st>>>(a, l);
  gpu::add_launch_count(t.L + (t.L - 1) + std::max(0, t.L - 2));
}

}  // namespace

bool System::fmm_tree() const { return fmm_ && fmm_->built && fmm_->d2d.L >= 0; }

int System::fmm_prepare() {
  if (fmm_ && fmm_->built) return kOk;
  if (!fmm_) {
    fmm_ = new FmmState();
    int st = build_tables(*fmm_, fmm_order_, st_);
    if (st) {
      free_fmm_state(fmm_);
      fmm_ = nullptr;
      return st == kErrCuda ? check(cudaGetLastError(), "FMM tables") : st;
    }
  }
  FmmState &f = *fmm_;
  FmmTree &t = f.d2d;
  const int n = d_.n;
  std::vector<double> xp(3 * (size_t)n);
  for (int j = 0; j < n; ++j)
    for (int d = 0; d < 3; ++d) xp[3 * (size_t)j + d] = m_.cmm[3 * (size_t)m_.polar_mm[j] + d];
  TreeLayout o;
  if (!plan_tree(n, xp.data(), 0, nullptr, std::max((double)std::sqrt(d_.damp_r2max32), fmm_min_leaf()), f.npairs,
                 o)) {
    t.L = -1;  // fewer than four damping ranges across: the direct sums serve
    f.built = true;
    log_msg(kVerbHigh, nullptr, "FMM: system too small for a tree with near field >= damping range; direct sums");
    return kOk;
  }
  std::vector<gpu::Pos64> spos(n);
  std::vector<double> sa(n);
  std::vector<float2> swa(n);
  for (int s = 0; s < n; ++s) {
    const int j = o.perm_s[s];
    const double w = 1.0 / m_.thole[m_.polar_mm[j]];
    spos[s] = gpu::Pos64{xp[3 * (size_t)j], xp[3 * (size_t)j + 1], xp[3 * (size_t)j + 2], w};
    sa[s] = m_.damping[j];
    swa[s] = make_float2((float)(w * w), (float)(m_.damping[j] * m_.damping[j]));
  }
  t.L = o.L;
  t.h0 = o.side;
  t.ox = o.lo[0], t.oy = o.lo[1], t.oz = o.lo[2];
  t.off = o.off;
  t.ncell = o.ncell;
  t.shared = true;
  int bad = upload(t.cnt, o.cnt_s, st_) | upload(t.leaf_start, o.start_s, st_) | upload(t.perm, o.perm_s, st_) |
            upload(t.spos, spos, st_) | upload(t.sa, sa, st_) | upload(t.swa, swa, st_);
  t.cnt_t = t.cnt, t.leaf_start_t = t.leaf_start, t.perm_t = t.perm, t.spos_t = t.spos, t.sa_t = t.sa, t.swa_t = t.swa;
  if (t.nalloc_cell < t.ncell) {
    if (t.M) cudaFree(t.M);
    if (t.Lc) cudaFree(t.Lc);
    t.M = t.Lc = nullptr;
    bad |= cudaMalloc((void **)&t.M, 2 * (size_t)t.ncell * f.K * (sizeof(double) + sizeof(float))) != cudaSuccess;
    bad |= cudaMalloc((void **)&t.Lc, 2 * (size_t)t.ncell * f.K * sizeof(double)) != cudaSuccess;
    t.M32 = t.M ? reinterpret_cast<float *>(t.M + 2 * (size_t)t.ncell * f.K) : nullptr;
    t.nalloc_cell = t.ncell;
  }
  if (f.field_n < 6 * (size_t)n) {
    if (f.field) cudaFree(f.field);
    f.field = nullptr;
    bad |= cudaMalloc((void **)&f.field, 6 * (size_t)n * sizeof(double)) != cudaSuccess;
    f.field_n = 6 * (size_t)n;
  }
  if (bad) {
    cudaGetLastError();
    t.nalloc_cell = 0;
    set_last_error("out of device memory for the FMM tree");
    return kErrMemory;
  }
  int st = check(cudaStreamSynchronize(st_), "FMM tree upload");  // host vectors die here
  if (st) return st;
  log_msg(kVerbHigh, nullptr, "FMM: order %d, %d levels, leaf side %.2f bohr, %d sites", f.p, t.L, t.h0 / (1 << t.L),
          n);
  t.built = true;
  f.built = true;
  return kOk;
}

int System::fmm_tmu(int ncol, const double *x, double *y, bool dodiag) {
  int st = fmm_prepare();
  if (st) return st;
  FmmState &f = *fmm_;
  FmmTree &t = f.d2d;
  if (t.L < 0) {
    set_last_error("FMM: no tree for this system");
    return kErrInput;
  }
  const int n = d_.n;
  const size_t nv = 3 * (size_t)n;
  const float thr2m = (float)(d_.damp_thr * d_.damp_thr * (1.0 + 1e-5));
  for (int c0 = 0; c0 < ncol; c0 += 2) {
    const int g = std::min(2, ncol - c0);
    gpu::FmmArgs a;
    tree_args(f, t, g, a);
    const double *xg = x + c0 * nv;
    cudaMemsetAsync(t.M, 0, 2 * (size_t)t.ncell * f.K * sizeof(double), st_);
    cudaMemsetAsync(t.Lc, 0, 2 * (size_t)t.ncell * f.K * sizeof(double), st_);
    const int nleaf = 1 << (3 * t.L);
    gpu::k_fmm_p2m<<<dim3(nleaf, g), gpu::FT, 0, st_>>>(a, xg, n);
    run_tree(f, t, a, g, st_);
    if (m_.amoeba)
      gpu::k_fmm_l2p<true><<<dim3(nleaf, g), gpu::FT, 0, st_>>>(a, xg, n, d_.damp_thr, thr2m, f.field);
    else
      gpu::k_fmm_l2p<false><<<dim3(nleaf, g), gpu::FT, 0, st_>>>(a, xg, n, d_.damp_thr, thr2m, f.field);
    gpu::add_launch_count(2);
    gpu::launch_tmu_finish64(d_, g, f.field, xg, dodiag, y + c0 * nv, st_);
  }
  return check(cudaGetLastError(), "FMM T.mu launch");
}

// E_M2D through the FMM: the static multipoles as sources, the polarizable
// sites as targets; done = false when the system is too small for a tree
int System::fmm_m2d(double *out, bool &done) {
  done = false;
  if (!fmms_) {  // tables of the static order
    fmms_ = new FmmState();
    int st = build_tables(*fmms_, fmm_order_static_, st_);
    if (st) {
      free_fmm_state(fmms_);
      fmms_ = nullptr;
      return st == kErrCuda ? check(cudaGetLastError(), "FMM tables") : st;
    }
  }
  int st = kOk;
  FmmState &f = *fmms_;
  FmmTree &t = f.m2d;
  const int n = d_.n, mm = d_.m, ld = m_.ld_cart;
  if (f.field_n < 3 * (size_t)n) {
    if (f.field) cudaFree(f.field);
    f.field = nullptr;
    if (cudaMalloc((void **)&f.field, 3 * (size_t)n * sizeof(double)) != cudaSuccess) {
      cudaGetLastError();
      f.field_n = 0;
      set_last_error("out of device memory for the FMM field");
      return kErrMemory;
    }
    f.field_n = 3 * (size_t)n;
  }
  if (!t.built) {
    std::vector<double> xp(3 * (size_t)n);
    for (int j = 0; j < n; ++j)
      for (int d = 0; d < 3; ++d) xp[3 * (size_t)j + d] = m_.cmm[3 * (size_t)m_.polar_mm[j] + d];
    TreeLayout o;
    if (!plan_tree(mm, m_.cmm.data(), n, xp.data(), std::max((double)std::sqrt(d_.m2d_r2max32), fmm_min_leaf()),
                   f.npairs, o)) {
      t.L = -1;
      t.built = true;
      return kOk;
    }
    const double inf = std::numeric_limits<double>::infinity();
    std::vector<gpu::Pos64> spos(mm), spos_t(n);
    std::vector<double> sa(mm), sa_t(n), sq((size_t)mm * ld);
    std::vector<float2> swa(mm), swa_t(n);
    std::vector<int> tmm(n);
    for (int s = 0; s < mm; ++s) {
      const int i = o.perm_s[s];
      const double th = m_.thole[i];
      const double w = th > 0.0 ? 1.0 / th : inf;
      const int pi = m_.mm_polar[i];
      const double a = pi >= 0 ? m_.damping[pi] : 0.0;
      spos[s] = gpu::Pos64{m_.cmm[3 * (size_t)i], m_.cmm[3 * (size_t)i + 1], m_.cmm[3 * (size_t)i + 2], w};
      sa[s] = a;
      swa[s] = make_float2((float)(w * w), (float)(a * a));
      for (int c = 0; c < ld; ++c) sq[(size_t)s * ld + c] = m_.q[(size_t)i * ld + c];
    }
    for (int s = 0; s < n; ++s) {
      const int j = o.perm_t[s];
      const double w = 1.0 / m_.thole[m_.polar_mm[j]];
      spos_t[s] = gpu::Pos64{xp[3 * (size_t)j], xp[3 * (size_t)j + 1], xp[3 * (size_t)j + 2], w};
      sa_t[s] = m_.damping[j];
      swa_t[s] = make_float2((float)(w * w), (float)(m_.damping[j] * m_.damping[j]));
      tmm[s] = m_.polar_mm[j];
    }
    t.L = o.L;
    t.h0 = o.side;
    t.ox = o.lo[0], t.oy = o.lo[1], t.oz = o.lo[2];
    t.off = o.off;
    t.ncell = o.ncell;
    t.shared = false;
    int bad = upload(t.cnt, o.cnt_s, st_) | upload(t.leaf_start, o.start_s, st_) | upload(t.perm, o.perm_s, st_) |
              upload(t.spos, spos, st_) | upload(t.sa, sa, st_) | upload(t.swa, swa, st_) | upload(t.sq, sq, st_) |
              upload(t.cnt_t, o.cnt_t, st_) | upload(t.leaf_start_t, o.start_t, st_) |
              upload(t.perm_t, o.perm_t, st_) | upload(t.spos_t, spos_t, st_) | upload(t.sa_t, sa_t, st_) |
              upload(t.swa_t, swa_t, st_) | upload(t.tmm, tmm, st_);
    if (t.nalloc_cell < t.ncell) {
      if (t.M) cudaFree(t.M);
      if (t.Lc) cudaFree(t.Lc);
      t.M = t.Lc = nullptr;
      bad |= cudaMalloc((void **)&t.M, (size_t)t.ncell * f.K * (sizeof(double) + sizeof(float))) != cudaSuccess;
      bad |= cudaMalloc((void **)&t.Lc, (size_t)t.ncell * f.K * sizeof(double)) != cudaSuccess;
      t.M32 = t.M ? reinterpret_cast<float *>(t.M + (size_t)t.ncell * f.K) : nullptr;
      t.nalloc_cell = t.ncell;
    }
    if (bad) {
      cudaGetLastError();
      t.nalloc_cell = 0;
      set_last_error("out of device memory for the FMM tree of the static multipoles");
      return kErrMemory;
    }
    st = check(cudaStreamSynchronize(st_), "FMM M2D tree upload");
    if (st) return st;
    t.built = true;
  }
  if (t.L < 0) return kOk;
  gpu::FmmArgs a;
  tree_args(f, t, 1, a);
  cudaMemsetAsync(t.M, 0, (size_t)t.ncell * f.K * sizeof(double), st_);
  cudaMemsetAsync(t.Lc, 0, (size_t)t.ncell * f.K * sizeof(double), st_);
  const int nleaf = 1 << (3 * t.L);
  if (m_.amoeba)
    gpu::k_fmm_p2m_mp<true><<<nleaf, gpu::FT, 0, st_>>>(a, t.sq);
  else
    gpu::k_fmm_p2m_mp<false><<<nleaf, gpu::FT, 0, st_>>>(a, t.sq);
  run_tree(f, t, a, 1, st_);
  const float thr2m = (float)(d_.damp_thr * d_.damp_thr * (1.0 + 1e-5));
  if (m_.amoeba)
    gpu::k_fmm_l2p_m2d<true><<<nleaf, gpu::FT, 0, st_>>>(a, t.leaf_start_t, t.perm_t, t.spos_t, t.sa_t, t.swa_t, t.tmm,
                                                         t.sq, d_.damp_thr, thr2m, f.field, flag_);
  else
    gpu::k_fmm_l2p_m2d<false><<<nleaf, gpu::FT, 0, st_>>>(a, t.leaf_start_t, t.perm_t, t.spos_t, t.sa_t, t.swa_t,
                                                          t.tmm, t.sq, d_.damp_thr, thr2m, f.field, flag_);
  gpu::add_launch_count(2);
  gpu::launch_m2d_finish(d_, out, f.field, 1, st_);
  done = true;
  return check(cudaGetLastError(), "FMM M2D launch");
}

}  // namespace ommp
