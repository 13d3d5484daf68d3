// Launch interface of the GB300 kernels (implemented in kernels.cu).
//
// Layout conventions (device memory, all 0-based):
//   site arrays are structure-of-arrays or packed Pos64 (x, y, z, w);
//   field / dipole vectors are [nrhs][n][3] contiguous (C order), the same
//   as the reference's Fortran (3, n, n_ipd) arrays seen from C.
#pragma once

#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

namespace ommp {
namespace gpu {

// One site: position and a per-site scalar, 32-byte aligned so that a tile
// load is two 16-byte transactions per thread.
struct __align__(32) Pos64 {
  double x, y, z, w;
};

// Immutable per-geometry device data of one system.
struct DevSites {
  int n = 0;      // polarizable sites
  int m = 0;      // MM (static) sites
  bool amoeba = false;
  // polarizable sites
  Pos64 *pol_pos = nullptr;   // x, y, z, 1/thole
  double *pol_a = nullptr;      // Thole damping a
  double *pol_alpha = nullptr;  // polarizability
  int *polar_mm = nullptr;      // mm index of each polarizable site
  float4 *pol_pos32 = nullptr;  // centred FP32 copy: x, y, z, 1/thole
  float4 *pol_pos32lo = nullptr;  // x, y, z - pol_pos32 (double-single low parts), w = 0
  float *pol_a32 = nullptr;
  float2 *pol_wa32 = nullptr;   // (1/thole)^2, a^2 in FP32: damping pre-test of the FP64 kernels
  float2 *mm_wa32 = nullptr;    // same for the static sites (inf when not polarizable)
  // static sites
  Pos64 *mm_pos = nullptr;    // x, y, z, thole (0 when not polarizable)
  double *mm_a = nullptr;       // damping a of the source (AMOEBA)
  double *mm_q = nullptr;       // [m][ld] lab-frame multipoles
  int ld = 1;
  // scaled pairs, target-major
  int *m2d_ri = nullptr, *m2d_src = nullptr;
  double *m2d_sP = nullptr, *m2d_sD = nullptr;
  int m2d_nnz = 0;
  int *d2d_ri = nullptr, *d2d_src = nullptr;
  double *d2d_s = nullptr;
  int d2d_nnz = 0;
  double damp_thr = 50.0;       // AMOEBA: damping applied when a u^3 < 50
  // FP32 operator: per 128-site tile the bounding box of pol_pos32 (lo, hi
  // pairs, [2*ntile]) and the squared distance beyond which no pair is damped
  float4 *tile_box32 = nullptr;
  int ntile = 0;
  float damp_r2max32 = 0.f;
  // double-single E_M2D: static-site positions (hi with w = 0, lo), their
  // tile boxes and the squared distance beyond which no M2D pair is damped
  float4 *mm_pos32 = nullptr, *mm_pos32lo = nullptr, *mm_tile_box32 = nullptr;
  float m2d_r2max32 = 0.f;
};

// ---- pair kernels ---------------------------------------------------------
// Permanent-multipole field at the polarizable sites (E_M2D), n_ipd sets:
// out [n_ipd][n][3]; scratch holds split partials (m2d_scratch_doubles()).
size_t m2d_scratch_doubles(const DevSites &s, int nsplit);
int m2d_pick_split(const DevSites &s, int sm_count);
void launch_m2d(const DevSites &s, double *out, double *scratch, int nsplit, int *err_flag,
                cudaStream_t st);
// the finishing pass alone: split partials [nsplit][n][3] summed, the
// scaled-pair corrections, out [n_ipd][n][3]
void launch_m2d_finish(const DevSites &s, double *out, const double *partial, int nsplit, cudaStream_t st);

// y = T x (dodiag) or y = -E_dd(x) (no diagonal); x,y [nrhs][n][3], FP64.
size_t tmu_scratch_doubles(const DevSites &s, int nrhs, int nsplit);
int tmu_pick_split(const DevSites &s, int nrhs, int sm_count, bool fp32);
void launch_tmu_f64(const DevSites &s, int nrhs, const double *x, double *y, bool dodiag,
                    double *scratch, int nsplit, cudaStream_t st);
// The finishing pass alone on a field partial [nrhs][n][3] (one split): the
// u-scaled pair corrections, the sign and the 1/alpha diagonal
void launch_tmu_finish64(const DevSites &s, int nrhs, const double *partial, const double *x, bool dodiag,
                         double *y, cudaStream_t st);
// FP32 finishing pass (partial [nrhs][n][3], one split; diagonal included)
void launch_tmu_finish32(const DevSites &s, int nrhs, const float *partial, const float *x, float *y,
                         cudaStream_t st);
// Same product with each unordered pair evaluated once (deterministic
// half-shell schedule); scratch of tmu_sym_scratch_doubles(s, nrhs_max).
size_t tmu_sym_scratch_doubles(const DevSites &s, int nrhs);
// gmax (1, 2 or 4): the widest column group the scratch was sized for
void launch_tmu_f64_sym(const DevSites &s, int nrhs, const double *x, double *y, bool dodiag, double *scratch,
                        cudaStream_t st, int gmax = 2);
// FP32 inner operator with compensated cross-tile sums; x,y float.  Columns
// go through the pair kernel in groups of up to gmax (8, 4, 2 or 1) sharing
// the pair geometry; scratch holds nsplit * nrhs * n * 3 floats.
// kver 1: one target per thread, per-pair damping test (kernels.cu);
// kver 2: the tile-classified kernel of tmu32.cu.
// kver 3: the symmetric kernel of tmu32.cu (each unordered pair once),
// columns in groups of gmax (1 or 2), sums in sym_scratch (laid out as for
// launch_tmu_f64_sym, tmu_sym_scratch_doubles(s, 2)); scratch unused.
void launch_tmu_f32(const DevSites &s, int nrhs, const float *x, float *y, float *scratch,
                    int nsplit, cudaStream_t st, int gmax = 4, int kver = 2, double *sym_scratch = nullptr);
// symmetric FP32 pair sums of g (1 or 2) columns into the fixed-point
// accumulators lo / hi [g][n][3] (zeroed here), read out into out [g][n][3]
void launch_tmu32_sym_pairs(const DevSites &s, int g, const float *x, unsigned long long *lo,
                            unsigned long long *hi, unsigned long long *bad, unsigned *next, float *out,
                            cudaStream_t st);
int tmu32_sym_resident(int g, bool amoeba);

// ---- multi-system symmetric products --------------------------------------
// One system's share of a launch that serves several systems (the products
// of uneven systems in one persistent kernel): the items [item0, item0 +
// count) of its product, whose item space (super-tile, chunk of slots) is
// fixed per system and product kind (*_sym_items), so that a product may be
// spread over several launches; its fixed-point accumulators [g][n][3] and
// error flag are zeroed by the caller before the first share.
// round_pairs: the pairs one round of a caller that spreads products over
// launches spends on this product kind; items are then cut to about a
// quarter of a resident CTA's share of such a round, so that a round keeps
// every CTA busy (0: items sized for one launch of the whole product).  The
// value is part of the item space and stays fixed for a product.
struct SymSlice {
  const DevSites *s;
  const void *x;  // [g][n][3]: float for the FP32 product, double otherwise
  unsigned long long *lo, *hi, *bad;
  int item0, count;
  double round_pairs = 0.0;
};
constexpr int kMaxSymSlices = 32;  // systems per launch
int tmu32_sym_items(const DevSites &s, int g, double round_pairs = 0.0);
// next: a device counter of the launch (zeroed by the launcher)
void launch_tmu32_sym_multi(int g, const SymSlice *sl, int nsl, unsigned *next, cudaStream_t st);
void launch_fixed_to_float(size_t total, const unsigned long long *lo, const unsigned long long *hi,
                           const unsigned long long *bad, float *out, cudaStream_t st);
// FP64 symmetric product (g = 1, 2 or 4; one damping kind per launch)
int tmu_f64_sym_items(const DevSites &s, int g, double round_pairs = 0.0);
void launch_tmu_f64_sym_multi(int g, bool amoeba, const SymSlice *sl, int nsl, unsigned *next, cudaStream_t st);
void launch_fixed_to_double(size_t total, const unsigned long long *lo, const unsigned long long *hi,
                            const unsigned long long *bad, double *out, cudaStream_t st);
// double-single symmetric product (g = 1 or 2; one damping kind per launch)
int tmu_ds_sym_items(const DevSites &s, int g, double round_pairs = 0.0);
void launch_tmu_ds_sym_multi(int g, bool amoeba, const SymSlice *sl, int nsl, unsigned *next, cudaStream_t st);
void launch_tmu32_pairs(const DevSites &s, int g, const float *x, float *partial, int nsplit, cudaStream_t st);
// source splits an FP32 scratch must hold (per column) for every shape the
// autotuner may pick
int tmu32_max_split(const DevSites &s, int sm_count);
// Split of the source range for the FP32 operator (tmu32.cu) and its tile
// boxes / undamped distance, computed on the host from the FP32 positions.
int tmu32_pick_split(const DevSites &s, int sm_count);
void tile_boxes32(const float4 *pos32, int n, float4 *boxes /*[2*ceil(n/128)]*/);
float damp_r2max32(bool amoeba, double damp_thr, const double *inv_thole, const double *a, int n);
// Double-single product (ds_kernels.cu): y = T x, columns in groups of two
// sharing the pair geometry, ~1e-13 relative accuracy on the FP32 pipes;
// scratch of nsplit * 2 * n * 3.
int tmu_ds_pick_split(const DevSites &s, int sm_count);
void launch_tmu_ds_pairs(const DevSites &s, int g, const double *x, double *partial, int nsplit, cudaStream_t st);
// sym_scratch (tmu_sym_scratch_doubles(s, 2), or null): from 2048 sites
// each unordered pair is evaluated once (launch_tmu_ds_sym_pairs)
void launch_tmu_ds(const DevSites &s, int nrhs, const double *x, double *y, bool dodiag, double *scratch,
                   int nsplit, double *sym_scratch, cudaStream_t st);
void launch_tmu_ds_sym_pairs(const DevSites &s, int g, const double *x, unsigned long long *lo,
                             unsigned long long *hi, unsigned long long *bad, unsigned *next, cudaStream_t st);
// E_M2D with the all-pairs part in double-single (scratch nsplit * n * 3)
int m2d_ds_pick_split(const DevSites &s, int sm_count);
void launch_m2d_ds_pairs(const DevSites &s, double *partial, int nsplit, int *err_flag, cudaStream_t st);
void launch_m2d_ds(const DevSites &s, double *out, double *scratch, int nsplit, int *err_flag, cudaStream_t st);
float m2d_r2max32(bool amoeba, double damp_thr, const double *pol_w, const double *pol_a, int n, const double *mm_w,
                  const double *mm_a, int m);
// Polarization-gradient pair sums in double-single (grad_ds.cu): the static
// multipoles' field gradient at the polarizable sites (partial [nsplit][6]
// [m], at each site's static index; which 0) and the induced dipoles' field
// gradients, field and quadrupole-contracted Hessian at the static sites
// (partial [nsplit][18 or 9][m]; which 1), unscaled
int grad_ds_pick_split(const DevSites &s, int which, int sm_count);
void launch_grad_ds_mp(const DevSites &s, double *partial, int nsplit, int *err, cudaStream_t st);
void launch_grad_ds_dip(const DevSites &s, const double *ipd, double *partial, int nsplit, int *err,
                        cudaStream_t st);
// z = M^-1 r for the block-Jacobi preconditioner (info / minv as built by
// build_block_jacobi), columns [ncol][n][3], FP32
void launch_block_apply(int ncol, int n, const int4 *info, const float *minv, const float *r, float *z,
                        cudaStream_t st);
// the Neumann step of the near-field preconditioner on z = B^-1 r:
// w = N z (near-field rows ri/ci/blk of build_near_field), z -= B^-1 w;
// w is a scratch of the same shape as z
void launch_near_correct(int ncol, int n, const int4 *info, const float *minv, const int *ri, const int *ci,
                         const float *blk, float *z, float *w, cudaStream_t st);
// batched fields: rhs[s*nf+f] = E_M2D[s] + field[f]; solution scatter to [f][s]
void launch_batch_rhs(int n, int nf, int nset, const double *e_m2d, const double *fields, double *rhs,
                      cudaStream_t st);
void launch_batch_scatter(int n, int nf, int nipd, int nsolved, const double *x, double *out, cudaStream_t st);

// ---- block CG (block_cg.cu) -----------------------------------------------
// out[a][b] = sum_i U[ua[a]][i] V[vb[b]][i] (FP32 tiles, FP64 across tiles,
// fixed order); partial of block_cg_gram_doubles(smax)
size_t block_cg_gram_doubles(int smax);
int block_cg_max_columns();
void launch_gram(size_t nv, int sa, const float *U, const int *ua, int sb, const float *V, const int *vb,
                 double *partial, double *out, cudaStream_t st);
// out[oc[k]] = base[bc[k]] + sum_j in[ic[j]] C[j][k], C [nin][nout] (device)
void launch_combine(size_t nv, int nin, const float *in, const int *ic, int nout, float *out, const int *oc,
                    const float *base, const int *bc, const float *C, cudaStream_t st);
void launch_scale_alpha32(int ncol, int n, const float *alpha, const float *r, float *z, cudaStream_t st);

// ---- dense T (incore matvec / inversion) ---------------------------------
void launch_build_tmat(const DevSites &s, double *tmat, cudaStream_t st);  // [3n][3n] col-major
void launch_gemv(int nn, const double *A, const double *x, double *y, bool dodiag,
                 const double *alpha, int nrhs, cudaStream_t st);
// LU with partial pivoting in place (column major); info (device int) 0 = ok.
void launch_lu_factor(int nn, double *A, int *piv, int *info, double *work, cudaStream_t st);
void launch_lu_solve(int nn, const double *A, const int *piv, double *b, cudaStream_t st);

// ---- BLAS-1 and reductions (deterministic) --------------------------------
constexpr int kRedBlocks = 456;  // 3 x 152 SMs
constexpr int kRedThreads = 256;
// partial[b][k] for k < ncol: sum over i of a[k*n+i]*b[k*n+i]
void launch_dots(int ncol, size_t n, const double *a, const double *b, double *partial,
                 cudaStream_t st);
// partial[b][k] = sum_i a[k*n+i] * v[i]  (one vector against ncol columns)
void launch_dots_bcast(int ncol, size_t n, const double *a, const double *v, double *partial,
                       cudaStream_t st);
void launch_dots_f32(int ncol, size_t n, const float *a, const float *b, double *partial,
                     cudaStream_t st);
// result[k] = sum_b partial[b][k]  (fixed order)
void launch_reduce_partials(int ncol, const double *partial, double *result, cudaStream_t st);

// misc elementwise
void launch_axpby(size_t n, double a, const double *x, double b, double *y, cudaStream_t st);
void launch_add(size_t n, const double *a, const double *b, double *out, cudaStream_t st);
void launch_scale_by_alpha(int nrhs, int n, const double *alpha, const double *x, double *y,
                           cudaStream_t st);
void launch_to_f32(size_t n, const double *x, const double *scale, float *y, cudaStream_t st);
// y[k][i] = x[k][i] * scale[k] for ncol columns of nv values (one launch)
void launch_to_f32_cols(int ncol, size_t nv, const double *x, const double *scale, float *y, cudaStream_t st);

// Multi-column PCG state kept on the device (one entry per column).
struct CgCol {
  double gold, gama, alpha, gnew, rms, beta;
  double tol;     // convergence threshold of this column (kept on the device
                  // so that a captured iteration graph stays valid)
  int active;     // column still iterating
  int quick;      // left through |p.Tp| < eps
  int converged;  // rms < tol
  int iters;
};
// cols[k] = {gold = dots[k], tol, active = dots[k] > 0} (inner PCG start)
void launch_cg_init(int ncol, const double *dots, CgCol *cols, double tol, cudaStream_t st);
// gama_k = (h.p)_k from reduced dots; alpha = gold/gama; quick-exit flags.
void launch_cg_alpha(int ncol, const double *dots, CgCol *cols, double eps, cudaStream_t st);
// x += alpha p; r -= alpha h; z = alpha_pol r; partial r.z per column
void launch_cg_update(int ncol, int n, double *x, double *r, const double *p, const double *h,
                      double *z, const double *alpha_pol, const CgCol *cols, double *partial,
                      cudaStream_t st);
// gnew = (r.z)_k, rms, convergence against cols[k].tol, beta; history
void launch_cg_gnew(int ncol, int n, const double *dots, CgCol *cols, double *hist, int hist_stride,
                    cudaStream_t st);
void launch_cg_pupdate(int ncol, int n, double *p, const double *z, const CgCol *cols,
                       cudaStream_t st);
// FP32 vectors, FP64 scalars (inner solver of the mixed-precision path)
void launch_cg_update_f32(int ncol, int n, float *x, float *r, const float *p, const float *h,
                          float *z, const float *alpha_pol, const CgCol *cols, double *partial,
                          cudaStream_t st);
void launch_cg_pupdate_f32(int ncol, int n, float *p, const float *z, const CgCol *cols,
                           cudaStream_t st);
// mu[k] += scale[k] * dmu32[k]  (IR correction, FP64 accumulate)
void launch_ir_accumulate(int ncol, int n, double *mu, const float *d32, const double *scale,
                          cudaStream_t st);
// r = rhs - Tmu (all columns), into r; and r32 = r / scale
void launch_residual(size_t total, const double *rhs, const double *tmu, double *r,
                     cudaStream_t st);
// r[k] -= scale[k] * t32[k]  (refinement residual updated by the FP32
// product of the correction instead of a recomputed product)
void launch_residual_update(int ncol, int n, double *r, const float *t32, const double *scale,
                            cudaStream_t st);
// DIIS: x_new = sum_i c_i X[:, i]
void launch_lincomb(int nvec, size_t n, const double *X, size_t ldx, const double *c, double *out,
                    cudaStream_t st);
// rms and max of (a - b): out[0] = sum sq, out[1] = max abs (per-block partials then reduce)
void launch_diff_norms(size_t n, const double *a, const double *b, double *partial,
                       cudaStream_t st);
void launch_reduce_norms(const double *partial, double *out, cudaStream_t st);
// NaN / Inf check: flag set to 1 when any entry is not finite
void launch_check_finite(size_t n, const double *x, int *flag, cudaStream_t st);
// flag set to 1 when a and b differ in any bit of any entry
void launch_any_diff(size_t n, const double *a, const double *b, int *flag, cudaStream_t st);

// Number of SMs of the current device (cached).
int sm_count();
// Kernels launched by this library since load (all streams); graph replays
// add the kernels of the replayed graph.
long long launch_count();
long long thread_launch_count();
void add_launch_count(long long k);
// FMA-chain kernel for the FP32 / FP64 pipe peak; returns its flop count.
double launch_fma_peak(bool fp64, int iters, void *out, cudaStream_t st);

}  // namespace gpu
}  // namespace ommp
