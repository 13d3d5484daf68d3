// Block preconditioned CG for the FP32 inner solve of batched right-hand
// sides (ommp_gpu_set_external_fields_batch in the mixed modes).
//
// The reference solves one right-hand side at a time with the scalar CG of
// src/mod_solvers.F90:86-216; the batch's columns (fields of several QM
// densities, say) share the matrix T, so here they share one Krylov space:
// every iteration multiplies a block of s search directions by T in one
// column-group product and minimises over all of them at once (O'Leary's
// block CG), so columns converge in fewer iterations than alone.
//
// Each iteration, with P the n x s directions, Q = T P, R and Z = M^-1 R
// the residuals of the active columns:
//   G = P^T Q, H = P^T R                  (Gram matrices, one launch each)
//   A = G^+ H                             (host, FP64; G^+ the pseudo-inverse
//                                          below drops directions that have
//                                          become dependent: rank-revealing
//                                          eigendecomposition of the
//                                          diagonally scaled G)
//   X += P A,  R -= Q A,  Z = M^-1 R
//   K = Q^T Z, rho_k = z_k . r_k          (convergence per column: the
//                                          scalar solver's rms of r.z)
//   P <- Z_active + P B,  B = -G^+ K      (new directions A-orthogonal to P)
// Converged columns leave the block (their X stays), so the block narrows as
// the columns converge.  The Gram matrices are accumulated in FP32 over tiles
// of 64 elements and in FP64 across tiles; the small matrices are solved on
// the host between the launches, so this iteration is not graph-captured.
#include <algorithm>
#include <cmath>
#include <vector>

#include "engine.h"
#include "log.h"

namespace ommp {
namespace gpu {
namespace {

constexpr int GT = 32;          // output tile of the Gram kernel (rows and columns)
constexpr int GE = 64;          // elements per staged tile
constexpr int kGramChunks = 152;  // element chunks (blocks along x)
constexpr int CK = 16;          // output columns per block of the combine kernel
constexpr int kMaxBlock = 128;  // widest block (columns)

// partial[c][a][b] = sum over chunk c of U[ua[a]][i] V[vb[b]][i]
__global__ void __launch_bounds__(256) k_gram(size_t nv, int sa, const float *__restrict__ U,
                                              const int *__restrict__ ua, int sb, const float *__restrict__ V,
                                              const int *__restrict__ vb, double *__restrict__ partial) {
  __shared__ float su[GT][GE + 1], sv[GT][GE + 1];
  const int a0 = blockIdx.y * GT, b0 = blockIdx.z * GT;
  const int tid = threadIdx.x, ta = tid >> 3, tb = (tid & 7) * 4;
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  const size_t chunk = (nv + gridDim.x - 1) / gridDim.x;
  const size_t i0 = (size_t)blockIdx.x * chunk;
  const size_t i1 = i0 + chunk < nv ? i0 + chunk : nv;
  for (size_t t = i0; t < i1; t += GE) {
    for (int q = tid; q < GT * GE; q += 256) {
      const int r = q / GE, e = q % GE;
      const size_t i = t + e;
      const int ar = a0 + r, br = b0 + r;
      su[r][e] = (ar < sa && i < i1) ? U[(size_t)ua[ar] * nv + i] : 0.f;
      sv[r][e] = (br < sb && i < i1) ? V[(size_t)vb[br] * nv + i] : 0.f;
    }
    __syncthreads();
    float f[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 8
    for (int e = 0; e < GE; ++e) {
      const float u = su[ta][e];
#pragma unroll
      for (int c = 0; c < 4; ++c) f[c] = fmaf(u, sv[tb + c][e], f[c]);
    }
#pragma unroll
    for (int c = 0; c < 4; ++c) acc[c] += (double)f[c];
    __syncthreads();
  }
  const int a = a0 + ta;
  if (a < sa)
#pragma unroll
    for (int c = 0; c < 4; ++c)
      if (b0 + tb + c < sb) partial[((size_t)blockIdx.x * sa + a) * sb + b0 + tb + c] = acc[c];
}

// out[k] = sum over chunks of partial[c][k], in chunk order
__global__ void k_gram_reduce(int nchunk, int total, const double *__restrict__ partial, double *__restrict__ out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= total) return;
  double s = 0.0;
  for (int c = 0; c < nchunk; ++c) s += partial[(size_t)c * total + k];
  out[k] = s;
}

// out[oc[k]][i] = base[bc[k]][i] + sum_j in[ic[j]][i] C[j][k]  (k < nout;
// C is [nin][nout]); out may be base (in-place update), never in
__global__ void __launch_bounds__(256) k_combine(size_t nv, int nin, const float *__restrict__ in,
                                                 const int *__restrict__ ic, int nout, float *out,
                                                 const int *__restrict__ oc, const float *base,
                                                 const int *__restrict__ bc, const float *__restrict__ C) {
  __shared__ float sC[kMaxBlock][CK];
  const int k0 = blockIdx.y * CK;
  const int kn = min(CK, nout - k0);
  for (int q = threadIdx.x; q < nin * CK; q += blockDim.x) {
    const int j = q / CK, kk = q % CK;
    sC[j][kk] = kk < kn ? C[(size_t)j * nout + k0 + kk] : 0.f;
  }
  __syncthreads();
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += (size_t)gridDim.x * blockDim.x) {
    float acc[CK];
#pragma unroll
    for (int kk = 0; kk < CK; ++kk) acc[kk] = kk < kn ? base[(size_t)bc[k0 + kk] * nv + i] : 0.f;
    for (int j = 0; j < nin; ++j) {
      const float x = in[(size_t)ic[j] * nv + i];
#pragma unroll
      for (int kk = 0; kk < CK; ++kk) acc[kk] = fmaf(x, sC[j][kk], acc[kk]);
    }
#pragma unroll
    for (int kk = 0; kk < CK; ++kk)
      if (kk < kn) out[(size_t)oc[k0 + kk] * nv + i] = acc[kk];
  }
}

// z = alpha r for ncol columns (the diagonal preconditioner of the reference)
__global__ void k_scale_alpha32(int ncol, int n, const float *__restrict__ alpha, const float *__restrict__ r,
                                float *__restrict__ z) {
  const size_t nv = 3 * (size_t)n, tot = nv * ncol;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < tot; i += (size_t)gridDim.x * blockDim.x)
    z[i] = alpha[(i % nv) / 3] * r[i];
}

}  // namespace

size_t block_cg_gram_doubles(int smax) { return (size_t)kGramChunks * smax * smax + (size_t)2 * smax * smax; }

void launch_gram(size_t nv, int sa, const float *U, const int *ua, int sb, const float *V, const int *vb,
                 double *partial, double *out, cudaStream_t st) {
  if (sa < 1 || sb < 1) return;
  add_launch_count(2);
  dim3 grid(kGramChunks, (sa + GT - 1) / GT, (sb + GT - 1) / GT);
  k_gram<<<grid, 256, 0, st>>>(nv, sa, U, ua, sb, V, vb, partial);
  const int total = sa * sb;
  k_gram_reduce<<<(total + 255) / 256, 256, 0, st>>>(kGramChunks, total, partial, out);
}

void launch_combine(size_t nv, int nin, const float *in, const int *ic, int nout, float *out, const int *oc,
                    const float *base, const int *bc, const float *C, cudaStream_t st) {
  if (nout < 1) return;
  add_launch_count(1);
  int bx = (int)std::min<size_t>((nv + 255) / 256, 4 * 152);
  dim3 grid(bx < 1 ? 1 : bx, (nout + CK - 1) / CK);
  k_combine<<<grid, 256, 0, st>>>(nv, nin, in, ic, nout, out, oc, base, bc, C);
}

void launch_scale_alpha32(int ncol, int n, const float *alpha, const float *r, float *z, cudaStream_t st) {
  add_launch_count(1);
  const size_t tot = 3 * (size_t)n * ncol;
  int b = (int)std::min<size_t>((tot + 255) / 256, 4 * 152 * 4);
  k_scale_alpha32<<<b < 1 ? 1 : b, 256, 0, st>>>(ncol, n, alpha, r, z);
}

int block_cg_max_columns() { return kMaxBlock; }

}  // namespace gpu

namespace {

// Pseudo-inverse of a symmetric positive semi-definite s x s matrix (row
// major) by cyclic Jacobi on its diagonally scaled form: eigenvalues below
// tau times the largest are dropped (dependent directions).  Returns the
// rank.
int psd_pinv(int s, const std::vector<double> &G, std::vector<double> &Gp, double tau) {
  std::vector<double> d(s), A((size_t)s * s), V((size_t)s * s, 0.0);
  for (int i = 0; i < s; ++i) d[i] = G[(size_t)i * s + i] > 0.0 ? 1.0 / std::sqrt(G[(size_t)i * s + i]) : 0.0;
  for (int i = 0; i < s; ++i)
    for (int j = 0; j < s; ++j) A[(size_t)i * s + j] = 0.5 * (G[(size_t)i * s + j] + G[(size_t)j * s + i]) * d[i] * d[j];
  for (int i = 0; i < s; ++i) V[(size_t)i * s + i] = 1.0;
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = 0.0, diag = 0.0;
    for (int i = 0; i < s; ++i)
      for (int j = 0; j < s; ++j) (i == j ? diag : off) += A[(size_t)i * s + j] * A[(size_t)i * s + j];
    if (off <= 1e-30 * (diag > 0.0 ? diag : 1.0)) break;
    for (int p = 0; p < s - 1; ++p)
      for (int q = p + 1; q < s; ++q) {
        const double apq = A[(size_t)p * s + q];
        if (std::fabs(apq) < 1e-300) continue;
        const double app = A[(size_t)p * s + p], aqq = A[(size_t)q * s + q];
        const double theta = 0.5 * (aqq - app) / apq;
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), sn = t * c;
        for (int k = 0; k < s; ++k) {
          const double akp = A[(size_t)k * s + p], akq = A[(size_t)k * s + q];
          A[(size_t)k * s + p] = c * akp - sn * akq;
          A[(size_t)k * s + q] = sn * akp + c * akq;
        }
        for (int k = 0; k < s; ++k) {
          const double apk = A[(size_t)p * s + k], aqk = A[(size_t)q * s + k];
          A[(size_t)p * s + k] = c * apk - sn * aqk;
          A[(size_t)q * s + k] = sn * apk + c * aqk;
        }
        for (int k = 0; k < s; ++k) {
          const double vkp = V[(size_t)k * s + p], vkq = V[(size_t)k * s + q];
          V[(size_t)k * s + p] = c * vkp - sn * vkq;
          V[(size_t)k * s + q] = sn * vkp + c * vkq;
        }
      }
  }
  double lmax = 0.0;
  for (int i = 0; i < s; ++i) lmax = std::max(lmax, A[(size_t)i * s + i]);
  Gp.assign((size_t)s * s, 0.0);
  int rank = 0;
  for (int e = 0; e < s; ++e) {
    const double l = A[(size_t)e * s + e];
    if (!(l > tau * lmax)) continue;
    ++rank;
    for (int i = 0; i < s; ++i)
      for (int j = 0; j < s; ++j) Gp[(size_t)i * s + j] += V[(size_t)i * s + e] * V[(size_t)j * s + e] / l;
  }
  for (int i = 0; i < s; ++i)
    for (int j = 0; j < s; ++j) Gp[(size_t)i * s + j] *= d[i] * d[j];
  return rank;
}

}  // namespace

// Block PCG on w.r32 (columns normalised to unit rms); result in w.x32.  Uses
// w.p32 / w.h32 as the compact direction blocks P / Q, w.t32 as the next P,
// w.gram for the Gram partials and results, w.bcoef / w.bidx for the
// coefficients and column maps.
int System::bpcg32_ws(Workspace &w, int ncol, int max_it, double eta) {
  const int n = d_.n;
  const size_t nv = 3 * (size_t)n;
  const int smax = gpu::block_cg_max_columns();
  if (ncol > smax || !w.t32 || !w.gram) {
    set_last_error("block CG: workspace without block buffers or more than 128 columns");
    return kErrBadArg;
  }
  // P and the next P swap buffers each iteration; the workspace keeps its own
  // pointers on return (the captured scalar iteration refers to them)
  struct Restore {
    Workspace &w;
    float *p, *t;
    ~Restore() { w.p32 = p, w.t32 = t; }
  } restore{w, w.p32, w.t32};
  F32Shape shape{1, 1, 2};
  int st = tune_f32(w, std::min(ncol, 8), shape);
  if (st) return st;
  const bool blocks = inner_precond_ >= 1 && blk_info_;
  const bool near = blocks && near_precond();
  auto precondition = [&](int nc) {
    if (blocks) {
      gpu::launch_block_apply(nc, n, blk_info_, blk_minv_, w.r32, w.z32, st_);
      // the next direction block (w.t32) is written only after this: scratch
      if (near)
        gpu::launch_near_correct(nc, n, blk_info_, blk_minv_, near_ri_, near_ci_, near_blk_, w.z32, w.t32, st_);
    } else {
      gpu::launch_scale_alpha32(nc, n, alpha32_, w.r32, w.z32, st_);
    }
  };
  // index maps in w.bidx: [0, smax) identity, then the active columns
  std::vector<int> idx(2 * (size_t)smax);
  for (int k = 0; k < smax; ++k) idx[k] = k;
  int *ident = w.bidx, *actd = w.bidx + smax;
  double *gpart = w.gram, *gout = w.gram + (size_t)gpu::block_cg_gram_doubles(smax) - 2 * (size_t)smax * smax;
  cudaMemsetAsync(w.x32, 0, ncol * nv * sizeof(float), st_);
  precondition(ncol);
  gpu::launch_dots_f32(ncol, nv, w.r32, w.z32, w.partial, st_);
  gpu::launch_reduce_partials(ncol, w.partial, w.dots, st_);
  cudaMemcpyAsync(w.scal_h, w.dots, ncol * sizeof(double), cudaMemcpyDeviceToHost, st_);
  st = check(cudaStreamSynchronize(st_), "block CG init");
  if (st) return st;
  std::vector<int> act;
  for (int k = 0; k < ncol; ++k)
    if (w.scal_h[k] > 0.0 && std::sqrt(w.scal_h[k] / (double)nv) >= eta) act.push_back(k);
  if (act.empty()) return kOk;
  int s = (int)act.size();
  // P = Z of the active columns
  for (int k = 0; k < s; ++k) idx[smax + k] = act[k];
  std::vector<float> C(2 * (size_t)smax * smax, 0.f);
  cudaMemcpyAsync(w.bidx, idx.data(), idx.size() * sizeof(int), cudaMemcpyHostToDevice, st_);
  cudaMemcpyAsync(w.bcoef, C.data(), (size_t)s * s * sizeof(float), cudaMemcpyHostToDevice, st_);
  gpu::launch_combine(nv, s, w.z32, actd, s, w.p32, ident, w.z32, actd, w.bcoef, st_);
  std::vector<double> G, H, K, Gp, A;
  int it = 0;
  const double tau = 1e-6;
  for (it = 1; it <= max_it; ++it) {
    // Q = T P (the column groups of the tuned FP32 kernel)
    KEv ev;
    if (ktime_on_) ev = kt_begin(1, s);
    f32_product(w, s, shape);
    if (ktime_on_) kt_end(ev);
    stats_.f32_matvecs += 1;
    const int sa = (int)act.size();
    gpu::launch_gram(nv, s, w.p32, ident, s, w.h32, ident, gpart, gout, st_);
    gpu::launch_gram(nv, s, w.p32, ident, sa, w.r32, actd, gpart, gout + (size_t)s * s, st_);
    G.resize((size_t)s * s);
    H.resize((size_t)s * sa);
    cudaMemcpyAsync(w.bscal_h, gout, ((size_t)s * s + (size_t)s * sa) * sizeof(double), cudaMemcpyDeviceToHost, st_);
    st = check(cudaStreamSynchronize(st_), "block CG Gram");
    if (st) return st;
    std::copy(w.bscal_h, w.bscal_h + (size_t)s * s, G.begin());
    std::copy(w.bscal_h + (size_t)s * s, w.bscal_h + (size_t)s * s + (size_t)s * sa, H.begin());
    const int rank = psd_pinv(s, G, Gp, tau);
    if (rank == 0) break;  // no direction left (exactly solved or broken down): the refinement continues
    // A = G^+ H; X += P A, R -= Q A
    A.assign((size_t)s * sa, 0.0);
    for (int i = 0; i < s; ++i)
      for (int j = 0; j < s; ++j) {
        const double g = Gp[(size_t)i * s + j];
        if (g == 0.0) continue;
        for (int k = 0; k < sa; ++k) A[(size_t)i * sa + k] += g * H[(size_t)j * sa + k];
      }
    for (size_t q = 0; q < (size_t)s * sa; ++q) {
      C[q] = (float)A[q];
      C[(size_t)s * sa + q] = (float)-A[q];
    }
    cudaMemcpyAsync(w.bcoef, C.data(), 2 * (size_t)s * sa * sizeof(float), cudaMemcpyHostToDevice, st_);
    gpu::launch_combine(nv, s, w.p32, ident, sa, w.x32, actd, w.x32, actd, w.bcoef, st_);
    gpu::launch_combine(nv, s, w.h32, ident, sa, w.r32, actd, w.r32, actd, w.bcoef + (size_t)s * sa, st_);
    precondition(ncol);
    // convergence of each column, and K = Q^T Z
    gpu::launch_dots_f32(ncol, nv, w.r32, w.z32, w.partial, st_);
    gpu::launch_reduce_partials(ncol, w.partial, w.dots, st_);
    gpu::launch_gram(nv, s, w.h32, ident, sa, w.z32, actd, gpart, gout, st_);
    cudaMemcpyAsync(w.bscal_h, gout, (size_t)s * sa * sizeof(double), cudaMemcpyDeviceToHost, st_);
    cudaMemcpyAsync(w.bscal_h + (size_t)s * sa, w.dots, ncol * sizeof(double), cudaMemcpyDeviceToHost, st_);
    st = check(cudaStreamSynchronize(st_), "block CG update");
    if (st) return st;
    K.assign(w.bscal_h, w.bscal_h + (size_t)s * sa);
    const double *rho = w.bscal_h + (size_t)s * sa;
    std::vector<int> keep;  // positions in act of the columns still above eta
    for (int k = 0; k < sa; ++k) {
      const double rms = std::sqrt(std::max(rho[act[k]], 0.0) / (double)nv);
      if (!std::isfinite(rms)) {
        set_last_error("non-finite residual in the block inner solver (coincident sites?)");
        return kErrNumeric;
      }
      if (rms >= eta) keep.push_back(k);
    }
    if (keep.empty()) break;
    // P <- Z_keep + P B, B = -G^+ K (restricted to the kept columns)
    const int sn = (int)keep.size();
    for (int i = 0; i < s; ++i)
      for (int kk = 0; kk < sn; ++kk) {
        double b = 0.0;
        for (int j = 0; j < s; ++j) b -= Gp[(size_t)i * s + j] * K[(size_t)j * sa + keep[kk]];
        C[(size_t)i * sn + kk] = (float)b;
      }
    std::vector<int> nact(sn);
    for (int kk = 0; kk < sn; ++kk) nact[kk] = act[keep[kk]];
    for (int kk = 0; kk < sn; ++kk) idx[smax + kk] = nact[kk];
    cudaMemcpyAsync(w.bcoef, C.data(), (size_t)s * sn * sizeof(float), cudaMemcpyHostToDevice, st_);
    cudaMemcpyAsync(actd, idx.data() + smax, sn * sizeof(int), cudaMemcpyHostToDevice, st_);
    gpu::launch_combine(nv, s, w.p32, ident, sn, w.t32, ident, w.z32, actd, w.bcoef, st_);
    std::swap(w.p32, w.t32);
    act.swap(nact);
    s = sn;
  }
  stats_.inner_iters += std::min(it, max_it);
  return check(cudaGetLastError(), "block CG");
}

}  // namespace ommp
