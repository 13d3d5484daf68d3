// Iterative solvers on a column workspace, and the batched solve.
//
//   cg64_ws      the reference's preconditioned CG (src/mod_solvers.F90:86-216)
//                for ncol independent columns sharing each T.mu product:
//                zero-norm guess replaced by alpha*x, quick exit when
//                |p.Tp| < 100 eps, convergence on sqrt(r.alpha r / n).
//   pcg32_ws     the FP32 inner solver of the mixed-precision path; one
//                iteration (FP32 T.mu, dots, updates, status copy) is captured
//                once as a CUDA graph and replayed.
//   mixed_ir_ws  iterative refinement: FP64 residual E - T mu, FP32 PCG on the
//                normalised residual, FP64 accumulation, FP64 convergence test.
//   tune_f32     picks the FP32 kernel's column-group width and source split
//                by timing the candidates on this system (cached per width).
//   solve_batch  nf fields at once (64 QM densities, say): one block of
//                columns through the same solvers.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>

#include "engine.h"
#include "log.h"

namespace ommp {

namespace {
template <typename T>
int walloc(T *&p, size_t count) {
  p = nullptr;
  if (count == 0) count = 1;
  return cudaMalloc((void **)&p, count * sizeof(T)) == cudaSuccess ? 0 : 1;
}
}  // namespace

void System::free_ws(Workspace &w) {
  if (w.graph) cudaGraphExecDestroy(w.graph);
  w.graph = nullptr;
  w.graph_ncol = -1;
  if (!w.owned) return;
  void *b[] = {w.x, w.r, w.p, w.h, w.z, w.rhs, w.fields, w.out, w.x32, w.r32, w.p32, w.h32, w.z32,
               w.scratch32, w.partial, w.dots, w.hist, w.cols, w.t32, w.gram, w.bcoef, w.bidx};
  for (void *p : b)
    if (p) cudaFree(p);
  if (st_) cudaStreamSynchronize(st_);  // read-backs into the pinned buffers
  pinned_free(w.cols_h);
  pinned_free(w.scal_h);
  pinned_free(w.bscal_h);
  w = Workspace();
}

int System::ensure_batch_ws(int ncol, int nf) {
  if (wsb_.cap >= ncol && wsb_.fcap >= nf) return kOk;
  cudaStreamSynchronize(st_);
  free_ws(wsb_);
  Workspace &w = wsb_;
  const size_t nv = 3 * (size_t)d_.n;
  const int nipd = m_.n_ipd;
  int s0 = gpu::tmu32_max_split(d_, gpu::sm_count());
  int bad = 0;
  bad |= walloc(w.x, ncol * nv) | walloc(w.r, ncol * nv) | walloc(w.p, ncol * nv) | walloc(w.h, ncol * nv) |
         walloc(w.z, ncol * nv) | walloc(w.rhs, ncol * nv);
  bad |= walloc(w.fields, nf * nv) | walloc(w.out, (size_t)nf * nipd * nv);
  bad |= walloc(w.x32, ncol * nv) | walloc(w.r32, ncol * nv) | walloc(w.p32, ncol * nv) |
         walloc(w.h32, ncol * nv) | walloc(w.z32, ncol * nv);
  bad |= walloc(w.scratch32, (size_t)s0 * ncol * nv);
  bad |= walloc(w.partial, (size_t)gpu::kRedBlocks * std::max(ncol, nf)) |
         walloc(w.dots, 3 * (size_t)ncol + nf) | walloc(w.cols, ncol);
  // block CG buffers (sized for the widest block)
  const int smax = gpu::block_cg_max_columns();
  bad |= walloc(w.t32, ncol * nv) | walloc(w.gram, gpu::block_cg_gram_doubles(smax)) |
         walloc(w.bcoef, 2 * (size_t)smax * smax) | walloc(w.bidx, 2 * (size_t)smax);
  if (bad || pinned_alloc((void **)&w.cols_h, ncol * sizeof(gpu::CgCol)) != cudaSuccess ||
      pinned_alloc((void **)&w.scal_h, (3 * (size_t)ncol + nf) * sizeof(double)) != cudaSuccess ||
      pinned_alloc((void **)&w.bscal_h, (2 * (size_t)smax * smax + smax) * sizeof(double)) != cudaSuccess) {
    w.owned = true;
    free_ws(w);
    set_last_error("out of device memory for the batch workspace");
    return kErrMemory;
  }
  w.cap = ncol;
  w.fcap = nf;
  w.scratch32_nsplit = s0;
  w.owned = true;
  return kOk;
}

// ---------------------------------------------------------------------------
// FP64 conjugate gradient (reference algorithm), ncol columns
// ---------------------------------------------------------------------------
int System::cg64_ws(Workspace &w, int matv, int ncol, const double *rhs, double *x, int set0) {
  const int n = d_.n;
  const size_t nv = 3 * (size_t)n;
  log_msg(kVerbLow, nullptr, "Solving linear system with CG solver");
  log_msg(kVerbLow, nullptr, "Max iter: %4d", maxiter_);
  log_msg(kVerbLow, nullptr, "Tolerance: %8.1E", tol_);
  // guess: a zero-norm input is replaced by precnd(x) = alpha * x (:151-157)
  gpu::launch_dots(ncol, nv, x, x, w.partial, st_);
  gpu::launch_reduce_partials(ncol, w.partial, w.dots, st_);
  cudaMemcpyAsync(w.scal_h, w.dots, ncol * sizeof(double), cudaMemcpyDeviceToHost, st_);
  int st = check(cudaStreamSynchronize(st_), "CG start");
  if (st) return st;
  bool all_zero = true;
  for (int k = 0; k < ncol; ++k) {
    if (w.scal_h[k] < kEpsRp) {
      log_msg(kVerbHigh, nullptr, "Input guess has zero norm, generating a guess from preconditioner.");
      gpu::launch_scale_by_alpha(1, n, d_.pol_alpha, x + k * nv, x + k * nv, st_);
    } else {
      log_msg(kVerbHigh, nullptr, "Using input guess as a starting point for iterative solver.");
    }
    if (w.scal_h[k] != 0.0) all_zero = false;
  }
  // r = rhs - T x; an exactly zero x gives T x = 0 without the pair sum
  if (all_zero) {
    cudaMemcpyAsync(w.r, rhs, ncol * nv * sizeof(double), cudaMemcpyDeviceToDevice, st_);
  } else {
    st = matvec64(matv, ncol, x, w.z, true);
    if (st) return st;
    gpu::launch_residual(ncol * nv, rhs, w.z, w.r, st_);
  }
  gpu::launch_scale_by_alpha(ncol, n, d_.pol_alpha, w.r, w.z, st_);
  cudaMemcpyAsync(w.p, w.z, ncol * nv * sizeof(double), cudaMemcpyDeviceToDevice, st_);
  gpu::launch_dots(ncol, nv, w.r, w.z, w.partial, st_);
  gpu::launch_reduce_partials(ncol, w.partial, w.dots, st_);
  cudaMemcpyAsync(w.scal_h, w.dots, ncol * sizeof(double), cudaMemcpyDeviceToHost, st_);
  st = check(cudaStreamSynchronize(st_), "CG init");
  if (st) return st;
  for (int k = 0; k < ncol; ++k) {
    gpu::CgCol c{};
    c.gold = w.scal_h[k];
    c.tol = tol_;
    c.active = 1;
    w.cols_h[k] = c;
  }
  cudaMemcpyAsync(w.cols, w.cols_h, ncol * sizeof(gpu::CgCol), cudaMemcpyHostToDevice, st_);
  double *hist = (set0 >= 0) ? w.hist : nullptr;
  for (int it = 1; it <= maxiter_; ++it) {
    st = matvec64(matv, ncol, w.p, w.h, true);
    if (st) return st;
    gpu::launch_dots(ncol, nv, w.h, w.p, w.partial, st_);
    gpu::launch_reduce_partials(ncol, w.partial, w.dots, st_);
    gpu::launch_cg_alpha(ncol, w.dots, w.cols, kEpsRp, st_);
    gpu::launch_cg_update(ncol, n, x, w.r, w.p, w.h, w.z, d_.pol_alpha, w.cols, w.partial, st_);
    gpu::launch_reduce_partials(ncol, w.partial, w.dots, st_);
    gpu::launch_cg_gnew(ncol, n, w.dots, w.cols, hist, maxhist_, st_);
    gpu::launch_cg_pupdate(ncol, n, w.p, w.z, w.cols, st_);
    cudaMemcpyAsync(w.cols_h, w.cols, ncol * sizeof(gpu::CgCol), cudaMemcpyDeviceToHost, st_);
    st = check(cudaStreamSynchronize(st_), "CG iteration");
    if (st) return st;
    bool any = false;
    for (int k = 0; k < ncol; ++k) {
      if (w.cols_h[k].active) any = true;
      if (log_level() >= kVerbHigh && w.cols_h[k].iters == it)
        log_msg(kVerbHigh, nullptr, "iter=%4d residual rms norm: %14.4E", it, w.cols_h[k].rms);
    }
    if (!any) break;
  }
  std::vector<double> h(maxhist_);
  int rc = kOk;
  for (int k = 0; k < ncol; ++k) {
    const gpu::CgCol &c = w.cols_h[k];
    if (set0 >= 0 && set0 + k < 2) {
      int set = set0 + k;
      stats_.iters[set] = c.iters;
      int nh = std::min(c.iters, maxhist_);
      cudaMemcpy(h.data(), w.hist + (size_t)k * maxhist_, nh * sizeof(double), cudaMemcpyDeviceToHost);
      stats_.hist[set].assign(h.begin(), h.begin() + nh);
    }
    if (c.quick) log_msg(kVerbHigh, nullptr, "Direction vector with zero norm, exiting iterative solver.");
    if (c.converged)
      log_msg(kVerbHigh, nullptr, "Required convergence threshold reached, exiting iterative solver.");
    if (!std::isfinite(c.rms)) {
      set_last_error("non-finite residual in the iterative solver (coincident sites?)");
      rc = kErrNumeric;
    } else if (!c.converged && !c.quick && c.rms > tol_ && std::fabs(c.gama) > kEpsRp) {
      set_last_error("Iterative solver did not converged");
      rc = kErrNotConverged;
    }
  }
  return rc;
}

// ---------------------------------------------------------------------------
// FP32 product with the tuned launch shape
// ---------------------------------------------------------------------------
void System::f32_product(Workspace &w, int ncol, const F32Shape &sh) {
  gpu::launch_tmu_f32(d_, ncol, w.p32, w.h32, w.scratch32, sh.nsplit, st_, sh.g, sh.kver, sym_scratch_);
}

int System::tune_f32(Workspace &w, int ncol, F32Shape &shape) {
  auto it = f32_tune_.find(ncol);
  if (it != f32_tune_.end() && it->second.nsplit <= w.scratch32_nsplit) {
    shape = it->second;
    return kOk;
  }
  const int sms = gpu::sm_count();
  const int tiles = (d_.n + 127) / 128;
  const int cap = std::min(w.scratch32_nsplit, tiles);
  std::vector<F32Shape> cands;
  std::vector<int> widths = {1};
  for (int g : {2, 4, 8})
    if (g <= ncol) widths.push_back(g);
  // kernel 1: one target per thread; kernel 2: tile-classified, two
  // targets per thread for one or two columns
  const int s1 = gpu::tmu_pick_split(d_, ncol, sms, true), s2 = gpu::tmu32_pick_split(d_, sms);
  for (int g : widths) {
    if (fp32_kernel_ == 0 || fp32_kernel_ == 1)
      for (int s : {s1, 2 * s1})
        if (s <= cap) cands.push_back({g, s, 1});
    if (fp32_kernel_ == 0 || fp32_kernel_ == 2)
      for (int s : {std::max(1, s2 / 2), s2, 2 * s2})
        if (s <= cap) cands.push_back({g, s, 2});
  }
  // kernel 3: each unordered pair once (tmu32.cu), column groups of 1 or 2,
  // from 2048 sites (or when forced); its accumulators are allocated here,
  // before any capture of the inner iteration
  if ((fp32_kernel_ == 3 || (fp32_kernel_ == 0 && d_.n >= 2048)) && ensure_sym_scratch() == kOk)
    for (int g : {1, 2})
      if (g <= ncol) cands.push_back({g, 1, 3});
  if (cands.empty()) cands.push_back({1, 1, fp32_kernel_ == 1 ? 1 : 2});
  const size_t nv = 3 * (size_t)d_.n;
  cudaMemsetAsync(w.p32, 0, ncol * nv * sizeof(float), st_);
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  float best = 1e30f;
  F32Shape pick = cands.front();
  for (const F32Shape &c : cands) {
    f32_product(w, ncol, c);  // warm-up
    cudaEventRecord(a, st_);
    f32_product(w, ncol, c);
    f32_product(w, ncol, c);
    cudaEventRecord(b, st_);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    if (ms < best) best = ms, pick = c;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  int st = check(cudaGetLastError(), "FP32 autotune");
  if (st) return st;
  f32_tune_[ncol] = pick;
  shape = pick;
  log_msg(kVerbHigh, nullptr,
          "autotuned FP32 T.mu for %d columns: kernel %d, %d per launch, %d source splits (%.3f ms)", ncol,
          pick.kver, pick.g, pick.nsplit, best / 2);
  return kOk;
}

// ---------------------------------------------------------------------------
// FP32 inner PCG on w.r32 (columns normalised to unit rms); result in w.x32
// ---------------------------------------------------------------------------
int System::pcg32_ws(Workspace &w, int ncol, int max_it, double eta) {
  const int n = d_.n;
  const size_t nv = 3 * (size_t)n;
  F32Shape shape{1, 1, 2};
  int st = tune_f32(w, ncol, shape);
  if (st) return st;
  // x = 0; p = h = 0 so that an update step with alpha = 0 only forms
  // z = alpha_pol r and the partial r.z
  cudaMemsetAsync(w.x32, 0, ncol * nv * sizeof(float), st_);
  cudaMemsetAsync(w.p32, 0, ncol * nv * sizeof(float), st_);
  cudaMemsetAsync(w.h32, 0, ncol * nv * sizeof(float), st_);
  for (int k = 0; k < ncol; ++k) {
    gpu::CgCol c{};
    c.active = 1;
    c.tol = eta;
    w.cols_h[k] = c;
  }
  cudaMemcpyAsync(w.cols, w.cols_h, ncol * sizeof(gpu::CgCol), cudaMemcpyHostToDevice, st_);
  // z = M^-1 r: the diagonal (fused in the update) or the block-Jacobi blocks
  const bool blocks = inner_precond_ >= 1 && blk_info_;
  const bool near = blocks && near_precond();
  auto precondition = [&]() {
    if (!blocks) return;
    gpu::launch_block_apply(ncol, n, blk_info_, blk_minv_, w.r32, w.z32, st_);
    // h32 (T p) is spent by the update above: scratch of the Neumann step
    if (near) gpu::launch_near_correct(ncol, n, blk_info_, blk_minv_, near_ri_, near_ci_, near_blk_, w.z32, w.h32, st_);
    gpu::launch_dots_f32(ncol, nv, w.r32, w.z32, w.partial, st_);
  };
  gpu::launch_cg_update_f32(ncol, n, w.x32, w.r32, w.p32, w.h32, w.z32, alpha32_, w.cols, w.partial, st_);
  precondition();
  gpu::launch_reduce_partials(ncol, w.partial, w.dots, st_);
  cudaMemcpyAsync(w.p32, w.z32, ncol * nv * sizeof(float), cudaMemcpyDeviceToDevice, st_);
  cudaMemcpyAsync(w.scal_h, w.dots, ncol * sizeof(double), cudaMemcpyDeviceToHost, st_);
  st = check(cudaStreamSynchronize(st_), "inner CG init");
  if (st) return st;
  for (int k = 0; k < ncol; ++k) {
    gpu::CgCol c{};
    c.gold = w.scal_h[k];
    c.tol = eta;
    c.active = w.scal_h[k] > 0.0 ? 1 : 0;
    w.cols_h[k] = c;
  }
  cudaMemcpyAsync(w.cols, w.cols_h, ncol * sizeof(gpu::CgCol), cudaMemcpyHostToDevice, st_);
  auto iteration = [&]() {
    f32_product(w, ncol, shape);
    gpu::launch_dots_f32(ncol, nv, w.h32, w.p32, w.partial, st_);
    gpu::launch_reduce_partials(ncol, w.partial, w.dots, st_);
    gpu::launch_cg_alpha(ncol, w.dots, w.cols, 1e-300, st_);
    gpu::launch_cg_update_f32(ncol, n, w.x32, w.r32, w.p32, w.h32, w.z32, alpha32_, w.cols, w.partial, st_);
    precondition();
    gpu::launch_reduce_partials(ncol, w.partial, w.dots, st_);
    gpu::launch_cg_gnew(ncol, n, w.dots, w.cols, nullptr, 0, st_);
    gpu::launch_cg_pupdate_f32(ncol, n, w.p32, w.z32, w.cols, st_);
    cudaMemcpyAsync(w.cols_h, w.cols, ncol * sizeof(gpu::CgCol), cudaMemcpyDeviceToHost, st_);
  };
  // capture one iteration as a graph (kernel arguments and buffers are fixed
  // per workspace, width and launch shape; the tolerance lives in w.cols)
  if (use_graphs_ && (w.graph_ncol != ncol || w.graph_gmax != shape.g || w.graph_nsplit != shape.nsplit ||
                     w.graph_kver != shape.kver || w.graph_prec != (near ? 2 : blocks ? 1 : 0))) {
    if (w.graph) cudaGraphExecDestroy(w.graph);
    w.graph = nullptr;
    w.graph_ncol = -1;
    cudaGraph_t g = nullptr;
    long long before = gpu::thread_launch_count();
    if (cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      iteration();
      cudaError_t e = cudaStreamEndCapture(st_, &g);
      long long kernels = gpu::thread_launch_count() - before;
      gpu::add_launch_count(-kernels);  // captured, not launched
      if (e == cudaSuccess && g && cudaGraphInstantiate(&w.graph, g, 0) == cudaSuccess) {
        w.graph_ncol = ncol;
        w.graph_gmax = shape.g;
        w.graph_nsplit = shape.nsplit;
        w.graph_kver = shape.kver;
        w.graph_prec = near ? 2 : blocks ? 1 : 0;
        w.graph_kernels = kernels;
      } else {
        w.graph = nullptr;
        cudaGetLastError();
        log_msg(kVerbHigh, nullptr, "CUDA graph capture of the inner iteration failed: direct launches");
      }
      if (g) cudaGraphDestroy(g);
    } else {
      cudaGetLastError();
    }
  }
  const bool graph = use_graphs_ && w.graph && w.graph_ncol == ncol;
  int it = 0;
  for (it = 1; it <= max_it; ++it) {
    KEv ev;
    if (ktime_on_) ev = kt_begin(1, ncol);
    if (graph) {
      cudaGraphLaunch(w.graph, st_);
      gpu::add_launch_count(w.graph_kernels);
    } else {
      iteration();
    }
    if (ktime_on_) kt_end(ev);
    stats_.f32_matvecs += 1;
    st = check(cudaStreamSynchronize(st_), "inner CG iteration");
    if (st) return st;
    bool any = false;
    for (int k = 0; k < ncol; ++k) any |= w.cols_h[k].active != 0;
    if (!any) break;
  }
  stats_.inner_iters += std::min(it, max_it);
  return kOk;
}

// ---------------------------------------------------------------------------
// Iterative refinement: FP64 residual, FP32 inner PCG, FP64 accumulation
// ---------------------------------------------------------------------------
// The refinement residual after a step may be updated, r -= T d, with the
// FP32 product of the step's correction d (rms times the inner solution)
// instead of recomputing E - T mu: the FP32 operator is within 1e-5 of T
// (relative, the tested bound), so the updated residual is within 1e-5 rms
// of the recomputed one, which must stay below a tenth of the tolerance for
// every unconverged column (a converged column's correction is zero).  The
// first step (r = E) never qualifies: its correction is the whole solution.
bool System::update_allowed(const std::vector<double> &rms) const {
  if (!residual_update()) return false;
  for (double r : rms)
    if (r >= tol_ && !(kResidualUpdateRel * r <= 0.1 * tol_)) return false;
  return true;
}

int System::mixed_ir_ws(Workspace &w, int ncol, const double *rhs, double *x, int set0, bool have_guess) {
  const int n = d_.n;
  const size_t nv = 3 * (size_t)n;
  const int max_outer = 30;
  const int cap = w.cap;
  log_msg(kVerbLow, nullptr, "Solving linear system with mixed-precision CG (FP32 inner, FP64 refinement)");
  {
    const int pst = ensure_near();
    if (pst) return pst;
  }
  if (have_guess) {
    int st0 = matvec_residual(ncol, x, w.h);
    if (st0) return st0;
    gpu::launch_residual(ncol * nv, rhs, w.h, w.r, st_);
  } else {
    cudaMemsetAsync(x, 0, ncol * nv * sizeof(double), st_);
    cudaMemcpyAsync(w.r, rhs, ncol * nv * sizeof(double), cudaMemcpyDeviceToDevice, st_);
  }
  if (set0 >= 0)
    for (int k = 0; k < ncol && set0 + k < 2; ++k) stats_.hist[set0 + k].clear();
  std::vector<double> rms(ncol);
  int outer = 0;
  bool done = false;
  while (true) {
    gpu::launch_scale_by_alpha(ncol, n, d_.pol_alpha, w.r, w.z, st_);
    gpu::launch_dots(ncol, nv, w.r, w.z, w.partial, st_);
    gpu::launch_reduce_partials(ncol, w.partial, w.dots, st_);
    cudaMemcpyAsync(w.scal_h, w.dots, ncol * sizeof(double), cudaMemcpyDeviceToHost, st_);
    int st = check(cudaStreamSynchronize(st_), "refinement residual");
    if (st) return st;
    done = true;
    for (int k = 0; k < ncol; ++k) {
      rms[k] = std::sqrt(std::max(w.scal_h[k], 0.0) / (double)nv);
      if (set0 >= 0 && set0 + k < 2) stats_.hist[set0 + k].push_back(rms[k]);
      if (!std::isfinite(rms[k])) {
        set_last_error("non-finite residual in the refinement loop (coincident sites?)");
        return kErrNumeric;
      }
      if (!(rms[k] < tol_)) done = false;
      if (log_level() >= kVerbHigh)
        log_msg(kVerbHigh, nullptr, "refinement step %3d column %d residual rms norm: %14.4E", outer, k, rms[k]);
    }
    if (done || outer >= max_outer) break;
    // normalise each unconverged column to unit preconditioned rms; converged
    // columns get a zero right-hand side (the inner CG leaves them at zero)
    double eta = 1e-5;
    for (int k = 0; k < ncol; ++k) {
      w.scal_h[cap + k] = rms[k] < tol_ ? 0.0 : 1.0 / rms[k];
      w.scal_h[2 * cap + k] = rms[k] < tol_ ? 0.0 : rms[k];
      if (rms[k] >= tol_) eta = std::max(eta, std::min(1e-2, 0.3 * tol_ / rms[k]));
    }
    cudaMemcpyAsync(w.dots + cap, w.scal_h + cap, 2 * cap * sizeof(double), cudaMemcpyHostToDevice, st_);
    gpu::launch_to_f32_cols(ncol, nv, w.r, w.dots + cap, w.r32, st_);
    // batches of at least 4 columns share one Krylov space (block CG)
    if (block_cg_ && w.t32 && ncol >= 4 && ncol <= gpu::block_cg_max_columns())
      st = bpcg32_ws(w, ncol, 200, eta);
    else
      st = pcg32_ws(w, ncol, 200, eta);
    if (st) return st;
    gpu::launch_ir_accumulate(ncol, n, x, w.x32, w.dots + 2 * cap, st_);
    if (update_allowed(rms)) {
      // r -= rms T32 x32: the FP32 product of this step's correction
      F32Shape shape{1, 1, 2};
      st = tune_f32(w, ncol, shape);
      if (st) return st;
      cudaMemcpyAsync(w.p32, w.x32, ncol * nv * sizeof(float), cudaMemcpyDeviceToDevice, st_);
      f32_product(w, ncol, shape);
      stats_.f32_matvecs += 1;
      stats_.updates += 1;
      gpu::launch_residual_update(ncol, n, w.r, w.h32, w.dots + 2 * cap, st_);
    } else {
      st = matvec_residual(ncol, x, w.h);
      if (st) return st;
      gpu::launch_residual(ncol * nv, rhs, w.h, w.r, st_);
    }
    ++outer;
  }
  stats_.outer += outer;
  if (set0 >= 0)
    for (int k = 0; k < ncol && set0 + k < 2; ++k) stats_.iters[set0 + k] = outer;
  if (!done) {
    set_last_error("Iterative solver did not converged");
    return kErrNotConverged;
  }
  return kOk;
}

// ---------------------------------------------------------------------------
// Batched fields
// ---------------------------------------------------------------------------
int System::solve_batch(int nf, const double *fields, double *out, double *energies) {
  if (nf < 1) {
    set_last_error("batch: the number of fields must be positive");
    return kErrBadArg;
  }
  const int n = d_.n;
  const size_t nv = 3 * (size_t)n;
  if (n == 0) {
    if (energies)
      for (int f = 0; f < nf; ++f) energies[f] = 0.0;
    return kOk;
  }
  int st = ensure_m2d();
  if (st) return st;
  const int nipd = m_.n_ipd;
  int nsets = nipd;
  if (nipd == 2) {
    // identical D and P right-hand sides: one set of columns (see polarization)
    int differ = 1;
    cudaMemsetAsync(flag_, 0, sizeof(int), st_);
    gpu::launch_any_diff(nv, e_m2d_, e_m2d_ + nv, flag_, st_);
    cudaMemcpyAsync(&differ, flag_, sizeof(int), cudaMemcpyDeviceToHost, st_);
    st = check(cudaStreamSynchronize(st_), "batch D/P comparison");
    if (st) return st;
    if (!differ) nsets = 1;
  }
  const int ncol = nf * nsets;
  st = ensure_batch_ws(ncol, nf);
  if (st) return st;
  Workspace &w = wsb_;
  stats_ = SolveStats();
  cudaEventRecord(ev0_, st_);
  gpu::launch_batch_rhs(n, nf, nsets, e_m2d_, fields, w.rhs, st_);
  cudaMemsetAsync(w.x, 0, ncol * nv * sizeof(double), st_);
  if (precision_ != kPrecFP64) {
    st = mixed_ir_ws(w, ncol, w.rhs, w.x, -1, false);
  } else {
    int matv = def_matv_ == kMatvIncore ? kMatvIncore : kMatvDirect;
    if (matv == kMatvIncore && ensure_tmat() != kOk) matv = kMatvDirect;
    st = cg64_ws(w, matv, nf, w.rhs, w.x, -1);
    if (!st && nsets == 2) {
      // P seeded with D (mod_polarization.F90:237-243)
      cudaMemcpyAsync(w.x + nf * nv, w.x, nf * nv * sizeof(double), cudaMemcpyDeviceToDevice, st_);
      st = cg64_ws(w, matv, nf, w.rhs + nf * nv, w.x + nf * nv, -1);
    }
  }
  if (st) return st;
  gpu::launch_batch_scatter(n, nf, nipd, nsets, w.x, out, st_);
  if (energies) {
    // -1/2 ipd(D) . E_M2D(P) per field (AMOEBA), -1/2 ipd . E_M2D otherwise
    const double *ef = m_.amoeba ? e_m2d_ + nv : e_m2d_;
    gpu::launch_dots_bcast(nf, nv, w.x, ef, w.partial, st_);
    gpu::launch_reduce_partials(nf, w.partial, w.dots, st_);
    cudaMemcpyAsync(w.scal_h, w.dots, nf * sizeof(double), cudaMemcpyDeviceToHost, st_);
  }
  cudaEventRecord(ev1_, st_);
  st = check(cudaStreamSynchronize(st_), "batch solve");
  if (st) return st;
  if (energies)
    for (int f = 0; f < nf; ++f) energies[f] = -0.5 * w.scal_h[f];
  cudaEventElapsedTime(&last_ms_, ev0_, ev1_);
  return kOk;
}

int System::solve_batch_host(int nf, const double *fields_host, double *out_host, double *energies) {
  if (nf < 1) {
    set_last_error("batch: the number of fields must be positive");
    return kErrBadArg;
  }
  const size_t nv = 3 * (size_t)d_.n;
  const int nsets_max = m_.n_ipd;
  int st = ensure_batch_ws(nf * nsets_max, nf);
  if (st) return st;
  cudaMemcpyAsync(wsb_.fields, fields_host, nf * nv * sizeof(double), cudaMemcpyHostToDevice, st_);
  st = solve_batch(nf, wsb_.fields, wsb_.out, energies);
  if (st) return st;
  cudaMemcpyAsync(out_host, wsb_.out, (size_t)nf * m_.n_ipd * nv * sizeof(double), cudaMemcpyDeviceToHost, st_);
  return check(cudaStreamSynchronize(st_), "batch copy-out");
}

}  // namespace ommp
