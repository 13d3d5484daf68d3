// Mixed-precision polarization solves of several systems advanced together.
//
// The reference solves one system per call (polarization,
// src/mod_polarization.F90:49-313, with the CG of src/mod_solvers.F90:86-216).
// A server holding many systems of very different sizes would otherwise run
// one solve per CUDA stream, and the symmetric pair kernels, persistent grids
// that fill the whole GPU, would run one system's product after another.
// Here one engine stream advances every queued solve in rounds:
//
//   * every solve is the iterative refinement of System::mixed_ir_ws (FP64 or
//     double-single residual E - T mu, convergence test on the reference's
//     rms of alpha r, FP32 inner PCG on the normalised residual, FP64
//     accumulation), written as a state machine;
//   * in each round, all systems that need a pair product share one launch
//     per product kind (FP32 inner product, FP64 or double-single residual
//     product) and column width: a persistent kernel whose work items are
//     (system, super-tile, chunk of slots), taken in order from one counter
//     (the launch_*_sym_multi kernels);
//   * a product gets a bounded share of each round (about 1.5 ms of work per
//     kind by default, set_round_ms: a fair share per system first, then the
//     shortest products), so
//     small systems finish their iterations while a large system's product
//     is spread over several rounds; its fixed-point sums simply continue;
//     work items are cut to a quarter of a resident CTA's share of a round
//     (SymSlice::round_pairs), so that every CTA stays busy for the whole
//     round whatever the systems' sizes;
//   * after the launches, every system whose product completed runs its CG
//     bookkeeping (finishing pass, dots, updates, convergence flags) on the
//     same stream, and one synchronisation per round brings the flags to
//     the host, where each solve takes its next step.
//
// Results equal those of the single-system solve to rounding: the products
// are the same symmetric kernels (the FP64 one also below 2048 sites, where
// the single-system path uses the target-outer kernel).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>

#include "../../include/openmmpol_gb300.h"
#include "log.h"
#include "multisolve.h"

namespace ommp {

namespace {
enum Stage {
  kStart,        // right-hand sides ready: first residual (or its product)
  kProduct,      // a pair product in progress
  kAwaitCheck,   // residual rms on its way to the host
  kInnerInit,    // start of an inner PCG
  kAwaitInner,   // inner PCG flags on their way to the host
  kAccumulate,   // inner PCG done: accumulate, then the residual product
  kFinalize,     // converged: dipoles, energy
  kAwaitDone,
  kFinished,
};
enum Kind { kNone, kF32, kF64, kDS };
constexpr int kMaxOuter = 30;
constexpr int kMaxInner = 200;
// pairs per millisecond of the symmetric kernels on GB300 per product kind
// (measured: FP32 8.6e11, FP64 1.76e10, double-single 8.6e10 pairs/s); a
// round's budget is round_ms_ of work per kind
constexpr double kPairsPerMs[4] = {0.0, 8.6e8, 1.76e7, 8.6e7};
}  // namespace

struct MultiSolver::Job {
  long long id = 0;
  System *s = nullptr;
  int ncol = 1;
  bool copy_p = false, guess = false;
  int stage = kStart;
  int kind = kNone, items = 0, done = 0, launches = 0;
  double round_pairs = 0.0;  // item size of the product in flight (SymSlice::round_pairs)
  bool update = false;       // the FP32 product in flight updates the residual
  std::vector<double> rms;   // residual rms of the last check, per column
  int outer = 0, inner = 0;
  double eta = 1e-5;
  int status = kOk;
  double energy = 0.0;
  std::string err;
};

MultiSolver::MultiSolver() {
  // the rounds run at the highest stream priority: their products and
  // bookkeeping go ahead of work queued on other streams (a request server's
  // uploads and permanent fields of new systems), which fills the gaps
  int least = 0, greatest = 0;
  cudaDeviceGetStreamPriorityRange(&least, &greatest);
  if (cudaStreamCreateWithPriority(&st_, cudaStreamNonBlocking, greatest) != cudaSuccess) {
    cudaGetLastError();
    cudaStreamCreateWithFlags(&st_, cudaStreamNonBlocking);
  }
  for (cudaEvent_t &e : ev_) cudaEventCreate(&e);
  cudaMalloc((void **)&counters_, 64 * sizeof(unsigned));
}

MultiSolver::~MultiSolver() {
  if (st_) cudaStreamSynchronize(st_);
  for (Job *j : pending_) delete j;
  for (Job *j : jobs_) delete j;
  for (auto &kv : done_) delete kv.second;
  if (counters_) cudaFree(counters_);
  for (cudaEvent_t e : ev_)
    if (e) cudaEventDestroy(e);
  if (st_) cudaStreamDestroy(st_);
}

long long MultiSolver::add(System *s, const double *ext_host, int &status) {
  status = kOk;
  if (!st_ || !counters_) {
    set_last_error("multi-system solver: no engine stream");
    status = kErrCuda;
    return -1;
  }
  if (s->precision_ == kPrecFP64 || s->fmm_on_) {
    set_last_error("multi-system solver: the mixed modes with direct products only");
    status = kErrBadArg;
    return -1;
  }
  const gpu::DevSites &d = s->d_;
  const size_t nv = 3 * (size_t)d.n;
  const int nipd = s->m_.n_ipd;
  s->stats_ = SolveStats();
  s->ipd_done_ = false;
  cudaStream_t sst = s->st_;
  int st = kOk;
  if (d.n > 0) {
    cudaMemcpyAsync(s->ext_, ext_host, nv * sizeof(double), cudaMemcpyHostToDevice, sst);
    st = s->ensure_m2d();
    if (!st) st = s->ensure_sym_scratch();
    if (!st) st = s->ensure_near();
  }
  auto *j = new Job();
  j->s = s;
  j->guess = s->ipd_use_guess_;
  if (!st && d.n > 0) {
    for (int k = 0; k < nipd; ++k) gpu::launch_add(nv, s->e_m2d_ + k * nv, s->ext_, s->rhs_ + k * nv, sst);
    cudaMemsetAsync(s->x_, 0, nv * nipd * sizeof(double), sst);
    if (j->guess) cudaMemcpyAsync(s->x_, s->ipd_, nv * nipd * sizeof(double), cudaMemcpyDeviceToDevice, sst);
    j->ncol = nipd;
    if (nipd == 2) {
      // identical D and P systems (AMOEBA water) are solved once
      cudaMemsetAsync(s->flag_, 0, sizeof(int), sst);
      gpu::launch_any_diff(nv, s->rhs_, s->rhs_ + nv, s->flag_, sst);
      if (j->guess) gpu::launch_any_diff(nv, s->x_, s->x_ + nv, s->flag_, sst);
      int differ = 1;
      cudaMemcpyAsync(&differ, s->flag_, sizeof(int), cudaMemcpyDeviceToHost, sst);
      st = s->check(cudaStreamSynchronize(sst), "D/P comparison");
      if (!differ) {
        j->ncol = 1;
        j->copy_p = true;
      }
    }
    if (!st) st = s->check(cudaStreamSynchronize(sst), "solve preparation");
  }
  if (st) {
    delete j;
    status = st;
    return -1;
  }
  if (d.n == 0) j->stage = kFinalize;
  std::lock_guard<std::mutex> lk(mu_);
  j->id = ++next_id_;
  pending_.push_back(j);
  return j->id;
}

void MultiSolver::set_round_ms(double ms) {
  std::lock_guard<std::mutex> lk(mu_);
  if (ms > 0.0 && std::isfinite(ms)) round_ms_ = ms;
}

double MultiSolver::round_pairs(int kind) {
  std::lock_guard<std::mutex> lk(mu_);
  return kPairsPerMs[kind] * round_ms_;
}

bool MultiSolver::idle() {
  std::lock_guard<std::mutex> lk(mu_);
  return pending_.empty() && jobs_.empty();
}

bool MultiSolver::take(long long id, int &status, double &energy, std::string &err) {
  std::lock_guard<std::mutex> lk(mu_);
  auto it = done_.find(id);
  if (it == done_.end()) return false;
  status = it->second->status;
  energy = it->second->energy;
  err = it->second->err;
  delete it->second;
  done_.erase(it);
  return true;
}

MultiSolver::Stats MultiSolver::stats() {
  std::lock_guard<std::mutex> lk(mu_);
  return stats_;
}

void MultiSolver::fail(Job &j, int status, const std::string &err) {
  j.status = status;
  j.err = err;
  j.stage = kFinished;
}

// Plan this round's share of every product in progress and launch it: one
// launch per kind, column width (and damping kind for the FP64 and
// double-single kernels) and group of at most kMaxSymSlices systems.
int MultiSolver::launch_products(std::vector<Job *> &active) {
  std::vector<Job *> prod;
  for (Job *j : active)
    if (j->stage == kProduct) prod.push_back(j);
  std::map<Job *, int> take;
  for (int kind = kF32; kind <= kDS; ++kind) {
    std::vector<Job *> js;
    for (Job *j : prod)
      if (j->kind == kind) js.push_back(j);
    if (js.empty()) continue;
    auto ppi = [](const Job *j) {
      const double n = j->s->d_.n;
      return std::max(1.0, 0.5 * n * (n - 1.0) / std::max(1, j->items));
    };
    const double budget = round_pairs(kind);
    double used = 0.0;
    const double share = budget / js.size();
    for (Job *j : js) {
      const int rem = j->items - j->done;
      const int t = (int)std::min((double)rem, std::max(1.0, std::floor(share / ppi(j))));
      take[j] = t;
      used += t * ppi(j);
    }
    // what is left goes to the shortest products first
    std::sort(js.begin(), js.end(), [&](const Job *a, const Job *b) {
      return (a->items - a->done) * ppi(a) < (b->items - b->done) * ppi(b);
    });
    for (Job *j : js) {
      if (used >= budget) break;
      const int rem = j->items - j->done - take[j];
      if (rem <= 0) continue;
      const int extra = (int)std::min((double)rem, std::floor((budget - used) / ppi(j)));
      take[j] += extra;
      used += extra * ppi(j);
    }
  }
  // zero the accumulators of products that start now
  for (auto &kv : take) {
    Job *j = kv.first;
    if (j->done > 0) continue;
    const size_t C = 3 * (size_t)j->ncol, n = j->s->d_.n;
    double *sym = j->s->sym_scratch_;
    cudaMemsetAsync(sym, 0, 2 * C * n * sizeof(unsigned long long), st_);
    cudaMemsetAsync(sym + 3 * C * n, 0, sizeof(unsigned long long), st_);
  }
  // group and launch
  struct Key {
    int kind, g, amoeba;
    bool operator<(const Key &o) const {
      return kind != o.kind ? kind < o.kind : (g != o.g ? g < o.g : amoeba < o.amoeba);
    }
  };
  std::map<Key, std::vector<Job *>> groups;
  for (auto &kv : take) {
    Job *j = kv.first;
    groups[{j->kind, j->ncol, j->kind == kF32 ? 0 : (j->s->d_.amoeba ? 1 : 0)}].push_back(j);
  }
  int nlaunch = 0;
  for (auto &kv : groups) {
    std::vector<Job *> &js = kv.second;
    for (size_t b = 0; b < js.size(); b += gpu::kMaxSymSlices) {
      std::vector<gpu::SymSlice> sl;
      for (size_t k = b; k < js.size() && k < b + gpu::kMaxSymSlices; ++k) {
        Job *j = js[k];
        System *s = j->s;
        const size_t C = 3 * (size_t)j->ncol, n = s->d_.n;
        unsigned long long *lo = reinterpret_cast<unsigned long long *>(s->sym_scratch_);
        const void *x = j->kind == kF32 ? static_cast<const void *>(s->ws_.p32) : static_cast<const void *>(s->x_);
        sl.push_back({&s->d_, x, lo, lo + C * n, reinterpret_cast<unsigned long long *>(s->sym_scratch_ + 3 * C * n),
                      j->done, take[j], j->round_pairs});
      }
      const int g = kv.first.g;
      if (kv.first.kind == kF32)
        gpu::launch_tmu32_sym_multi(g, sl.data(), (int)sl.size(), counters_, st_);
      else if (kv.first.kind == kF64)
        gpu::launch_tmu_f64_sym_multi(g, kv.first.amoeba != 0, sl.data(), (int)sl.size(), counters_, st_);
      else
        gpu::launch_tmu_ds_sym_multi(g, kv.first.amoeba != 0, sl.data(), (int)sl.size(), counters_, st_);
      ++nlaunch;
      std::lock_guard<std::mutex> lk(mu_);
      stats_.launches += 1;
      if (sl.size() >= 2) stats_.shared_launches += 1;
      stats_.max_systems = std::max<long long>(stats_.max_systems, (long long)sl.size());
    }
  }
  for (auto &kv : take) {
    kv.first->done += kv.second;
    kv.first->launches += 1;
  }
  return nlaunch;
}

// The bookkeeping after a system's product (which 0: the rest of the FP32
// inner PCG iteration; 1: the refinement residual and its rms; 2: the
// residual updated by the FP32 product of the correction), on the engine
// stream, launched directly.  Capturing it as a CUDA graph per system and
// column count was measured slower in a request stream: every new system
// paid the graph's instantiation, more than its replays saved.
void MultiSolver::enqueue_tail(Job &j, int which) {
  System &s = *j.s;
  const gpu::DevSites &d = s.d_;
  const int n = d.n, ncol = j.ncol;
  const size_t nv = 3 * (size_t)n, C = 3 * (size_t)ncol;
  Workspace &w = s.ws_;
  unsigned long long *lo = reinterpret_cast<unsigned long long *>(s.sym_scratch_);
  unsigned long long *hi = lo + C * n;
  unsigned long long *bad = reinterpret_cast<unsigned long long *>(s.sym_scratch_ + 3 * C * n);
  if (which == 2) {
    // r -= rms T32 d: the FP32 product of the correction (System::update_allowed)
    float *e = reinterpret_cast<float *>(s.sym_scratch_ + 2 * C * n);
    gpu::launch_fixed_to_float(C * n, lo, hi, bad, e, st_);
    gpu::launch_tmu_finish32(d, ncol, e, w.p32, w.h32, st_);
    gpu::launch_residual_update(ncol, n, w.r, w.h32, w.dots + 2 * w.cap, st_);
    gpu::launch_scale_by_alpha(ncol, n, d.pol_alpha, w.r, w.z, st_);
    gpu::launch_dots(ncol, nv, w.r, w.z, w.partial, st_);
    gpu::launch_reduce_partials(ncol, w.partial, w.dots, st_);
    cudaMemcpyAsync(w.scal_h, w.dots, ncol * sizeof(double), cudaMemcpyDeviceToHost, st_);
  } else if (which == 0) {
    float *e = reinterpret_cast<float *>(s.sym_scratch_ + 2 * C * n);
    gpu::launch_fixed_to_float(C * n, lo, hi, bad, e, st_);
    gpu::launch_tmu_finish32(d, ncol, e, w.p32, w.h32, st_);
    // the rest of pcg32_ws's iteration
    gpu::launch_dots_f32(ncol, nv, w.h32, w.p32, w.partial, st_);
    gpu::launch_reduce_partials(ncol, w.partial, w.dots, st_);
    gpu::launch_cg_alpha(ncol, w.dots, w.cols, 1e-300, st_);
    gpu::launch_cg_update_f32(ncol, n, w.x32, w.r32, w.p32, w.h32, w.z32, s.alpha32_, w.cols, w.partial, st_);
    if (s.inner_precond_ >= 1 && s.blk_info_) {
      gpu::launch_block_apply(ncol, n, s.blk_info_, s.blk_minv_, w.r32, w.z32, st_);
      if (s.near_precond())
        gpu::launch_near_correct(ncol, n, s.blk_info_, s.blk_minv_, s.near_ri_, s.near_ci_, s.near_blk_, w.z32, w.h32,
                                 st_);
      gpu::launch_dots_f32(ncol, nv, w.r32, w.z32, w.partial, st_);
    }
    gpu::launch_reduce_partials(ncol, w.partial, w.dots, st_);
    gpu::launch_cg_gnew(ncol, n, w.dots, w.cols, nullptr, 0, st_);
    gpu::launch_cg_pupdate_f32(ncol, n, w.p32, w.z32, w.cols, st_);
    cudaMemcpyAsync(w.cols_h, w.cols, ncol * sizeof(gpu::CgCol), cudaMemcpyDeviceToHost, st_);
  } else {
    double *e = s.sym_scratch_ + 2 * C * n;
    gpu::launch_fixed_to_double(C * n, lo, hi, bad, e, st_);
    gpu::launch_tmu_finish64(d, ncol, e, s.x_, true, w.h, st_);
    gpu::launch_residual(ncol * nv, s.rhs_, w.h, w.r, st_);
    gpu::launch_scale_by_alpha(ncol, n, d.pol_alpha, w.r, w.z, st_);
    gpu::launch_dots(ncol, nv, w.r, w.z, w.partial, st_);
    gpu::launch_reduce_partials(ncol, w.partial, w.dots, st_);
    cudaMemcpyAsync(w.scal_h, w.dots, ncol * sizeof(double), cudaMemcpyDeviceToHost, st_);
  }
}

int MultiSolver::tick() {
  {
    std::lock_guard<std::mutex> lk(mu_);
    for (Job *j : pending_) jobs_.push_back(j);
    pending_.clear();
  }
  if (jobs_.empty()) return 0;
  const auto wall0 = std::chrono::steady_clock::now();
  bool work = false;
  // ---- steps decided in the previous round ----------------------------------
  for (Job *jp : jobs_) {
    Job &j = *jp;
    System &s = *j.s;
    const gpu::DevSites &d = s.d_;
    const int n = d.n, ncol = j.ncol, cap = s.ws_.cap;
    const size_t nv = 3 * (size_t)n;
    Workspace &w = s.ws_;
    switch (j.stage) {
      case kStart:
        if (j.guess) {
          j.stage = kProduct;
          j.kind = s.precision_ == kPrecMixedDS ? kDS : kF64;
          j.round_pairs = round_pairs(j.kind);
          j.items = j.kind == kDS ? gpu::tmu_ds_sym_items(d, ncol, j.round_pairs)
                                  : gpu::tmu_f64_sym_items(d, ncol, j.round_pairs);
          j.done = j.launches = 0;
        } else {
          cudaMemcpyAsync(w.r, s.rhs_, ncol * nv * sizeof(double), cudaMemcpyDeviceToDevice, st_);
          gpu::launch_scale_by_alpha(ncol, n, d.pol_alpha, w.r, w.z, st_);
          gpu::launch_dots(ncol, nv, w.r, w.z, w.partial, st_);
          gpu::launch_reduce_partials(ncol, w.partial, w.dots, st_);
          cudaMemcpyAsync(w.scal_h, w.dots, ncol * sizeof(double), cudaMemcpyDeviceToHost, st_);
          j.stage = kAwaitCheck;
          work = true;
        }
        break;
      case kInnerInit: {
        // pcg32_ws's start, with the first r.z kept on the device
        cudaMemcpyAsync(w.dots + cap, w.scal_h + cap, 2 * cap * sizeof(double), cudaMemcpyHostToDevice, st_);
        gpu::launch_to_f32_cols(ncol, nv, w.r, w.dots + cap, w.r32, st_);
        cudaMemsetAsync(w.x32, 0, ncol * nv * sizeof(float), st_);
        cudaMemsetAsync(w.p32, 0, ncol * nv * sizeof(float), st_);
        cudaMemsetAsync(w.h32, 0, ncol * nv * sizeof(float), st_);
        for (int k = 0; k < ncol; ++k) {
          gpu::CgCol c{};
          c.active = 1;
          c.tol = j.eta;
          w.cols_h[k] = c;
        }
        cudaMemcpyAsync(w.cols, w.cols_h, ncol * sizeof(gpu::CgCol), cudaMemcpyHostToDevice, st_);
        gpu::launch_cg_update_f32(ncol, n, w.x32, w.r32, w.p32, w.h32, w.z32, s.alpha32_, w.cols, w.partial, st_);
        if (s.inner_precond_ >= 1 && s.blk_info_) {
          gpu::launch_block_apply(ncol, n, s.blk_info_, s.blk_minv_, w.r32, w.z32, st_);
          if (s.near_precond())
            gpu::launch_near_correct(ncol, n, s.blk_info_, s.blk_minv_, s.near_ri_, s.near_ci_, s.near_blk_, w.z32,
                                     w.h32, st_);
          gpu::launch_dots_f32(ncol, nv, w.r32, w.z32, w.partial, st_);
        }
        gpu::launch_reduce_partials(ncol, w.partial, w.dots, st_);
        cudaMemcpyAsync(w.p32, w.z32, ncol * nv * sizeof(float), cudaMemcpyDeviceToDevice, st_);
        gpu::launch_cg_init(ncol, w.dots, w.cols, j.eta, st_);
        j.stage = kProduct;
        j.kind = kF32;
        j.round_pairs = round_pairs(kF32);
        j.items = gpu::tmu32_sym_items(d, ncol, j.round_pairs);
        j.done = j.launches = 0;
        j.inner = 1;
        work = true;
        break;
      }
      case kAccumulate:
        gpu::launch_ir_accumulate(ncol, n, s.x_, w.x32, w.dots + 2 * cap, st_);
        j.stage = kProduct;
        j.update = s.update_allowed(j.rms);
        if (j.update) {
          // the residual is updated by the FP32 product of the correction
          cudaMemcpyAsync(w.p32, w.x32, ncol * nv * sizeof(float), cudaMemcpyDeviceToDevice, st_);
          j.kind = kF32;
          j.round_pairs = round_pairs(kF32);
          j.items = gpu::tmu32_sym_items(d, ncol, j.round_pairs);
        } else {
          j.kind = s.precision_ == kPrecMixedDS ? kDS : kF64;
          j.round_pairs = round_pairs(j.kind);
          j.items = j.kind == kDS ? gpu::tmu_ds_sym_items(d, ncol, j.round_pairs)
                                  : gpu::tmu_f64_sym_items(d, ncol, j.round_pairs);
        }
        j.done = j.launches = 0;
        ++j.outer;
        work = true;
        break;
      case kFinalize: {
        const int nipd = s.m_.n_ipd;
        if (n > 0) {
          if (j.copy_p) cudaMemcpyAsync(s.x_ + nv, s.x_, nv * sizeof(double), cudaMemcpyDeviceToDevice, st_);
          cudaMemcpyAsync(s.ipd_, s.x_, nv * nipd * sizeof(double), cudaMemcpyDeviceToDevice, st_);
          const double *ef = s.m_.amoeba ? s.e_m2d_ + nv : s.e_m2d_;
          gpu::launch_dots(1, nv, s.ipd_, ef, w.partial, st_);
          gpu::launch_reduce_partials(1, w.partial, w.dots, st_);
          cudaMemcpyAsync(w.scal_h, w.dots, sizeof(double), cudaMemcpyDeviceToHost, st_);
          cudaMemcpyAsync(s.ipd_h_.data(), s.ipd_, s.ipd_h_.size() * sizeof(double), cudaMemcpyDeviceToHost, st_);
        } else {
          w.scal_h[0] = 0.0;
        }
        j.stage = kAwaitDone;
        work = true;
        break;
      }
      default:
        break;
    }
  }
  // ---- this round's share of every product -----------------------------------
  cudaEventRecord(ev_[0], st_);
  const bool launched = launch_products(jobs_) > 0;
  if (launched) work = true;
  cudaEventRecord(ev_[1], st_);
  // ---- bookkeeping of the products that completed ----------------------------
  for (Job *jp : jobs_) {
    Job &j = *jp;
    if (j.stage != kProduct || j.done < j.items) continue;
    System &s = *j.s;
    if (j.launches > 1) {
      std::lock_guard<std::mutex> lk(mu_);
      stats_.spread_products += 1;
    }
    if (j.kind == kF32 && j.update) {
      s.stats_.f32_matvecs += 1;
      s.stats_.updates += 1;
      enqueue_tail(j, 2);
      j.update = false;
      j.stage = kAwaitCheck;
    } else if (j.kind == kF32) {
      s.stats_.f32_matvecs += 1;
      enqueue_tail(j, 0);
      j.stage = kAwaitInner;
    } else {
      if (j.kind == kDS)
        s.stats_.ds_matvecs += 1;
      else
        s.stats_.f64_matvecs += 1;
      enqueue_tail(j, 1);
      j.stage = kAwaitCheck;
    }
    j.kind = kNone;
    work = true;
  }
  cudaEventRecord(ev_[2], st_);
  if (work) {
    cudaError_t e = cudaStreamSynchronize(st_);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) {
      float pm = 0.f, tm = 0.f;
      cudaEventElapsedTime(&pm, ev_[0], ev_[1]);
      cudaEventElapsedTime(&tm, ev_[1], ev_[2]);
      std::lock_guard<std::mutex> lk(mu_);
      stats_.product_ms += pm;
      stats_.tail_ms += tm;
    }
    if (e != cudaSuccess) {
      const std::string msg = std::string("multi-system solver: ") + cudaGetErrorString(e);
      for (Job *j : jobs_) fail(*j, kErrCuda, msg);
    }
  }
  // ---- decisions -----------------------------------------------------------------
  for (Job *jp : jobs_) {
    Job &j = *jp;
    if (j.stage == kFinished) continue;
    System &s = *j.s;
    const int n = s.d_.n, ncol = j.ncol, cap = s.ws_.cap;
    const size_t nv = 3 * (size_t)n;
    Workspace &w = s.ws_;
    if (j.stage == kAwaitCheck) {
      bool done = true;
      std::vector<double> rms(ncol);
      for (int k = 0; k < ncol; ++k) {
        rms[k] = std::sqrt(std::max(w.scal_h[k], 0.0) / (double)nv);
        if (k < 2) s.stats_.hist[k].push_back(rms[k]);
        if (!(rms[k] < s.tol_)) done = false;
      }
      j.rms = rms;
      bool finite = true;
      for (double r : rms) finite = finite && std::isfinite(r);
      if (!finite) {
        fail(j, kErrNumeric, "non-finite residual in the refinement loop (coincident sites?)");
      } else if (done) {
        j.stage = kFinalize;
      } else if (j.outer >= kMaxOuter) {
        fail(j, kErrNotConverged, "Iterative solver did not converged");
      } else {
        double eta = 1e-5;
        for (int k = 0; k < ncol; ++k) {
          w.scal_h[cap + k] = rms[k] < s.tol_ ? 0.0 : 1.0 / rms[k];
          w.scal_h[2 * cap + k] = rms[k] < s.tol_ ? 0.0 : rms[k];
          if (rms[k] >= s.tol_) eta = std::max(eta, std::min(1e-2, 0.3 * s.tol_ / rms[k]));
        }
        j.eta = eta;
        j.stage = kInnerInit;
      }
    } else if (j.stage == kAwaitInner) {
      bool any = false;
      for (int k = 0; k < ncol; ++k) any |= w.cols_h[k].active != 0;
      if (any && j.inner < kMaxInner) {
        j.stage = kProduct;
        j.kind = kF32;
        j.round_pairs = round_pairs(kF32);
        j.items = gpu::tmu32_sym_items(s.d_, ncol, j.round_pairs);
        j.done = j.launches = 0;
        ++j.inner;
      } else {
        s.stats_.inner_iters += j.inner;
        j.stage = kAccumulate;
      }
    } else if (j.stage == kAwaitDone) {
      j.energy = -0.5 * w.scal_h[0];
      s.stats_.outer = j.outer;
      s.stats_.iters[0] = j.outer;
      if (j.copy_p || ncol == 2) s.stats_.iters[1] = j.outer;
      if (j.copy_p) s.stats_.hist[1] = s.stats_.hist[0];
      s.ipd_done_ = true;
      s.ipd_use_guess_ = true;
      j.stage = kFinished;
    }
  }
  // ---- hand over the finished jobs -------------------------------------------
  int finished = 0;
  std::vector<Job *> keep;
  std::lock_guard<std::mutex> lk(mu_);
  stats_.ticks += 1;
  stats_.wall_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - wall0).count();
  for (Job *j : jobs_) {
    if (j->stage == kFinished) {
      done_[j->id] = j;
      ++finished;
      stats_.finished += 1;
    } else {
      keep.push_back(j);
    }
  }
  jobs_.swap(keep);
  return finished;
}

}  // namespace ommp

using ommp::MultiSolver;

extern "C" {

// No counterpart in the reference: the solves of several systems, each with
// its own field [pol_atoms][3] (host), advanced together with shared
// multi-system product launches.  energies [nsys]; stats5 (may be NULL):
// rounds, product launches, launches that served two or more systems, most
// systems in one launch, products spread over several launches.
int32_t ommp_gpu_solve_multi(int32_t nsys, OMMP_SYSTEM_PRT *systems, const double *const *fields, double *energies,
                             int64_t *stats5) {
  if (nsys < 1 || !systems || !fields) {
    ommp::set_last_error("solve_multi: no systems");
    return ommp::kErrBadArg;
  }
  MultiSolver ms;
  std::vector<long long> ids(nsys, -1);
  int rc = ommp::kOk;
  for (int k = 0; k < nsys && !rc; ++k) {
    int st = ommp::kOk;
    ids[k] = ms.add(static_cast<ommp::System *>(systems[k]), fields[k], st);
    if (st) rc = st;
  }
  std::string first_err = rc ? ommp::last_error() : "";
  while (!ms.idle()) ms.tick();
  for (int k = 0; k < nsys; ++k) {
    if (ids[k] < 0) continue;
    int st = ommp::kOk;
    double e = 0.0;
    std::string err;
    ms.take(ids[k], st, e, err);
    if (energies) energies[k] = e;
    if (st && !rc) {
      rc = st;
      first_err = err;
    }
  }
  if (stats5) {
    const MultiSolver::Stats s = ms.stats();
    stats5[0] = s.ticks, stats5[1] = s.launches, stats5[2] = s.shared_launches, stats5[3] = s.max_systems,
    stats5[4] = s.spread_products;
  }
  if (rc) ommp::set_last_error(first_err);
  return rc;
}

}  // extern "C"
