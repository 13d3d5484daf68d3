// Request server: continuous admission of polarization solves on one GPU.
//
// Requests are either "new" (a system read from a .mmp file: host setup,
// device upload, E_M2D, solve) or "follow-up" (a new field on a resident
// instance, warm-started from its last dipoles, as in successive SCF
// iterations of a QM/MM calculation; the reference's ipd_use_guess,
// src/mod_polarization.F90:195-210).  Worker slots each carry one request at
// a time: host setup, admission, upload and E_M2D on the instance's own CUDA
// stream.  In the mixed modes the solve itself then joins the multi-system
// engine (multisolve.cu), whose rounds advance every admitted solve together
// on one stream, the pair products of all of them sharing persistent
// multi-system launches, so a request that arrives while others are on the
// GPU starts iterating at the next round; in FP64 the worker solves on the
// instance's stream.  A request is admitted as soon as a slot is free and its
// device memory fits the budget; idle resident instances are evicted
// least-recently-used first to make room.  Instances allocate and free their
// device memory stream-ordered (cudaMallocAsync / cudaFreeAsync), so
// admission and eviction do not synchronise the device.  Follow-ups on one
// instance run in submission order.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <set>
#include <string>
#include <thread>
#include <vector>

#include "../../include/openmmpol_gb300.h"
#include "engine.h"
#include "log.h"
#include "multisolve.h"

namespace ommp {
namespace {

double now_ms() {
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

struct Request {
  long long id = 0;
  bool followup = false;
  std::string path;
  long long instance = -1;
  int pol_atoms = 0;
  std::vector<double> field;
  // a new system whose host setup is done, waiting for device memory
  std::unique_ptr<System> staged;
  size_t need = 0;
  // results
  std::vector<double> ipd;
  double energy = 0.0;
  int status = kOk;
  std::string err;
  double t_submit = 0, t_done = 0;
  // phases of a new system: worker picked it up, host setup done, admitted
  // to device memory, uploaded, permanent field and right-hand side formed
  double t_setup0 = 0, t_setup1 = 0, t_admit = 0, t_upload = 0, t_field = 0;
  bool done = false;
};

struct Instance {
  long long id = 0;
  std::unique_ptr<System> sys;
  size_t bytes = 0;
  bool busy = false;
  bool released = false;
  double last_use = 0;
};

class Server {
 public:
  Server(size_t budget, int slots, int precision, double tol)
      : budget_(budget), precision_(precision), tol_(tol), use_engine_(precision != kPrecFP64) {
    if (use_engine_) engine_thread_ = std::thread([this] { engine_loop(); });
    for (int k = 0; k < slots; ++k) workers_.emplace_back([this] { work(); });
  }
  ~Server() {
    {
      std::lock_guard<std::mutex> lk(mu_);
      stop_ = true;
    }
    cv_.notify_all();
    for (auto &t : workers_) t.join();
    if (use_engine_) {
      {
        std::lock_guard<std::mutex> lk(emu_);
        estop_ = true;
      }
      ecv_.notify_all();
      engine_thread_.join();
    }
  }

  void set_round_ms(double ms) { engine_.set_round_ms(ms); }

  void engine_stats(long long *out) {
    MultiSolver::Stats s = engine_.stats();
    out[0] = s.ticks, out[1] = s.launches, out[2] = s.shared_launches, out[3] = s.max_systems,
    out[4] = s.spread_products;
  }

  void engine_times(double *out) {
    MultiSolver::Stats s = engine_.stats();
    out[0] = s.product_ms, out[1] = s.tail_ms, out[2] = s.wall_ms;
  }

  long long submit(Request *r) {
    std::lock_guard<std::mutex> lk(mu_);
    r->id = ++next_id_;
    r->t_submit = now_ms();
    reqs_[r->id].reset(r);
    queue_.push_back(r);
    if (r->followup) ++pending_[r->instance];
    cv_.notify_all();
    return r->id;
  }

  int wait(long long id, double *ipd, double *energy, long long *instance, double *latency_ms) {
    std::unique_lock<std::mutex> lk(mu_);
    auto it = reqs_.find(id);
    if (it == reqs_.end()) {
      set_last_error("server: unknown request id");
      return kErrBadArg;
    }
    Request *r = it->second.get();
    cv_.wait(lk, [&] { return r->done; });
    if (ipd && r->status == kOk) std::memcpy(ipd, r->ipd.data(), r->ipd.size() * sizeof(double));
    if (energy) *energy = r->energy;
    if (instance) *instance = r->instance;
    if (latency_ms) *latency_ms = r->t_done - r->t_submit;
    int st = r->status;
    if (st) set_last_error(r->err);
    reqs_.erase(it);
    return st;
  }

  int cancel(long long id) {
    std::lock_guard<std::mutex> lk(mu_);
    auto it = std::find_if(queue_.begin(), queue_.end(), [&](Request *r) { return r->id == id; });
    if (it == queue_.end()) {
      set_last_error("server: the request is not queued (running, done or unknown)");
      return kErrBadArg;
    }
    Request *r = *it;
    queue_.erase(it);
    if (r->followup) --pending_[r->instance];
    r->staged.reset();
    finish_locked(r, kErrCancelled, "server: request cancelled");
    return kOk;
  }

  void release(long long inst) {
    std::lock_guard<std::mutex> lk(mu_);
    auto it = inst_.find(inst);
    if (it != inst_.end()) it->second.released = true;
    cv_.notify_all();
  }

  // sums over the new systems that completed without error: count, then the
  // milliseconds waiting for a worker, in host setup, waiting for admission,
  // uploading, forming the permanent field and right-hand side, solving
  void phase_stats(double *out) {
    std::lock_guard<std::mutex> lk(mu_);
    for (int k = 0; k < 7; ++k) out[k] = phase_sum_[k];
  }

  void stats(double *out) {
    std::lock_guard<std::mutex> lk(mu_);
    out[0] = (double)used_;
    out[1] = (double)peak_used_;
    out[2] = (double)inst_.size();
    out[3] = (double)evictions_;
    out[4] = (double)peak_running_;
    out[5] = (double)completed_;
    out[6] = (double)budget_;
  }

 private:
  // an instance may be evicted when idle and no follow-up for it is queued
  bool evictable_locked(const Instance &in) const {
    if (in.busy) return false;
    auto p = pending_.find(in.id);
    return p == pending_.end() || p->second == 0;
  }

  bool fits_locked(size_t need) const {
    size_t avail = budget_ - std::min(budget_, used_);
    for (auto &kv : inst_)
      if (evictable_locked(kv.second)) avail += kv.second.bytes;
    return avail >= need;
  }

  // First queued request that can start now (nullptr if none).  Follow-ups
  // keep their per-instance order and wait while their instance is busy;
  // staged new systems start in arrival order once they fit; a new system
  // without host setup can always start (the setup needs no device memory).
  Request *pick_locked() {
    std::set<long long> seen;
    bool staged_blocked = false;
    for (auto it = queue_.begin(); it != queue_.end(); ++it) {
      Request *r = *it;
      if (r->followup) {
        if (!seen.insert(r->instance).second) continue;
        auto in = inst_.find(r->instance);
        if (in != inst_.end() && in->second.busy) continue;
      } else if (r->staged) {
        if (staged_blocked) continue;
        if (!fits_locked(r->need)) {
          staged_blocked = true;
          continue;
        }
      }
      queue_.erase(it);
      if (r->followup) --pending_[r->instance];
      return r;
    }
    return nullptr;
  }

  // evict evictable instances (released first, then least recently used)
  // until `need` more bytes fit the budget
  void make_room_locked(size_t need) {
    while (used_ + need > budget_) {
      Instance *victim = nullptr;
      for (auto &kv : inst_) {
        Instance &in = kv.second;
        if (!evictable_locked(in)) continue;
        bool better = !victim || (in.released && !victim->released) ||
                      (in.released == victim->released && in.last_use < victim->last_use);
        if (better) victim = &in;
      }
      if (!victim) return;
      used_ -= victim->bytes;
      ++evictions_;
      pending_.erase(victim->id);
      retired_.push_back(std::move(victim->sys));
      inst_.erase(victim->id);
    }
  }

  void start_locked() {
    ++running_;
    peak_running_ = std::max(peak_running_, running_);
  }

  void work() {
    std::unique_lock<std::mutex> lk(mu_);
    while (true) {
      Request *r = nullptr;
      cv_.wait(lk, [&] { return stop_ || (r = pick_locked()) != nullptr; });
      if (!r) return;  // stopping
      if (r->followup) {
        auto in = inst_.find(r->instance);
        if (in == inst_.end()) {
          finish_locked(r, kErrBadArg, "server: the instance of this follow-up is not resident");
          continue;
        }
        Instance &inst = in->second;
        inst.busy = true;
        start_locked();
        System *s = inst.sys.get();
        lk.unlock();
        int st = run(s, r);
        std::string err = st ? last_error() : "";
        lk.lock();
        Instance &after = inst_.at(r->instance);  // busy instances are never evicted
        after.busy = false;
        after.last_use = now_ms();
        --running_;
        finish_locked(r, st, err);
        continue;
      }
      if (!r->staged) {
        // host setup (file parse, topology, pair lists) outside the lock,
        // then back to the head of the queue to wait for device memory
        lk.unlock();
        r->t_setup0 = now_ms();
        std::string err;
        int st = kOk;
        std::unique_ptr<System> sys(System::load_host(r->path, err, st));
        r->t_setup1 = now_ms();
        size_t need = sys ? sys->device_bytes_estimate() : 0;
        lk.lock();
        if (!sys) {
          finish_locked(r, st ? st : kErrInput, err);
        } else if (need > budget_) {
          finish_locked(r, kErrMemory,
                        "server: the system needs " + std::to_string(need >> 20) +
                            " MiB of device memory, more than the whole budget");
        } else {
          r->staged = std::move(sys);
          r->need = need;
          queue_.push_front(r);
        }
        cv_.notify_all();
        continue;
      }
      // admitted: make room, account, attach and solve
      make_room_locked(r->need);
      std::vector<std::unique_ptr<System>> dead;
      dead.swap(retired_);
      size_t need = r->need;
      used_ += need;
      peak_used_ = std::max(peak_used_, used_);
      long long id = ++next_inst_;
      std::unique_ptr<System> sys = std::move(r->staged);
      start_locked();
      lk.unlock();
      r->t_admit = now_ms();
      dead.clear();  // free evicted systems' device memory outside the lock
      sys->set_async_alloc(true);
      int st = sys->attach_device();
      r->t_upload = now_ms();
      if (st == kOk) {
        sys->set_precision(precision_);
        sys->set_tol(tol_);
        st = run(sys.get(), r);
      }
      std::string err = st ? last_error() : "";
      if (!(st == kOk || st == kErrNotConverged || st == kErrNumeric)) sys.reset();
      lk.lock();
      --running_;
      if (st == kOk) {
        const double t_field = r->t_field > 0 ? r->t_field : r->t_upload;
        const double ph[6] = {r->t_setup0 - r->t_submit, r->t_setup1 - r->t_setup0, r->t_admit - r->t_setup1,
                              r->t_upload - r->t_admit, t_field - r->t_upload, now_ms() - t_field};
        phase_sum_[0] += 1.0;
        for (int k = 0; k < 6; ++k) phase_sum_[k + 1] += ph[k];
      }
      if (sys) {
        Instance &inst = inst_[id];
        inst.id = id;
        inst.sys = std::move(sys);
        inst.bytes = need;
        inst.last_use = now_ms();
        r->instance = id;
      } else {
        used_ -= need;
      }
      finish_locked(r, st, err);
    }
  }

  // the engine thread: one round at a time while any solve is admitted
  void engine_loop() {
    std::unique_lock<std::mutex> lk(emu_);
    while (true) {
      ecv_.wait(lk, [&] { return estop_ || !engine_.idle(); });
      if (estop_ && engine_.idle()) return;
      lk.unlock();
      engine_.tick();
      lk.lock();
      ecv_.notify_all();
    }
  }

  int run(System *s, Request *r) {
    const int n = s->model().npol;
    if (r->pol_atoms != n) {
      set_last_error("server: the field has " + std::to_string(r->pol_atoms) + " sites, the system " +
                     std::to_string(n));
      return kErrBadArg;
    }
    if (use_engine_) {
      int st = kOk;
      const long long id = engine_.add(s, r->field.data(), st);
      if (id < 0) return st;
      if (!r->followup) r->t_field = now_ms();
      int jst = kOk;
      double e = 0.0;
      std::string err;
      {
        std::unique_lock<std::mutex> lk(emu_);
        ecv_.notify_all();
        ecv_.wait(lk, [&] { return engine_.take(id, jst, e, err); });
      }
      if (jst) {
        set_last_error(err);
        return jst;
      }
      r->energy = e;
      const int nipd = s->model().n_ipd;
      r->ipd.assign(s->ipd_host(), s->ipd_host() + (size_t)nipd * n * 3);
      return kOk;
    }
    int st = s->set_external_field(r->field.data(), kSolverNone, kMatvNone, true);
    if (st) return st;
    double e = 0.0;
    st = s->polelec_energy(e);
    if (st) return st;
    r->energy = e;
    const int nipd = s->model().n_ipd;
    r->ipd.assign(s->ipd_host(), s->ipd_host() + (size_t)nipd * n * 3);
    return kOk;
  }

  void finish_locked(Request *r, int st, const std::string &err) {
    r->status = st;
    r->err = err;
    r->t_done = now_ms();
    r->done = true;
    r->field.clear();
    r->field.shrink_to_fit();
    ++completed_;
    cv_.notify_all();
  }

  size_t budget_, used_ = 0, peak_used_ = 0;
  int precision_;
  double tol_;
  bool use_engine_;
  MultiSolver engine_;
  std::thread engine_thread_;
  std::mutex emu_;
  std::condition_variable ecv_;  // work for the engine / a round finished
  bool estop_ = false;
  std::mutex mu_;
  std::condition_variable cv_;
  std::deque<Request *> queue_;
  std::map<long long, std::unique_ptr<Request>> reqs_;
  std::map<long long, Instance> inst_;
  std::map<long long, int> pending_;  // queued follow-ups per instance
  std::vector<std::unique_ptr<System>> retired_;
  std::vector<std::thread> workers_;
  long long next_id_ = 0, next_inst_ = 0, evictions_ = 0, completed_ = 0;
  double phase_sum_[7] = {0, 0, 0, 0, 0, 0, 0};
  int running_ = 0, peak_running_ = 0;
  bool stop_ = false;
};

}  // namespace
}  // namespace ommp

using ommp::Server;

extern "C" {

int32_t ommp_gpu_server_create(int64_t hbm_budget_bytes, int32_t slots, int32_t precision, double tol,
                               void **server) {
  *server = nullptr;
  if (hbm_budget_bytes <= 0 || slots < 1 || slots > 64 || precision < 0 || precision > 2) {
    ommp::set_last_error("server: budget must be positive, slots 1..64 and precision 0..2");
    return ommp::kErrBadArg;
  }
  *server = new Server((size_t)hbm_budget_bytes, slots, precision, tol);
  return ommp::kOk;
}

void ommp_gpu_server_destroy(void *server) { delete static_cast<Server *>(server); }

int32_t ommp_gpu_server_submit(void *server, const char *mmp_path, const double *field, int32_t pol_atoms,
                               int64_t *request_id) {
  auto *r = new ommp::Request();
  r->path = mmp_path ? mmp_path : "";
  r->pol_atoms = pol_atoms;
  r->field.assign(field, field + 3 * (size_t)pol_atoms);
  *request_id = static_cast<Server *>(server)->submit(r);
  return ommp::kOk;
}

int32_t ommp_gpu_server_submit_followup(void *server, int64_t instance, const double *field, int32_t pol_atoms,
                                        int64_t *request_id) {
  auto *r = new ommp::Request();
  r->followup = true;
  r->instance = instance;
  r->pol_atoms = pol_atoms;
  r->field.assign(field, field + 3 * (size_t)pol_atoms);
  *request_id = static_cast<Server *>(server)->submit(r);
  return ommp::kOk;
}

int32_t ommp_gpu_server_wait(void *server, int64_t request_id, double *ipd_out, double *energy, int64_t *instance,
                             double *latency_ms) {
  long long inst = -1;
  int st = static_cast<Server *>(server)->wait(request_id, ipd_out, energy, &inst, latency_ms);
  if (instance) *instance = inst;
  return st;
}

void ommp_gpu_server_release(void *server, int64_t instance) { static_cast<Server *>(server)->release(instance); }

int32_t ommp_gpu_server_cancel(void *server, int64_t request_id) {
  return static_cast<Server *>(server)->cancel(request_id);
}

void ommp_gpu_server_stats(void *server, double *out7) { static_cast<Server *>(server)->stats(out7); }

int32_t ommp_gpu_server_set_round_ms(void *server, double ms) {
  if (!(ms > 0.0) || !(ms < 1e6)) {
    ommp::set_last_error("server: the round length must be a positive number of milliseconds");
    return ommp::kErrBadArg;
  }
  static_cast<Server *>(server)->set_round_ms(ms);
  return ommp::kOk;
}

void ommp_gpu_server_engine_times(void *server, double *out3) {
  static_cast<Server *>(server)->engine_times(out3);
}

void ommp_gpu_server_phase_stats(void *server, double *out7) {
  static_cast<Server *>(server)->phase_stats(out7);
}

void ommp_gpu_server_engine_stats(void *server, int64_t *out5) {
  long long v[5] = {0, 0, 0, 0, 0};
  static_cast<Server *>(server)->engine_stats(v);
  for (int k = 0; k < 5; ++k) out5[k] = v[k];
}

}  // extern "C"
