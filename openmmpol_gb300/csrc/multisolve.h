// Mixed-precision solves of several systems advanced together on one stream,
// their pair products sharing persistent multi-system launches
// (multisolve.cu).
#pragma once

#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "engine.h"

namespace ommp {

class MultiSolver {
 public:
  struct Stats {
    long long ticks = 0;
    long long launches = 0;        // multi-system product launches
    long long shared_launches = 0; // launches that served two or more systems
    long long max_systems = 0;     // most systems served by one launch
    long long spread_products = 0; // products spread over more than one launch
    long long finished = 0;
    // where the rounds' time went: GPU time of the product launches and of
    // the per-system bookkeeping after them (CUDA events on the engine
    // stream), and host wall time of the rounds (from the start of a round's
    // preparation steps to its decisions)
    double product_ms = 0.0, tail_ms = 0.0, wall_ms = 0.0;
  };

  MultiSolver();
  ~MultiSolver();
  MultiSolver(const MultiSolver &) = delete;
  MultiSolver &operator=(const MultiSolver &) = delete;

  // Queue the solve of system s for the field ext_host [pol_atoms][3] (host
  // memory): the permanent field, right-hand sides and starting guess are
  // prepared on the system's own stream by the calling thread, then the
  // solve joins the next round.  The system must stay idle (no other call on
  // it) until the job is taken.  Returns the job id, or -1 with the status in
  // `status` (the message in last_error()).
  long long add(System *s, const double *ext_host, int &status);
  // One round: pending preparation steps, one launch per product kind and
  // column width for every system that needs a product (a bounded share of
  // each product per round), the CG bookkeeping of every system whose product
  // completed, one synchronisation, the decisions.  Returns the jobs that
  // finished in this round.  Called by one thread.
  int tick();
  bool idle();
  // work per product kind in one round, in milliseconds of GPU time at the
  // symmetric kernels' measured pair rates (default 1.5): shorter rounds let
  // small systems iterate faster beside large ones, longer rounds spend less
  // of the GPU on the per-round bookkeeping
  void set_round_ms(double ms);
  // a finished job's status, energy and error text; false while running
  bool take(long long id, int &status, double &energy, std::string &err);
  Stats stats();

 private:
  struct Job;
  int launch_products(std::vector<Job *> &active);
  void enqueue_tail(Job &j, int which);
  double round_pairs(int kind);  // pairs of one round's budget for a product kind
  void fail(Job &j, int status, const std::string &err);

  cudaStream_t st_ = nullptr;
  cudaEvent_t ev_[3] = {nullptr, nullptr, nullptr};  // products start / end, bookkeeping end
  unsigned *counters_ = nullptr;  // one work counter per launch of a round
  std::mutex mu_;
  std::vector<Job *> pending_;    // added, not yet in a round
  std::vector<Job *> jobs_;       // in rounds (engine thread only)
  std::map<long long, Job *> done_;
  long long next_id_ = 0;
  double round_ms_ = 1.5;
  Stats stats_;
};

}  // namespace ommp
