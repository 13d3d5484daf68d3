// Device-resident system and the polarization solvers (FP64 CG, Jacobi/DIIS,
// inversion, and the FP32-inner / FP64-refinement solver).
#pragma once

#include <map>
#include <string>
#include <utility>
#include <vector>

#include "kernels.h"
#include "ommp_internal.h"

namespace ommp {

enum Status : int {
  kOk = 0,
  kErrInput = 1,
  kErrNotConverged = 2,
  kErrBadArg = 3,
  kErrNumeric = 4,
  kErrCuda = 5,
  kErrMemory = 6,
  kErrCancelled = 7,
};

// Column buffers of one solve: a view of a system's default two-column
// buffers, or the batch buffers (grown on demand).  Columns are [cap][n][3].
struct Workspace {
  int cap = 0;
  int fcap = 0;  // batch: fields the staging buffers hold
  double *x = nullptr, *r = nullptr, *p = nullptr, *h = nullptr, *z = nullptr, *rhs = nullptr;
  double *fields = nullptr, *out = nullptr;  // batch staging
  float *x32 = nullptr, *r32 = nullptr, *p32 = nullptr, *h32 = nullptr, *z32 = nullptr;
  float *scratch32 = nullptr;
  int scratch32_nsplit = 0;  // source splits the FP32 scratch holds for cap columns
  double *partial = nullptr;  // kRedBlocks x cap
  double *dots = nullptr;     // 3 x cap (+ fcap)
  double *hist = nullptr;     // cap x maxhist, or none
  // block CG of the batch (block_cg.cu): next directions, Gram partials and
  // results, coefficients, column maps, pinned host copy of the small matrices
  float *t32 = nullptr;
  double *gram = nullptr;
  float *bcoef = nullptr;
  int *bidx = nullptr;
  double *bscal_h = nullptr;
  gpu::CgCol *cols = nullptr;
  gpu::CgCol *cols_h = nullptr;  // pinned
  double *scal_h = nullptr;      // pinned 3 x cap (+ fcap)
  bool owned = false;
  // captured inner FP32 iteration (CUDA graph) and what it was built for
  cudaGraphExec_t graph = nullptr;
  int graph_ncol = -1, graph_gmax = 0, graph_nsplit = 0, graph_kver = 0, graph_prec = -1;
  long long graph_kernels = 0;
};

// device data of the polarization gradient (grad.cu) and of the fast
// multipole method (fmm.cu)
struct GradState;
void free_grad_state(GradState *g);
struct FmmState;
void free_fmm_state(FmmState *f);

struct SolveStats {
  int iters[2] = {0, 0};
  std::vector<double> hist[2];
  int outer = 0;          // refinement steps of the mixed solver
  int inner_iters = 0;    // FP32 iterations summed over outer steps
  int f64_matvecs = 0;
  int f32_matvecs = 0;
  int ds_matvecs = 0;     // double-single residual products
  int updates = 0;        // refinement residuals updated by an FP32 product
};

// relative accuracy of the FP32 operator against T assumed by the residual
// update (the bound its accuracy tests hold it to)
constexpr double kResidualUpdateRel = 1e-5;

class MultiSolver;

class System {
  friend class MultiSolver;

 public:
  ~System();
  static System *from_mmp(const std::string &path, std::string &err, int &status);
  // two-phase creation for admission control: parse and set up on the host,
  // then (once memory is granted) allocate and upload the device arrays
  static System *load_host(const std::string &path, std::string &err, int &status);
  int attach_device();
  size_t device_bytes_estimate() const;
  // stream-ordered allocation (cudaMallocAsync / cudaFreeAsync on the
  // system's own stream, from the device's default pool) of the system's
  // resident buffers, for systems admitted and evicted by the request server
  // while other systems' kernels run: cudaMalloc and cudaFree synchronise the
  // device.  Set before attach_device.
  void set_async_alloc(bool on) { async_alloc_ = on; }

  // --- reference API semantics -------------------------------------------------
  int set_external_field(const double *ext_host, int solver, int matv, bool add_mm);
  int set_external_field_device(const double *ext_dev, int solver, int matv, bool add_mm);
  int polelec_energy(double &e);
  // interaction energy of the static multipoles (once per geometry)
  int fixedelec_energy(double &e);
  int update_coordinates(const double *c_host);
  int set_default_solver(int s);
  int set_default_matv(int m);

  // --- extensions --------------------------------------------------------------
  // nf independent fields solved together (cold start, system state untouched):
  // fields [nf][n][3], out [nf][n_ipd][n][3] (device or host), energies [nf] host
  int solve_batch(int nf, const double *fields_dev, double *out_dev, double *energies);
  int solve_batch_host(int nf, const double *fields_host, double *out_host, double *energies);
  void set_use_graphs(bool on) { use_graphs_ = on; }
  // block CG for the FP32 inner solve of batches of at least 4 columns
  // (default on); off: independent scalar PCG per column
  void set_block_cg(bool on) { block_cg_ = on; }
  // refinement residuals of the mixed modes after a recomputed one: -1 by
  // mode (update in mixed-ds, recompute in the strict mixed mode), 0 always
  // recompute E - T mu with the residual product, 1 update r -= T32 d by the
  // FP32 product of the correction d when its error bound allows
  int set_residual_update(int mode);
  bool residual_update() const {
    return residual_update_ < 0 ? precision_ == kPrecMixedDS : residual_update_ == 1;
  }
  int tmatvec(const double *x_host, double *y_host, int nrhs, bool dodiag, int matv);
  int tmatvec_f32(const double *x_host, double *y_host, int nrhs);
  int tmatvec_ds(const double *x_host, double *y_host, int nrhs);
  // potential (field = false, out [n]) or field (out [n][3]) at the points
  // cext [n][3], added into out; which 0 all, 1 static, 2 induced
  int ext_props(int which, bool field, int n, const double *cext_host, double *out_host);
  int e_m2d(double *out_host);
  // geometric gradient of the polarization energy, out [mm][3] (overwritten)
  int polelec_geomgrad(double *grad_host);
  // forces of the frame rotation of the static multipoles in a given field
  // E [mm][3] and field gradient G [mm][6], out [mm][3] (overwritten)
  int rotation_geomgrad(const double *E_host, const double *G_host, double *grad_host);
  // gradient of the static multipole energy, out [mm][3] (overwritten)
  int fixedelec_geomgrad(double *grad_host);
  // fast multipole method for the FP64 T.mu products (expansion order 2..12)
  int set_fmm(bool on, int order);
  bool fmm_on() const { return fmm_on_; }
  int fmm_order() const { return fmm_order_; }
  // the reference's FMM settings (mod_c_interface.F90:1781-1841): expansion
  // order of the induced-dipole products (lmax_pol) and of the permanent
  // field (lmax), near-field distance and minimum cell size (bohr), mapped
  // onto this FMM's orders and the leaf side of its uniform octree
  int set_fmm_order_pol(int order);
  int set_fmm_order_static(int order);
  int set_fmm_distance(double d);
  int set_fmm_min_cell_size(double d);
  int fmm_order_static() const { return fmm_order_static_; }
  double fmm_min_leaf() const;
  void clear_guess() { ipd_use_guess_ = false; }
  void set_tol(double t) { tol_ = t; }
  void set_maxiter(int n) { maxiter_ = n; }
  void set_precision(int p) {
    if (p >= kPrecFP64 && p <= kPrecMixedDS) precision_ = p;
  }
  // FP64 direct product: 0 auto (symmetric from 2048 sites), 1 all ordered
  // pairs (target-outer), 2 symmetric (unordered pairs)
  int set_fp64_kernel(int mode);
  int set_fp32_kernel(int mode);
  int fp32_shape(int ncol, int32_t *shape) const;
  int set_inner_preconditioner(int mode);
  // runs of the block-Jacobi inner preconditioner: at most max_sites
  // consecutive polarizable sites, each within link_bohr of an earlier one
  int set_inner_blocks(int max_sites, double link_bohr);
  int matvec_residual(int ncol, const double *x, double *y);
  int ensure_ds_scratch();
  int ensure_sym_scratch();
  int precision() const { return precision_; }
  double tol() const { return tol_; }
  const SolveStats &stats() const { return stats_; }
  float last_solve_ms() const { return last_ms_; }
  int sync();

  // kernel timing of the dominant pair kernels (CUDA events on the stream,
  // resolved lazily so that timing adds no synchronisation)
  void enable_kernel_timing(bool on) { ktime_on_ = on; }
  void kernel_stats(int which, long long &launches, double &ms, long long &columns);
  void reset_kernel_stats();
  // stream-ordered event timers (slots 0..7) and an L2 flush on the stream
  int timer_record(int slot);
  int timer_elapsed(int a, int b, double &ms);
  int flush_l2(size_t bytes);

  const HostModel &model() const { return m_; }
  double *ipd_host() { return ipd_h_.data(); }
  double *cpol_host() { return cpol_h_.data(); }
  int *polar_mm_host() { return polar_mm_h_.data(); }
  double *cmm_host() { return m_.cmm.data(); }
  double *q_host() { return m_.q.data(); }
  cudaStream_t stream() const { return st_; }
  const gpu::DevSites &dev() const { return d_; }
  bool ipd_done() const { return ipd_done_; }
  int *flag_dev() { return flag_; }  // device error flag of the system's stream

 private:
  System() = default;
  template <typename T>
  int alloc(T *&p, size_t count);
  void release(void *p);
  // host-to-device copy of set-up data through a page-locked pool buffer
  // (h2d), returned to the pool by h2d_release once the stream has caught up
  void h2d(void *dst, const void *src, size_t bytes);
  void h2d_release();
  std::vector<void *> staged_;
  bool async_alloc_ = false;
  std::vector<void *> async_bufs_;
  int upload_static();
  int upload_geometry();
  int ensure_m2d();
  int ensure_tmat();
  int polarization(const double *e_dev, int solver, int matv, const bool *mask);
  int matvec64(int matv, int ncol, const double *x, double *y, bool dodiag);
  int cg64(int matv, int ncol, const double *rhs, double *x, int set0) { return cg64_ws(ws_, matv, ncol, rhs, x, set0); }
  int diis64(int matv, const double *rhs, double *x, int set);
  int inversion64(const double *rhs, double *x);
  int mixed_ir(int ncol, const double *rhs, double *x, int set0, bool have_guess) {
    return mixed_ir_ws(ws_, ncol, rhs, x, set0, have_guess);
  }
  // solvers.cu: the same solvers on any workspace
  int cg64_ws(Workspace &w, int matv, int ncol, const double *rhs, double *x, int set0);
  int pcg32_ws(Workspace &w, int ncol, int max_it, double eta);
  int bpcg32_ws(Workspace &w, int ncol, int max_it, double eta);
  int mixed_ir_ws(Workspace &w, int ncol, const double *rhs, double *x, int set0, bool have_guess);
  struct F32Shape {
    int g, nsplit, kver;  // group width, source splits, kernel version
  };
  int tune_f32(Workspace &w, int ncol, F32Shape &shape);
  bool update_allowed(const std::vector<double> &rms) const;
  void f32_product(Workspace &w, int ncol, const F32Shape &shape);
  int ensure_batch_ws(int ncol, int nf);
  void free_ws(Workspace &w);
  int check(cudaError_t e, const char *what);
  int fetch_ipd();

  HostModel m_;
  ScaledPairs m2d_pairs_, d2d_pairs_;
  gpu::DevSites d_;
  cudaStream_t st_ = nullptr;
  cudaEvent_t ev0_ = nullptr, ev1_ = nullptr;
  // solver state
  int def_solver_ = kSolverCG, def_matv_ = kMatvDirect;
  int precision_ = kPrecFP64;
  double tol_ = 1e-8;
  int maxiter_ = 200;
  int diis_max_ = 20;
  bool m2d_done_ = false, ipd_done_ = false, ipd_use_guess_ = false;
  // device buffers
  double *e_m2d_ = nullptr;   // [n_ipd][n][3]
  double *ipd_ = nullptr;     // [n_ipd][n][3]
  double *rhs_ = nullptr;     // [2][n][3] right-hand sides of the solve
  double *ext_ = nullptr;     // [n][3] staging of a host external field
  double *x_ = nullptr, *r_ = nullptr, *p_ = nullptr, *h_ = nullptr, *z_ = nullptr;  // [2][n][3]
  float *x32_ = nullptr, *r32_ = nullptr, *p32_ = nullptr, *h32_ = nullptr, *z32_ = nullptr;
  float *alpha32_ = nullptr;
  double *scratch_ = nullptr;  // pair-kernel split partials
  size_t scratch_n_ = 0;
  double *sym_scratch_ = nullptr;  // symmetric-kernel partials (allocated on first use)
  int fp64_kernel_ = 0;
  int4 *blk_info_ = nullptr;   // block-Jacobi preconditioner (build_block_jacobi)
  float *blk_minv_ = nullptr;
  int *near_ri_ = nullptr, *near_ci_ = nullptr;  // near-field couplings (build_near_field)
  float *near_blk_ = nullptr;
  std::vector<int> blk_runs_;  // the runs of the block preconditioner (host copy of its info)
  int ensure_near();
  // FP32 inner solver: 0 diagonal, 1 block Jacobi, 2 block Jacobi with the
  // near-field Neumann step (default)
  int inner_precond_ = 2;
  bool near_precond() const { return inner_precond_ == 2 && blk_info_ && near_ri_; }
  int blk_max_ = kMaxBlock;
  double blk_link_ = kBlockLinkBohr;
  int build_blocks();
  double *ext_buf_ = nullptr;  // external points: coordinates, partials, output, dipoles
  size_t ext_cap_ = 0;
  double *ds_scratch_ = nullptr;  // split partials of the double-single kernels
  int nsplit_ds_ = 1, nsplit_m2d_ds_ = 1;
  // how the cached E_M2D was computed
  static constexpr int kM2dDirect = 0, kM2dDS = 1, kM2dFMM = 2;
  int m2d_method_ = kM2dDirect;
  int fp32_kernel_ = 0;  // 0 autotuned, else the forced kernel version
  float *scratch32_ = nullptr;
  double *partial_ = nullptr;  // reduction partials [kRedBlocks][8]
  double *dots_ = nullptr;     // [8]
  double *hist_ = nullptr;     // [2][maxhist]
  gpu::CgCol *cols_ = nullptr;
  gpu::CgCol *cols_h_ = nullptr;  // pinned
  double *scal_h_ = nullptr;      // pinned scalars
  int *flag_ = nullptr;
  double *tmat_ = nullptr;
  int *piv_ = nullptr;
  int *info_ = nullptr;
  bool tmat_ok_ = false, lu_ok_ = false;
  double *diis_x_ = nullptr, *diis_e_ = nullptr;
  int nsplit_m2d_ = 1, nsplit_tmu_ = 1, nsplit_tmu32_ = 1;
  int maxhist_ = 1024;
  // host mirrors
  std::vector<double> ipd_h_, cpol_h_;
  std::vector<int> polar_mm_h_;
  SolveStats stats_;
  float last_ms_ = 0.f;
  bool ktime_on_ = false;
  // kernel timing: 0 FP64, 1 FP32, 2 double-single T.mu, 3 gradient pair pass
  long long klaunch_[4] = {0, 0, 0, 0};
  long long kcols_[4] = {0, 0, 0, 0};
  double kms_[4] = {0, 0, 0, 0};
  struct KEv {
    cudaEvent_t a, b;
    int kind;
    int cols;  // right-hand sides carried by the timed launch
  };
  std::vector<KEv> kpending_, kfree_;
  KEv kt_begin(int kind, int cols);
  void kt_end(KEv &e);
  void kt_resolve();
  bool fixedelec_done_ = false;
  double fixedelec_ = 0.0;
  bool fixedelec_grad_done_ = false;
  std::vector<double> fixedelec_grad_;
  int m2m_launch(bool grad, double **buf, double **site, double **E, double **G, double **base);
  GradState *grad_ = nullptr;
  int ensure_grad_state();
  int frame_forces(const double *E_dev, const double *G_dev, const double *base_dev, double *grad_host);
  FmmState *fmm_ = nullptr;   // induced-dipole products: tables of fmm_order_, the T.mu tree
  FmmState *fmms_ = nullptr;  // permanent field: tables of fmm_order_static_, the M2D tree
  bool fmm_on_ = false;
  int fmm_order_ = 10;  // total order |g| + |h| <= 10 of the Cartesian M2L
  int fmm_order_static_ = 10;
  double fmm_dfar_ = 0.0, fmm_mincell_ = 0.0;  // 0: leaf side from the damping range alone
  void fmm_drop_static();
  int fmm_prepare();
  void fmm_invalidate();
  bool fmm_tree() const;  // the prepared FMM has a tree (else direct sums)
  int fmm_tmu(int ncol, const double *x, double *y, bool dodiag);
  int fmm_m2d(double *out, bool &done);
  Workspace ws_;   // view of the default two-column buffers
  Workspace wsb_;  // batch buffers
  std::map<int, F32Shape> f32_tune_;  // columns -> tuned FP32 launch shape
  bool use_graphs_ = true;
  bool block_cg_ = true;
  int residual_update_ = -1;
  cudaEvent_t tev_[8] = {};
  void *flush_buf_ = nullptr;
  size_t flush_bytes_ = 0;
  unsigned flush_tag_ = 0;
};

// process-wide: systems created while this is on get the FMM switched on when
// they have more than 1,000 MM atoms, as the reference does by default
// (src/mod_electrostatics.F90:294-306, OMMP_FMM_ENABLE_THR)
void set_fmm_auto(bool on);
bool fmm_auto();

// resolves the static scratch of ommp_gpu_tmatvec_noalloc on the current
// device (noalloc.cu); called once per system set-up
int noalloc_prepare_device();

// process-wide error text of the last failing call
void set_last_error(const std::string &s);
const char *last_error();

// Page-locked host buffers for the solvers' small asynchronous read-backs,
// from a process-wide pool: a buffer returned by pinned_free is kept for the
// next pinned_alloc of its size class instead of being released, because
// cudaFreeHost waits for the whole device (a request server freeing an
// evicted system would stall every solve in flight).  The caller must have
// completed all copies into or out of a buffer before returning it.
cudaError_t pinned_alloc(void **p, size_t bytes);
void pinned_free(void *p);

}  // namespace ommp
