// extern "C" entry points of libommp_gb300.so (declared in
// include/openmmpol_gb300.h).  The legacy names keep the reference's
// behaviour: no return status, and a message plus exit(1) on error
// (src/mod_io.F90:155-175).  The ommp_gpu_* names return a status instead.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/openmmpol_gb300.h"
#include "engine.h"
#include "log.h"
#include "qm_helper.h"

using ommp::QMHelper;
using ommp::System;

namespace {
System *S(OMMP_SYSTEM_PRT p) { return static_cast<System *>(p); }
QMHelper *Q(OMMP_QM_HELPER_PRT p) { return static_cast<QMHelper *>(p); }

void fatal_if(int st) {
  if (st != ommp::kOk) ommp::log_fatal(ommp::last_error());
}

// timer stack of ommp_time_push / ommp_time_pull (src/mod_profiling.F90:19-70)
std::vector<std::chrono::steady_clock::time_point> g_timers;
}  // namespace

extern "C" {

int32_t ommp_gpu_init_mmp(const char *filename, OMMP_SYSTEM_PRT *out) {
  *out = nullptr;
  std::string err;
  int st = ommp::kOk;
  System *s = System::from_mmp(filename ? filename : "", err, st);
  if (!s) {
    ommp::set_last_error(err);
    return st ? st : ommp::kErrInput;
  }
  *out = s;
  return ommp::kOk;
}

OMMP_SYSTEM_PRT ommp_init_mmp(const char *filename) {
  OMMP_SYSTEM_PRT s = nullptr;
  fatal_if(ommp_gpu_init_mmp(filename, &s));
  return s;
}

void ommp_terminate(OMMP_SYSTEM_PRT s) { delete S(s); }

int32_t ommp_gpu_set_default_solver(OMMP_SYSTEM_PRT s, int32_t solver) { return S(s)->set_default_solver(solver); }
int32_t ommp_gpu_set_default_matv(OMMP_SYSTEM_PRT s, int32_t matv) { return S(s)->set_default_matv(matv); }
void ommp_set_default_solver(OMMP_SYSTEM_PRT s, int32_t solver) { fatal_if(ommp_gpu_set_default_solver(s, solver)); }
void ommp_set_default_matv(OMMP_SYSTEM_PRT s, int32_t matv) { fatal_if(ommp_gpu_set_default_matv(s, matv)); }

void ommp_set_verbose(int32_t level) { ommp::log_set_level(level); }
void ommp_set_outputfile(const char *path) { ommp::log_set_file(path); }
void ommp_close_outputfile(void) { ommp::log_close_file(); }
void ommp_message(const char *msg, int32_t level, const char *tag) {
  ommp::log_msg(level, (tag && tag[0]) ? tag : nullptr, "%s", msg);
}
void ommp_fatal(const char *msg) { ommp::log_fatal(msg); }
void ommp_time_push(void) {
  if (g_timers.size() >= 128) ommp::log_fatal("time_push Cannot push another time in the buffer.");
  g_timers.push_back(std::chrono::steady_clock::now());
}
void ommp_time_pull(const char *label) {
  if (g_timers.empty()) ommp::log_fatal("time_pull Cannot pull any value.");
  double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - g_timers.back()).count();
  g_timers.pop_back();
  std::string bar(g_timers.size(), '-');
  ommp::log_msg(ommp::kVerbHigh, "time", "%s> %s: %14.6E s", bar.c_str(), label, el);
}

int32_t ommp_gpu_set_external_field(OMMP_SYSTEM_PRT s, const double *ef, int32_t solver, int32_t matv,
                                    int32_t add_mm) {
  return S(s)->set_external_field(ef, solver, matv, add_mm != 0);
}
int32_t ommp_gpu_set_external_field_status(OMMP_SYSTEM_PRT s, const double *ef, int32_t solver, int32_t matv,
                                           int32_t add_mm) {
  return ommp_gpu_set_external_field(s, ef, solver, matv, add_mm);
}
int32_t ommp_gpu_set_external_field_device(OMMP_SYSTEM_PRT s, const double *ef, int32_t solver, int32_t matv,
                                           int32_t add_mm) {
  return S(s)->set_external_field_device(ef, solver, matv, add_mm != 0);
}
void ommp_set_external_field(OMMP_SYSTEM_PRT s, const double *ef, int32_t solver, int32_t matv) {
  fatal_if(ommp_gpu_set_external_field(s, ef, solver, matv, 1));
}
void ommp_set_external_field_nomm(OMMP_SYSTEM_PRT s, const double *ef, int32_t solver, int32_t matv) {
  fatal_if(ommp_gpu_set_external_field(s, ef, solver, matv, 0));
}

int32_t ommp_gpu_get_fixedelec_energy(OMMP_SYSTEM_PRT s, double *e) {
  ommp_time_push();
  int st = S(s)->fixedelec_energy(*e);
  if (st == ommp::kOk) ommp_time_pull("Fixed electrostatic energy");
  return st;
}
double ommp_get_fixedelec_energy(OMMP_SYSTEM_PRT s) {
  double e = 0.0;
  fatal_if(ommp_gpu_get_fixedelec_energy(s, &e));
  return e;
}
double ommp_get_full_ele_energy(OMMP_SYSTEM_PRT s) {
  double em = 0.0, ep = 0.0;
  fatal_if(ommp_gpu_get_fixedelec_energy(s, &em));
  fatal_if(ommp_gpu_get_polelec_energy(s, &ep));
  return em + ep;
}
int32_t ommp_gpu_get_polelec_energy(OMMP_SYSTEM_PRT s, double *e) {
  ommp_time_push();
  int st = S(s)->polelec_energy(*e);
  if (st == ommp::kOk) ommp_time_pull("Polarizable Electrostatic energy");
  else g_timers.pop_back();
  return st;
}
double ommp_get_polelec_energy(OMMP_SYSTEM_PRT s) {
  double e = 0.0;
  fatal_if(ommp_gpu_get_polelec_energy(s, &e));
  return e;
}

bool ommp_ff_is_amoeba(OMMP_SYSTEM_PRT s) { return S(s)->model().amoeba; }
int32_t ommp_get_n_ipd(OMMP_SYSTEM_PRT s) { return S(s)->model().n_ipd; }
int32_t ommp_get_ld_cart(OMMP_SYSTEM_PRT s) { return S(s)->model().ld_cart; }
int32_t ommp_get_mm_atoms(OMMP_SYSTEM_PRT s) { return S(s)->model().mm; }
int32_t ommp_get_pol_atoms(OMMP_SYSTEM_PRT s) { return S(s)->model().npol; }
double *ommp_get_cmm(OMMP_SYSTEM_PRT s) { return S(s)->cmm_host(); }
double *ommp_get_cpol(OMMP_SYSTEM_PRT s) { return S(s)->cpol_host(); }
double *ommp_get_q(OMMP_SYSTEM_PRT s) { return S(s)->q_host(); }
double *ommp_get_ipd(OMMP_SYSTEM_PRT s) { return S(s)->ipd_host(); }
int32_t *ommp_get_polar_mm(OMMP_SYSTEM_PRT s) { return S(s)->polar_mm_host(); }

int32_t ommp_gpu_update_coordinates(OMMP_SYSTEM_PRT s, const double *c) { return S(s)->update_coordinates(c); }
void ommp_update_coordinates(OMMP_SYSTEM_PRT s, const double *c) { fatal_if(ommp_gpu_update_coordinates(s, c)); }

int32_t ommp_gpu_potential_ext(OMMP_SYSTEM_PRT s, int32_t which, int32_t n, const double *cext, double *v) {
  return S(s)->ext_props(which, false, n, cext, v);
}
int32_t ommp_gpu_field_ext(OMMP_SYSTEM_PRT s, int32_t which, int32_t n, const double *cext, double *e) {
  return S(s)->ext_props(which, true, n, cext, e);
}
void ommp_potential_mmpol2ext(OMMP_SYSTEM_PRT s, int32_t n, const double *c, double *v) {
  fatal_if(S(s)->ext_props(0, false, n, c, v));
}
void ommp_potential_mm2ext(OMMP_SYSTEM_PRT s, int32_t n, const double *c, double *v) {
  fatal_if(S(s)->ext_props(1, false, n, c, v));
}
void ommp_potential_pol2ext(OMMP_SYSTEM_PRT s, int32_t n, const double *c, double *v) {
  fatal_if(S(s)->ext_props(2, false, n, c, v));
}
void ommp_field_mmpol2ext(OMMP_SYSTEM_PRT s, int32_t n, const double *c, double *e) {
  fatal_if(S(s)->ext_props(0, true, n, c, e));
}
void ommp_field_mm2ext(OMMP_SYSTEM_PRT s, int32_t n, const double *c, double *e) {
  fatal_if(S(s)->ext_props(1, true, n, c, e));
}
void ommp_field_pol2ext(OMMP_SYSTEM_PRT s, int32_t n, const double *c, double *e) {
  fatal_if(S(s)->ext_props(2, true, n, c, e));
}
int32_t ommp_gpu_polelec_geomgrad(OMMP_SYSTEM_PRT s, double *grd) {
  ommp_time_push();
  int st = S(s)->polelec_geomgrad(grd);
  if (st == ommp::kOk) ommp_time_pull("Polarizable Elctrostatic grad");
  return st;
}
void ommp_polelec_geomgrad(OMMP_SYSTEM_PRT s, double *grd) { fatal_if(ommp_gpu_polelec_geomgrad(s, grd)); }
int32_t ommp_gpu_fixedelec_geomgrad(OMMP_SYSTEM_PRT s, double *grd) {
  ommp_time_push();
  int st = S(s)->fixedelec_geomgrad(grd);
  if (st == ommp::kOk) ommp_time_pull("Fixed Elctrostatic grad");
  return st;
}
void ommp_fixedelec_geomgrad(OMMP_SYSTEM_PRT s, double *grd) { fatal_if(ommp_gpu_fixedelec_geomgrad(s, grd)); }
int32_t ommp_gpu_rotation_geomgrad(OMMP_SYSTEM_PRT s, const double *E, const double *Egrd, double *grd) {
  ommp_time_push();
  int st = S(s)->rotation_geomgrad(E, Egrd, grd);
  if (st == ommp::kOk) ommp_time_pull("Multipole rotation grad");
  return st;
}
void ommp_rotation_geomgrad(OMMP_SYSTEM_PRT s, const double *E, const double *Egrd, double *grd) {
  fatal_if(ommp_gpu_rotation_geomgrad(s, E, Egrd, grd));
}

int32_t ommp_gpu_init_qm_helper(int32_t n, const double *cqm, const double *qqm, const int32_t *zqm,
                                OMMP_QM_HELPER_PRT *out) {
  *out = nullptr;
  if (n < 0 || (n > 0 && (!cqm || !qqm || !zqm))) {
    ommp::set_last_error("QM helper: n >= 0 and coordinates, charges and atomic numbers are required");
    return ommp::kErrBadArg;
  }
  *out = new QMHelper(n, cqm, qqm, zqm);
  return ommp::kOk;
}
OMMP_QM_HELPER_PRT ommp_init_qm_helper(int32_t n, const double *cqm, const double *qqm, const int32_t *zqm) {
  OMMP_QM_HELPER_PRT h = nullptr;
  fatal_if(ommp_gpu_init_qm_helper(n, cqm, qqm, zqm, &h));
  return h;
}
void ommp_terminate_qm_helper(OMMP_QM_HELPER_PRT qm) { delete Q(qm); }
void ommp_qm_helper_update_coord(OMMP_QM_HELPER_PRT qm, const double *c) { Q(qm)->update_coord(c); }
int32_t ommp_gpu_prepare_qm_ele_ene(OMMP_SYSTEM_PRT s, OMMP_QM_HELPER_PRT qm) { return Q(qm)->prepare_ene(*S(s)); }
int32_t ommp_gpu_prepare_qm_ele_grd(OMMP_SYSTEM_PRT s, OMMP_QM_HELPER_PRT qm) { return Q(qm)->prepare_grd(*S(s)); }
void ommp_prepare_qm_ele_ene(OMMP_SYSTEM_PRT s, OMMP_QM_HELPER_PRT qm) { fatal_if(ommp_gpu_prepare_qm_ele_ene(s, qm)); }
void ommp_prepare_qm_ele_grd(OMMP_SYSTEM_PRT s, OMMP_QM_HELPER_PRT qm) { fatal_if(ommp_gpu_prepare_qm_ele_grd(s, qm)); }
double *ommp_qm_helper_get_V_m2n(OMMP_QM_HELPER_PRT qm) { return Q(qm)->V_m2n(); }
double *ommp_qm_helper_get_V_p2n(OMMP_QM_HELPER_PRT qm) { return Q(qm)->V_p2n(); }
double *ommp_qm_helper_get_E_m2n(OMMP_QM_HELPER_PRT qm) { return Q(qm)->E_m2n(); }
double *ommp_qm_helper_get_E_p2n(OMMP_QM_HELPER_PRT qm) { return Q(qm)->E_p2n(); }
double *ommp_qm_helper_get_E_n2p(OMMP_QM_HELPER_PRT qm) { return Q(qm)->E_n2p(); }
double *ommp_qm_helper_get_G_n2p(OMMP_QM_HELPER_PRT qm) { return Q(qm)->G_n2p(); }
double *ommp_qm_helper_get_E_n2m(OMMP_QM_HELPER_PRT qm) { return Q(qm)->E_n2m(); }
double *ommp_qm_helper_get_G_n2m(OMMP_QM_HELPER_PRT qm) { return Q(qm)->G_n2m(); }
double *ommp_qm_helper_get_H_n2m(OMMP_QM_HELPER_PRT qm) { return Q(qm)->H_n2m(); }
double *ommp_qm_helper_get_cqm(OMMP_QM_HELPER_PRT qm) { return Q(qm)->cqm(); }
int32_t ommp_qm_helper_get_npol(OMMP_QM_HELPER_PRT qm) { return Q(qm)->npol(); }
int32_t ommp_qm_helper_get_nmm(OMMP_QM_HELPER_PRT qm) { return Q(qm)->nmm(); }
int32_t ommp_qm_helper_get_qm_atoms(OMMP_QM_HELPER_PRT qm) { return Q(qm)->qm_atoms(); }

void ommp_enable_fmm(OMMP_SYSTEM_PRT s) { fatal_if(S(s)->set_fmm(true, S(s)->fmm_order())); }
void ommp_disable_fmm(OMMP_SYSTEM_PRT s) { fatal_if(S(s)->set_fmm(false, S(s)->fmm_order())); }
bool ommp_use_fmm(OMMP_SYSTEM_PRT s) { return S(s)->fmm_on(); }
int32_t ommp_gpu_set_fmm(OMMP_SYSTEM_PRT s, int32_t on, int32_t order) { return S(s)->set_fmm(on != 0, order); }
void ommp_set_fmm_lmax_pol(OMMP_SYSTEM_PRT s, int32_t l) { fatal_if(S(s)->set_fmm_order_pol(l)); }
void ommp_set_fmm_lmax(OMMP_SYSTEM_PRT s, int32_t l) { fatal_if(S(s)->set_fmm_order_static(l)); }
void ommp_set_fmm_distance(OMMP_SYSTEM_PRT s, double d) { fatal_if(S(s)->set_fmm_distance(d)); }
void ommp_set_fmm_min_cell_size(OMMP_SYSTEM_PRT s, double d) { fatal_if(S(s)->set_fmm_min_cell_size(d)); }
int32_t ommp_gpu_set_fmm_lmax_pol(OMMP_SYSTEM_PRT s, int32_t l) { return S(s)->set_fmm_order_pol(l); }
int32_t ommp_gpu_set_fmm_lmax(OMMP_SYSTEM_PRT s, int32_t l) { return S(s)->set_fmm_order_static(l); }
int32_t ommp_gpu_set_fmm_distance(OMMP_SYSTEM_PRT s, double d) { return S(s)->set_fmm_distance(d); }
int32_t ommp_gpu_set_fmm_min_cell_size(OMMP_SYSTEM_PRT s, double d) { return S(s)->set_fmm_min_cell_size(d); }
void ommp_gpu_get_fmm_settings(OMMP_SYSTEM_PRT s, int32_t *lmax_pol, int32_t *lmax, double *min_leaf) {
  if (lmax_pol) *lmax_pol = S(s)->fmm_order();
  if (lmax) *lmax = S(s)->fmm_order_static();
  if (min_leaf) *min_leaf = S(s)->fmm_min_leaf();
}
void ommp_gpu_set_fmm_auto(int32_t on) { ommp::set_fmm_auto(on != 0); }

const char *ommp_gpu_last_error(void) { return ommp::last_error(); }
void ommp_gpu_set_solver_tol(OMMP_SYSTEM_PRT s, double tol) { S(s)->set_tol(tol); }
void ommp_gpu_set_solver_maxiter(OMMP_SYSTEM_PRT s, int32_t n) { S(s)->set_maxiter(n); }
void ommp_gpu_set_precision(OMMP_SYSTEM_PRT s, int32_t mode) { S(s)->set_precision(mode); }
int32_t ommp_gpu_set_fp64_kernel(OMMP_SYSTEM_PRT s, int32_t mode) { return S(s)->set_fp64_kernel(mode); }
int32_t ommp_gpu_set_fp32_kernel(OMMP_SYSTEM_PRT s, int32_t mode) { return S(s)->set_fp32_kernel(mode); }
int32_t ommp_gpu_get_fp32_shape(OMMP_SYSTEM_PRT s, int32_t ncol, int32_t *shape) {
  return S(s)->fp32_shape(ncol, shape);
}
int32_t ommp_gpu_set_inner_preconditioner(OMMP_SYSTEM_PRT s, int32_t mode) {
  return S(s)->set_inner_preconditioner(mode);
}
int32_t ommp_gpu_set_inner_blocks(OMMP_SYSTEM_PRT s, int32_t max_sites, double link_bohr) {
  return S(s)->set_inner_blocks(max_sites, link_bohr);
}
void ommp_gpu_set_use_graphs(OMMP_SYSTEM_PRT s, int32_t on) { S(s)->set_use_graphs(on != 0); }
void ommp_gpu_set_block_cg(OMMP_SYSTEM_PRT s, int32_t on) { S(s)->set_block_cg(on != 0); }
int32_t ommp_gpu_set_residual_update(OMMP_SYSTEM_PRT s, int32_t mode) { return S(s)->set_residual_update(mode); }
int32_t ommp_gpu_set_external_fields_batch(OMMP_SYSTEM_PRT s, int32_t nfields, const double *fields, double *ipd_out,
                                           double *energies) {
  return S(s)->solve_batch_host(nfields, fields, ipd_out, energies);
}
int32_t ommp_gpu_set_external_fields_batch_device(OMMP_SYSTEM_PRT s, int32_t nfields, const double *fields_dev,
                                                  double *ipd_out_dev, double *energies) {
  return S(s)->solve_batch(nfields, fields_dev, ipd_out_dev, energies);
}
void ommp_gpu_clear_guess(OMMP_SYSTEM_PRT s) { S(s)->clear_guess(); }

int32_t ommp_gpu_get_iterations(OMMP_SYSTEM_PRT s, int32_t set) { return S(s)->stats().iters[set & 1]; }
int32_t ommp_gpu_get_residual_history(OMMP_SYSTEM_PRT s, int32_t set, double *out, int32_t maxn) {
  const auto &h = S(s)->stats().hist[set & 1];
  int32_t n = (int32_t)h.size();
  for (int32_t i = 0; i < n && i < maxn; ++i) out[i] = h[i];
  return n;
}
int64_t ommp_gpu_get_counter(OMMP_SYSTEM_PRT s, int32_t which) {
  const auto &st = S(s)->stats();
  switch (which) {
    case 0: return st.f64_matvecs;
    case 1: return st.f32_matvecs;
    case 2: return st.outer;
    case 3: return st.inner_iters;
    case 4: return st.ds_matvecs;
    case 5: return st.updates;
    default: return -1;
  }
}
double ommp_gpu_last_solve_ms(OMMP_SYSTEM_PRT s) { return S(s)->last_solve_ms(); }

int32_t ommp_gpu_get_e_m2d(OMMP_SYSTEM_PRT s, double *out) { return S(s)->e_m2d(out); }
int32_t ommp_gpu_tmatvec(OMMP_SYSTEM_PRT s, const double *x, double *y, int32_t nrhs, int32_t dodiag, int32_t matv) {
  return S(s)->tmatvec(x, y, nrhs, dodiag != 0, matv);
}
int32_t ommp_gpu_tmatvec_ds(OMMP_SYSTEM_PRT s, const double *x, double *y, int32_t nrhs) {
  return S(s)->tmatvec_ds(x, y, nrhs);
}
int32_t ommp_gpu_tmatvec_fp32(OMMP_SYSTEM_PRT s, const double *x, double *y, int32_t nrhs) {
  return S(s)->tmatvec_f32(x, y, nrhs);
}
void ommp_gpu_enable_kernel_timing(OMMP_SYSTEM_PRT s, int32_t on) { S(s)->enable_kernel_timing(on != 0); }
void ommp_gpu_kernel_stats(OMMP_SYSTEM_PRT s, int32_t which, int64_t *launches, double *total_ms,
                           int64_t *columns) {
  long long l = 0, c = 0;
  double ms = 0;
  S(s)->kernel_stats(which, l, ms, c);
  *launches = l;
  *total_ms = ms;
  if (columns) *columns = c;
}
int32_t ommp_gpu_synchronize(OMMP_SYSTEM_PRT s) { return S(s)->sync(); }
void ommp_gpu_reset_kernel_stats(OMMP_SYSTEM_PRT s) { S(s)->reset_kernel_stats(); }
int32_t ommp_gpu_timer_record(OMMP_SYSTEM_PRT s, int32_t slot) { return S(s)->timer_record(slot); }
int32_t ommp_gpu_timer_elapsed(OMMP_SYSTEM_PRT s, int32_t a, int32_t b, double *ms) {
  return S(s)->timer_elapsed(a, b, *ms);
}
int32_t ommp_gpu_flush_l2(OMMP_SYSTEM_PRT s, int64_t bytes) { return S(s)->flush_l2((size_t)bytes); }
int64_t ommp_gpu_kernel_launch_count(void) { return ommp::gpu::launch_count(); }

int32_t ommp_gpu_device_alloc(int64_t bytes, void **ptr) {
  *ptr = nullptr;
  cudaError_t e = cudaMalloc(ptr, (size_t)(bytes > 0 ? bytes : 1));
  if (e != cudaSuccess) {
    ommp::set_last_error(std::string("cudaMalloc: ") + cudaGetErrorString(e));
    return ommp::kErrMemory;
  }
  return ommp::kOk;
}
int32_t ommp_gpu_device_free(void *ptr) {
  return cudaFree(ptr) == cudaSuccess ? ommp::kOk : ommp::kErrCuda;
}
int32_t ommp_gpu_copy_to_device(void *dst, const void *src, int64_t bytes) {
  cudaError_t e = cudaMemcpy(dst, src, (size_t)bytes, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    ommp::set_last_error(std::string("cudaMemcpy: ") + cudaGetErrorString(e));
    return ommp::kErrCuda;
  }
  return ommp::kOk;
}
int32_t ommp_gpu_copy_to_host(void *dst, const void *src, int64_t bytes) {
  cudaError_t e = cudaMemcpy(dst, src, (size_t)bytes, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) {
    ommp::set_last_error(std::string("cudaMemcpy: ") + cudaGetErrorString(e));
    return ommp::kErrCuda;
  }
  return ommp::kOk;
}
int32_t ommp_gpu_device_mem_info(int64_t *free_bytes, int64_t *total_bytes) {
  size_t f = 0, t = 0;
  cudaError_t e = cudaMemGetInfo(&f, &t);
  *free_bytes = (int64_t)f;
  *total_bytes = (int64_t)t;
  if (e != cudaSuccess) {
    ommp::set_last_error(std::string("cudaMemGetInfo: ") + cudaGetErrorString(e));
    return ommp::kErrCuda;
  }
  return ommp::kOk;
}
int32_t ommp_gpu_measure_pipe_peak(int32_t fp64, double *tflops) {
  *tflops = 0.0;
  void *out = nullptr;
  if (cudaMalloc(&out, 1 << 20) != cudaSuccess) return ommp::kErrMemory;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  int iters = fp64 ? 100 : 4000;  // a few hundred ms per launch on GB300
  ommp::gpu::launch_fma_peak(fp64 != 0, iters, out, 0);  // warm-up
  double best = 0.0;
  for (int rep = 0; rep < 5; ++rep) {
    cudaEventRecord(a, 0);
    double flop = ommp::gpu::launch_fma_peak(fp64 != 0, iters, out, 0);
    cudaEventRecord(b, 0);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    if (ms > 0) best = std::max(best, flop / (ms * 1e-3) / 1e12);
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(out);
  *tflops = best;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    ommp::set_last_error(std::string("peak kernel: ") + cudaGetErrorString(e));
    return ommp::kErrCuda;
  }
  return ommp::kOk;
}
int32_t ommp_gpu_device_sm_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return 0;
  return ommp::gpu::sm_count();
}

}  // extern "C"
