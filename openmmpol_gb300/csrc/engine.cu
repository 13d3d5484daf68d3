// System lifetime, device residency and the polarization solvers.
//
// Solver semantics follow the reference (file:line in OpenMMPol):
//   polarization driver     src/mod_polarization.F90:49-313
//   conjugate gradient      src/mod_solvers.F90:86-216
//   Jacobi + Pulay DIIS     src/mod_solvers.F90:218-469
//   inversion               src/mod_solvers.F90:41-84
//   set_external_field      src/mod_interface.F90:184-233
//   get_polelec_energy      src/mod_interface.F90:343-370, energy_MM_pol
//                           src/mod_electrostatics.F90:943-976
//   update_coordinates      src/mod_mmpol.F90:325-371
// Every vector lives on the device; the host reads one small status record
// per iteration to decide when to stop.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <mutex>

#include "engine.h"
#include "log.h"

namespace ommp {

namespace {
thread_local std::string g_last_error;  // per host thread (the server runs workers)
constexpr size_t kMaxDenseBytes = size_t(24) << 30;  // incore T / inversion budget

template <typename T>
int dalloc(T *&p, size_t count) {
  p = nullptr;
  if (count == 0) count = 1;
  return cudaMalloc((void **)&p, count * sizeof(T)) == cudaSuccess ? 0 : 1;
}
}  // namespace

void set_last_error(const std::string &s) { g_last_error = s; }
const char *last_error() { return g_last_error.c_str(); }

namespace {
std::mutex g_pin_mu;
std::map<size_t, std::vector<void *>> g_pin_free;  // size class -> returned buffers
std::map<void *, size_t> g_pin_class;               // every pool buffer -> its size class
size_t pin_class(size_t bytes) {
  size_t c = 256;
  while (c < bytes) c <<= 1;
  return c;
}
}  // namespace

cudaError_t pinned_alloc(void **p, size_t bytes) {
  const size_t c = pin_class(bytes);
  {
    std::lock_guard<std::mutex> lk(g_pin_mu);
    std::vector<void *> &fl = g_pin_free[c];
    if (!fl.empty()) {
      *p = fl.back();
      fl.pop_back();
      return cudaSuccess;
    }
  }
  cudaError_t e = cudaMallocHost(p, c);
  if (e == cudaSuccess) {
    std::lock_guard<std::mutex> lk(g_pin_mu);
    g_pin_class[*p] = c;
  }
  return e;
}

void pinned_free(void *p) {
  if (!p) return;
  std::lock_guard<std::mutex> lk(g_pin_mu);
  auto it = g_pin_class.find(p);
  if (it != g_pin_class.end()) g_pin_free[it->second].push_back(p);
}

int System::check(cudaError_t e, const char *what) {
  if (e == cudaSuccess) return kOk;
  set_last_error(std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e));
  return kErrCuda;
}

template <typename T>
int System::alloc(T *&p, size_t count) {
  p = nullptr;
  if (count == 0) count = 1;
  if (async_alloc_ && st_) {
    static std::once_flag pool_once;
    std::call_once(pool_once, [] {
      // keep freed memory in the pool: returning it to the driver would
      // synchronise
      int dev = 0;
      cudaMemPool_t pool;
      if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
        unsigned long long thr = ~0ull;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
      }
      cudaGetLastError();
    });
    if (cudaMallocAsync((void **)&p, count * sizeof(T), st_) != cudaSuccess) {
      cudaGetLastError();
      p = nullptr;
      return 1;
    }
    async_bufs_.push_back((void *)p);
    return 0;
  }
  return cudaMalloc((void **)&p, count * sizeof(T)) == cudaSuccess ? 0 : 1;
}

void System::release(void *p) {
  if (!p) return;
  auto it = std::find(async_bufs_.begin(), async_bufs_.end(), p);
  if (it != async_bufs_.end()) {
    cudaFreeAsync(p, st_);
    async_bufs_.erase(it);
  } else {
    cudaFree(p);
  }
}

System::~System() {
  if (st_) cudaStreamSynchronize(st_);
  free_ws(ws_);
  free_ws(wsb_);
  void *bufs[] = {d_.pol_pos, d_.pol_a, d_.pol_alpha, d_.polar_mm, d_.pol_pos32, d_.pol_pos32lo, d_.pol_a32,
                  d_.pol_wa32, ds_scratch_, d_.mm_pos32, d_.mm_pos32lo, d_.mm_tile_box32,
                  d_.mm_wa32, d_.mm_pos,
                  d_.mm_a, d_.mm_q, d_.m2d_ri, d_.m2d_src, d_.m2d_sP, d_.m2d_sD, d_.d2d_ri, d_.d2d_src,
                  d_.d2d_s, e_m2d_, ipd_, rhs_, ext_, x_, r_, p_, h_, z_, x32_, r32_, p32_, h32_, z32_,
                  alpha32_, scratch_, scratch32_, partial_, dots_, hist_, cols_, flag_, tmat_, piv_,
                  info_, diis_x_, diis_e_, d_.tile_box32, ext_buf_, blk_info_, blk_minv_, near_ri_, near_ci_,
                  near_blk_};
  for (void *b : bufs) release(b);
  if (flush_buf_) cudaFree(flush_buf_);
  release(sym_scratch_);
  free_grad_state(grad_);
  free_fmm_state(fmm_);
  free_fmm_state(fmms_);
  kt_resolve();
  for (auto &e : kfree_) {
    cudaEventDestroy(e.a);
    cudaEventDestroy(e.b);
  }
  for (auto ev : tev_)
    if (ev) cudaEventDestroy(ev);
  if (ev0_) cudaEventDestroy(ev0_);
  if (ev1_) cudaEventDestroy(ev1_);
  if (st_) cudaStreamSynchronize(st_);  // stream-ordered frees and read-backs
  pinned_free(cols_h_);
  pinned_free(scal_h_);
  if (st_) cudaStreamDestroy(st_);
}

System *System::from_mmp(const std::string &path, std::string &err, int &status) {
  System *s = load_host(path, err, status);
  if (!s) return nullptr;
  status = s->attach_device();
  if (status != kOk) {
    err = last_error();
    delete s;
    return nullptr;
  }
  return s;
}

System *System::load_host(const std::string &path, std::string &err, int &status) {
  System *s = new System();
  if (!read_mmp(path, s->m_, err) || !prepare_model(s->m_, err)) {
    status = kErrInput;
    delete s;
    return nullptr;
  }
  build_m2d_pairs(s->m_, s->m2d_pairs_);
  build_d2d_pairs(s->m_, s->d2d_pairs_);
  if (s->m_.fmm_requested && fmm_auto()) {
    s->fmm_on_ = true;
    log_msg(kVerbHigh, nullptr, "More than 1000 MM atoms: FMM enabled (ommp_gpu_set_fmm_auto is on).");
  } else if (s->m_.fmm_requested) {
    log_msg(kVerbHigh, nullptr,
            "More than 1000 MM atoms: the reference would enable FMM here; this library keeps the "
            "direct sums unless ommp_enable_fmm or ommp_gpu_set_fmm_auto is called.");
  }
  status = kOk;
  return s;
}

int System::attach_device() { return upload_static(); }

size_t System::device_bytes_estimate() const {
  const size_t n = m_.npol, m = m_.mm, nv = 3 * n, nipd = m_.n_ipd;
  const size_t nm2d = m2d_pairs_.src.size(), nd2d = d2d_pairs_.src.size();
  gpu::DevSites d;
  d.n = (int)n;
  d.m = (int)m;
  int sms = gpu::sm_count();
  size_t s32 = gpu::tmu_scratch_doubles(d, 2, gpu::tmu32_max_split(d, sms)) + 8 * ((n + 127) / 128);
  size_t s64 = std::max(gpu::m2d_scratch_doubles(d, gpu::m2d_pick_split(d, sms)),
                        gpu::tmu_scratch_doubles(d, 2, gpu::tmu_pick_split(d, 2, sms, false)));
  size_t sym = n >= 2048 ? gpu::tmu_sym_scratch_doubles(d, 4) : 0;
  size_t bytes = 8 * (6 * n + 5 * m + m * m_.ld_cart + 2 * nm2d + nd2d + nv * (2 * nipd + 3 + 10)) +
                 4 * (9 * n + 2 * m + 10 * nv + 2 * (n + 1) + nm2d + nd2d) + 4 * s32 + 8 * s64 + 8 * sym +
                 8 * (gpu::kRedBlocks * 32 + 64 + 2 * (size_t)maxhist_);
  // double-single copies of the positions, static-site tile boxes, and the
  // double-single kernels' split partials (allocated in that mode only)
  const size_t ds_split = std::max(2 * gpu::tmu_ds_pick_split(d, sms), gpu::m2d_ds_pick_split(d, sms));
  bytes += 16 * (n + 2 * m + 2 * ((m + 127) / 128)) + 8 * ds_split * nv;
  // near-field couplings of the Neumann step (about a dozen per site in water)
  if (inner_precond_ == 2) bytes += 4 * (n + 1) + 40 * 24 * n;
  return bytes + (size_t(4) << 20);  // events, flags, rounding
}

// A copy from pageable memory is staged by the driver on the calling thread
// and, in a request server, held up the engine thread's launches (uploads of
// new systems took 20-40 ms under load against 2-6 ms alone); from a
// page-locked buffer the copy is asynchronous.  The buffer comes from the
// process-wide pool and goes back at h2d_release(), after a synchronisation
// of the system's stream.
void System::h2d(void *dst, const void *src, size_t bytes) {
  if (!bytes) return;
  void *buf = nullptr;
  if (pinned_alloc(&buf, bytes) != cudaSuccess) {
    cudaGetLastError();
    cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st_);
    return;
  }
  std::memcpy(buf, src, bytes);
  cudaMemcpyAsync(dst, buf, bytes, cudaMemcpyHostToDevice, st_);
  staged_.push_back(buf);
}

void System::h2d_release() {
  for (void *b : staged_) pinned_free(b);
  staged_.clear();
}

int System::upload_static() {
  const HostModel &m = m_;
  int n = m.npol, mm = m.mm;
  int st = check(cudaStreamCreateWithFlags(&st_, cudaStreamNonBlocking), "stream");
  if (st) return st;
  cudaEventCreate(&ev0_);
  cudaEventCreate(&ev1_);
  d_.n = n;
  d_.m = mm;
  d_.amoeba = m.amoeba;
  d_.ld = m.ld_cart;
  int sms = gpu::sm_count();
  nsplit_m2d_ = gpu::m2d_pick_split(d_, sms);
  nsplit_tmu_ = gpu::tmu_pick_split(d_, 2, sms, false);
  nsplit_tmu32_ = gpu::tmu32_pick_split(d_, sms);
  const int f32_splits = gpu::tmu32_max_split(d_, sms);
  d_.ntile = (n + 127) / 128;
  size_t nv = 3 * (size_t)n;
  int nipd = m.n_ipd;
  int bad = 0;
  bad |= alloc(d_.pol_pos, n) | alloc(d_.pol_a, n) | alloc(d_.pol_alpha, n) | alloc(d_.polar_mm, n);
  bad |= alloc(d_.pol_pos32, n) | alloc(d_.pol_pos32lo, n) | alloc(d_.pol_a32, n) | alloc(alpha32_, n);
  bad |= alloc(d_.pol_wa32, n) | alloc(d_.mm_wa32, mm);
  bad |= alloc(d_.mm_pos, mm) | alloc(d_.mm_a, mm) | alloc(d_.mm_q, (size_t)mm * m.ld_cart);
  bad |= alloc(d_.m2d_ri, n + 1) | alloc(d_.m2d_src, m2d_pairs_.src.size()) |
         alloc(d_.m2d_sP, m2d_pairs_.src.size()) | alloc(d_.m2d_sD, m2d_pairs_.src.size());
  bad |= alloc(d_.d2d_ri, n + 1) | alloc(d_.d2d_src, d2d_pairs_.src.size()) |
         alloc(d_.d2d_s, d2d_pairs_.src.size());
  bad |= alloc(e_m2d_, nv * nipd) | alloc(ipd_, nv * nipd) | alloc(rhs_, nv * 2) | alloc(ext_, nv);
  bad |= alloc(x_, nv * 2) | alloc(r_, nv * 2) | alloc(p_, nv * 2) | alloc(h_, nv * 2) | alloc(z_, nv * 2);
  bad |= alloc(x32_, nv * 2) | alloc(r32_, nv * 2) | alloc(p32_, nv * 2) | alloc(h32_, nv * 2) |
         alloc(z32_, nv * 2);
  scratch_n_ = std::max(gpu::m2d_scratch_doubles(d_, nsplit_m2d_), gpu::tmu_scratch_doubles(d_, 2, nsplit_tmu_));
  // FP32 scratch for twice the default source split (the autotuner tries both)
  bad |= alloc(scratch_, scratch_n_) | alloc(scratch32_, gpu::tmu_scratch_doubles(d_, 2, f32_splits));
  bad |= alloc(d_.tile_box32, 2 * (size_t)d_.ntile);
  bad |= alloc(d_.mm_pos32, mm) | alloc(d_.mm_pos32lo, mm) | alloc(d_.mm_tile_box32, 2 * (size_t)((mm + 127) / 128));
  bad |= alloc(partial_, (size_t)gpu::kRedBlocks * 32) | alloc(dots_, 64) | alloc(hist_, 2 * (size_t)maxhist_);
  bad |= alloc(cols_, 2) | alloc(flag_, 1) | alloc(info_, 1);
  if (bad || pinned_alloc((void **)&cols_h_, 2 * sizeof(gpu::CgCol)) != cudaSuccess ||
      pinned_alloc((void **)&scal_h_, 64 * sizeof(double)) != cudaSuccess) {
    set_last_error("out of device memory while allocating the system");
    return kErrMemory;
  }
  ws_.cap = 2;
  ws_.x = x_, ws_.r = r_, ws_.p = p_, ws_.h = h_, ws_.z = z_, ws_.rhs = rhs_;
  ws_.x32 = x32_, ws_.r32 = r32_, ws_.p32 = p32_, ws_.h32 = h32_, ws_.z32 = z32_;
  ws_.scratch32 = scratch32_;
  ws_.scratch32_nsplit = f32_splits;
  ws_.partial = partial_, ws_.dots = dots_, ws_.hist = hist_;
  ws_.cols = cols_, ws_.cols_h = cols_h_, ws_.scal_h = scal_h_;
  ws_.owned = false;
  d_.m2d_nnz = (int)m2d_pairs_.src.size();
  d_.d2d_nnz = (int)d2d_pairs_.src.size();
  auto up = [&](void *dst, const void *src, size_t bytes) { h2d(dst, src, bytes); };
  up(d_.m2d_ri, m2d_pairs_.ri.data(), (n + 1) * sizeof(int));
  up(d_.m2d_src, m2d_pairs_.src.data(), m2d_pairs_.src.size() * sizeof(int));
  up(d_.m2d_sP, m2d_pairs_.sP.data(), m2d_pairs_.sP.size() * sizeof(double));
  up(d_.m2d_sD, m2d_pairs_.sD.data(), m2d_pairs_.sD.size() * sizeof(double));
  up(d_.d2d_ri, d2d_pairs_.ri.data(), (n + 1) * sizeof(int));
  up(d_.d2d_src, d2d_pairs_.src.data(), d2d_pairs_.src.size() * sizeof(int));
  up(d_.d2d_s, d2d_pairs_.sP.data(), d2d_pairs_.sP.size() * sizeof(double));
  std::vector<double> alpha(m.pol), a(m.damping);
  std::vector<float> alpha32(n), a32(n);
  for (int k = 0; k < n; ++k) {
    alpha32[k] = (float)alpha[k];
    a32[k] = (float)a[k];
  }
  up(d_.pol_alpha, alpha.data(), n * sizeof(double));
  up(d_.pol_a, a.data(), n * sizeof(double));
  up(alpha32_, alpha32.data(), n * sizeof(float));
  up(d_.pol_a32, a32.data(), n * sizeof(float));
  up(d_.polar_mm, m.polar_mm.data(), n * sizeof(int));
  // FP32 damping pre-test data: (1/thole)^2 and a^2 (inf / 0 for static sites)
  std::vector<float2> pwa(n), mwa(mm);
  for (int j = 0; j < n; ++j) {
    double w = 1.0 / m.thole[m.polar_mm[j]];
    pwa[j] = make_float2((float)(w * w), (float)(m.damping[j] * m.damping[j]));
  }
  for (int i = 0; i < mm; ++i) {
    int p = m.mm_polar[i];
    double w = m.thole[i] > 0.0 ? 1.0 / m.thole[i] : std::numeric_limits<double>::infinity();
    double a = p >= 0 ? m.damping[p] : 0.0;
    mwa[i] = make_float2((float)(w * w), (float)(a * a));
  }
  up(d_.pol_wa32, pwa.data(), n * sizeof(float2));
  {
    std::vector<double> w(n);
    for (int j = 0; j < n; ++j) w[j] = 1.0 / m.thole[m.polar_mm[j]];
    d_.damp_r2max32 = gpu::damp_r2max32(m.amoeba, d_.damp_thr, w.data(), m.damping.data(), n);
    std::vector<double> mw(mm), ma(mm, 0.0);
    for (int i = 0; i < mm; ++i) {
      mw[i] = m.thole[i] > 0.0 ? 1.0 / m.thole[i] : std::numeric_limits<double>::infinity();
      if (m.mm_polar[i] >= 0) ma[i] = m.damping[m.mm_polar[i]];
    }
    d_.m2d_r2max32 = gpu::m2d_r2max32(m.amoeba, d_.damp_thr, w.data(), m.damping.data(), n, mw.data(), ma.data(), mm);
  }
  up(d_.mm_wa32, mwa.data(), mm * sizeof(float2));
  cudaMemsetAsync(ipd_, 0, nv * nipd * sizeof(double), st_);
  cudaMemsetAsync(e_m2d_, 0, nv * nipd * sizeof(double), st_);
  ipd_h_.assign(nv * nipd, 0.0);
  polar_mm_h_ = m.polar_mm;
  st = upload_geometry();
  if (st) return st;
  // place the no-allocation entry point's static scratch on this device now,
  // while the system allocates anyway (a failure here is retried by that call)
  noalloc_prepare_device();
  st = check(cudaStreamSynchronize(st_), "upload");
  h2d_release();
  return st;
}

int System::upload_geometry() {
  const HostModel &m = m_;
  int n = m.npol, mm = m.mm;
  const double inf = std::numeric_limits<double>::infinity();
  std::vector<gpu::Pos64> pp(n), mp(mm);
  std::vector<float4> pp32(n), pp32lo(n);
  std::vector<double> ma(mm, 0.0);
  double c[3] = {0, 0, 0};
  for (int i = 0; i < mm; ++i)
    for (int k = 0; k < 3; ++k) c[k] += m.cmm[3 * (size_t)i + k] / mm;
  cpol_h_.resize(3 * (size_t)n);
  for (int j = 0; j < n; ++j) {
    int a = m.polar_mm[j];
    const double *x = &m.cmm[3 * (size_t)a];
    double w = 1.0 / m.thole[a];
    pp[j] = gpu::Pos64{x[0], x[1], x[2], w};
    const double xc[3] = {x[0] - c[0], x[1] - c[1], x[2] - c[2]};
    pp32[j] = make_float4((float)xc[0], (float)xc[1], (float)xc[2], (float)w);
    pp32lo[j] = make_float4((float)(xc[0] - (double)pp32[j].x), (float)(xc[1] - (double)pp32[j].y),
                            (float)(xc[2] - (double)pp32[j].z), 0.f);
    for (int k = 0; k < 3; ++k) cpol_h_[3 * (size_t)j + k] = x[k];
  }
  for (int i = 0; i < mm; ++i) {
    const double *x = &m.cmm[3 * (size_t)i];
    double t = m.thole[i];
    mp[i] = gpu::Pos64{x[0], x[1], x[2], t > 0.0 ? 1.0 / t : inf};
    if (m.mm_polar[i] >= 0) ma[i] = m.damping[m.mm_polar[i]];
  }
  h2d(d_.pol_pos, pp.data(), n * sizeof(gpu::Pos64));
  h2d(d_.pol_pos32, pp32.data(), n * sizeof(float4));
  h2d(d_.pol_pos32lo, pp32lo.data(), n * sizeof(float4));
  std::vector<float4> boxes(2 * (size_t)d_.ntile);
  gpu::tile_boxes32(pp32.data(), n, boxes.data());
  if (n) h2d(d_.tile_box32, boxes.data(), boxes.size() * sizeof(float4));
  // static sites in double-single for the double-single E_M2D
  std::vector<float4> mp32(mm), mp32lo(mm);
  for (int i = 0; i < mm; ++i) {
    const double *x = &m.cmm[3 * (size_t)i];
    const double xc[3] = {x[0] - c[0], x[1] - c[1], x[2] - c[2]};
    mp32[i] = make_float4((float)xc[0], (float)xc[1], (float)xc[2], 0.f);
    mp32lo[i] = make_float4((float)(xc[0] - (double)mp32[i].x), (float)(xc[1] - (double)mp32[i].y),
                            (float)(xc[2] - (double)mp32[i].z), 0.f);
  }
  std::vector<float4> mboxes(2 * (size_t)((mm + 127) / 128));
  gpu::tile_boxes32(mp32.data(), mm, mboxes.data());
  if (mm) {
    h2d(d_.mm_pos32, mp32.data(), mm * sizeof(float4));
    h2d(d_.mm_pos32lo, mp32lo.data(), mm * sizeof(float4));
    h2d(d_.mm_tile_box32, mboxes.data(), mboxes.size() * sizeof(float4));
  }
  h2d(d_.mm_pos, mp.data(), mm * sizeof(gpu::Pos64));
  h2d(d_.mm_a, ma.data(), mm * sizeof(double));
  h2d(d_.mm_q, m.q.data(), m.q.size() * sizeof(double));
  // the host vectors above die at return: wait for the copies
  fmm_invalidate();  // the tree follows the geometry
  // block-Jacobi preconditioner of the FP32 inner solver (geometry-dependent)
  int bst = build_blocks();
  if (bst) return bst;
  const int st = check(cudaStreamSynchronize(st_), "geometry upload");
  h2d_release();
  return st;
}

int System::build_blocks() {
  const int n = m_.npol;
  std::vector<int> info;
  std::vector<float> minv;
  build_block_jacobi(m_, d2d_pairs_, d_.damp_thr, blk_max_, blk_link_, info, minv);
  cudaStreamSynchronize(st_);
  // a captured inner iteration holds the preconditioner's device pointers:
  // drop it before the buffers are replaced (it is captured again)
  for (Workspace *w : {&ws_, &wsb_}) {
    if (w->graph) cudaGraphExecDestroy(w->graph);
    w->graph = nullptr;
    w->graph_ncol = -1;
  }
  release(blk_info_);
  release(blk_minv_);
  blk_info_ = nullptr;
  blk_minv_ = nullptr;
  if (n > 0) {
    if (alloc(blk_info_, (size_t)n) || alloc(blk_minv_, minv.size())) {
      set_last_error("out of device memory for the block preconditioner");
      return kErrMemory;
    }
    h2d(blk_info_, info.data(), info.size() * sizeof(int));
    h2d(blk_minv_, minv.data(), minv.size() * sizeof(float));
  }
  // the near-field couplings follow the geometry: built again at the next
  // mixed solve (ensure_near)
  release(near_ri_);
  release(near_ci_);
  release(near_blk_);
  near_ri_ = near_ci_ = nullptr;
  near_blk_ = nullptr;
  blk_runs_.assign(info.begin(), info.end());
  // the host vectors die at return
  const int st = check(cudaStreamSynchronize(st_), "block preconditioner upload");
  h2d_release();
  return st;
}

// The near-field couplings of the Neumann step, built before the first mixed
// solve that uses them (on the calling thread: a request server's worker,
// not the engine), so that systems solved in FP64 never pay for them.
int System::ensure_near() {
  if (inner_precond_ != 2 || near_ri_ || !blk_info_ || d_.n == 0) return kOk;
  std::vector<int> ri, ci;
  std::vector<float> blk;
  build_near_field(m_, d2d_pairs_, d_.damp_thr, blk_runs_, kNearBohr, ri, ci, blk);
  if (alloc(near_ri_, ri.size()) || alloc(near_ci_, ci.size()) || alloc(near_blk_, blk.size())) {
    set_last_error("out of device memory for the near-field preconditioner");
    return kErrMemory;
  }
  // a captured inner iteration was built without the Neumann step
  for (Workspace *w : {&ws_, &wsb_}) {
    if (w->graph) cudaGraphExecDestroy(w->graph);
    w->graph = nullptr;
    w->graph_ncol = -1;
  }
  h2d(near_ri_, ri.data(), ri.size() * sizeof(int));
  h2d(near_ci_, ci.data(), ci.size() * sizeof(int));
  h2d(near_blk_, blk.data(), blk.size() * sizeof(float));
  const int st = check(cudaStreamSynchronize(st_), "near-field preconditioner upload");
  h2d_release();
  return st;
}

int System::set_inner_blocks(int max_sites, double link_bohr) {
  if (max_sites < 1 || max_sites > kMaxBlockLimit || !(link_bohr >= 0.0)) {
    set_last_error("inner blocks: 1 <= max_sites <= 32 and link distance >= 0 bohr");
    return kErrBadArg;
  }
  blk_max_ = max_sites;
  blk_link_ = link_bohr;
  return build_blocks();
}

int System::sync() {
  int st = check(cudaStreamSynchronize(st_), "synchronize");
  return st;
}

System::KEv System::kt_begin(int kind, int cols) {
  KEv e;
  if (!kfree_.empty()) {
    e = kfree_.back();
    kfree_.pop_back();
  } else {
    cudaEventCreate(&e.a);
    cudaEventCreate(&e.b);
  }
  e.kind = kind;
  e.cols = cols;
  cudaEventRecord(e.a, st_);
  return e;
}

void System::kt_end(KEv &e) {
  cudaEventRecord(e.b, st_);
  kpending_.push_back(e);
  if (kpending_.size() > 4096) kt_resolve();
}

void System::kt_resolve() {
  for (auto &e : kpending_) {
    cudaEventSynchronize(e.b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e.a, e.b);
    klaunch_[e.kind] += 1;
    kcols_[e.kind] += e.cols;
    kms_[e.kind] += ms;
    kfree_.push_back(e);
  }
  kpending_.clear();
}

void System::kernel_stats(int which, long long &launches, double &ms, long long &columns) {
  kt_resolve();
  const int k = which >= 0 && which < 4 ? which : 0;
  launches = klaunch_[k];
  ms = kms_[k];
  columns = kcols_[k];
}

void System::reset_kernel_stats() {
  kt_resolve();
  for (int k = 0; k < 4; ++k) {
    klaunch_[k] = 0;
    kcols_[k] = 0;
    kms_[k] = 0.0;
  }
}

int System::timer_record(int slot) {
  if (slot < 0 || slot > 7) {
    set_last_error("timer slot must be 0..7");
    return kErrBadArg;
  }
  if (!tev_[slot]) cudaEventCreate(&tev_[slot]);
  return check(cudaEventRecord(tev_[slot], st_), "timer record");
}

int System::timer_elapsed(int a, int b, double &ms) {
  if (a < 0 || a > 7 || b < 0 || b > 7 || !tev_[a] || !tev_[b]) {
    set_last_error("timer slots not recorded");
    return kErrBadArg;
  }
  int st = check(cudaEventSynchronize(tev_[b]), "timer sync");
  if (st) return st;
  float f = 0.f;
  st = check(cudaEventElapsedTime(&f, tev_[a], tev_[b]), "timer elapsed");
  ms = f;
  return st;
}

int System::flush_l2(size_t bytes) {
  if (bytes > flush_bytes_) {
    if (flush_buf_) cudaFree(flush_buf_);
    flush_buf_ = nullptr;
    flush_bytes_ = 0;
    if (cudaMalloc(&flush_buf_, bytes) != cudaSuccess) {
      set_last_error("out of device memory for the L2 flush buffer");
      return kErrMemory;
    }
    flush_bytes_ = bytes;
  }
  return check(cudaMemsetAsync(flush_buf_, (int)(++flush_tag_ & 0xff), bytes, st_), "L2 flush");
}

int System::ensure_m2d() {
  // the method the mode asks for: double-single in the mixed-ds mode, the
  // FMM when it is switched on, else the direct FP64 sums; a cached field
  // serves if it came from that method or from the direct FP64 sums
  const bool ds = precision_ == kPrecMixedDS;
  const int want = ds ? kM2dDS : (fmm_on_ ? kM2dFMM : kM2dDirect);
  if (m2d_done_ && (m2d_method_ == want || m2d_method_ == kM2dDirect)) return kOk;
  cudaMemsetAsync(flag_, 0, sizeof(int), st_);
  int method = kM2dDirect;
  if (ds) {
    int st = ensure_ds_scratch();
    if (st) return st;
    gpu::launch_m2d_ds(d_, e_m2d_, ds_scratch_, nsplit_m2d_ds_, flag_, st_);
    method = kM2dDS;
  } else {
    bool done = false;
    if (fmm_on_) {  // the fast multipole method (too small a system: direct)
      int st = fmm_m2d(e_m2d_, done);
      if (st) return st;
    }
    if (done)
      method = kM2dFMM;
    else
      gpu::launch_m2d(d_, e_m2d_, scratch_, nsplit_m2d_, flag_, st_);
  }
  m2d_method_ = method;
  int flag = 0;
  cudaMemcpyAsync(&flag, flag_, sizeof(int), cudaMemcpyDeviceToHost, st_);
  int st = check(cudaStreamSynchronize(st_), "M2D field");
  if (st) return st;
  if (flag) {
    set_last_error(
        "Requesting Coulomb kernel for two atoms placed in the same point, this could be an internal bug or "
        "a problem in your input file, please check.");
    return kErrNumeric;
  }
  m2d_done_ = true;
  return kOk;
}

int System::e_m2d(double *out) {
  int st = ensure_m2d();
  if (st) return st;
  size_t bytes = 3 * (size_t)d_.n * m_.n_ipd * sizeof(double);
  cudaMemcpyAsync(out, e_m2d_, bytes, cudaMemcpyDeviceToHost, st_);
  return check(cudaStreamSynchronize(st_), "E_M2D copy");
}

int System::ensure_tmat() {
  if (tmat_ok_) return kOk;
  size_t nn = 3 * (size_t)d_.n;
  if (nn * nn * sizeof(double) > kMaxDenseBytes) {
    set_last_error("the dense T matrix does not fit the in-core budget");
    return kErrMemory;
  }
  if (!tmat_) {
    if (dalloc(tmat_, nn * nn) || dalloc(piv_, nn)) {
      set_last_error("out of device memory for the dense T matrix");
      return kErrMemory;
    }
  }
  gpu::launch_build_tmat(d_, tmat_, st_);
  tmat_ok_ = true;
  lu_ok_ = false;
  return check(cudaGetLastError(), "T matrix");
}

int System::matvec64(int matv, int ncol, const double *x, double *y, bool dodiag) {
  if (matv == kMatvIncore && tmat_ok_) {
    gpu::launch_gemv(3 * d_.n, tmat_, x, y, dodiag, d_.pol_alpha, ncol, st_);
    return kOk;
  }
  if (fmm_on_) {
    int st = fmm_prepare();
    if (st) return st;
    if (fmm_tree()) {  // else too small for a tree: the direct sums below
      KEv e;
      if (ktime_on_) e = kt_begin(0, ncol);
      st = fmm_tmu(ncol, x, y, dodiag);
      if (ktime_on_) kt_end(e);
      if (st) return st;
      stats_.f64_matvecs += 1;
      return kOk;
    }
  }
  {
    bool sym = fp64_kernel_ == 2 || (fp64_kernel_ == 0 && d_.n >= 2048);
    if (sym && ensure_sym_scratch() != kOk) {
      sym = false;  // not enough memory for the partials: all-ordered-pairs kernel
      log_msg(kVerbHigh, nullptr, "symmetric T.mu scratch does not fit: using the target-outer kernel");
    }
    KEv e;
    if (ktime_on_) e = kt_begin(0, ncol);
    if (sym) {
      gpu::launch_tmu_f64_sym(d_, ncol, x, y, dodiag, sym_scratch_, st_, 4);
    } else {
      // the split partials hold two columns: larger blocks go two at a time
      const size_t nv = 3 * (size_t)d_.n;
      for (int c0 = 0; c0 < ncol; c0 += 2)
        gpu::launch_tmu_f64(d_, std::min(2, ncol - c0), x + c0 * nv, y + c0 * nv, dodiag, scratch_, nsplit_tmu_,
                            st_);
    }
    if (ktime_on_) kt_end(e);
    stats_.f64_matvecs += 1;
  }
  return kOk;
}

// fixed-point accumulators of the symmetric products (FP64, double-single
// and FP32 share them: they run one after another on the system's stream)
int System::ensure_sym_scratch() {
  if (sym_scratch_) return kOk;
  if (alloc(sym_scratch_, gpu::tmu_sym_scratch_doubles(d_, 4))) {
    sym_scratch_ = nullptr;
    cudaGetLastError();
    set_last_error("out of device memory for the symmetric-product accumulators");
    return kErrMemory;
  }
  return kOk;
}

// FP64-accurate product for the refinement residual: the FP64 kernel, or in
// the double-single mode the double-single kernel (one column at a time)
int System::ensure_ds_scratch() {
  if (ds_scratch_) return kOk;
  nsplit_ds_ = gpu::tmu_ds_pick_split(d_, gpu::sm_count());
  nsplit_m2d_ds_ = gpu::m2d_ds_pick_split(d_, gpu::sm_count());
  if (alloc(ds_scratch_, (size_t)std::max(2 * nsplit_ds_, nsplit_m2d_ds_) * 3 * d_.n)) {
    ds_scratch_ = nullptr;
    set_last_error("out of device memory for the double-single kernels");
    return kErrMemory;
  }
  return kOk;
}

int System::matvec_residual(int ncol, const double *x, double *y) {
  if (precision_ != kPrecMixedDS) return matvec64(kMatvDirect, ncol, x, y, true);
  int st = ensure_ds_scratch();
  if (st) return st;
  // the symmetric double-single kernel shares the FP64 one's fixed-point
  // scratch (without it: the target-outer double-single kernel)
  if (d_.n >= 2048 && ensure_sym_scratch() != kOk)
    log_msg(kVerbHigh, nullptr, "symmetric T.mu scratch does not fit: using the target-outer kernel");
  KEv e;
  if (ktime_on_) e = kt_begin(2, ncol);
  gpu::launch_tmu_ds(d_, ncol, x, y, true, ds_scratch_, nsplit_ds_, sym_scratch_, st_);
  if (ktime_on_) kt_end(e);
  stats_.ds_matvecs += 1;
  return kOk;
}

// Pulay DIIS extrapolation state lives on the host (tiny B matrix).
namespace {
int small_lu_solve(int n, std::vector<double> &a, std::vector<double> &b) {
  // column-major a (n x n), partial pivoting; returns 0 on success
  for (int k = 0; k < n; ++k) {
    int pr = k;
    double mx = std::fabs(a[(size_t)k * n + k]);
    for (int r = k + 1; r < n; ++r)
      if (std::fabs(a[(size_t)k * n + r]) > mx) mx = std::fabs(a[(size_t)k * n + r]), pr = r;
    if (a[(size_t)k * n + pr] == 0.0) return k + 1;
    if (pr != k) {
      for (int c = 0; c < n; ++c) std::swap(a[(size_t)c * n + k], a[(size_t)c * n + pr]);
      std::swap(b[k], b[pr]);
    }
    double d = a[(size_t)k * n + k];
    for (int r = k + 1; r < n; ++r) a[(size_t)k * n + r] /= d;
    for (int c = k + 1; c < n; ++c) {
      double f = a[(size_t)c * n + k];
      if (f != 0.0)
        for (int r = k + 1; r < n; ++r) a[(size_t)c * n + r] -= a[(size_t)k * n + r] * f;
    }
  }
  for (int k = 0; k < n; ++k)
    for (int r = k + 1; r < n; ++r) b[r] -= a[(size_t)k * n + r] * b[k];
  for (int k = n - 1; k >= 0; --k) {
    b[k] /= a[(size_t)k * n + k];
    for (int r = 0; r < k; ++r) b[r] -= a[(size_t)k * n + r] * b[k];
  }
  return 0;
}
}  // namespace

int System::diis64(int matv, const double *rhs, double *x, int set) {
  const int n = d_.n;
  const size_t nv = 3 * (size_t)n;
  const int nd = diis_max_;
  log_msg(kVerbLow, nullptr, "Solving linear system with jacobi solver");
  log_msg(kVerbLow, nullptr, "Max iter: %4d", maxiter_);
  log_msg(kVerbLow, nullptr, "Tolerance: %8.1E", tol_);
  log_msg(kVerbLow, nullptr, "DIIS is enabled with n = %4d", nd);
  if (!diis_x_ && (dalloc(diis_x_, nv * nd) || dalloc(diis_e_, nv * nd))) {
    set_last_error("out of device memory for the DIIS history");
    return kErrMemory;
  }
  double *xnew = z_, *y = h_;
  std::vector<double> B((size_t)(nd + 1) * (nd + 1), 0.0);
  auto Bat = [&](int r, int c) -> double & { return B[(size_t)c * (nd + 1) + r]; };
  gpu::launch_dots(1, nv, x, x, partial_, st_);
  gpu::launch_reduce_partials(1, partial_, dots_, st_);
  cudaMemcpyAsync(scal_h_, dots_, sizeof(double), cudaMemcpyDeviceToHost, st_);
  int st = check(cudaStreamSynchronize(st_), "DIIS start");
  if (st) return st;
  if (scal_h_[0] < kEpsRp) gpu::launch_scale_by_alpha(1, n, d_.pol_alpha, rhs, x, st_);
  int nmat = 1;
  double mx = 0.0;
  stats_.hist[set].clear();
  stats_.iters[set] = 0;
  for (int it = 1; it <= maxiter_; ++it) {
    int mst = matvec64(matv, 1, x, y, false);
    if (mst) return mst;
    gpu::launch_residual(nv, rhs, y, y, st_);
    gpu::launch_scale_by_alpha(1, n, d_.pol_alpha, y, xnew, st_);
    if (nd > 0) {
      cudaMemcpyAsync(diis_x_ + (size_t)(nmat - 1) * nv, xnew, nv * sizeof(double), cudaMemcpyDeviceToDevice, st_);
      // error vector e = xnew - x
      cudaMemcpyAsync(diis_e_ + (size_t)(nmat - 1) * nv, xnew, nv * sizeof(double), cudaMemcpyDeviceToDevice, st_);
      gpu::launch_axpby(nv, -1.0, x, 1.0, diis_e_ + (size_t)(nmat - 1) * nv, st_);
      if (nmat >= nd) {  // drop the ten oldest points
        for (int j = 2; j <= nmat - 10; ++j)
          for (int k = 2; k <= nmat - 10; ++k) Bat(j - 1, k - 1) = Bat(j + 10 - 1, k + 10 - 1);
        size_t cnt = (size_t)(nmat - 10) * nv;
        cudaMemcpyAsync(diis_x_, diis_x_ + 10 * nv, cnt * sizeof(double), cudaMemcpyDeviceToDevice, st_);
        cudaMemcpyAsync(diis_e_, diis_e_ + 10 * nv, cnt * sizeof(double), cudaMemcpyDeviceToDevice, st_);
        nmat -= 10;
      }
      // makeb: new row/column of B from dots against the newest error vector
      gpu::launch_dots_bcast(nmat, nv, diis_e_, diis_e_ + (size_t)(nmat - 1) * nv, partial_, st_);
      gpu::launch_reduce_partials(nmat, partial_, dots_, st_);
      cudaMemcpyAsync(scal_h_, dots_, nmat * sizeof(double), cudaMemcpyDeviceToHost, st_);
      st = check(cudaStreamSynchronize(st_), "DIIS dots");
      if (st) return st;
      if (nmat == 1) {
        Bat(0, 0) = 0.0;
        Bat(0, 1) = 1.0;
        Bat(1, 0) = 1.0;
        Bat(1, 1) = scal_h_[0];
      } else {
        Bat(nmat, 0) = 1.0;
        Bat(0, nmat) = 1.0;
        for (int i = 1; i <= nmat - 1; ++i) Bat(nmat, i) = Bat(i, nmat) = scal_h_[i - 1];
        Bat(nmat, nmat) = scal_h_[nmat - 1];
      }
      int nm1 = nmat + 1;
      std::vector<double> bl((size_t)nm1 * nm1), cex(nm1, 0.0);
      for (int c = 0; c < nm1; ++c)
        for (int r = 0; r < nm1; ++r) bl[(size_t)c * nm1 + r] = Bat(r, c);
      cex[0] = 1.0;
      if (small_lu_solve(nm1, bl, cex) != 0) {
        nmat = 1;
      } else {
        cudaMemcpyAsync(dots_, cex.data() + 1, nmat * sizeof(double), cudaMemcpyHostToDevice, st_);
        gpu::launch_lincomb(nmat, nv, diis_x_, nv, dots_, xnew, st_);
        nmat += 1;
      }
    }
    gpu::launch_diff_norms(nv, xnew, x, partial_, st_);
    gpu::launch_reduce_norms(partial_, dots_ + 32, st_);
    cudaMemcpyAsync(x, xnew, nv * sizeof(double), cudaMemcpyDeviceToDevice, st_);
    cudaMemcpyAsync(scal_h_, dots_ + 32, 2 * sizeof(double), cudaMemcpyDeviceToHost, st_);
    st = check(cudaStreamSynchronize(st_), "DIIS iteration");
    if (st) return st;
    double rms = std::sqrt(scal_h_[0] / (double)nv);
    mx = scal_h_[1];
    stats_.hist[set].push_back(mx);
    stats_.iters[set] = it;
    log_msg(kVerbHigh, nullptr, "iter=%4d residual norm (rms, max): %14.4E%14.4E", it, rms, mx);
    if (!std::isfinite(mx)) {
      set_last_error("non-finite increment in the Jacobi/DIIS solver");
      return kErrNumeric;
    }
    if (mx < tol_) {
      log_msg(kVerbHigh, nullptr, "Required convergence threshold reached, exiting iterative solver.");
      break;
    }
  }
  if (mx > tol_) {
    set_last_error("Iterative solver did not converged");
    return kErrNotConverged;
  }
  return kOk;
}

int System::inversion64(const double *rhs, double *x) {
  int st = ensure_tmat();
  if (st) return st;
  size_t nn = 3 * (size_t)d_.n;
  if (!lu_ok_) {
    double *lu = nullptr;
    if (dalloc(lu, nn * nn)) {
      set_last_error("out of device memory for the LU factors");
      return kErrMemory;
    }
    cudaMemcpyAsync(lu, tmat_, nn * nn * sizeof(double), cudaMemcpyDeviceToDevice, st_);
    gpu::launch_lu_factor((int)nn, lu, piv_, info_, nullptr, st_);
    int info = 0;
    cudaMemcpyAsync(&info, info_, sizeof(int), cudaMemcpyDeviceToHost, st_);
    st = check(cudaStreamSynchronize(st_), "LU");
    if (st) {
      cudaFree(lu);
      return st;
    }
    if (info) {
      cudaFree(lu);
      set_last_error("inversion solver: singular interaction matrix");
      return kErrNumeric;
    }
    // the factors replace T; an in-core matvec rebuilds T on demand
    std::swap(lu, tmat_);
    cudaFree(lu);
    tmat_ok_ = false;
    lu_ok_ = true;
  }
  cudaMemcpyAsync(x, rhs, nn * sizeof(double), cudaMemcpyDeviceToDevice, st_);
  gpu::launch_lu_solve((int)nn, tmat_, piv_, x, st_);
  return check(cudaStreamSynchronize(st_), "LU solve");
}

int System::polarization(const double *e, int solver, int matv, const bool *mask_in) {
  const int n = d_.n;
  const size_t nv = 3 * (size_t)n;
  if (n == 0) return kOk;
  if (solver == kSolverNone) solver = def_solver_;
  if (matv == kMatvNone) matv = def_matv_;
  bool mask[2] = {true, true};
  if (mask_in && m_.n_ipd > 1) mask[0] = mask_in[0], mask[1] = mask_in[1];
  const int nipd = m_.n_ipd;
  stats_ = SolveStats();
  if (matv == kMatvIncore || solver == kSolverInversion) {
    int st = ensure_tmat();
    if (st == kErrMemory && solver != kSolverInversion) {
      log_msg(kVerbHigh, nullptr, "In-core T does not fit the memory budget: using the direct matrix-vector product");
      matv = kMatvDirect;
    } else if (st) {
      return st;
    }
    if (matv == kMatvIncore && !tmat_ok_) {
      st = ensure_tmat();
      if (st) return st;
    }
  }
  cudaEventRecord(ev0_, st_);
  cudaMemsetAsync(x_, 0, nv * nipd * sizeof(double), st_);
  if (solver != kSolverInversion) {
    if (ipd_use_guess_)
      for (int k = 0; k < nipd; ++k)
        if (mask[k]) cudaMemcpyAsync(x_ + k * nv, ipd_ + k * nv, nv * sizeof(double), cudaMemcpyDeviceToDevice, st_);
    if (matv == kMatvIncore)
      log_msg(kVerbHigh, nullptr, "Matrix-Vector will be performed in-memory");
    else if (matv == kMatvDirect)
      log_msg(kVerbHigh, nullptr, "Matrix-Vector will be performed on-the-fly");
    else {
      set_last_error("Unknown matrix-vector method requested");
      return kErrBadArg;
    }
  }
  int st = kOk;
  if (solver == kSolverCG || solver == kSolverDIIS) {
    bool mixed = solver == kSolverCG && precision_ != kPrecFP64 && matv == kMatvDirect;
    if (mixed) {
      if (nipd == 2 && mask[0] && mask[1]) {
        // Identical D and P systems (right-hand sides and starting guesses
        // equal bit for bit, as for AMOEBA water where both fields exclude
        // the whole molecule) have identical solutions: the reference's P
        // solve seeded with the D dipoles returns them unchanged
        // (mod_polarization.F90:237-243).  Solve once and copy.
        cudaMemsetAsync(flag_, 0, sizeof(int), st_);
        gpu::launch_any_diff(nv, e, e + nv, flag_, st_);
        if (ipd_use_guess_) gpu::launch_any_diff(nv, x_, x_ + nv, flag_, st_);
        int differ = 1;
        cudaMemcpyAsync(&differ, flag_, sizeof(int), cudaMemcpyDeviceToHost, st_);
        st = check(cudaStreamSynchronize(st_), "D/P comparison");
        if (st) return st;
        if (differ) {
          // both sets share every pair evaluation
          st = mixed_ir(2, e, x_, 0, ipd_use_guess_);
        } else {
          st = mixed_ir(1, e, x_, 0, ipd_use_guess_);
          if (!st) {
            cudaMemcpyAsync(x_ + nv, x_, nv * sizeof(double), cudaMemcpyDeviceToDevice, st_);
            stats_.hist[1] = stats_.hist[0];
            stats_.iters[1] = stats_.iters[0];
          }
        }
      } else {
        for (int k = 0; k < nipd && !st; ++k)
          if (mask[k]) st = mixed_ir(1, e + k * nv, x_ + k * nv, k, ipd_use_guess_);
      }
    } else {
      auto run = [&](int k) {
        return solver == kSolverCG ? cg64(matv, 1, e + k * nv, x_ + k * nv, k) : diis64(matv, e + k * nv, x_ + k * nv, k);
      };
      if (nipd == 2) {
        if (mask[0]) st = run(0);
        // without a guess, D seeds P (:237-243)
        if (!st && mask[0] && mask[1] && !ipd_use_guess_)
          cudaMemcpyAsync(x_ + nv, x_, nv * sizeof(double), cudaMemcpyDeviceToDevice, st_);
        if (!st && mask[1]) st = run(1);
      } else {
        st = run(0);
      }
    }
  } else if (solver == kSolverInversion) {
    for (int k = 0; k < nipd && !st; ++k)
      if (mask[k]) st = inversion64(e + k * nv, x_ + k * nv);
  } else {
    set_last_error("Unknown solver for calculation of the induced point dipoles");
    return kErrBadArg;
  }
  if (st) return st;
  cudaMemcpyAsync(ipd_, x_, nv * nipd * sizeof(double), cudaMemcpyDeviceToDevice, st_);
  cudaEventRecord(ev1_, st_);
  ipd_done_ = true;
  ipd_use_guess_ = true;
  st = fetch_ipd();
  cudaEventElapsedTime(&last_ms_, ev0_, ev1_);
  return st;
}

int System::fetch_ipd() {
  size_t bytes = ipd_h_.size() * sizeof(double);
  cudaMemcpyAsync(ipd_h_.data(), ipd_, bytes, cudaMemcpyDeviceToHost, st_);
  return check(cudaStreamSynchronize(st_), "dipole copy");
}

int System::set_external_field(const double *ext_host, int solver, int matv, bool add_mm) {
  const size_t nv = 3 * (size_t)d_.n;
  cudaMemcpyAsync(ext_, ext_host, nv * sizeof(double), cudaMemcpyHostToDevice, st_);
  return set_external_field_device(ext_, solver, matv, add_mm);
}

int System::set_external_field_device(const double *ext, int solver, int matv, bool add_mm) {
  const size_t nv = 3 * (size_t)d_.n;
  ipd_done_ = false;
  if (d_.n == 0) return kOk;
  int st = kOk;
  if (add_mm) {
    st = ensure_m2d();
    if (st) return st;
    // rhs_[k] = E_M2D[k] + ext
    for (int k = 0; k < m_.n_ipd; ++k) gpu::launch_add(nv, e_m2d_ + k * nv, ext, rhs_ + k * nv, st_);
    // the reference does not forward matv on this path (mod_interface.F90:222)
    return polarization(rhs_, solver, kMatvNone, nullptr);
  }
  if (ext != rhs_) cudaMemcpyAsync(rhs_, ext, nv * sizeof(double), cudaMemcpyDeviceToDevice, st_);
  if (m_.n_ipd == 2) cudaMemsetAsync(rhs_ + nv, 0, nv * sizeof(double), st_);
  bool mask[2] = {true, false};
  return polarization(rhs_, solver, matv, mask);
}

int System::polelec_energy(double &e) {
  e = 0.0;
  const int n = d_.n;
  if (n == 0) return kOk;
  const size_t nv = 3 * (size_t)n;
  int st;
  if (!ipd_done_) {
    st = ensure_m2d();
    if (st) return st;
    st = polarization(e_m2d_, kSolverNone, kMatvNone, nullptr);
    if (st) return st;
  }
  st = ensure_m2d();
  if (st) return st;
  // -1/2 sum ipd(D) . E_M2D(P) for AMOEBA, -1/2 sum ipd . E_M2D otherwise
  const double *ef = m_.amoeba ? e_m2d_ + nv : e_m2d_;
  gpu::launch_dots(1, nv, ipd_, ef, partial_, st_);
  gpu::launch_reduce_partials(1, partial_, dots_, st_);
  cudaMemcpyAsync(scal_h_, dots_, sizeof(double), cudaMemcpyDeviceToHost, st_);
  st = check(cudaStreamSynchronize(st_), "energy");
  if (st) return st;
  e = -0.5 * scal_h_[0];
  return kOk;
}

int System::update_coordinates(const double *c) {
  std::copy(c, c + 3 * (size_t)m_.mm, m_.cmm.begin());
  std::string err;
  if (m_.amoeba && !rotate_multipoles(m_, err)) {
    set_last_error(err);
    return kErrInput;
  }
  m2d_done_ = ipd_done_ = ipd_use_guess_ = false;
  fixedelec_done_ = false;
  fixedelec_grad_done_ = false;
  tmat_ok_ = lu_ok_ = false;
  return upload_geometry();
}

int System::set_fp64_kernel(int mode) {
  if (mode < 0 || mode > 2) {
    set_last_error("FP64 kernel mode must be 0 (auto), 1 (all ordered pairs) or 2 (symmetric)");
    return kErrBadArg;
  }
  fp64_kernel_ = mode;
  return kOk;
}

int System::set_inner_preconditioner(int mode) {
  if (mode < 0 || mode > 2) {
    set_last_error("inner preconditioner must be 0 (diagonal), 1 (block Jacobi) or 2 (block Jacobi with the "
                   "near-field Neumann step)");
    return kErrBadArg;
  }
  inner_precond_ = mode;
  return kOk;
}

int System::set_fp32_kernel(int mode) {
  if (mode < 0 || mode > 3) {
    set_last_error("FP32 kernel mode must be 0 (autotuned), 1, 2 or 3");
    return kErrBadArg;
  }
  if (mode != fp32_kernel_) f32_tune_.clear();
  fp32_kernel_ = mode;
  return kOk;
}

int System::set_residual_update(int mode) {
  if (mode < -1 || mode > 1) {
    set_last_error("residual update mode must be -1 (by precision mode), 0 or 1");
    return kErrBadArg;
  }
  residual_update_ = mode;
  return kOk;
}

int System::fp32_shape(int ncol, int32_t *shape) const {
  if (!shape) {
    set_last_error("fp32_shape: null output");
    return kErrBadArg;
  }
  const auto it = f32_tune_.find(ncol);
  shape[0] = it == f32_tune_.end() ? 0 : it->second.kver;
  shape[1] = it == f32_tune_.end() ? 0 : it->second.g;
  shape[2] = it == f32_tune_.end() ? 0 : it->second.nsplit;
  return kOk;
}

int System::set_default_solver(int s) {
  if (s != kSolverCG && s != kSolverInversion && s != kSolverDIIS) {
    set_last_error("Unrecognized setting for default solver method");
    return kErrBadArg;
  }
  def_solver_ = s;
  return kOk;
}

int System::set_default_matv(int mv) {
  if (mv != kMatvIncore && mv != kMatvDirect) {
    set_last_error("Unrecognized setting for default matrix-vector method");
    return kErrBadArg;
  }
  def_matv_ = mv;
  return kOk;
}

int System::tmatvec(const double *xh, double *yh, int nrhs, bool dodiag, int matv) {
  const size_t nv = 3 * (size_t)d_.n;
  if (nrhs < 1 || nrhs > 2) {
    set_last_error("tmatvec: nrhs must be 1 or 2");
    return kErrBadArg;
  }
  if (matv == kMatvNone) matv = def_matv_;
  if (matv == kMatvIncore) {
    int st = ensure_tmat();
    if (st) return st;
  }
  cudaMemcpyAsync(p_, xh, nrhs * nv * sizeof(double), cudaMemcpyHostToDevice, st_);
  int mst = matvec64(matv, nrhs, p_, h_, dodiag);
  if (mst) return mst;
  cudaMemcpyAsync(yh, h_, nrhs * nv * sizeof(double), cudaMemcpyDeviceToHost, st_);
  return check(cudaStreamSynchronize(st_), "tmatvec");
}

int System::tmatvec_ds(const double *xh, double *yh, int nrhs) {
  const size_t nv = 3 * (size_t)d_.n;
  if (nrhs < 1 || nrhs > 2) {
    set_last_error("tmatvec_ds: nrhs must be 1 or 2");
    return kErrBadArg;
  }
  cudaMemcpyAsync(p_, xh, nrhs * nv * sizeof(double), cudaMemcpyHostToDevice, st_);
  const int keep = precision_;
  precision_ = kPrecMixedDS;
  int st = matvec_residual(nrhs, p_, h_);
  precision_ = keep;
  if (st) return st;
  cudaMemcpyAsync(yh, h_, nrhs * nv * sizeof(double), cudaMemcpyDeviceToHost, st_);
  return check(cudaStreamSynchronize(st_), "tmatvec_ds");
}

int System::tmatvec_f32(const double *xh, double *yh, int nrhs) {
  const size_t nv = 3 * (size_t)d_.n;
  if (nrhs < 1 || nrhs > 2) {
    set_last_error("tmatvec_f32: nrhs must be 1 or 2");
    return kErrBadArg;
  }
  cudaMemcpyAsync(p_, xh, nrhs * nv * sizeof(double), cudaMemcpyHostToDevice, st_);
  gpu::launch_to_f32(nrhs * nv, p_, nullptr, p32_, st_);
  int kver = fp32_kernel_ ? fp32_kernel_ : 2;
  if (kver == 3 && ensure_sym_scratch() != kOk) kver = 2;
  const int split = kver == 2 ? nsplit_tmu32_ : gpu::tmu_pick_split(d_, nrhs, gpu::sm_count(), true);
  gpu::launch_tmu_f32(d_, nrhs, p32_, h32_, scratch32_, split, st_, kver == 3 ? 2 : 4, kver, sym_scratch_);
  std::vector<float> tmp(nrhs * nv);
  cudaMemcpyAsync(tmp.data(), h32_, tmp.size() * sizeof(float), cudaMemcpyDeviceToHost, st_);
  int st = check(cudaStreamSynchronize(st_), "tmatvec_f32");
  for (size_t i = 0; i < tmp.size(); ++i) yh[i] = tmp[i];
  return st;
}

}  // namespace ommp
