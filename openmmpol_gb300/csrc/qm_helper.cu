// QM helper: the electrostatic quantities a QM code needs from the MM side
// (mod_qm_helper, src/mod_qm_helper.F90:14-106,118-161,336-520).
//
//   prepare_qm_ele_ene  E_n2p  field of the QM nuclei at the polarizable sites
//                       V_m2n  potential of the static multipoles at the nuclei
//                       V_p2n  potential of the induced dipoles at the nuclei
//                              (once the system holds dipoles)
//   prepare_qm_ele_grd  E_n2m, G_n2m, H_n2m  field, field gradient and field
//                              Hessian of the nuclei at every static site,
//                       G_n2p  G_n2m at the polarizable sites
//                       E_m2n, E_p2n  field of the static multipoles / of the
//                              induced dipoles at the nuclei
// The nuclear fields are point-charge sums (undamped coulomb_kernel,
// q_elec_prop src/mod_electrostatics.F90:978-1016,1097-1176) over all nuclei
// for every site: k_nuclei_fields, one site per thread, the nuclei staged in
// shared memory and summed in their input order.  The MM-side quantities are
// the external-point kernels of external.cu (System::ext_props).
// Flags follow the reference: the energy quantities are computed once and
// kept until update_coord (which leaves V_p2n as it is, as the reference
// does); the gradient quantities are recomputed at every call.  Results are
// host arrays in the reference's Fortran order ([n][3], [n][6], [n][10]).
#include <cmath>
#include <vector>

#include "engine.h"
#include "qm_helper.h"

namespace ommp {

namespace gpu {
namespace {

constexpr int QTPB = 128;

// E (and G, H when GRAD) of nq point charges (x, y, z, q) at the sites
// pos[idx ? idx[j] : j], j < nt
template <bool GRAD>
__global__ void __launch_bounds__(QTPB) k_nuclei_fields(int nt, const Pos64 *__restrict__ pos,
                                                        const int *__restrict__ idx, int nq,
                                                        const Pos64 *__restrict__ nuc, double *__restrict__ E,
                                                        double *__restrict__ G, double *__restrict__ H, int *err) {
  __shared__ Pos64 s_n[QTPB];
  const int j = blockIdx.x * QTPB + threadIdx.x;
  const bool valid = j < nt;
  const Pos64 p = valid ? pos[idx ? idx[j] : j] : Pos64{0, 0, 0, 0};
  double e[3] = {0, 0, 0}, g[6] = {0, 0, 0, 0, 0, 0}, h[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  int bad = 0;
  for (int t0 = 0; t0 < nq; t0 += QTPB) {
    __syncthreads();
    if (t0 + threadIdx.x < nq) s_n[threadIdx.x] = nuc[t0 + threadIdx.x];
    __syncthreads();
    const int cnt = min(QTPB, nq - t0);
    if (!valid) continue;
    for (int k = 0; k < cnt; ++k) {
      const Pos64 n = s_n[k];
      const double dx = p.x - n.x, dy = p.y - n.y, dz = p.z - n.z;
      const double r2 = dx * dx + dy * dy + dz * dz;
      if (r2 < 4.9e-28) {  // |r| < 100 eps: the reference stops here
        bad = 1;
        continue;
      }
      const double r = sqrt(r2), k1 = 1.0 / r, ir2 = k1 * k1;
      const double k3 = k1 * ir2, q = n.w;
      const double qk3 = q * k3;
      e[0] += qk3 * dx;
      e[1] += qk3 * dy;
      e[2] += qk3 * dz;
      if (!GRAD) continue;
      const double k5 = k3 * ir2, k7 = k5 * ir2;
      const double d[3] = {dx, dy, dz};
      const double a5 = 3.0 * q * k5;
      // xx, xy, yy, xz, yz, zz
      g[0] += a5 * dx * dx - qk3;
      g[1] += a5 * dx * dy;
      g[2] += a5 * dy * dy - qk3;
      g[3] += a5 * dx * dz;
      g[4] += a5 * dy * dz;
      g[5] += a5 * dz * dz - qk3;
      // 15 q k7 d_a d_b d_c - 3 q k5 (delta_ab d_c + delta_ac d_b + delta_bc d_a)
      const double a7 = 15.0 * q * k7;
      const int A[10] = {0, 0, 0, 0, 0, 0, 1, 1, 1, 2}, B[10] = {0, 0, 0, 1, 1, 2, 1, 1, 2, 2},
                C[10] = {0, 1, 2, 1, 2, 2, 1, 2, 2, 2};
#pragma unroll
      for (int c = 0; c < 10; ++c) {
        const int a = A[c], b = B[c], cc = C[c];
        const double t = (a == b ? d[cc] : 0.0) + (a == cc ? d[b] : 0.0) + (b == cc ? d[a] : 0.0);
        h[c] += a7 * d[a] * d[b] * d[cc] - a5 * t;
      }
    }
  }
  if (bad) atomicOr(err, 1);
  if (!valid) return;
  for (int c = 0; c < 3; ++c) E[3 * (size_t)j + c] = e[c];
  if (GRAD) {
    for (int c = 0; c < 6; ++c) G[6 * (size_t)j + c] = g[c];
    for (int c = 0; c < 10; ++c) H[10 * (size_t)j + c] = h[c];
  }
}

}  // namespace
}  // namespace gpu

QMHelper::QMHelper(int n, const double *cqm, const double *qqm, const int *zqm)
    : nq_(n), cqm_(cqm, cqm + 3 * (size_t)n), qqm_(qqm, qqm + n), zqm_(zqm, zqm + n) {}

QMHelper::~QMHelper() {
  if (dbuf_) cudaFree(dbuf_);
}

void QMHelper::update_coord(const double *c) {
  std::copy(c, c + 3 * (size_t)nq_, cqm_.begin());
  // src/mod_qm_helper.F90:143-149 (V_p2n and E_p2n keep their flags)
  e_n2p_done_ = g_n2p_done_ = e_n2m_done_ = g_n2m_done_ = h_n2m_done_ = v_m2n_done_ = e_m2n_done_ = false;
}

int QMHelper::nuclear_fields(System &s, bool grad) {
  const gpu::DevSites &d = s.dev();
  const int nt = grad ? d.m : d.n;
  const size_t per = grad ? 19 : 3;
  const size_t need = 4 * (size_t)nq_ + per * (size_t)nt;
  if (need > cap_) {
    if (dbuf_) cudaFree(dbuf_);
    dbuf_ = nullptr;
    cap_ = 0;
    if (cudaMalloc((void **)&dbuf_, need * sizeof(double)) != cudaSuccess) {
      cudaGetLastError();
      set_last_error("out of device memory for the QM helper");
      return kErrMemory;
    }
    cap_ = need;
  }
  std::vector<gpu::Pos64> nuc(nq_);
  for (int i = 0; i < nq_; ++i) nuc[i] = gpu::Pos64{cqm_[3 * i], cqm_[3 * i + 1], cqm_[3 * i + 2], qqm_[i]};
  gpu::Pos64 *dn = reinterpret_cast<gpu::Pos64 *>(dbuf_);
  double *E = dbuf_ + 4 * (size_t)nq_, *G = E + 3 * (size_t)nt, *H = G + 6 * (size_t)nt;
  cudaStream_t st = s.stream();
  int *flag = s.flag_dev();
  cudaMemcpyAsync(dn, nuc.data(), nq_ * sizeof(gpu::Pos64), cudaMemcpyHostToDevice, st);
  cudaMemsetAsync(flag, 0, sizeof(int), st);
  const int blocks = (nt + gpu::QTPB - 1) / gpu::QTPB;
  if (nt > 0) {
    if (grad)
      gpu::k_nuclei_fields<true><<<blocks, gpu::QTPB, 0, st>>>(nt, d.mm_pos, nullptr, nq_, dn, E, G, H, flag);
    else
      gpu::k_nuclei_fields<false><<<blocks, gpu::QTPB, 0, st>>>(nt, d.mm_pos, d.polar_mm, nq_, dn, E, G, H, flag);
    gpu::add_launch_count(1);
  }
  int bad = 0;
  std::vector<double> &e = grad ? e_n2m_ : e_n2p_;
  e.assign(3 * (size_t)nt, 0.0);
  cudaMemcpyAsync(e.data(), E, e.size() * sizeof(double), cudaMemcpyDeviceToHost, st);
  if (grad) {
    g_n2m_.assign(6 * (size_t)nt, 0.0);
    h_n2m_.assign(10 * (size_t)nt, 0.0);
    cudaMemcpyAsync(g_n2m_.data(), G, g_n2m_.size() * sizeof(double), cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(h_n2m_.data(), H, h_n2m_.size() * sizeof(double), cudaMemcpyDeviceToHost, st);
  }
  cudaMemcpyAsync(&bad, flag, sizeof(int), cudaMemcpyDeviceToHost, st);
  cudaError_t ce = cudaStreamSynchronize(st);
  if (ce != cudaSuccess) {
    set_last_error(std::string("CUDA error in the QM helper: ") + cudaGetErrorString(ce));
    return kErrCuda;
  }
  if (bad) {
    set_last_error(
        "Requesting Coulomb kernel for two atoms placed in the same point, this could be an internal bug or a "
        "problem in your input file, please check.");
    return kErrNumeric;
  }
  return kOk;
}

// electrostatic_for_ene, src/mod_qm_helper.F90:356-433
int QMHelper::prepare_ene(System &s) {
  int st;
  if (!e_n2p_done_) {
    st = nuclear_fields(s, false);
    if (st) return st;
    e_n2p_done_ = true;
  }
  if (!v_m2n_done_) {
    v_m2n_.assign(nq_, 0.0);
    st = s.ext_props(1, false, nq_, cqm_.data(), v_m2n_.data());
    if (st) return st;
    v_m2n_done_ = true;
  }
  if (!v_p2n_done_ && s.ipd_done()) {
    v_p2n_.assign(nq_, 0.0);
    st = s.ext_props(2, false, nq_, cqm_.data(), v_p2n_.data());
    if (st) return st;
    v_p2n_done_ = true;
  }
  return kOk;
}

// electrostatic_for_grad, src/mod_qm_helper.F90:435-520
int QMHelper::prepare_grd(System &s) {
  int st = nuclear_fields(s, true);
  if (st) return st;
  e_n2m_done_ = g_n2m_done_ = h_n2m_done_ = true;
  const HostModel &m = s.model();
  g_n2p_.assign(6 * (size_t)m.npol, 0.0);
  for (int j = 0; j < m.npol; ++j)
    for (int c = 0; c < 6; ++c) g_n2p_[6 * (size_t)j + c] = g_n2m_[6 * (size_t)m.polar_mm[j] + c];
  g_n2p_done_ = true;
  e_m2n_.assign(3 * (size_t)nq_, 0.0);
  st = s.ext_props(1, true, nq_, cqm_.data(), e_m2n_.data());
  if (st) return st;
  e_m2n_done_ = true;
  e_p2n_.assign(3 * (size_t)nq_, 0.0);
  st = s.ext_props(2, true, nq_, cqm_.data(), e_p2n_.data());
  if (st) return st;
  e_p2n_done_ = true;
  return kOk;
}

}  // namespace ommp
