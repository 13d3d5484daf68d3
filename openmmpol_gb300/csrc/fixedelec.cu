// Interaction energy of the static multipoles, ommp_get_fixedelec_energy
// (energy_MM_MM, src/mod_electrostatics.F90:899-941, on elec_prop_M2M's
// direct path :1678-1952 with the m-scaled pair list list_S_S :597-648).
//
//   k_m2m_pairs    per static target, unscaled sums over every other static
//                  site of the potential, field and field gradient of its
//                  multipoles (undamped: the static-static interaction has no
//                  Thole damping), split over source ranges
//   k_m2m_finish   partials summed in a fixed order, the m-scaled pairs
//                  corrected by (s - 1) times their terms, and the site's
//                  energy term q V - mu.E + Q:G (the off-diagonal quadrupole
//                  components counted twice)
// The energy is half the sum of the site terms, added on the host in site
// order (deterministic).  Computed once per geometry.
//
// Gradient, ommp_fixedelec_geomgrad (fixedelec_geomgrad,
// src/mod_geomgrad.F90:17-111, on elec_prop_M2M with field gradients and
// Hessians): the same two kernels with the GRAD flag accumulate per static
// target the field E, the field gradient G and h_a = sum_bc Q_bc H_bca, the
// field Hessian H of all other static multipoles contracted with the
// target's own quadrupole Q (the reference's q/mu/quad_elec_prop Hessians,
// :1097-1405, as closed tensor expressions).  The finish writes E, G and
// the site term -q E + mu.G - h; the frame forces of the rotated multipoles
// in E and G (rotation_geomgrad) are added by the polarization gradient's
// frame kernels.
#include <algorithm>
#include <cmath>
#include <vector>

#include "engine.h"
#include "grad_math.cuh"
#include "pair_math.cuh"

namespace ommp {

namespace gpu {
namespace {

constexpr int MTPB = 128;

struct M2mArgs {
  int mm, nsplit;
  const Pos64 *pos;
  const double *q;
  const int *ri, *src;
  const double *sc;
  double *partial;  // [nsplit][NV][mm]
  double *site;     // [mm] energy terms
  double *E, *G;    // [mm][3], [mm][6] field and field gradient (gradient pass)
  double *base;     // [mm][3] site gradient terms (gradient pass)
  int *err;
};

// accumulators of one target: energy pass V (+ E, G); gradient pass E, G, h
template <bool AMOEBA, bool GRAD>
struct M2mNV {
  static constexpr int N = GRAD ? (AMOEBA ? 12 : 3) : (AMOEBA ? 10 : 1);
};

// potential, field and (AMOEBA) field gradient of the multipole q at
// d = target - source with undamped r^-1 .. r^-9
template <bool AMOEBA>
__device__ __forceinline__ void m2m_pair(const double *q, double dx, double dy, double dz, double rinv, double w,
                                         double *acc) {
  const double ir2 = rinv * rinv, k3 = rinv * ir2, k5 = k3 * ir2;
  if (!AMOEBA) {
    acc[0] += w * q[0] * rinv;
    return;
  }
  const double k7 = k5 * ir2, k9 = k7 * ir2;
  const double md = q[1] * dx + q[2] * dy + q[3] * dz;
  const double tx = q[4] * dx + q[5] * dy + q[7] * dz;
  const double ty = q[5] * dx + q[6] * dy + q[8] * dz;
  const double tz = q[7] * dx + q[8] * dy + q[9] * dz;
  const double s = tx * dx + ty * dy + tz * dz;
  acc[0] += w * (q[0] * rinv + md * k3 + 3.0 * s * k5);
  const double c = q[0] * k3 + 3.0 * md * k5 + 15.0 * s * k7;
  acc[1] += w * (c * dx - q[1] * k3 - 6.0 * k5 * tx);
  acc[2] += w * (c * dy - q[2] * k3 - 6.0 * k5 * ty);
  acc[3] += w * (c * dz - q[3] * k3 - 6.0 * k5 * tz);
  gradmath::multipole_grad<true>(q, dx, dy, dz, k3, k5, k7, k9, w, acc + 4);
}

// field E, field gradient G and (AMOEBA) h_a = sum_bc Qt_bc H_bca of the
// multipole q at d = target - source (undamped), added with weight w;
// Qt (xx, xy, yy, xz, yz, zz) and trq are the target's quadrupole and trace.
// Field Hessians of a charge, dipole and quadrupole contracted with Qt
// (u = Qt d, sg = d.Qt.d; source t = Qs d, s = d.Qs.d):
//   charge      q (15 k7 sg d - 3 k5 (2 u + trq d))
//   dipole      gradmath::dipole_hess_q
//   quadrupole  945 k11 s sg d - 105 k9 (s (2 u + trq d) + 2 sg t + 4 (t.u) d)
//               + 30 k7 (2 Qs u + (Qs:Qt) d + 2 Qt t + trq t)
template <bool AMOEBA>
__device__ __forceinline__ void m2m_pair_grad(const double *q, double dx, double dy, double dz, double rinv,
                                              double w, const double *Qt, double trq, double *acc) {
  const double ir2 = rinv * rinv, k3 = rinv * ir2;
  if (!AMOEBA) {
    const double c = w * q[0] * k3;
    acc[0] += c * dx;
    acc[1] += c * dy;
    acc[2] += c * dz;
    return;
  }
  const double k5 = k3 * ir2, k7 = k5 * ir2, k9 = k7 * ir2, k11 = k9 * ir2;
  const double md = q[1] * dx + q[2] * dy + q[3] * dz;
  const double tx = q[4] * dx + q[5] * dy + q[7] * dz;
  const double ty = q[5] * dx + q[6] * dy + q[8] * dz;
  const double tz = q[7] * dx + q[8] * dy + q[9] * dz;
  const double s = tx * dx + ty * dy + tz * dz;
  const double c = q[0] * k3 + 3.0 * md * k5 + 15.0 * s * k7;
  acc[0] += w * (c * dx - q[1] * k3 - 6.0 * k5 * tx);
  acc[1] += w * (c * dy - q[2] * k3 - 6.0 * k5 * ty);
  acc[2] += w * (c * dz - q[3] * k3 - 6.0 * k5 * tz);
  gradmath::multipole_grad<true>(q, dx, dy, dz, k3, k5, k7, k9, w, acc + 3);
  // h: target quadrupole against the source's field Hessian
  const double ux = Qt[0] * dx + Qt[1] * dy + Qt[3] * dz;
  const double uy = Qt[1] * dx + Qt[2] * dy + Qt[4] * dz;
  const double uz = Qt[3] * dx + Qt[4] * dy + Qt[5] * dz;
  const double sg = ux * dx + uy * dy + uz * dz;
  const double tu = tx * ux + ty * uy + tz * uz;
  const double qq = q[4] * Qt[0] + q[6] * Qt[2] + q[9] * Qt[5] + 2.0 * (q[5] * Qt[1] + q[7] * Qt[3] + q[8] * Qt[4]);
  // Qs u and Qt t
  const double px = q[4] * ux + q[5] * uy + q[7] * uz;
  const double py = q[5] * ux + q[6] * uy + q[8] * uz;
  const double pz = q[7] * ux + q[8] * uy + q[9] * uz;
  const double ox = Qt[0] * tx + Qt[1] * ty + Qt[3] * tz;
  const double oy = Qt[1] * tx + Qt[2] * ty + Qt[4] * tz;
  const double oz = Qt[3] * tx + Qt[4] * ty + Qt[5] * tz;
  const double cd = 15.0 * k7 * q[0] * sg - 3.0 * k5 * q[0] * trq + 945.0 * k11 * s * sg -
                    105.0 * k9 * (s * trq + 4.0 * tu) + 30.0 * k7 * qq;
  const double cu = -6.0 * k5 * q[0] - 210.0 * k9 * s;
  const double ct = -210.0 * k9 * sg + 30.0 * k7 * trq;
  const double cp = 60.0 * k7;
  double h[3] = {0.0, 0.0, 0.0};
  h[0] = cd * dx + cu * ux + ct * tx + cp * (px + ox);
  h[1] = cd * dy + cu * uy + ct * ty + cp * (py + oy);
  h[2] = cd * dz + cu * uz + ct * tz + cp * (pz + oz);
  gradmath::dipole_hess_q(&q[1], md, dx, dy, dz, Qt, trq, k5, k7, k9, 1.0, h);
  acc[9] += w * h[0];
  acc[10] += w * h[1];
  acc[11] += w * h[2];
}

template <bool AMOEBA, bool GRAD>
__device__ __forceinline__ void m2m_any(const double *q, double dx, double dy, double dz, double rinv, double w,
                                        const double *Qt, double trq, double *acc) {
  if (GRAD)
    m2m_pair_grad<AMOEBA>(q, dx, dy, dz, rinv, w, Qt, trq, acc);
  else
    m2m_pair<AMOEBA>(q, dx, dy, dz, rinv, w, acc);
}

template <bool AMOEBA, bool GRAD>
__global__ void __launch_bounds__(MTPB) k_m2m_pairs(M2mArgs a, int per_split) {
  constexpr int LD = AMOEBA ? 10 : 1;
  constexpr int NV = M2mNV<AMOEBA, GRAD>::N;
  __shared__ Pos64 s_pos[MTPB];
  __shared__ double s_q[MTPB * LD];
  const int t = blockIdx.x * MTPB + threadIdx.x;
  const bool valid = t < a.mm;
  const Pos64 pt = valid ? a.pos[t] : Pos64{0, 0, 0, 0};
  double Qt[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  if (GRAD && AMOEBA && valid)
    for (int c = 0; c < 6; ++c) Qt[c] = a.q[(size_t)t * LD + 4 + c];
  const double trq = Qt[0] + Qt[2] + Qt[5];
  double acc[NV];
#pragma unroll
  for (int c = 0; c < NV; ++c) acc[c] = 0.0;
  int bad = 0;
  const int s0 = blockIdx.y * per_split, s1 = min(a.mm, s0 + per_split);
  for (int t0 = s0; t0 < s1; t0 += MTPB) {
    __syncthreads();
    const int i = t0 + threadIdx.x;
    if (i < s1) {
      s_pos[threadIdx.x] = a.pos[i];
      for (int c = 0; c < LD; ++c) s_q[threadIdx.x * LD + c] = a.q[(size_t)i * LD + c];
    }
    __syncthreads();
    if (!valid) continue;
    const int cnt = min(MTPB, s1 - t0);
    for (int k = 0; k < cnt; ++k) {
      if (t0 + k == t) continue;
      const Pos64 ps = s_pos[k];
      const double dx = pt.x - ps.x, dy = pt.y - ps.y, dz = pt.z - ps.z;
      const double r2 = dx * dx + dy * dy + dz * dz;
      if (coincident(r2)) {
        bad = 1;
        continue;
      }
      m2m_any<AMOEBA, GRAD>(&s_q[k * LD], dx, dy, dz, rinv_f64(r2, r2_f32(r2)), 1.0, Qt, trq, acc);
    }
  }
  if (bad) atomicOr(a.err, 1);
  if (valid)
    for (int c = 0; c < NV; ++c) a.partial[((size_t)blockIdx.y * NV + c) * a.mm + t] = acc[c];
}

template <bool AMOEBA, bool GRAD>
__global__ void k_m2m_finish(M2mArgs a) {
  constexpr int LD = AMOEBA ? 10 : 1;
  constexpr int NV = M2mNV<AMOEBA, GRAD>::N;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= a.mm) return;
  double Qt[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  if (GRAD && AMOEBA)
    for (int c = 0; c < 6; ++c) Qt[c] = a.q[(size_t)t * LD + 4 + c];
  const double trq = Qt[0] + Qt[2] + Qt[5];
  double acc[NV];
  for (int c = 0; c < NV; ++c) {
    double s = 0.0;
    for (int p = 0; p < a.nsplit; ++p) s += a.partial[((size_t)p * NV + c) * a.mm + t];
    acc[c] = s;
  }
  const Pos64 pt = a.pos[t];
  for (int k = a.ri[t]; k < a.ri[t + 1]; ++k) {
    const int i = a.src[k];
    const Pos64 ps = a.pos[i];
    const double dx = pt.x - ps.x, dy = pt.y - ps.y, dz = pt.z - ps.z;
    const double r2 = dx * dx + dy * dy + dz * dz;
    if (r2 < 4.9e-28) continue;  // flagged by the pair pass
    m2m_any<AMOEBA, GRAD>(&a.q[(size_t)i * LD], dx, dy, dz, 1.0 / sqrt(r2), a.sc[k] - 1.0, Qt, trq, acc);
  }
  const double *q = &a.q[(size_t)t * LD];
  if (GRAD) {
    double g[3];
    for (int c = 0; c < 3; ++c) {
      a.E[3 * (size_t)t + c] = acc[c];
      g[c] = -q[0] * acc[c];
    }
    if (AMOEBA) {
      double mg[3];
      gradmath::sym_apply(acc + 3, q + 1, mg);
      for (int c = 0; c < 6; ++c) a.G[6 * (size_t)t + c] = acc[3 + c];
      for (int c = 0; c < 3; ++c) g[c] += mg[c] - acc[9 + c];
    }
    for (int c = 0; c < 3; ++c) a.base[3 * (size_t)t + c] = g[c];
    return;
  }
  double e = q[0] * acc[0];
  if (AMOEBA) {
    e -= q[1] * acc[1] + q[2] * acc[2] + q[3] * acc[3];
    const double *g = acc + (GRAD ? 3 : 4);
    e += q[4] * g[0] + q[6] * g[2] + q[9] * g[5] + 2.0 * (q[5] * g[1] + q[7] * g[3] + q[8] * g[4]);
  }
  a.site[t] = e;
}

}  // namespace
}  // namespace gpu

namespace {

// list_S_S: pairs within four bonds whose m-scale is not 1, by target
void build_ss(const HostModel &m, int mm, std::vector<int> &ri, std::vector<int> &src, std::vector<double> &sc) {
  ri.assign(mm + 1, 0);
  src.clear();
  sc.clear();
  for (int i = 0; i < mm; ++i) {
    for (int l = 0; l < 4; ++l)
      for (int k = m.conn[l].ri[i]; k < m.conn[l].ri[i + 1]; ++k) {
        const double s = m.mscale[l];
        if (std::fabs(s - 1.0) > kEpsRp) {
          src.push_back(m.conn[l].ci[k]);
          sc.push_back(s);
        }
      }
    ri[i + 1] = (int)src.size();
  }
}

}  // namespace

// The pair and finish passes of the energy (grad false) or of the gradient
// (grad true: E, G and the site terms into e_out, g_out, base_out).  buf
// receives the device block to free after the stream is synchronised.
int System::m2m_launch(bool grad, double **buf_out, double **site_out, double **e_out, double **g_out,
                       double **base_out) {
  const int mm = d_.m;
  const bool amoeba = m_.amoeba;
  const int nv = grad ? (amoeba ? 12 : 3) : (amoeba ? 10 : 1);
  std::vector<int> ri, src;
  std::vector<double> sc;
  build_ss(m_, mm, ri, src, sc);
  const int tiles = (mm + gpu::MTPB - 1) / gpu::MTPB;
  const int tblocks = tiles;
  int nsplit = std::max(1, std::min(tiles, (6 * gpu::sm_count() + tblocks - 1) / tblocks));
  const size_t out = grad ? 12 * (size_t)mm : (size_t)mm;  // E, G, base | site
  const size_t need = (size_t)nsplit * nv * mm + out + ri.size() + 2 * src.size() + 1;
  double *buf = nullptr;
  if (cudaMalloc((void **)&buf, need * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    set_last_error("out of device memory for the static multipole field");
    return kErrMemory;
  }
  gpu::M2mArgs a{};
  a.mm = mm;
  a.nsplit = nsplit;
  a.pos = d_.mm_pos;
  a.q = d_.mm_q;
  a.partial = buf;
  double *o = buf + (size_t)nsplit * nv * mm;
  if (grad) {
    a.E = o;
    a.G = o + 3 * (size_t)mm;
    a.base = o + 9 * (size_t)mm;
  } else {
    a.site = o;
  }
  double *sc_d = o + out;
  int *ri_d = reinterpret_cast<int *>(sc_d + std::max<size_t>(sc.size(), 1));
  int *src_d = ri_d + ri.size();
  a.ri = ri_d;
  a.src = src_d;
  a.sc = sc_d;
  a.err = flag_;
  cudaMemcpyAsync(sc_d, sc.data(), sc.size() * sizeof(double), cudaMemcpyHostToDevice, st_);
  cudaMemcpyAsync(ri_d, ri.data(), ri.size() * sizeof(int), cudaMemcpyHostToDevice, st_);
  cudaMemcpyAsync(src_d, src.data(), src.size() * sizeof(int), cudaMemcpyHostToDevice, st_);
  cudaMemsetAsync(flag_, 0, sizeof(int), st_);
  const int per = ((tiles + nsplit - 1) / nsplit) * gpu::MTPB;
  const dim3 grid(tblocks, nsplit);
  const int fb = (mm + 127) / 128;
  if (amoeba && grad) {
    gpu::k_m2m_pairs<true, true><<<grid, gpu::MTPB, 0, st_>>>(a, per);
    gpu::k_m2m_finish<true, true><<<fb, 128, 0, st_>>>(a);
  } else if (amoeba) {
    gpu::k_m2m_pairs<true, false><<<grid, gpu::MTPB, 0, st_>>>(a, per);
    gpu::k_m2m_finish<true, false><<<fb, 128, 0, st_>>>(a);
  } else if (grad) {
    gpu::k_m2m_pairs<false, true><<<grid, gpu::MTPB, 0, st_>>>(a, per);
    gpu::k_m2m_finish<false, true><<<fb, 128, 0, st_>>>(a);
  } else {
    gpu::k_m2m_pairs<false, false><<<grid, gpu::MTPB, 0, st_>>>(a, per);
    gpu::k_m2m_finish<false, false><<<fb, 128, 0, st_>>>(a);
  }
  gpu::add_launch_count(2);
  // host vectors above die at return: wait for their copies
  int flag = 0;
  cudaMemcpyAsync(&flag, flag_, sizeof(int), cudaMemcpyDeviceToHost, st_);
  int st = check(cudaStreamSynchronize(st_), "static multipole field");
  if (st) {
    cudaFree(buf);
    return st;
  }
  if (flag) {
    cudaFree(buf);
    set_last_error(
        "Requesting Coulomb kernel for two atoms placed in the same point, this could be an internal bug or "
        "a problem in your input file, please check.");
    return kErrNumeric;
  }
  *buf_out = buf;
  if (site_out) *site_out = a.site;
  if (e_out) *e_out = a.E;
  if (g_out) *g_out = a.G;
  if (base_out) *base_out = a.base;
  return kOk;
}

int System::fixedelec_energy(double &energy) {
  energy = 0.0;
  const int mm = d_.m;
  if (mm == 0) return kOk;
  if (fixedelec_done_) {
    energy = fixedelec_;
    return kOk;
  }
  double *buf = nullptr, *site_d = nullptr;
  int st = m2m_launch(false, &buf, &site_d, nullptr, nullptr, nullptr);
  if (st) return st;
  std::vector<double> site(mm);
  cudaMemcpyAsync(site.data(), site_d, mm * sizeof(double), cudaMemcpyDeviceToHost, st_);
  st = check(cudaStreamSynchronize(st_), "static multipole energy");
  cudaFree(buf);
  if (st) return st;
  double e = 0.0;
  for (int t = 0; t < mm; ++t) e += site[t];
  fixedelec_ = 0.5 * e;
  fixedelec_done_ = true;
  energy = fixedelec_;
  return kOk;
}

int System::fixedelec_geomgrad(double *grad_h) {
  const int mm = d_.m;
  std::fill(grad_h, grad_h + 3 * (size_t)mm, 0.0);
  if (mm == 0) return kOk;
  if (fixedelec_grad_done_) {
    std::copy(fixedelec_grad_.begin(), fixedelec_grad_.end(), grad_h);
    return kOk;
  }
  double *buf = nullptr, *E = nullptr, *G = nullptr, *base = nullptr;
  int st = m2m_launch(true, &buf, nullptr, &E, &G, &base);
  if (st) return st;
  st = frame_forces(E, G, base, grad_h);  // synchronises the stream
  cudaFree(buf);
  if (st) return st;
  fixedelec_grad_.assign(grad_h, grad_h + 3 * (size_t)mm);
  fixedelec_grad_done_ = true;
  return kOk;
}

}  // namespace ommp
