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
  double *site;     // [mm]
  int *err;
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

template <bool AMOEBA>
__global__ void __launch_bounds__(MTPB) k_m2m_pairs(M2mArgs a, int per_split) {
  constexpr int LD = AMOEBA ? 10 : 1;
  constexpr int NV = AMOEBA ? 10 : 1;  // V, E[3], G[6]
  __shared__ Pos64 s_pos[MTPB];
  __shared__ double s_q[MTPB * LD];
  const int t = blockIdx.x * MTPB + threadIdx.x;
  const bool valid = t < a.mm;
  const Pos64 pt = valid ? a.pos[t] : Pos64{0, 0, 0, 0};
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
      if (r2 < 4.9e-28) {  // |r| < 100 eps: coincident sites
        bad = 1;
        continue;
      }
      m2m_pair<AMOEBA>(&s_q[k * LD], dx, dy, dz, rinv_f64(r2, (float)r2), 1.0, acc);
    }
  }
  if (bad) atomicOr(a.err, 1);
  if (valid)
    for (int c = 0; c < NV; ++c) a.partial[((size_t)blockIdx.y * NV + c) * a.mm + t] = acc[c];
}

template <bool AMOEBA>
__global__ void k_m2m_finish(M2mArgs a) {
  constexpr int LD = AMOEBA ? 10 : 1;
  constexpr int NV = AMOEBA ? 10 : 1;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= a.mm) return;
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
    m2m_pair<AMOEBA>(&a.q[(size_t)i * LD], dx, dy, dz, 1.0 / sqrt(r2), a.sc[k] - 1.0, acc);
  }
  const double *q = &a.q[(size_t)t * LD];
  double e = q[0] * acc[0];
  if (AMOEBA) {
    e -= q[1] * acc[1] + q[2] * acc[2] + q[3] * acc[3];
    const double *g = acc + 4;
    e += q[4] * g[0] + q[6] * g[2] + q[9] * g[5] + 2.0 * (q[5] * g[1] + q[7] * g[3] + q[8] * g[4]);
  }
  a.site[t] = e;
}

}  // namespace
}  // namespace gpu

int System::fixedelec_energy(double &energy) {
  energy = 0.0;
  const int mm = d_.m;
  if (mm == 0) return kOk;
  if (fixedelec_done_) {
    energy = fixedelec_;
    return kOk;
  }
  const bool amoeba = m_.amoeba;
  const int nv = amoeba ? 10 : 1;
  // list_S_S: pairs within four bonds whose m-scale is not 1, by target
  std::vector<int> ri(mm + 1, 0), src;
  std::vector<double> sc;
  for (int i = 0; i < mm; ++i) {
    for (int l = 0; l < 4; ++l)
      for (int k = m_.conn[l].ri[i]; k < m_.conn[l].ri[i + 1]; ++k) {
        const double s = m_.mscale[l];
        if (std::fabs(s - 1.0) > kEpsRp) {
          src.push_back(m_.conn[l].ci[k]);
          sc.push_back(s);
        }
      }
    ri[i + 1] = (int)src.size();
  }
  const int tiles = (mm + gpu::MTPB - 1) / gpu::MTPB;
  const int tblocks = tiles;
  int nsplit = std::max(1, std::min(tiles, (6 * gpu::sm_count() + tblocks - 1) / tblocks));
  const size_t need = (size_t)nsplit * nv * mm + mm + ri.size() + 2 * src.size() + 1;
  double *buf = nullptr;
  if (cudaMalloc((void **)&buf, need * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    set_last_error("out of device memory for the static multipole energy");
    return kErrMemory;
  }
  gpu::M2mArgs a{};
  a.mm = mm;
  a.nsplit = nsplit;
  a.pos = d_.mm_pos;
  a.q = d_.mm_q;
  a.partial = buf;
  a.site = buf + (size_t)nsplit * nv * mm;
  double *sc_d = a.site + mm;
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
  if (amoeba) {
    gpu::k_m2m_pairs<true><<<grid, gpu::MTPB, 0, st_>>>(a, per);
    gpu::k_m2m_finish<true><<<(mm + 127) / 128, 128, 0, st_>>>(a);
  } else {
    gpu::k_m2m_pairs<false><<<grid, gpu::MTPB, 0, st_>>>(a, per);
    gpu::k_m2m_finish<false><<<(mm + 127) / 128, 128, 0, st_>>>(a);
  }
  gpu::add_launch_count(2);
  std::vector<double> site(mm);
  int flag = 0;
  cudaMemcpyAsync(site.data(), a.site, mm * sizeof(double), cudaMemcpyDeviceToHost, st_);
  cudaMemcpyAsync(&flag, flag_, sizeof(int), cudaMemcpyDeviceToHost, st_);
  int st = check(cudaStreamSynchronize(st_), "static multipole energy");
  cudaFree(buf);
  if (st) return st;
  if (flag) {
    set_last_error(
        "Requesting Coulomb kernel for two atoms placed in the same point, this could be an internal bug or "
        "a problem in your input file, please check.");
    return kErrNumeric;
  }
  double e = 0.0;
  for (int t = 0; t < mm; ++t) e += site[t];
  fixedelec_ = 0.5 * e;
  fixedelec_done_ = true;
  energy = fixedelec_;
  return kOk;
}

}  // namespace ommp
