// Block-Jacobi preconditioner of the mixed-precision inner solver.
//
// The reference preconditions its CG with the diagonal of T (z = alpha r,
// src/mod_polarization.F90:535-557), and the plain FP64 solver here keeps
// exactly that.  The FP32 inner solve of the mixed modes is this library's
// own, so it may use a stronger preconditioner without changing what is
// solved: the outer FP64 refinement and its convergence test (the
// reference's rms of alpha r) are untouched.  The sites are cut into short
// runs of consecutive polarizable sites that are chemically bonded or very
// close (water molecules, chain segments; at most kMaxBlock sites), and each
// run's diagonal block of T -- 1/alpha on the diagonal, minus the damped and
// scaled dipole-field tensor between its sites, the same terms as the
// matrix-vector product -- is inverted in FP64 and stored in FP32.  Any such
// partition gives a symmetric positive-definite preconditioner; on AMOEBA
// water it cuts the CG iterations by about a quarter.
#include <algorithm>
#include <cmath>
#include <thread>
#include <vector>

#include "engine.h"

namespace ommp {

namespace {

// damped dipole-field factors k3 = lambda3 / r^3, k5 = lambda5 / r^5 (the
// Thole damping of the reference, src/mod_electrostatics.F90:1018-1095)
void damped_k35(bool amoeba, double r2, double wt, double ws, double at, double as, double thr, double &k3,
                double &k5) {
  const double r = std::sqrt(r2), rinv = 1.0 / r;
  k3 = rinv * rinv * rinv;
  k5 = k3 * rinv * rinv;
  const double u = r * wt * ws;
  if (amoeba) {
    const double au3 = std::min(at, as) * u * u * u;
    if (au3 < thr) {
      const double e = std::exp(-au3);
      k3 *= 1.0 - e;
      k5 *= 1.0 - (1.0 + au3) * e;
    }
  } else if (u < 1.0) {
    const double u3 = u * u * u, u4 = u3 * u;
    k3 *= 4.0 * u3 - 3.0 * u4;
    k5 *= u4;
  }
}

// in-place inverse of the dim x dim matrix a (row-major), partial pivoting;
// false if singular
bool invert(std::vector<double> &a, int dim) {
  std::vector<double> inv(dim * dim, 0.0);
  for (int i = 0; i < dim; ++i) inv[i * dim + i] = 1.0;
  for (int c = 0; c < dim; ++c) {
    int p = c;
    for (int r = c + 1; r < dim; ++r)
      if (std::fabs(a[r * dim + c]) > std::fabs(a[p * dim + c])) p = r;
    if (!(std::fabs(a[p * dim + c]) > 0.0)) return false;
    if (p != c)
      for (int k = 0; k < dim; ++k) {
        std::swap(a[p * dim + k], a[c * dim + k]);
        std::swap(inv[p * dim + k], inv[c * dim + k]);
      }
    const double d = 1.0 / a[c * dim + c];
    for (int k = 0; k < dim; ++k) {
      a[c * dim + k] *= d;
      inv[c * dim + k] *= d;
    }
    for (int r = 0; r < dim; ++r) {
      if (r == c) continue;
      const double f = a[r * dim + c];
      if (f == 0.0) continue;
      for (int k = 0; k < dim; ++k) {
        a[r * dim + k] -= f * a[c * dim + k];
        inv[r * dim + k] -= f * inv[c * dim + k];
      }
    }
  }
  a.swap(inv);
  return true;
}

}  // namespace

void build_block_jacobi(const HostModel &m, const ScaledPairs &d2d, double damp_thr, int max_sites,
                        double link_bohr, std::vector<int> &info, std::vector<float> &minv) {
  const int n = m.npol;
  info.assign(4 * (size_t)n, 0);
  minv.clear();
  const double link2 = link_bohr * link_bohr;
  auto pos = [&](int j) { return &m.cmm[3 * (size_t)m.polar_mm[j]]; };
  auto dist2 = [&](int i, int j) {
    const double *a = pos(i), *b = pos(j);
    const double dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
    return dx * dx + dy * dy + dz * dz;
  };
  // runs: grow while the next site is close to one already in the run
  std::vector<int> run_start, run_off;
  size_t total = 0;
  for (int start = 0; start < n;) {
    int end = start + 1;
    while (end < n && end - start < max_sites) {
      bool linked = false;
      for (int i = start; i < end && !linked; ++i) linked = dist2(i, end) < link2;
      if (!linked) break;
      ++end;
    }
    run_start.push_back(start);
    run_off.push_back((int)total);
    total += 9 * (size_t)(end - start) * (end - start);
    start = end;
  }
  const int nrun = (int)run_start.size();
  run_start.push_back(n);
  minv.resize(total);
  // each run's block: built, inverted and stored independently (threads)
  auto work = [&](int r0, int r1) {
    std::vector<double> a, inv;
    for (int r = r0; r < r1; ++r) {
      const int start = run_start[r], s = run_start[r + 1] - start, dim = 3 * s, off = run_off[r];
      a.assign((size_t)dim * dim, 0.0);
      for (int jl = 0; jl < s; ++jl) {
        const int j = start + jl;
        for (int c = 0; c < 3; ++c) a[(3 * jl + c) * dim + 3 * jl + c] = 1.0 / m.pol[j];
        for (int il = 0; il < s; ++il) {
          if (il == jl) continue;
          const int i = start + il;
          double sc = 1.0;  // scale of source i in target j's row
          for (int k = d2d.ri[j]; k < d2d.ri[j + 1]; ++k)
            if (d2d.src[k] == i) sc = d2d.sP[k];
          if (sc == 0.0) continue;
          const double *pj = pos(j), *pi = pos(i);
          const double d[3] = {pj[0] - pi[0], pj[1] - pi[1], pj[2] - pi[2]};
          const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
          const double wt = 1.0 / m.thole[m.polar_mm[j]], ws = 1.0 / m.thole[m.polar_mm[i]];
          const double at = m.amoeba ? m.damping[j] : 0.0, as = m.amoeba ? m.damping[i] : 0.0;
          double k3, k5;
          damped_k35(m.amoeba, r2, wt, ws, at, as, damp_thr, k3, k5);
          // T_ji = -s (3 k5 d d^T - k3 I)
          for (int p = 0; p < 3; ++p)
            for (int q = 0; q < 3; ++q)
              a[(3 * jl + p) * dim + 3 * il + q] = -sc * (3.0 * k5 * d[p] * d[q] - (p == q ? k3 : 0.0));
        }
      }
      inv = a;
      const bool ok = invert(inv, dim);
      for (int rr = 0; rr < dim; ++rr)
        for (int cc = 0; cc < dim; ++cc) {
          double v;
          if (ok)
            v = 0.5 * (inv[rr * dim + cc] + inv[cc * dim + rr]);  // symmetric in FP32 too
          else
            v = (rr == cc) ? 1.0 / a[rr * dim + rr] : 0.0;  // fall back to the diagonal
          minv[off + rr * dim + cc] = (float)v;
        }
      for (int jl = 0; jl < s; ++jl) {
        int *e = &info[4 * (size_t)(start + jl)];
        e[0] = start;
        e[1] = s;
        e[2] = off;
        e[3] = jl;
      }
    }
  };
  const int nt = std::max(1, std::min<int>((int)std::thread::hardware_concurrency(), nrun / 1024));
  std::vector<std::thread> th;
  for (int t = 1; t < nt; ++t) th.emplace_back(work, (int)((long)nrun * t / nt), (int)((long)nrun * (t + 1) / nt));
  work(0, (int)((long)nrun / nt));
  for (auto &x : th) x.join();
}


// Near-field couplings (build_near_field): the sites are binned in cubic
// cells of side rc and packed in cell order (position, Thole factor, damping
// a, run, index), so that the candidates of a row are contiguous records;
// each row scans the 27 cells around its own in a fixed order, so the lists
// are the same on any number of threads.  Rows are counted in a first pass
// and filled in a second.
void build_near_field(const HostModel &m, const ScaledPairs &d2d, double damp_thr, const std::vector<int> &info,
                      double rc, std::vector<int> &ri, std::vector<int> &ci, std::vector<float> &blk) {
  const int n = m.npol;
  ri.assign((size_t)n + 1, 0);
  ci.clear();
  blk.clear();
  if (n == 0) return;
  struct Site {
    double x, y, z, w, a;
    int run, idx;
  };
  auto pos = [&](int j) { return &m.cmm[3 * (size_t)m.polar_mm[j]]; };
  double lo[3] = {pos(0)[0], pos(0)[1], pos(0)[2]}, hi[3] = {lo[0], lo[1], lo[2]};
  for (int j = 1; j < n; ++j)
    for (int c = 0; c < 3; ++c) lo[c] = std::min(lo[c], pos(j)[c]), hi[c] = std::max(hi[c], pos(j)[c]);
  long dim[3];
  for (int c = 0; c < 3; ++c) dim[c] = std::max(1L, std::min(1024L, (long)((hi[c] - lo[c]) / rc) + 1));
  auto cell_of = [&](const double *p, long *q) {
    for (int c = 0; c < 3; ++c) q[c] = std::min(dim[c] - 1, std::max(0L, (long)((p[c] - lo[c]) / rc)));
    return (size_t)((q[2] * dim[1] + q[1]) * dim[0] + q[0]);
  };
  const size_t ncell = (size_t)dim[0] * dim[1] * dim[2];
  std::vector<int> cstart(ncell + 1, 0), cell(n);
  for (int j = 0; j < n; ++j) {
    long q[3];
    cell[j] = (int)cell_of(pos(j), q);
    ++cstart[cell[j] + 1];
  }
  for (size_t c = 0; c < ncell; ++c) cstart[c + 1] += cstart[c];
  std::vector<Site> site(n);
  {
    std::vector<int> fill(cstart.begin(), cstart.end() - 1);
    for (int j = 0; j < n; ++j) {
      const double *p = pos(j);
      site[fill[cell[j]]++] = Site{p[0], p[1], p[2], 1.0 / m.thole[m.polar_mm[j]], m.amoeba ? m.damping[j] : 0.0,
                                   info[4 * (size_t)j], j};
    }
  }
  const double rc2 = rc * rc;
  // visit the candidates of site s (a packed record) in a fixed order
  auto scan = [&](const Site &sj, auto &&f) {
    long q[3];
    const double pj[3] = {sj.x, sj.y, sj.z};
    cell_of(pj, q);
    for (long z = std::max(0L, q[2] - 1); z <= std::min(dim[2] - 1, q[2] + 1); ++z)
      for (long y = std::max(0L, q[1] - 1); y <= std::min(dim[1] - 1, q[1] + 1); ++y) {
        const size_t row = (z * dim[1] + y) * dim[0];
        const int k0 = cstart[row + std::max(0L, q[0] - 1)], k1 = cstart[row + std::min(dim[0] - 1, q[0] + 1) + 1];
        for (int k = k0; k < k1; ++k) {
          const Site &si = site[k];
          if (si.run == sj.run) continue;  // same run: in the block
          const double d[3] = {sj.x - si.x, sj.y - si.y, sj.z - si.z};
          const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
          if (r2 < rc2) f(si, d, r2);
        }
      }
  };
  auto scale = [&](int j, int i) {
    for (int k = d2d.ri[j]; k < d2d.ri[j + 1]; ++k)
      if (d2d.src[k] == i) return d2d.sP[k];
    return 1.0;
  };
  const int nt = std::max(1, std::min<int>((int)std::thread::hardware_concurrency(), n / 4096));
  auto parallel = [&](auto &&body) {
    std::vector<std::thread> th;
    for (int t = 1; t < nt; ++t) th.emplace_back(body, (int)((long)n * t / nt), (int)((long)n * (t + 1) / nt));
    body(0, (int)((long)n / nt));
    for (auto &x : th) x.join();
  };
  // rows in cell order (packed index s), written at their site's place
  parallel([&](int s0, int s1) {
    for (int s = s0; s < s1; ++s) {
      const Site &sj = site[s];
      int cnt = 0;
      scan(sj, [&](const Site &si, const double *, double) { cnt += scale(sj.idx, si.idx) != 0.0; });
      ri[sj.idx + 1] = cnt;
    }
  });
  for (int j = 0; j < n; ++j) ri[j + 1] += ri[j];
  ci.resize(ri[n]);
  blk.resize(9 * (size_t)ri[n]);
  parallel([&](int s0, int s1) {
    for (int s = s0; s < s1; ++s) {
      const Site &sj = site[s];
      int e = ri[sj.idx];
      scan(sj, [&](const Site &si, const double *d, double r2) {
        const double sc = scale(sj.idx, si.idx);
        if (sc == 0.0) return;
        double k3, k5;
        damped_k35(m.amoeba, r2, sj.w, si.w, sj.a, si.a, damp_thr, k3, k5);
        ci[e] = si.idx;
        for (int p = 0; p < 3; ++p)
          for (int q = 0; q < 3; ++q)
            blk[9 * (size_t)e + 3 * p + q] = (float)(-sc * (3.0 * k5 * d[p] * d[q] - (p == q ? k3 : 0.0)));
        ++e;
      });
    }
  });
}

}  // namespace ommp
