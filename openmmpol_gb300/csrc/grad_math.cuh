// Pair and frame formulas of the polarization-energy geometric gradient,
// shared by the GPU kernels (grad.cu) and usable from host code.
//
// Restated from the reference's field-gradient / Hessian formulas
// (q_elec_prop, mu_elec_prop, quad_elec_prop with derivatives,
// src/mod_electrostatics.F90:1097-1405), damped_coulomb_kernel (:1018-1095)
// and the frame dependence of the rotated multipoles (rotation_geomgrad,
// src/rotate_multipoles.F90:298-643).  The formulas are written as closed
// tensor expressions:
//   field gradient of a static multipole (q, mu, Q) at d = target - source
//     G_ab = A d_a d_b + B delta_ab + v_a d_b + v_b d_a + 6 k5 Q_ab
//     A = 3 q k5 + 15 k7 (mu.d) + 105 k9 (d.Q.d)
//     B = -q k3 - 3 k5 (mu.d) - 15 k7 (d.Q.d)
//     v = -3 k5 mu - 30 k7 Q d
//   the field Hessian of a dipole is only needed contracted with the target's
//   own quadrupole, h_a = sum_bc Q_bc H_abc, which is accumulated directly;
//   the frame term is the reverse-mode pullback of the energy's dependence on
//   the rotation matrix through the frame construction (ez from u, ex by
//   Gram-Schmidt of v, ey = ez x ex) onto the four frame atoms.
// Symmetric 3x3 tensors are stored xx, xy, yy, xz, yz, zz (the reference's
// component order).
#pragma once

#include <cmath>

#if defined(__CUDACC__)
#define OMMP_HD __host__ __device__ __forceinline__
#else
#define OMMP_HD inline
#endif

namespace ommp {
namespace gradmath {

// Damped inverse odd powers of one pair: k3 = l3/r^3 ... k9 = l9/r^9.
// ww = 1/(thole_t thole_s) (inf when either site has no Thole factor), a the
// AMOEBA damping exponent of the pair, thr the AMOEBA damping threshold.
template <bool AMOEBA>
OMMP_HD void damped_k(double r2, double rinv, double ww, double a, double thr, bool test, double &k3, double &k5,
                      double &k7, double &k9) {
  const double ir2 = rinv * rinv;
  k3 = rinv * ir2;
  k5 = k3 * ir2;
  k7 = k5 * ir2;
  k9 = k7 * ir2;
  if (!test) return;
  const double u = r2 * rinv * ww;  // r / (thole_t thole_s)
  if (AMOEBA) {
    const double au3 = a * u * u * u;
    if (au3 < thr) {
      const double e = exp(-au3);
      const double au6 = au3 * au3;
      k3 *= 1.0 - e;
      k5 *= 1.0 - (1.0 + au3) * e;
      k7 *= 1.0 - (1.0 + au3 + 0.6 * au6) * e;
      k9 *= 1.0 - (1.0 + au3 + (18.0 / 35.0) * au6 + (9.0 / 35.0) * au6 * au3) * e;
    }
  } else if (u < 1.0) {
    const double u3 = u * u * u, u4 = u3 * u;
    k3 *= 4.0 * u3 - 3.0 * u4;
    k5 *= u4;
    k7 *= 0.2 * u4;
  }
}

// The tensor formulas below are templates over the scalar type T (double,
// or the double-single type of the FP32-pipe kernels) and the weight type W
// (a scalar, or One for a unit weight that costs nothing).  Constants are
// written as floats: all are exact in single precision.
struct One {};
template <typename T>
OMMP_HD T operator*(One, T x) {
  return x;
}

// g += w * (A d d^T + B I + v d^T + d v^T)
template <typename T, typename W>
OMMP_HD void sym_add(T A, T B, T vx, T vy, T vz, T dx, T dy, T dz, W w, T *g) {
  const T px = A * dx + vx, py = A * dy + vy, pz = A * dz + vz;
  g[0] += w * (px * dx + vx * dx + B);
  g[1] += w * (px * dy + vy * dx);
  g[2] += w * (py * dy + vy * dy + B);
  g[3] += w * (px * dz + vz * dx);
  g[4] += w * (py * dz + vz * dy);
  g[5] += w * (pz * dz + vz * dz + B);
}

// field gradient of a static multipole q[0..ld-1] (charge; + dipole and
// quadrupole when AMOEBA), added with weight w
template <bool AMOEBA, typename T, typename W>
OMMP_HD void multipole_grad(const T *q, T dx, T dy, T dz, T k3, T k5, T k7, T k9, W w, T *g) {
  if (!AMOEBA) {
    const T z = 0.0f * dx;
    sym_add(3.0f * q[0] * k5, -(q[0] * k3), z, z, z, dx, dy, dz, w, g);
    return;
  }
  const T md = q[1] * dx + q[2] * dy + q[3] * dz;
  const T tx = q[4] * dx + q[5] * dy + q[7] * dz;
  const T ty = q[5] * dx + q[6] * dy + q[8] * dz;
  const T tz = q[7] * dx + q[8] * dy + q[9] * dz;
  const T s = tx * dx + ty * dy + tz * dz;
  const T A = 3.0f * q[0] * k5 + 15.0f * k7 * md + 105.0f * k9 * s;
  const T B = -(q[0] * k3 + 3.0f * k5 * md + 15.0f * k7 * s);
  const T c5 = -3.0f * k5, c7 = -30.0f * k7;
  sym_add(A, B, c5 * q[1] + c7 * tx, c5 * q[2] + c7 * ty, c5 * q[3] + c7 * tz, dx, dy, dz, w, g);
  const T C = 6.0f * k5;
  g[0] += w * (C * q[4]);
  g[1] += w * (C * q[5]);
  g[2] += w * (C * q[6]);
  g[3] += w * (C * q[7]);
  g[4] += w * (C * q[8]);
  g[5] += w * (C * q[9]);
}

// field gradient of a point dipole mu (md = mu.d), weight w
template <typename T, typename W>
OMMP_HD void dipole_grad(const T *mu, T md, T dx, T dy, T dz, T k5, T k7, W w, T *g) {
  const T c = -3.0f * k5;
  sym_add(15.0f * k7 * md, c * md, c * mu[0], c * mu[1], c * mu[2], dx, dy, dz, w, g);
}

// field of a point dipole, weight w
template <typename T, typename W>
OMMP_HD void dipole_field(const T *mu, T md, T dx, T dy, T dz, T k3, T k5, W w, T *e) {
  const T c = 3.0f * md * k5;
  e[0] += w * (c * dx - k3 * mu[0]);
  e[1] += w * (c * dy - k3 * mu[1]);
  e[2] += w * (c * dz - k3 * mu[2]);
}

// h_a += w * sum_bc Q_bc H_abc, H the field Hessian of the dipole mu and Q
// (6 components, trace trq) the target's quadrupole
template <typename T, typename W>
OMMP_HD void dipole_hess_q(const T *mu, T md, T dx, T dy, T dz, const T *Q, T trq, T k5, T k7, T k9, W w, T *h) {
  const T tx = Q[0] * dx + Q[1] * dy + Q[3] * dz;
  const T ty = Q[1] * dx + Q[2] * dy + Q[4] * dz;
  const T tz = Q[3] * dx + Q[4] * dy + Q[5] * dz;
  const T s = tx * dx + ty * dy + tz * dz;
  const T wx = Q[0] * mu[0] + Q[1] * mu[1] + Q[3] * mu[2];
  const T wy = Q[1] * mu[0] + Q[2] * mu[1] + Q[4] * mu[2];
  const T wz = Q[3] * mu[0] + Q[4] * mu[1] + Q[5] * mu[2];
  const T mt = mu[0] * tx + mu[1] * ty + mu[2] * tz;
  const T cd = 105.0f * k9 * md * s - 30.0f * k7 * mt - 15.0f * k7 * md * trq;
  const T cm = 3.0f * k5 * trq - 15.0f * k7 * s;
  const T ct = -30.0f * k7 * md;
  const T cw = 6.0f * k5;
  h[0] += w * (cd * dx + cm * mu[0] + ct * tx + cw * wx);
  h[1] += w * (cd * dy + cm * mu[1] + ct * ty + cw * wy);
  h[2] += w * (cd * dz + cm * mu[2] + ct * tz + cw * wz);
}

// sum_b x_b G_ab for a symmetric G (6 components)
OMMP_HD void sym_apply(const double *G, const double *x, double *out) {
  out[0] = G[0] * x[0] + G[1] * x[1] + G[3] * x[2];
  out[1] = G[1] * x[0] + G[2] * x[1] + G[4] * x[2];
  out[2] = G[3] * x[0] + G[4] * x[1] + G[5] * x[2];
}

OMMP_HD double dot3(const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
OMMP_HD void cross3(const double *a, const double *b, double *o) {
  o[0] = a[1] * b[2] - a[2] * b[1];
  o[1] = a[2] * b[0] - a[0] * b[2];
  o[2] = a[0] * b[1] - a[1] * b[0];
}

// Forces of the frame dependence of one site's rotated multipoles.  The
// site's lab-frame dipole R mu0 and quadrupole R Q0 R^T sit in the field E
// and field gradient G (6 components); the energy term -E.(R mu0) +
// (R Q0 R^T):G is differentiated with respect to the positions of the site
// (c) and its z, x, y frame atoms (cz, cx, cy); out[0..3] receive the
// gradient on c, cz, cx, cy.  Frames: 0 none, 1 z-then-x, 2 bisector,
// 3 z-only, 4 z-bisector, 5 3-fold (the construction of rotate_multipoles,
// src/rotate_multipoles.F90:3-230).  Returns false for a degenerate frame.
OMMP_HD bool frame_pullback(int frame, const double *c, const double *cz, const double *cx, const double *cy,
                            const double *q0, const double *E, const double *G, double out[4][3]) {
  for (int w = 0; w < 4; ++w) out[w][0] = out[w][1] = out[w][2] = 0.0;
  if (frame < 1 || frame > 5) return true;
  double a[3], b[3], d[3];
  for (int k = 0; k < 3; ++k) {
    a[k] = cz[k] - c[k];
    b[k] = cx[k] - c[k];
    d[k] = cy[k] - c[k];
  }
  const double na = sqrt(dot3(a, a)), nb = sqrt(dot3(b, b)), nd = sqrt(dot3(d, d));
  double u[3] = {0, 0, 0}, v[3] = {0, 0, 0};
  for (int k = 0; k < 3; ++k) {
    switch (frame) {
      case 1:
        u[k] = a[k], v[k] = b[k];
        break;
      case 2:
        u[k] = nb * a[k] + na * b[k], v[k] = b[k];
        break;
      case 3:
        u[k] = a[k];
        break;
      case 4:
        u[k] = a[k], v[k] = nd * b[k] + nb * d[k];
        break;
      default:
        u[k] = nb * nd * a[k] + na * nd * b[k] + na * nb * d[k], v[k] = b[k];
        break;
    }
  }
  if (frame == 3) {  // a fixed lab axis, chosen as the construction does
    if (u[2] / na <= 0.866 && fabs(u[1]) > 2.220446049250313e-14)
      v[0] = 1.0;
    else
      v[1] = 1.0;
  }
  const double nu = sqrt(dot3(u, u));
  if (!(nu > 0.0)) return false;
  double ez[3], ex[3], ey[3];
  for (int k = 0; k < 3; ++k) ez[k] = u[k] / nu;
  const double vez = dot3(v, ez);
  double wv[3];
  for (int k = 0; k < 3; ++k) wv[k] = v[k] - vez * ez[k];
  const double nw = sqrt(dot3(wv, wv));
  if (!(nw > 0.0)) return false;
  for (int k = 0; k < 3; ++k) ex[k] = wv[k] / nw;
  cross3(ez, ex, ey);
  // dPhi/dR for Phi = -E.(R mu0) + (R Q0 R^T):G  ->  W = -E mu0^T + 2 G R Q0
  const double Q0[3][3] = {{q0[4], q0[5], q0[7]}, {q0[5], q0[6], q0[8]}, {q0[7], q0[8], q0[9]}};
  const double Gm[3][3] = {{G[0], G[1], G[3]}, {G[1], G[2], G[4]}, {G[3], G[4], G[5]}};
  const double R[3][3] = {{ex[0], ey[0], ez[0]}, {ex[1], ey[1], ez[1]}, {ex[2], ey[2], ez[2]}};
  double RQ[3][3], W[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) RQ[i][j] = R[i][0] * Q0[0][j] + R[i][1] * Q0[1][j] + R[i][2] * Q0[2][j];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      W[i][j] = -E[i] * q0[1 + j] + 2.0 * (Gm[i][0] * RQ[0][j] + Gm[i][1] * RQ[1][j] + Gm[i][2] * RQ[2][j]);
  double gx[3] = {W[0][0], W[1][0], W[2][0]}, gy[3] = {W[0][1], W[1][1], W[2][1]},
         gz[3] = {W[0][2], W[1][2], W[2][2]};
  // ey = ez x ex
  double t[3];
  cross3(ex, gy, t);
  for (int k = 0; k < 3; ++k) gz[k] += t[k];
  cross3(gy, ez, t);
  for (int k = 0; k < 3; ++k) gx[k] += t[k];
  // ex = wv / |wv|
  const double xg = dot3(ex, gx);
  double gw[3];
  for (int k = 0; k < 3; ++k) gw[k] = (gx[k] - ex[k] * xg) / nw;
  // wv = v - (v.ez) ez
  const double wz = dot3(gw, ez);
  double gv[3];
  for (int k = 0; k < 3; ++k) {
    gv[k] = gw[k] - wz * ez[k];
    gz[k] += -wz * v[k] - vez * gw[k];
  }
  // ez = u / |u|
  const double zg = dot3(ez, gz);
  double gu[3];
  for (int k = 0; k < 3; ++k) gu[k] = (gz[k] - ez[k] * zg) / nu;
  // u, v as functions of a = cz - c, b = cx - c, d = cy - c
  double ga[3] = {0, 0, 0}, gb[3] = {0, 0, 0}, gd[3] = {0, 0, 0};
  switch (frame) {
    case 1:
      for (int k = 0; k < 3; ++k) ga[k] = gu[k], gb[k] = gv[k];
      break;
    case 2: {
      const double ub = dot3(gu, b) / na, ua = dot3(gu, a) / nb;
      for (int k = 0; k < 3; ++k) {
        ga[k] = nb * gu[k] + ub * a[k];
        gb[k] = na * gu[k] + ua * b[k] + gv[k];
      }
      break;
    }
    case 3:
      for (int k = 0; k < 3; ++k) ga[k] = gu[k];
      break;
    case 4: {
      const double vd = dot3(gv, d) / nb, vb = dot3(gv, b) / nd;
      for (int k = 0; k < 3; ++k) {
        ga[k] = gu[k];
        gb[k] = nd * gv[k] + vd * b[k];
        gd[k] = nb * gv[k] + vb * d[k];
      }
      break;
    }
    default: {
      const double ua = dot3(gu, a), ub = dot3(gu, b), ud = dot3(gu, d);
      const double fa = (ub * nd + ud * nb) / na, fb = (ua * nd + ud * na) / nb, fd = (ua * nb + ub * na) / nd;
      for (int k = 0; k < 3; ++k) {
        ga[k] = nb * nd * gu[k] + fa * a[k];
        gb[k] = na * nd * gu[k] + fb * b[k] + gv[k];
        gd[k] = na * nb * gu[k] + fd * d[k];
      }
      break;
    }
  }
  for (int k = 0; k < 3; ++k) {
    out[0][k] = -(ga[k] + gb[k] + gd[k]);
    out[1][k] = ga[k];
    out[2][k] = gb[k];
    out[3][k] = gd[k];
  }
  return true;
}

}  // namespace gradmath
}  // namespace ommp
