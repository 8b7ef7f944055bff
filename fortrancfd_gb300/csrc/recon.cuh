// Face reconstruction of primitive variables (device).
//
// Restates SRC/muscl.f90 (muscl3 with minmod / superbee / MC limiters,
// kappa = 1/3) and SRC/weno.f90 (weno3z, weno5 JS/Z, weno7z) for the fused
// stage kernel. The limiter arithmetic is reorganised to spend as few FP64
// instructions as possible: minmod is evaluated with integer compares and
// the kappa blend is folded into two FMAs, which changes results only at
// the level of rounding.
#pragma once

#include "edyn_dev.cuh"

namespace edyn {

enum Acu : int { ACU_FIRST = 0, ACU_MUSCL = 1, ACU_WENO3 = 2, ACU_WENO5 = 3, ACU_WENO7 = 4 };

// Ghost depth per scheme (SRC/params.f90:161-173).
__host__ __device__ constexpr int acu_lvir(int acu) {
  return acu == ACU_FIRST ? 1 : acu == ACU_MUSCL ? 2 : acu == ACU_WENO3 ? 2 : acu == ACU_WENO5 ? 3 : 4;
}

#ifdef __CUDACC__

// b = (3 - kappa) / (1 - kappa) evaluated as the reference does.
__device__ __forceinline__ double muscl_b() { return (3.0 - 1.0 / 3.0) / (1.0 - 1.0 / 3.0); }

__device__ __forceinline__ double superbee_f(double x, double y) {
  return fmax(fmax(0.0, fmin(x, 2.0 * y)), fmin(2.0 * x, y));
}
__device__ __forceinline__ double mc_f(double x, double y) {
  return fmax(0.0, fmin(fmin(2.0 * x, 2.0 * y), 0.5 * (x + y)));
}

// s points at q(i-1); faces between q(i) and q(i+1). LIM: 1 none, 2 minmod,
// 3 superbee, 4 MC.
template <int LIM>
__device__ __forceinline__ void muscl3_d(const double* s, int stride, double& sl, double& sr) {
  const double s0 = s[0], s1 = s[stride], s2 = s[2 * stride], s3 = s[3 * stride];
  const double cm = 0.25 * (1.0 - 1.0 / 3.0), cp = 0.25 * (1.0 + 1.0 / 3.0);
  const double dm_i = s1 - s0, dp_i = s2 - s1, dp_ip = s3 - s2;
  const double dm_ip = dp_i;
  if (LIM == 1) {
    sl = fma(cp, dp_i, fma(cm, dm_i, s1));
    sr = s2 - fma(cp, dm_ip, cm * dp_ip);
    return;
  }
  const double b = muscl_b();
  const double bdm_i = b * dm_i, bdp_i = b * dp_i, bdp_ip = b * dp_ip;
  double lp_i, lm_i, lp_ip, lm_ip;
  if (LIM == 2) {
    lp_i = minmod_i(dp_i, bdm_i);
    lm_i = minmod_i(dm_i, bdp_i);
    lp_ip = minmod_i(dp_ip, bdp_i);  // b * dminus_ip == b * dplus_i
    lm_ip = minmod_i(dm_ip, bdp_ip);
  } else if (LIM == 3) {
    lp_i = superbee_f(dp_i, bdm_i);
    lm_i = superbee_f(dm_i, bdp_i);
    lp_ip = superbee_f(dp_ip, bdp_i);
    lm_ip = superbee_f(dm_ip, bdp_ip);
  } else {
    lp_i = mc_f(dp_i, bdm_i);
    lm_i = mc_f(dm_i, bdp_i);
    lp_ip = mc_f(dp_ip, bdp_i);
    lm_ip = mc_f(dm_ip, bdp_ip);
  }
  sl = fma(cp, lp_i, fma(cm, lm_i, s1));
  sr = s2 - fma(cp, lm_ip, cm * lp_ip);
}

// weno3z, s points at q(i-1).
__device__ __forceinline__ void weno3z_d(const double* s, int st, double& sl, double& sr) {
  const double eps = 1.0e-6;
  const double s0 = s[0], s1 = s[st], s2 = s[2 * st], s3 = s[3 * st];
  double b2 = (s0 - s1) * (s0 - s1), b1 = (s1 - s2) * (s1 - s2);
  double tau = fabs(b2 - b1);
  double q2 = tau / (eps + b2), q1 = tau / (eps + b1);
  double a2 = 2.0 * fma(q2, q2, 1.0), a1 = fma(q1, q1, 1.0);
  sl = 0.5 * (a2 * (3.0 * s1 - s0) + a1 * (s1 + s2)) / (a2 + a1);
  b2 = (s3 - s2) * (s3 - s2);
  b1 = (s2 - s1) * (s2 - s1);
  tau = fabs(b2 - b1);
  q2 = tau / (eps + b2);
  q1 = tau / (eps + b1);
  a2 = 2.0 * fma(q2, q2, 1.0);
  a1 = fma(q1, q1, 1.0);
  sr = 0.5 * (a2 * (3.0 * s2 - s3) + a1 * (s1 + s2)) / (a2 + a1);
}

template <int FLAG>  // 2 JS, 3 Z
__device__ __forceinline__ void weno5_side(double p0, double p1, double p2, double p3, double p4, double& out) {
  // p0..p4 ordered away from the face: candidate stencils as SRC/weno.f90:79-116.
  const double eps = 1.0e-6, c13 = 13.0 / 12.0;
  double t3a = p0 - 2.0 * p1 + p2, t3b = p0 - 4.0 * p1 + 3.0 * p2;
  double t2a = p1 - 2.0 * p2 + p3, t2b = p1 - p3;
  double t1a = p2 - 2.0 * p3 + p4, t1b = 3.0 * p2 - 4.0 * p3 + p4;
  double b3 = fma(c13 * t3a, t3a, 0.25 * t3b * t3b);
  double b2 = fma(c13 * t2a, t2a, 0.25 * t2b * t2b);
  double b1 = fma(c13 * t1a, t1a, 0.25 * t1b * t1b);
  double w3, w2, w1;
  if (FLAG == 2) {
    double e3 = eps + b3, e2 = eps + b2, e1 = eps + b1;
    w3 = 1.0 / (e3 * e3);
    w2 = 6.0 / (e2 * e2);
    w1 = 3.0 / (e1 * e1);
  } else {
    double tau = fabs(b3 - b1);
    double q3 = tau / (eps + b3), q2 = tau / (eps + b2), q1 = tau / (eps + b1);
    w3 = fma(q3, q3, 1.0);
    w2 = 6.0 * fma(q2, q2, 1.0);
    w1 = 3.0 * fma(q1, q1, 1.0);
  }
  double v3 = 2.0 * p0 - 7.0 * p1 + 11.0 * p2;
  double v2 = -p1 + 5.0 * p2 + 2.0 * p3;
  double v1 = 2.0 * p2 + 5.0 * p3 - p4;
  out = (w3 * v3 + w2 * v2 + w1 * v1) / (6.0 * (w3 + w2 + w1));
}

// weno5, s points at q(i-2).
template <int FLAG>
__device__ __forceinline__ void weno5_d(const double* s, int st, double& sl, double& sr) {
  const double q0 = s[0], q1 = s[st], q2 = s[2 * st], q3 = s[3 * st], q4 = s[4 * st], q5 = s[5 * st];
  weno5_side<FLAG>(q0, q1, q2, q3, q4, sl);
  weno5_side<FLAG>(q5, q4, q3, q2, q1, sr);
}

// weno7z, s points at q(i-3); the eighth point repeats q(i+3) as the
// reference does (SRC/flux.f90:231-232). The smoothness indicators are sums
// of O(1e4) q^2 terms that cancel almost completely where the data are
// smooth; their weights then amplify rounding, so they are evaluated in the
// reference's operation order without FMA contraction.
__device__ __forceinline__ double m_(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double a_(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double s_(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double w7beta(double p0, double p1, double p2, double p3, double c00, double c01,
                                         double c02, double c03, double c11, double c12, double c13, double c22,
                                         double c23, double c33) {
  // p0*(c00 p0 + c01 p1 + c02 p2 + c03 p3) + p1*(c11 p1 + c12 p2 + c13 p3) + p2*(c22 p2 + c23 p3) + c33 p3^2
  double t0 = a_(a_(a_(m_(c00, p0), m_(c01, p1)), m_(c02, p2)), m_(c03, p3));
  double t1 = a_(a_(m_(c11, p1), m_(c12, p2)), m_(c13, p3));
  double t2 = a_(m_(c22, p2), m_(c23, p3));
  return a_(a_(a_(m_(p0, t0), m_(p1, t1)), m_(p2, t2)), m_(c33, m_(p3, p3)));
}
// One WENO7-Z face value from p[0..6] ordered toward the face, in the
// reference's operation order.
__device__ __forceinline__ double weno7z_side(const double* p) {
  const double eps = 1.0e-6;
  const double b4 = w7beta(p[0], p[1], p[2], p[3], 547.0, -3882.0, 4642.0, -1854.0, 7043.0, -17246.0, 7042.0,
                           11003.0, -9402.0, 2107.0);
  const double b3 = w7beta(p[1], p[2], p[3], p[4], 267.0, -1642.0, 1602.0, -494.0, 2843.0, -5966.0, 1922.0,
                           3443.0, -2522.0, 547.0);
  const double b2 = w7beta(p[2], p[3], p[4], p[5], 547.0, -2522.0, 1922.0, -494.0, 3443.0, -5966.0, 1602.0,
                           2843.0, -1642.0, 267.0);
  const double b1 = w7beta(p[3], p[4], p[5], p[6], 2107.0, -9402.0, 7042.0, -1854.0, 11003.0, -17246.0, 4642.0,
                           7043.0, -3882.0, 547.0);
  const double tau = fabs(s_(b4, b1));
  const double r4 = tau / a_(eps, b4), r3 = tau / a_(eps, b3), r2 = tau / a_(eps, b2), r1 = tau / a_(eps, b1);
  const double a4 = m_(1.0 / 35.0, a_(1.0, m_(r4, r4))), a3 = m_(12.0 / 35.0, a_(1.0, m_(r3, r3)));
  const double a2 = m_(18.0 / 35.0, a_(1.0, m_(r2, r2))), a1 = m_(4.0 / 35.0, a_(1.0, m_(r1, r1)));
  const double al = 1.0 / a_(a_(a_(a4, a3), a2), a1);
  const double v4 = a_(a_(a_(m_(-3.0, p[0]), m_(13.0, p[1])), m_(-23.0, p[2])), m_(25.0, p[3]));
  const double v3 = a_(a_(a_(m_(1.0, p[1]), m_(-5.0, p[2])), m_(13.0, p[3])), m_(3.0, p[4]));
  const double v2 = a_(a_(a_(m_(-1.0, p[2]), m_(7.0, p[3])), m_(7.0, p[4])), m_(-1.0, p[5]));
  const double v1 = a_(a_(a_(m_(3.0, p[3]), m_(13.0, p[4])), m_(-5.0, p[5])), m_(1.0, p[6]));
  return m_(m_(1.0 / 12.0, al), a_(a_(a_(m_(a4, v4), m_(a3, v3)), m_(a2, v2)), m_(a1, v1)));
}

__device__ __forceinline__ void weno7z_d(const double* s, int st, double& sl, double& sr) {
  double q[8];
#pragma unroll
  for (int j = 0; j < 7; ++j) q[j] = s[j * st];
  q[7] = q[6];
  double p[7];
#pragma unroll
  for (int j = 0; j < 7; ++j) p[j] = q[j];
  sl = weno7z_side(p);
#pragma unroll
  for (int j = 0; j < 7; ++j) p[j] = q[7 - j];
  sr = weno7z_side(p);
}

// ---------------------------------------------------------------------------
// Cell-centred reconstruction: both face values of cell j from its own
// stencil (radius lvir - 1): vr at face j+1/2 (the left state there), vl at
// face j-1/2 (the right state there). What a cell's two faces share is
// computed once: MUSCL's limited slopes, WENO3's smoothness quotients (both
// bit-identical to the face-by-face forms), WENO5's smoothness indicators
// and weights (the mirrored indicators are the same quantities in another
// summation order, so results move at the rounding level), with the WENO5
// divisions merged into two reciprocals. WENO7-Z keeps the face-by-face
// arithmetic in the reference's order.
// ---------------------------------------------------------------------------
template <int LIM>
__device__ __forceinline__ void muscl_cell(const double* s, double& vr, double& vl) {
  // s points at q(j-1)
  const double s0 = s[0], s1 = s[1], s2 = s[2];
  const double cm = 0.25 * (1.0 - 1.0 / 3.0), cp = 0.25 * (1.0 + 1.0 / 3.0);
  const double dm = s1 - s0, dp = s2 - s1;
  if (LIM == 1) {
    vr = fma(cp, dp, fma(cm, dm, s1));
    vl = s1 - fma(cp, dm, cm * dp);
    return;
  }
  const double b = muscl_b();
  const double bdm = b * dm, bdp = b * dp;
  double lp, lm;
  if (LIM == 2) {
    lp = minmod_i(dp, bdm);
    lm = minmod_i(dm, bdp);
  } else if (LIM == 3) {
    lp = superbee_f(dp, bdm);
    lm = superbee_f(dm, bdp);
  } else {
    lp = mc_f(dp, bdm);
    lm = mc_f(dm, bdp);
  }
  vr = fma(cp, lp, fma(cm, lm, s1));
  vl = s1 - fma(cp, lm, cm * lp);
}

__device__ __forceinline__ void weno3z_cell(const double* s, double& vr, double& vl) {
  // s points at q(j-1)
  const double eps = 1.0e-6;
  const double s0 = s[0], s1 = s[1], s2 = s[2];
  const double bl = (s0 - s1) * (s0 - s1), br = (s1 - s2) * (s1 - s2);
  const double tau = fabs(bl - br);
  const double ql = tau / (eps + bl), qr = tau / (eps + br);
  double a2 = 2.0 * fma(ql, ql, 1.0), a1 = fma(qr, qr, 1.0);
  vr = 0.5 * (a2 * (3.0 * s1 - s0) + a1 * (s1 + s2)) / (a2 + a1);
  a2 = 2.0 * fma(qr, qr, 1.0);
  a1 = fma(ql, ql, 1.0);
  vl = 0.5 * (a2 * (3.0 * s1 - s2) + a1 * (s0 + s1)) / (a2 + a1);
}

template <int FLAG>  // 2 JS, 3 Z
__device__ __forceinline__ void weno5_cell(const double* s, double& vr, double& vl) {
  // s points at q(j-2); stencils S3 = {j-2..j}, S2 = {j-1..j+1}, S1 = {j..j+2}
  const double eps = 1.0e-6, c13 = 13.0 / 12.0;
  const double p0 = s[0], p1 = s[1], p2 = s[2], p3 = s[3], p4 = s[4];
  const double t3a = p0 - 2.0 * p1 + p2, t3b = p0 - 4.0 * p1 + 3.0 * p2;
  const double t2a = p1 - 2.0 * p2 + p3, t2b = p1 - p3;
  const double t1a = p2 - 2.0 * p3 + p4, t1b = 3.0 * p2 - 4.0 * p3 + p4;
  const double b3 = fma(c13 * t3a, t3a, 0.25 * t3b * t3b);
  const double b2 = fma(c13 * t2a, t2a, 0.25 * t2b * t2b);
  const double b1 = fma(c13 * t1a, t1a, 0.25 * t1b * t1b);
  const double e3 = eps + b3, e2 = eps + b2, e1 = eps + b1;
  // 1/e_k from one division
  const double e32 = e3 * e2;
  const double r = 1.0 / (e32 * e1);
  const double i3 = r * (e2 * e1), i2 = r * (e3 * e1), i1 = r * e32;
  double w3, w2, w1, u3, u2, u1;  // right-face weights (w) and left-face weights (u)
  if (FLAG == 2) {
    const double k3 = i3 * i3, k2 = i2 * i2, k1 = i1 * i1;
    w3 = k3;
    w2 = 6.0 * k2;
    w1 = 3.0 * k1;
    u3 = k1;
    u2 = w2;
    u1 = 3.0 * k3;
  } else {
    const double tau = fabs(b3 - b1);
    const double q3 = tau * i3, q2 = tau * i2, q1 = tau * i1;
    const double z3 = fma(q3, q3, 1.0), z2 = fma(q2, q2, 1.0), z1 = fma(q1, q1, 1.0);
    w3 = z3;
    w2 = 6.0 * z2;
    w1 = 3.0 * z1;
    u3 = z1;
    u2 = w2;
    u1 = 3.0 * z3;
  }
  const double v3 = 2.0 * p0 - 7.0 * p1 + 11.0 * p2, v2 = -p1 + 5.0 * p2 + 2.0 * p3, v1 = 2.0 * p2 + 5.0 * p3 - p4;
  const double x3 = 2.0 * p4 - 7.0 * p3 + 11.0 * p2, x2 = -p3 + 5.0 * p2 + 2.0 * p1, x1 = 2.0 * p2 + 5.0 * p1 - p0;
  const double sr = 6.0 * (w3 + w2 + w1), sl = 6.0 * (u3 + u2 + u1);
  const double rr = 1.0 / (sr * sl);
  vr = (w3 * v3 + w2 * v2 + w1 * v1) * (rr * sl);
  vl = (u3 * x3 + u2 * x2 + u1 * x1) * (rr * sr);
}

__device__ __forceinline__ void weno7z_cell(const double* s, double& vr, double& vl) {
  // s points at q(j-3); the left face repeats q(j+2) as its first two points,
  // the reference's stencil (SRC/flux.f90:231-232) seen from the cell
  double p[7];
#pragma unroll
  for (int k = 0; k < 7; ++k) p[k] = s[k];
  vr = weno7z_side(p);
  p[0] = s[5];
  p[1] = s[5];
  p[2] = s[4];
  p[3] = s[3];
  p[4] = s[2];
  p[5] = s[1];
  p[6] = s[0];
  vl = weno7z_side(p);
}

// Both face values of one variable of the cell at row index c (radius lvir - 1).
template <int ACU, int LIM, int WFLAG>
__device__ __forceinline__ void recon_cell(const double* row, int c, double& vr, double& vl) {
  if (ACU == ACU_FIRST) {
    vr = row[c];
    vl = row[c];
  } else if (ACU == ACU_MUSCL) {
    muscl_cell<LIM>(row + c - 1, vr, vl);
  } else if (ACU == ACU_WENO3) {
    weno3z_cell(row + c - 1, vr, vl);
  } else if (ACU == ACU_WENO5) {
    weno5_cell<WFLAG>(row + c - 2, vr, vl);
  } else {
    weno7z_cell(row + c - 3, vr, vl);
  }
}

// Reconstructs one variable at face f (between cells f-1 and f). `row`
// points at the shared-memory row of the variable, `c` is the row index of
// cell f-1.
template <int ACU, int LIM, int WFLAG>
__device__ __forceinline__ void recon(const double* row, int c, double& l, double& r) {
  if (ACU == ACU_FIRST) {
    l = row[c];
    r = row[c + 1];
  } else if (ACU == ACU_MUSCL) {
    muscl3_d<LIM>(row + c - 1, 1, l, r);
  } else if (ACU == ACU_WENO3) {
    weno3z_d(row + c - 1, 1, l, r);
  } else if (ACU == ACU_WENO5) {
    weno5_d<WFLAG>(row + c - 2, 1, l, r);
  } else {
    weno7z_d(row + c - 3, 1, l, r);
  }
}

#endif

}  // namespace edyn
