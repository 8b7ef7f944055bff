/*
 * Oracle (test infrastructure only): reconstruction, fluxes, time
 * integration, boundaries and the time-step restriction of the reference's
 * fluid path, restated in plain C FP64 with the reference's operation order.
 *
 * The reference stores the tube as 10-cell blocks with their own ghost
 * cells. With equal cell sizes, the inter-block ghost copy
 * (interpolation_block, SRC/block.f90:490-497) replaces a ghost by the
 * neighbour's conserved state and QcToqf then rebuilds the same primitive
 * state, so the block structure is equivalent to one contiguous array with
 * lvir ghost cells at each end; that array is what is kept here.
 */
#include "edyn_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

int or_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ---- SRC/muscl.f90 ---- */

static double minmod(double x, double y) {
  /* SRC/muscl.f90:79-93 */
  return copysign(1.0, x) * fmax(0.0, fmin(fabs(x), copysign(1.0, x) * y));
}
static double superbee(double x, double y) {
  /* SRC/muscl.f90:96-121 */
  return fmax(fmax(0.0, fmin(x, 2.0 * y)), fmin(2.0 * x, y));
}
static double mc(double x, double y) {
  /* SRC/muscl.f90:124-142 */
  return fmax(0.0, fmin(fmin(2.0 * x, 2.0 * y), 0.5 * (x + y)));
}

/* muscl3, SRC/muscl.f90:9-76 (kappa = 1/3) */
void or_muscl3(const double* s, double* sl, double* sr, int flag_muscl) {
  const double k = 1.0 / 3.0;
  const double b = (3.0 - k) / (1.0 - k);
  double dminus_i = s[1] - s[0];
  double dplus_i = s[2] - s[1];
  double dminus_ip = s[2] - s[1];
  double dplus_ip = s[3] - s[2];
  if (flag_muscl == 1) {
    *sl = s[1] + (1.0 / 4.0) * ((1.0 - k) * dminus_i + (1.0 + k) * dplus_i);
    *sr = s[2] - (1.0 / 4.0) * ((1.0 - k) * dplus_ip + (1.0 + k) * dminus_ip);
    return;
  }
  double lp_i, lm_i, lp_ip, lm_ip;
  if (flag_muscl == 2) {
    lp_i = minmod(dplus_i, b * dminus_i);
    lm_i = minmod(dminus_i, b * dplus_i);
    lp_ip = minmod(dplus_ip, b * dminus_ip);
    lm_ip = minmod(dminus_ip, b * dplus_ip);
  } else if (flag_muscl == 3) {
    lp_i = superbee(dplus_i, b * dminus_i);
    lm_i = superbee(dminus_i, b * dplus_i);
    lp_ip = superbee(dplus_ip, b * dminus_ip);
    lm_ip = superbee(dminus_ip, b * dplus_ip);
  } else {
    lp_i = mc(dplus_i, b * dminus_i);
    lm_i = mc(dminus_i, b * dplus_i);
    lp_ip = mc(dplus_ip, b * dminus_ip);
    lm_ip = mc(dminus_ip, b * dplus_ip);
  }
  *sl = s[1] + (1.0 / 4.0) * ((1.0 - k) * lm_i + (1.0 + k) * lp_i);
  *sr = s[2] - (1.0 / 4.0) * ((1.0 - k) * lp_ip + (1.0 + k) * lm_ip);
}

/* ---- SRC/weno.f90 ---- */

/* weno3z, SRC/weno.f90:11-65 */
void or_weno3z(const double* s, double* sl, double* sr) {
  const double eps = 1.0e-6;
  double b2 = (s[0] - s[1]) * (s[0] - s[1]);
  double b1 = (s[1] - s[2]) * (s[1] - s[2]);
  double tau = fabs(b2 - b1);
  b2 = 1.0 + (tau / (eps + b2)) * (tau / (eps + b2));
  b1 = 1.0 + (tau / (eps + b1)) * (tau / (eps + b1));
  double a2 = 2.0 * b2, a1 = 1.0 * b1;
  double a = 1.0 / (a2 + a1);
  double v2 = -s[0] + 3.0 * s[1], v1 = s[1] + s[2];
  *sl = 0.5 * a * (a2 * v2 + a1 * v1);
  b2 = (s[3] - s[2]) * (s[3] - s[2]);
  b1 = (s[2] - s[1]) * (s[2] - s[1]);
  tau = fabs(b2 - b1);
  b2 = 1.0 + (tau / (eps + b2)) * (tau / (eps + b2));
  b1 = 1.0 + (tau / (eps + b1)) * (tau / (eps + b1));
  a2 = 2.0 * b2;
  a1 = 1.0 * b1;
  a = 1.0 / (a2 + a1);
  v2 = 3.0 * s[2] - s[3];
  v1 = s[1] + s[2];
  *sr = 0.5 * a * (a2 * v2 + a1 * v1);
}

static void weno5_weights(double* b3, double* b2, double* b1, int flag_weno) {
  const double eps = 1.0e-6;
  if (flag_weno == 2) {
    *b3 = 1.0 / ((eps + *b3) * (eps + *b3));
    *b2 = 1.0 / ((eps + *b2) * (eps + *b2));
    *b1 = 1.0 / ((eps + *b1) * (eps + *b1));
  } else if (flag_weno == 3) {
    double tau = fabs(*b3 - *b1);
    *b3 = 1.0 + (tau / (eps + *b3)) * (tau / (eps + *b3));
    *b2 = 1.0 + (tau / (eps + *b2)) * (tau / (eps + *b2));
    *b1 = 1.0 + (tau / (eps + *b1)) * (tau / (eps + *b1));
  }
}

static double sq(double v) { return v * v; }

/* weno5 (JS flag 2, Z flag 3), SRC/weno.f90:68-166 */
void or_weno5(const double* s, double* sl, double* sr, int flag_weno) {
  const double c13 = 13.0 / 12.0;
  double b3 = c13 * sq(s[0] - 2.0 * s[1] + s[2]) + 0.25 * sq(s[0] - 4.0 * s[1] + 3.0 * s[2]);
  double b2 = c13 * sq(s[1] - 2.0 * s[2] + s[3]) + 0.25 * (s[1] - s[3]) * (s[1] - s[3]);
  double b1 = c13 * sq(s[2] - 2.0 * s[3] + s[4]) + 0.25 * sq(3.0 * s[2] - 4.0 * s[3] + s[4]);
  weno5_weights(&b3, &b2, &b1, flag_weno);
  double a3 = b3, a2 = 6.0 * b2, a1 = 3.0 * b1;
  double a = 1.0 / (a3 + a2 + a1);
  double v3 = 2.0 * s[0] - 7.0 * s[1] + 11.0 * s[2];
  double v2 = -s[1] + 5.0 * s[2] + 2.0 * s[3];
  double v1 = 2.0 * s[2] + 5.0 * s[3] - s[4];
  *sl = (1.0 / 6.0) * a * (a3 * v3 + a2 * v2 + a1 * v1);

  b3 = c13 * sq(s[5] - 2.0 * s[4] + s[3]) + 0.25 * sq(s[5] - 4.0 * s[4] + 3.0 * s[3]);
  b2 = c13 * sq(s[4] - 2.0 * s[3] + s[2]) + 0.25 * (s[4] - s[2]) * (s[4] - s[2]);
  b1 = c13 * sq(s[3] - 2.0 * s[2] + s[1]) + 0.25 * sq(3.0 * s[3] - 4.0 * s[2] + s[1]);
  weno5_weights(&b3, &b2, &b1, flag_weno);
  a3 = b3;
  a2 = 6.0 * b2;
  a1 = 3.0 * b1;
  a = 1.0 / (a3 + a2 + a1);
  v3 = 11.0 * s[3] - 7.0 * s[4] + 2.0 * s[5];
  v2 = -s[4] + 5.0 * s[3] + 2.0 * s[2];
  v1 = 2.0 * s[3] + 5.0 * s[2] - s[1];
  *sr = (1.0 / 6.0) * a * (a3 * v3 + a2 * v2 + a1 * v1);
}

/* weno7z, SRC/weno.f90:169-267 */
void or_weno7z(const double* s, double* sl, double* sr) {
  const double eps = 1.0e-6;
  const double w[4] = {1.0 / 35.0, 12.0 / 35.0, 18.0 / 35.0, 4.0 / 35.0};
  double b[5], a[5], v[5];
  for (int side = 0; side < 2; ++side) {
    double q[8];
    for (int j = 0; j < 8; ++j) q[j] = side == 0 ? s[j] : s[7 - j];
    b[4] = q[0] * (547.0 * q[0] - 3882.0 * q[1] + 4642.0 * q[2] - 1854.0 * q[3]) +
           q[1] * (7043.0 * q[1] - 17246.0 * q[2] + 7042.0 * q[3]) + q[2] * (11003.0 * q[2] - 9402.0 * q[3]) +
           2107.0 * (q[3] * q[3]);
    b[3] = q[1] * (267.0 * q[1] - 1642.0 * q[2] + 1602.0 * q[3] - 494.0 * q[4]) +
           q[2] * (2843.0 * q[2] - 5966.0 * q[3] + 1922.0 * q[4]) + q[3] * (3443.0 * q[3] - 2522.0 * q[4]) +
           547.0 * (q[4] * q[4]);
    b[2] = q[2] * (547.0 * q[2] - 2522.0 * q[3] + 1922.0 * q[4] - 494.0 * q[5]) +
           q[3] * (3443.0 * q[3] - 5966.0 * q[4] + 1602.0 * q[5]) + q[4] * (2843.0 * q[4] - 1642.0 * q[5]) +
           267.0 * (q[5] * q[5]);
    b[1] = q[3] * (2107.0 * q[3] - 9402.0 * q[4] + 7042.0 * q[5] - 1854.0 * q[6]) +
           q[4] * (11003.0 * q[4] - 17246.0 * q[5] + 4642.0 * q[6]) + q[5] * (7043.0 * q[5] - 3882.0 * q[6]) +
           547.0 * (q[6] * q[6]);
    double tau = fabs(b[4] - b[1]);
    for (int j = 4; j >= 1; --j) b[j] = 1.0 + (tau / (eps + b[j])) * (tau / (eps + b[j]));
    a[4] = w[0] * b[4];
    a[3] = w[1] * b[3];
    a[2] = w[2] * b[2];
    a[1] = w[3] * b[1];
    double al = 1.0 / (a[4] + a[3] + a[2] + a[1]);
    v[4] = -3.0 * q[0] + 13.0 * q[1] - 23.0 * q[2] + 25.0 * q[3];
    v[3] = 1.0 * q[1] - 5.0 * q[2] + 13.0 * q[3] + 3.0 * q[4];
    v[2] = -1.0 * q[2] + 7.0 * q[3] + 7.0 * q[4] - 1.0 * q[5];
    v[1] = 3.0 * q[3] + 13.0 * q[4] - 5.0 * q[5] + 1.0 * q[6];
    double r = (1.0 / 12.0) * al * (a[4] * v[4] + a[3] * v[3] + a[2] * v[2] + a[1] * v[1]);
    if (side == 0) *sl = r; else *sr = r;
  }
}

/* ---- tube state ---- */

#define QF(t, i) ((t)->qf + (size_t)((i) + (t)->lvir) * (t)->nequ)
#define QC(t, i) ((t)->qc + (size_t)((i) + (t)->lvir) * (t)->nequ)

or_tube* or_tube_create(const or_mech* m, int n, int lvir, const int* iflags, const double* rparams,
                        const double* x_in) {
  or_tube* t = (or_tube*)calloc(1, sizeof(or_tube));
  t->m = m;
  t->n = n;
  t->lvir = lvir;
  t->nspe = m->kk;
  t->nequ = m->kk + 3;
  t->select_time = iflags[0];
  t->select_riemann = iflags[1];
  t->flag_acu = iflags[2];
  t->flag_muscl = iflags[3];
  t->flag_weno = iflags[4];
  t->flag_lbound = iflags[5];
  t->flag_rbound = iflags[6];
  t->do_reaction = iflags[7];
  t->dx = rparams[0];
  t->p_out = rparams[1];
  t->t_in = rparams[2];
  t->rho_u_in = rparams[3];
  t->rtol = rparams[4];
  t->atol = rparams[5];
  if (x_in) {
    for (int k = 0; k < m->kk; ++k) t->x_in[k] = x_in[k];
    or_ckxty(m, t->x_in, t->y_in);
  }
  size_t tot = (size_t)(n + 2 * lvir) * t->nequ;
  t->qf = (double*)calloc(tot, sizeof(double));
  t->qc = (double*)calloc(tot, sizeof(double));
  t->q0 = (double*)calloc((size_t)n * t->nequ, sizeof(double));
  t->fplus = (double*)calloc((size_t)(n + 1) * t->nequ, sizeof(double));
  t->pgod = (double*)calloc((size_t)(n + 1), sizeof(double));
  t->hrr = (double*)calloc((size_t)n, sizeof(double));
  t->hrr_dot = (double*)calloc((size_t)n, sizeof(double));
  t->qrad = (double*)calloc((size_t)n, sizeof(double));
  t->qtw = (double*)calloc((size_t)n, sizeof(double));
  return t;
}

void or_tube_destroy(or_tube* t) {
  if (!t) return;
  free(t->qf);
  free(t->qc);
  free(t->q0);
  free(t->fplus);
  free(t->pgod);
  free(t->hrr);
  free(t->hrr_dot);
  free(t->qrad);
  free(t->qtw);
  free(t);
}

void or_tube_set_interior(or_tube* t, const double* qf, const double* qc) {
  memcpy(QF(t, 0), qf, sizeof(double) * (size_t)t->n * t->nequ);
  memcpy(QC(t, 0), qc, sizeof(double) * (size_t)t->n * t->nequ);
  /* main.f90:107-121: boundary + ghost QcToqf after set_block_params */
  or_update_boundary(t);
}

void or_tube_get_interior(const or_tube* t, double* qf, double* qc) {
  if (qf) memcpy(qf, QF(t, 0), sizeof(double) * (size_t)t->n * t->nequ);
  if (qc) memcpy(qc, QC(t, 0), sizeof(double) * (size_t)t->n * t->nequ);
}

void or_tube_get_all(const or_tube* t, double* qf, double* qc) {
  size_t tot = (size_t)(t->n + 2 * t->lvir) * t->nequ;
  if (qf) memcpy(qf, t->qf, sizeof(double) * tot);
  if (qc) memcpy(qc, t->qc, sizeof(double) * tot);
}

/* ---- SRC/boundary.f90 ---- */

static void lbound_wall(or_tube* t) {
  /* SRC/boundary.f90:152-174 */
  for (int l = 1; l <= t->lvir; ++l) {
    memcpy(QC(t, -l), QC(t, l - 1), sizeof(double) * t->nequ);
    QC(t, -l)[1] = -QC(t, l - 1)[1];
  }
}

static void rbound_wall(or_tube* t) {
  /* SRC/boundary.f90:177-199 */
  int e = t->n - 1;
  for (int l = 1; l <= t->lvir; ++l) {
    memcpy(QC(t, e + l), QC(t, e - l + 1), sizeof(double) * t->nequ);
    QC(t, e + l)[1] = -QC(t, e - l + 1)[1];
  }
}

static void lbound_inlet(or_tube* t) {
  /* SRC/boundary.f90:70-103 */
  const or_mech* m = t->m;
  for (int l = 1; l <= t->lvir; ++l) {
    double rho_in = QC(t, l - 1)[0];
    double p_in = or_pressure(m, rho_in, t->t_in, t->x_in);
    (void)p_in;
    double* g = QC(t, -l);
    g[0] = rho_in;
    g[1] = t->rho_u_in;
    double u_in = t->rho_u_in / rho_in;
    double e_in = or_specific_energy(m, t->t_in, t->x_in);
    g[2] = rho_in * (e_in + 0.5 * (u_in * u_in));
    for (int k = 0; k < t->nspe; ++k) g[3 + k] = rho_in * t->y_in[k];
  }
}

static void rbound_outlet(or_tube* t) {
  /* SRC/boundary.f90:106-149 */
  const or_mech* m = t->m;
  int e = t->n - 1;
  double x[OR_MAXSP], y[OR_MAXSP];
  for (int l = 1; l <= t->lvir; ++l) {
    const double* in = QC(t, e - l + 1);
    double* g = QC(t, e + l);
    g[1] = -in[1];
    double u_out = in[1] / in[0];
    double e_out = in[2] / in[0] - 0.5 * (u_out * u_out);
    for (int k = 0; k < t->nspe; ++k) y[k] = in[3 + k] / in[0];
    or_ckytx(m, y, x);
    double t_out = or_temperature_con(m, e_out, x, NULL);
    double rho_out = or_density(m, t->p_out, t_out, x);
    g[0] = rho_out;
    g[1] = rho_out * u_out;
    e_out = or_specific_energy(m, t_out, x);
    g[2] = rho_out * (e_out + 0.5 * (u_out * u_out));
    for (int k = 0; k < t->nspe; ++k) g[3 + k] = rho_out * y[k];
  }
}

/* update_boundary, SRC/boundary.f90:12-67: ghost Qc from the boundary rule,
 * then QcToqf on the ghost cells of both domain ends. */
void or_update_boundary(or_tube* t) {
  /* an SMR block's side that faces another block takes its ghosts from
   * interpolation_block, not from a boundary rule */
  if (!t->smr_left) {
    if (t->flag_lbound == 0) lbound_wall(t);
    else if (t->flag_lbound == 1) lbound_inlet(t);
    for (int l = 1; l <= t->lvir; ++l) or_qc_to_qf(t->m, QC(t, -l), QF(t, -l));
  }
  if (!t->smr_right) {
    if (t->flag_rbound == 0) rbound_wall(t);
    else if (t->flag_rbound == 1) rbound_outlet(t);
    for (int l = 1; l <= t->lvir; ++l) or_qc_to_qf(t->m, QC(t, t->n - 1 + l), QF(t, t->n - 1 + l));
  }
}

void or_ghost_qf(or_tube* t) { or_update_boundary(t); }

/* The largest signal speed max(|u - a|, |u|, |u + a|) of calc_dt. */
static double or_cvel(or_tube* t);

/* calc_dt, SRC/update.f90:13-59 (the all-reduce is a no-op on one rank). */
double or_calc_dt(or_tube* t, double cfl) { return (cfl * t->dx) / or_cvel(t); }

static double or_cvel(or_tube* t) {
  const or_mech* m = t->m;
  double cvel = 0.0;
#pragma omp parallel for reduction(max : cvel) schedule(static)
  for (int i = 0; i < t->n; ++i) {
    double x[OR_MAXSP];
    const double* q = QF(t, i);
    or_ckytx(m, q + 3, x);
    double rho = q[0], temp = q[2];
    double pres = or_pressure(m, rho, temp, x);
    double a = or_sonic_speed(m, rho, pres, temp, x);
    double aupc = fmax(fmax(fabs(q[1] - a), fabs(q[1])), fabs(q[1] + a));
    if (aupc > cvel) cvel = aupc;
  }
  return cvel;
}

/* calc_flux_advection, SRC/flux.f90:130-373 (Cartesian). Face f lies
 * between cells f-1 and f; the flux is added to Fplus (SRC/flux.f90:358). */
static void or_calc_flux_advection_add(or_tube* t) {
  const or_mech* m = t->m;
  const int ns = t->nspe, ne = t->nequ;
#pragma omp parallel for schedule(static)
  for (int f = 0; f <= t->n; ++f) {
    double qfl[OR_MAXSP + 3], qfr[OR_MAXSP + 3], qcl[OR_MAXSP + 3], qcr[OR_MAXSP + 3];
    double fl[OR_MAXSP + 3], fr[OR_MAXSP + 3], flux[OR_MAXSP + 3], vec[OR_MAXSP + 3];
    double xl[OR_MAXSP], xr[OR_MAXSP];
    int i = f - 1; /* reference face index i: between cells i and i+1 */
    for (int n = 0; n < ne; ++n) {
      double s[8];
      if (t->flag_acu == 1) {
        for (int j = 0; j < 4; ++j) s[j] = QF(t, i - 1 + j)[n];
        or_muscl3(s, &qfl[n], &qfr[n], t->flag_muscl);
      } else if (t->flag_acu == 2 && t->flag_weno == 1) {
        for (int j = 0; j < 4; ++j) s[j] = QF(t, i - 1 + j)[n];
        or_weno3z(s, &qfl[n], &qfr[n]);
      } else if (t->flag_acu == 2 && (t->flag_weno == 2 || t->flag_weno == 3)) {
        for (int j = 0; j < 6; ++j) s[j] = QF(t, i - 2 + j)[n];
        or_weno5(s, &qfl[n], &qfr[n], t->flag_weno);
      } else if (t->flag_acu == 2 && t->flag_weno == 4) {
        for (int j = 0; j < 7; ++j) s[j] = QF(t, i - 3 + j)[n];
        s[7] = QF(t, i + 3)[n]; /* the reference repeats q(i+3), SRC/flux.f90:232 */
        or_weno7z(s, &qfl[n], &qfr[n]);
      }
    }
    if (t->flag_acu == 0) {
      memcpy(qfl, QF(t, i), sizeof(double) * ne);
      memcpy(qfr, QF(t, i + 1), sizeof(double) * ne);
    }
    or_qf_to_qc(m, qfl, qcl);
    or_qf_to_qc(m, qfr, qcr);
    or_ckytx(m, qfl + 3, xl);
    or_ckytx(m, qfr + 3, xr);
    or_adjust_sum(ns, xl);
    or_adjust_sum(ns, xr);
    double rhol = qfl[0], rhor = qfr[0], ul = qfl[1], ur = qfr[1], tl = qfl[2], tr = qfr[2];
    double pl = or_pressure(m, rhol, tl, xl), pr = or_pressure(m, rhor, tr, xr);
    double al = or_sonic_speed(m, rhol, pl, tl, xl), ar = or_sonic_speed(m, rhor, pr, tr, xr);
    double el = qcl[2], er = qcr[2];
    double hl = (el + pl) / rhol, hr = (er + pr) / rhor;
    fl[0] = rhol * ul;
    fr[0] = rhor * ur;
    if (t->is_spherical) { /* SRC/flux.f90:272-278 */
      fl[1] = rhol * ul * ul;
      fr[1] = rhor * ur * ur;
    } else {
      fl[1] = rhol * ul * ul + pl;
      fr[1] = rhor * ur * ur + pr;
    }
    fl[2] = (el + pl) * ul;
    fr[2] = (er + pr) * ur;
    for (int k = 0; k < ns; ++k) {
      fl[3 + k] = rhol * qfl[3 + k] * ul;
      fr[3 + k] = rhor * qfr[3 + k] * ur;
    }
    if (t->select_riemann == 0) {
      double lamL = fmax(fmax(fabs(ul - al), fabs(ul)), fabs(ul + al));
      double lamR = fmax(fmax(fabs(ur - ar), fabs(ur)), fabs(ur + ar));
      double alpha = fmax(lamL, lamR);
      for (int n = 0; n < ne; ++n) flux[n] = 0.5 * (fl[n] + fr[n] - alpha * (qcr[n] - qcl[n]));
    } else {
      double rt = sqrt(rhor / rhol);
      double u_roe = (ul + rt * ur) / (1.0 + rt);
      double h_roe = (hl + rt * hr) / (1.0 + rt);
      double a_roe = (al + rt * ar) / (1.0 + rt);
      (void)h_roe;
      double sL = fmin(ul - al, u_roe - a_roe);
      double sR = fmax(ur + ar, u_roe + a_roe);
      if (t->select_riemann == 1) {
        if (0.0 <= sL) {
          memcpy(flux, fl, sizeof(double) * ne);
        } else if (sL <= 0.0 && 0.0 <= sR) {
          for (int n = 0; n < ne; ++n) flux[n] = (sR * fl[n] - sL * fr[n] + sL * sR * (qcr[n] - qcl[n])) / (sR - sL);
        } else {
          memcpy(flux, fr, sizeof(double) * ne);
        }
      } else {
        double sM = (pl - pr + rhor * ur * (sR - ur) - rhol * ul * (sL - ul)) / (rhor * (sR - ur) - rhol * (sL - ul));
        if (0.0 <= sL) {
          memcpy(flux, fl, sizeof(double) * ne);
        } else if (sL <= 0.0 && 0.0 <= sM) {
          vec[0] = 1.0;
          vec[1] = sM;
          vec[2] = el / rhol + (sM - ul) * (sM + pl / (rhol * (sL - ul)));
          for (int k = 0; k < ns; ++k) vec[3 + k] = qcl[3 + k] / rhol;
          double fac = rhol * (sL - ul) / (sL - sM);
          for (int n = 0; n < ne; ++n) flux[n] = fl[n] + sL * (fac * vec[n] - qcl[n]);
        } else if (sM <= 0.0 && 0.0 <= sR) {
          vec[0] = 1.0;
          vec[1] = sM;
          vec[2] = er / rhor + (sM - ur) * (sM + pr / (rhor * (sR - ur)));
          for (int k = 0; k < ns; ++k) vec[3 + k] = qcr[3 + k] / rhor;
          double fac = rhor * (sR - ur) / (sR - sM);
          for (int n = 0; n < ne; ++n) flux[n] = fr[n] + sR * (fac * vec[n] - qcr[n]);
        } else {
          memcpy(flux, fr, sizeof(double) * ne);
        }
      }
    }
    /* the face's Roe-averaged pressure (godunov_state, SRC/flux.f90:360-367) */
    {
      double rt = sqrt(rhor / rhol);
      t->pgod[f] = (pl + rt * pr) / (1.0 + rt);
    }
    double* fp = t->fplus + (size_t)f * ne;
    for (int n = 0; n < ne; ++n) fp[n] = fp[n] + flux[n];
  }
}

void or_tube_set_transport(or_tube* t, const or_tran* tr) { t->tran = tr; }

/* calc_flux_tran, SRC/flux.f90:18-127: every face i (between cells i and
 * i+1 of the reference, f-1 and f here, ghosts included) from the current
 * conserved state, added to fplus. */
void or_calc_flux_tran(or_tube* t) {
  const int ne = t->nequ;
#pragma omp parallel for schedule(dynamic, 4)
  for (int f = 0; f <= t->n; ++f)
    or_face_flux_tran(t->m, t->tran, QC(t, f - 1), QC(t, f), t->dx, t->fplus + (size_t)f * ne);
}

/* The flux of a stage (SRC/timeintegration.f90:31-47): Fplus = 0, then the
 * transport flux when do_tran = 1, then the advective flux added. */
static void calc_fluxes(or_tube* t) {
  memset(t->fplus, 0, sizeof(double) * (size_t)(t->n + 1) * t->nequ);
  if (t->tran) or_calc_flux_tran(t);
  or_calc_flux_advection_add(t);
}

void or_calc_flux_advection(or_tube* t) {
  memset(t->fplus, 0, sizeof(double) * (size_t)(t->n + 1) * t->nequ);
  or_calc_flux_advection_add(t);
}

/* QcToqf on every cell including the ghosts (SRC/timeintegration.f90:211-215). */
static void all_qc_to_qf(or_tube* t) {
#pragma omp parallel for schedule(static)
  for (int i = -t->lvir; i < t->n + t->lvir; ++i) or_qc_to_qf(t->m, QC(t, i), QF(t, i));
}

/* boundary + ghost copy + boundary + QcToqf, the tail of every stage. */
static void stage_tail(or_tube* t) {
  or_update_boundary(t);
  or_update_boundary(t);
  all_qc_to_qf(t);
}

/* explicit_euler, SRC/timeintegration.f90:12-96 */
/* The spherical update of cell i (SRC/timeintegration.f90:58-75, 177-198):
 * q = h1 q0 + h2 (q - dt/dV (Ar F_i - Al F_{i-1})) (Euler: q - dt/dV (...)),
 * then the momentum's face-pressure gradient, after the combination. */
static void spherical_update(or_tube* t, int i, double dt, double h1, double h2, const double* q0, int euler) {
  const int ne = t->nequ;
  double dx = t->dx, rm = t->x0 + (i + 0.5) * dx;
  double Al = (rm - (dx / 2.0)) * (rm - (dx / 2.0));
  double Ar = (rm + (dx / 2.0)) * (rm + (dx / 2.0));
  double dV = rm * rm * dx;
  double* q = QC(t, i);
  const double* fp = t->fplus + (size_t)(i + 1) * ne;
  const double* fm = t->fplus + (size_t)i * ne;
  for (int n = 0; n < ne; ++n) {
    double d = (dt / dV) * (Ar * fp[n] - Al * fm[n]);
    q[n] = euler ? q[n] - d : h1 * q0[n] + h2 * (q[n] - d);
  }
  q[1] = q[1] - (dt / dx) * (t->pgod[i + 1] - t->pgod[i]);
}

void or_tube_set_spherical(or_tube* t, int on) { t->is_spherical = on; }

static void euler_update(or_tube* t, double dt) {
  const int ne = t->nequ;
  calc_fluxes(t);
  double c = dt / t->dx;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < t->n; ++i) {
    if (t->is_spherical) {
      spherical_update(t, i, dt, 1.0, 1.0, NULL, 1);
      continue;
    }
    double* q = QC(t, i);
    const double* fp = t->fplus + (size_t)(i + 1) * ne;
    const double* fm = t->fplus + (size_t)i * ne;
    for (int n = 0; n < ne; ++n) q[n] = q[n] - c * (fp[n] - fm[n]);
  }
}

static void explicit_euler(or_tube* t, double dt) {
  euler_update(t, dt);
  stage_tail(t);
}

/* One TVDRK3 stage's fluxes and update, without the stage tail
 * (SRC/timeintegration.f90:131-198); stage 1 also saves Q0. */
static void tvdrk3_update(or_tube* t, int stage, double dt) {
  const int ne = t->nequ;
  if (stage == 1) memcpy(t->q0, QC(t, 0), sizeof(double) * (size_t)t->n * ne);
  {
    calc_fluxes(t);
    double h1, h2;
    if (stage == 1) {
      h1 = 1.0;
      h2 = 1.0;
      memset(t->qc, 0, sizeof(double) * (size_t)(t->n + 2 * t->lvir) * ne);
    } else if (stage == 2) {
      h1 = 3.0 / 4.0;
      h2 = 1.0 / 4.0;
    } else {
      h1 = 1.0 / 3.0;
      h2 = 2.0 / 3.0;
    }
    double c = dt / t->dx;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < t->n; ++i) {
      double* q = QC(t, i);
      const double* q0 = t->q0 + (size_t)i * ne;
      const double* fp = t->fplus + (size_t)(i + 1) * ne;
      const double* fm = t->fplus + (size_t)i * ne;
      if (t->is_spherical) {
        spherical_update(t, i, dt, h1, h2, q0, 0);
        continue;
      }
      for (int n = 0; n < ne; ++n) q[n] = h1 * q0[n] + h2 * (q[n] - c * (fp[n] - fm[n]));
    }
  }
}

/* TVDRK3, SRC/timeintegration.f90:99-219 */
static void tvdrk3(or_tube* t, double dt) {
  for (int stage = 1; stage <= 3; ++stage) {
    tvdrk3_update(t, stage, dt);
    stage_tail(t);
  }
}

/* RK4, SRC/timeintegration.f90:222-356. The interior primitive state is
 * not refreshed between the four flux evaluations in the reference; only the
 * ghost cells are (update_boundary), and that is restated as is. */
static void rk4(or_tube* t, double dt) {
  const int ne = t->nequ, n = t->n;
  double* k[4];
  for (int s = 0; s < 4; ++s) k[s] = (double*)malloc(sizeof(double) * (size_t)n * ne);
  memcpy(t->q0, QC(t, 0), sizeof(double) * (size_t)n * ne);
  for (int s = 0; s < 4; ++s) {
    calc_fluxes(t);
    for (int i = 0; i < n; ++i) {
      double* q = QC(t, i);
      const double* fp = t->fplus + (size_t)(i + 1) * ne;
      const double* fm = t->fplus + (size_t)i * ne;
      for (int v = 0; v < ne; ++v) {
        k[s][(size_t)i * ne + v] = -(dt / t->dx) * (fp[v] - fm[v]);
        if (s < 2) q[v] = q[v] - 0.5 * (0.5 * dt / t->dx) * (fp[v] - fm[v]);
        else if (s == 2) q[v] = q[v] - (dt / t->dx) * (fp[v] - fm[v]);
      }
    }
    if (s < 3) or_update_boundary(t);
  }
  for (int i = 0; i < n; ++i) {
    double* q = QC(t, i);
    for (int v = 0; v < ne; ++v) {
      size_t o = (size_t)i * ne + v;
      q[v] = t->q0[o] + (1.0 / 6.0) * (k[0][o] + 2.0 * k[1][o] + 2.0 * k[2][o] + k[3][o]);
    }
  }
  or_update_boundary(t);
  for (int s = 0; s < 4; ++s) free(k[s]);
  all_qc_to_qf(t);
}

void or_tube_get_source(const or_tube* t, double* hrr, double* hrr_dot) {
  for (int i = 0; i < t->n; ++i) {
    if (hrr) hrr[i] = t->hrr[i];
    if (hrr_dot) hrr_dot[i] = t->hrr_dot[i];
  }
}

/* solve_fluid, SRC/update.f90:62-97 */
void or_solve_fluid(or_tube* t, double dt) {
  if (t->select_time == 0) explicit_euler(t, dt);
  else if (t->select_time == 1) tvdrk3(t, dt);
  else if (t->select_time == 2) rk4(t, dt);
}

/* The post-step block of the time loop, SRC/main.f90:149-163. */
void or_post_step(or_tube* t) { stage_tail(t); }

/* solve_source -> reaction_macks, SRC/update.f90:100-150 and
 * SRC/source.f90:17-84, with the project's FP64 integrator as "macks". */
static void or_solve_reaction(or_tube* t, double dt);

void or_tube_set_sources(or_tube* t, const or_sources* s) { t->src = *s; }
void or_tube_set_time(or_tube* t, double time) { t->time = time; }
int or_sources_sizeof(void) { return (int)sizeof(or_sources); }

/* QcToqf of every interior cell, as each energy source ends (SRC/source.f90:130-134). */
static void interior_qc_to_qf(or_tube* t) {
#pragma omp parallel for schedule(static)
  for (int i = 0; i < t->n; ++i) or_qc_to_qf(t->m, QC(t, i), QF(t, i));
}

/* radiation_heat_loss, SRC/radiation.f90:74-121 */
static double rad_loss(const or_sources* s, double p, double T, const double* x) {
  const double stefan_boltzmann = 5.6703744191844294e-08;
  double T1 = T, T2 = T1 * T1, T3 = T2 * T1, T4 = T3 * T1, T5 = T4 * T1;
  double T0 = 300.0, T04 = T0 * T0 * T0 * T0;
  double kp = 0.0;
  for (int r = 0; r < s->nrad; ++r) {
    const double* c = s->rad_coef[r];
    double kpi = c[0] + c[1] * T1 + c[2] * T2 + c[3] * T3 + c[4] * T4 + c[5] * T5;
    kp = kp + kpi * x[s->rad_sp[r]] * (p / 101325.0);
  }
  return -4.0 * kp * stefan_boltzmann * (T4 - T04);
}

/* heat_transfer + Tw, SRC/mfr.f90:41-78 (thermal_conductivity, SRC/trans.f90:63-77) */
static double wall_heat(const or_sources* s, double T, const double* x, double xm) {
  double lambda = or_thermal_conductivity(s->tran, T, x);
  double A = 0.5 * (s->tw_max - s->tw_min), B = 0.5 * (s->tw_max + s->tw_min);
  double tw = A * tanh(s->alpha * (xm - s->beta)) + B;
  return -4.0 * lambda * s->nu * (T - tw) / (s->d_m * s->d_m);
}

/* add_igsource (type 1) and add_igsource_WZhang (type 2), SRC/ignitionsource.f90:150-262 */
static double ignition(const or_sources* s, double time, double rm) {
  const double pi = 3.14159265359;
  double eadd = 0.0;
  for (int g = 0; g < s->n_ig; ++g) {
    double e = s->ig_e[g], r = s->ig_r[g], tg = s->ig_t[g], t0 = s->ig_t0[g];
    if (t0 < time && time < t0 + tg) {
      if (s->ig_type == 1) {
        double vol = 4.0 * pi * (r * r * r) / 3.0;
        double w = rm / r, w2 = w * w;
        eadd = e / (vol * tg) * exp(-(pi / 4.0) * (w2 * w2 * w2));
      } else {
        double w = rm / r;
        eadd = e / (pow(pi, 1.5) * (r * r * r) * tg) * exp(-(w * w));
      }
    }
  }
  return eadd;
}

/* heat_transfer_radiation, heat_transfer_mfr, energy_source
 * (SRC/source.f90:88-239) in the order of solve_source (SRC/update.f90:126-147). */
static void energy_sources(or_tube* t, double dt) {
  const or_mech* m = t->m;
  const or_sources* s = &t->src;
  for (int src = 0; src < 3; ++src) {
    if ((src == 0 && !s->nrad) || (src == 1 && !s->wall) || (src == 2 && !s->ig_type)) continue;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < t->n; ++i) {
      const double* q = QF(t, i);
      double x[OR_MAXSP], add;
      double xm = t->x0 + (i + 0.5) * t->dx;
      if (src == 2) {
        add = ignition(s, t->time, xm);
      } else {
        or_ckytx(m, q + 3, x);
        double p = or_pressure(m, q[0], q[2], x);
        add = src == 0 ? rad_loss(s, p, q[2], x) : wall_heat(s, q[2], x, xm);
        if (src == 0) t->qrad[i] = add;
        else t->qtw[i] = add;
      }
      QC(t, i)[2] = QC(t, i)[2] + dt * add;
    }
    interior_qc_to_qf(t);
  }
}

/* set_eos_params (SRC/block.f90:434-470) per cell: X = CKYTX(Y),
 * p = pressure(rho, T, X), ek = u^2/2, ei = specific_energy(T, X),
 * et = Qc(iuener) / rho; then the rows in write_hdf5_b's order
 * (SRC/write_hdf5.f90:140-162), Tw from the wall profile when it is set
 * (SRC/params.f90:495-499), else 0. Cell centres (i + 1/2) dx. */
void or_output_rows(const or_tube* t, double* rows) {
  const or_mech* m = t->m;
  const int n = t->n, ns = t->nspe;
  const or_sources* s = &t->src;
  for (int i = 0; i < n; ++i) {
    const double* q = QF(t, i);
    const double* c = QC(t, i);
    double x[OR_MAXSP];
    or_ckytx(m, q + 3, x);
    const double xm = t->x0 + (i + 0.5) * t->dx;
    double* o = rows + i;
    o[0] = q[0];
    o[(size_t)n] = q[1];
    o[2 * (size_t)n] = q[2];
    o[3 * (size_t)n] = or_pressure(m, q[0], q[2], x);
    o[4 * (size_t)n] = c[2] / q[0];
    o[5 * (size_t)n] = 0.5 * (q[1] * q[1]);
    o[6 * (size_t)n] = or_specific_energy(m, q[2], x);
    o[7 * (size_t)n] = t->hrr[i];
    o[8 * (size_t)n] = t->hrr_dot[i];
    o[9 * (size_t)n] = t->qrad[i];
    o[10 * (size_t)n] = s->wall ? 0.5 * (s->tw_max - s->tw_min) * tanh(s->alpha * (xm - s->beta)) +
                                      0.5 * (s->tw_max + s->tw_min)
                                : 0.0;
    o[11 * (size_t)n] = t->qtw[i];
    o[12 * (size_t)n] = xm;
    o[13 * (size_t)n] = t->dx;
    o[14 * (size_t)n] = (double)(i + 1);
    for (int k = 0; k < ns; ++k) o[(size_t)(OR_OUT_FIXED + k) * n] = x[k];
  }
}

void or_solve_source(or_tube* t, double dt) {
  or_solve_reaction(t, dt);
  energy_sources(t, dt);
}

static void or_solve_reaction(or_tube* t, double dt) {
  if (!t->do_reaction) return;
  const or_mech* m = t->m;
  const int ns = t->nspe;
  long rhs_sum = 0, step_sum = 0;
/* chunks of one cell: the costly cells of a reaction front are neighbours */
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : rhs_sum, step_sum)
  for (int i = 0; i < t->n; ++i) {
    double* q = QF(t, i);
    double y0[OR_MAXSP], y[OR_MAXSP], yit[OR_MAXSP + 1];
    for (int k = 0; k < ns; ++k) y0[k] = q[3 + k];
    double rho = q[0], temp = q[2];
    for (int k = 0; k < ns; ++k) y[k] = q[3 + k];
    or_adjust_sum(ns, y);
    for (int k = 0; k < ns; ++k) yit[k] = y[k];
    yit[ns] = temp;
    or_chem_stats st = {0, 0, 0, 0, 0};
    or_reactor(m, rho, dt, yit, t->rtol, t->atol, &st);
    rhs_sum += st.rhs;
    step_sum += st.steps;
    for (int k = 0; k < ns; ++k) y[k] = yit[k];
    temp = yit[ns];
    or_adjust_sum(ns, y);
    q[2] = temp;
    for (int k = 0; k < ns; ++k) q[3 + k] = y[k];
    /* heat_release_rate, SRC/thermo.f90:83-103 */
    double rho_cgs = rho * 1e-3, s = 0.0;
    for (int k = 0; k < ns; ++k) s = s + rho_cgs * m->hf298[k] * (q[3 + k] - y0[k]) / dt;
    t->hrr[i] = -s * 1e-1;
    /* heat_release_rate_omegadot, SRC/thermo.f90:105-134 */
    double cdot[OR_MAXSP], ddot[OR_MAXSP];
    or_ckcdyr(m, rho_cgs, temp, q + 3, cdot, ddot);
    s = 0.0;
    for (int k = 0; k < ns; ++k) s = s + m->wt[k] * m->hf298[k] * (cdot[k] - ddot[k]);
    t->hrr_dot[i] = -s * 1e-1;
  }
  t->chem_rhs_evals += rhs_sum;
  t->chem_steps += step_sum;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < t->n; ++i) or_qf_to_qc(m, QF(t, i), QC(t, i));
}

/* One pass of the time loop body, SRC/main.f90:130-163. */
double or_step(or_tube* t, double cfl) {
  double dt = or_calc_dt(t, cfl);
  t->time = t->time + dt;
  or_solve_fluid(t, dt);
  or_solve_source(t, dt);
  or_post_step(t);
  return dt;
}

/* ---- SMR blocks: SRC/block.f90:475-569 (interpolation_block) and the
 * stage tails of SRC/timeintegration.f90 and SRC/main.f90:149-163 ----
 * Segments are runs of equal-dx blocks (whose ghost exchange is a plain copy,
 * the same as one contiguous array); consecutive segments differ in dx. */

struct or_smr {
  int nseg;
  or_tube* seg[OR_MAXSEG];
  double dx_comp;
};

/* minmod slope of interpolation_block: 0.5 (sign(1, m) + sign(1, p)) min(|m|, |p|) */
static double smr_slope(double m, double p) {
  return 0.5 * (copysign(1.0, m) + copysign(1.0, p)) * fmin(fabs(m), fabs(p));
}

static void smr_interface(or_tube* a, or_tube* b) {
  const int ne = a->nequ, lv = a->lvir;
  const int ea = a->n - 1; /* iend of the left block; ista of the right is 0 */
  if (a->dx == b->dx) {
    for (int l = 1; l <= lv; ++l) {
      memcpy(QC(b, -l), QC(a, ea - l + 1), sizeof(double) * ne);
      memcpy(QC(a, ea + l), QC(b, l - 1), sizeof(double) * ne);
    }
  } else if (a->dx > b->dx) {
    /* left coarse, right fine: restriction into the left's ghosts, then
     * prolongation of the left (ghosts included) into the right's */
    for (int l = 1; l <= lv; ++l)
      for (int v = 0; v < ne; ++v)
        QC(a, ea + l)[v] = (QC(b, 2 * (l - 1))[v] + QC(b, 2 * (l - 1) + 1)[v]) / 2.0;
    for (int l = 1; l <= lv; ++l) {
      int ic = -((l - 1) / 2);
      for (int v = 0; v < ne; ++v) {
        double m = QC(a, ea + ic)[v] - QC(a, ea + ic - 1)[v];
        double p = QC(a, ea + ic + 1)[v] - QC(a, ea + ic)[v];
        double d = smr_slope(m, p);
        QC(b, -l)[v] = (l % 2 == 1) ? QC(a, ea + ic)[v] + 0.25 * d : QC(a, ea + ic)[v] - 0.25 * d;
      }
    }
  } else {
    /* left fine, right coarse */
    for (int l = 1; l <= lv; ++l)
      for (int v = 0; v < ne; ++v)
        QC(b, -l)[v] = (QC(a, ea - 2 * (l - 1))[v] + QC(a, ea - 2 * (l - 1) - 1)[v]) / 2.0;
    for (int l = 1; l <= lv; ++l) {
      int ic = (l - 1) / 2;
      for (int v = 0; v < ne; ++v) {
        double m = QC(b, ic)[v] - QC(b, ic - 1)[v];
        double p = QC(b, ic + 1)[v] - QC(b, ic)[v];
        double d = smr_slope(m, p);
        QC(a, ea + l)[v] = (l % 2 == 1) ? QC(b, ic)[v] - 0.25 * d : QC(b, ic)[v] + 0.25 * d;
      }
    }
  }
}

/* update_boundary, interpolation_block, update_boundary, QcToqf of every
 * cell with its ghosts */
static void smr_tail(or_smr* s) {
  for (int g = 0; g < s->nseg; ++g) or_update_boundary(s->seg[g]);
  for (int g = 0; g + 1 < s->nseg; ++g) smr_interface(s->seg[g], s->seg[g + 1]);
  for (int g = 0; g < s->nseg; ++g) or_update_boundary(s->seg[g]);
  for (int g = 0; g < s->nseg; ++g) all_qc_to_qf(s->seg[g]);
}

or_smr* or_smr_create(const or_mech* m, int nseg, const int* ncell, const double* dx, int lvir, const int* iflags,
                      const double* rparams, const double* x_in) {
  if (nseg < 1 || nseg > OR_MAXSEG) return NULL;
  or_smr* s = (or_smr*)calloc(1, sizeof(or_smr));
  s->nseg = nseg;
  s->dx_comp = rparams[0];
  /* x = 0 where the left SMR zone (the leading segments coarser than
   * dx_comp) ends, SRC/block.f90:236-237, 296-304 */
  double x = 0.0;
  for (int g = 0; g < nseg && dx[g] != s->dx_comp; ++g) x -= ncell[g] * dx[g];
  for (int g = 0; g < nseg; ++g) {
    double rp[6];
    for (int j = 0; j < 6; ++j) rp[j] = rparams[j];
    rp[0] = dx[g];
    s->seg[g] = or_tube_create(m, ncell[g], lvir, iflags, rp, x_in);
    s->seg[g]->smr_left = g > 0;
    s->seg[g]->smr_right = g + 1 < nseg;
    s->seg[g]->x0 = x;
    x += ncell[g] * dx[g];
  }
  return s;
}

void or_smr_destroy(or_smr* s) {
  if (!s) return;
  for (int g = 0; g < s->nseg; ++g) or_tube_destroy(s->seg[g]);
  free(s);
}

void or_smr_set_interior(or_smr* s, const double* qf, const double* qc) {
  size_t off = 0;
  for (int g = 0; g < s->nseg; ++g) {
    or_tube* t = s->seg[g];
    memcpy(QF(t, 0), qf + off, sizeof(double) * (size_t)t->n * t->nequ);
    memcpy(QC(t, 0), qc + off, sizeof(double) * (size_t)t->n * t->nequ);
    off += (size_t)t->n * t->nequ;
  }
  /* SRC/main.f90:95-113: boundary, interpolation, boundary, then QcToqf of
   * every block's ghost cells (the interior keeps its qf) */
  for (int g = 0; g < s->nseg; ++g) or_update_boundary(s->seg[g]);
  for (int g = 0; g + 1 < s->nseg; ++g) smr_interface(s->seg[g], s->seg[g + 1]);
  for (int g = 0; g < s->nseg; ++g) {
    or_tube* t = s->seg[g];
    or_update_boundary(t);
    for (int l = 1; l <= t->lvir; ++l) {
      or_qc_to_qf(t->m, QC(t, -l), QF(t, -l));
      or_qc_to_qf(t->m, QC(t, t->n - 1 + l), QF(t, t->n - 1 + l));
    }
  }
}

/* do_tran on every block (NULL: off). */
void or_smr_set_transport(or_smr* s, const or_tran* tr) {
  for (int g = 0; g < s->nseg; ++g) s->seg[g]->tran = tr;
}

void or_smr_set_spherical(or_smr* s, int on) {
  for (int g = 0; g < s->nseg; ++g) s->seg[g]->is_spherical = on;
}

void or_smr_set_sources(or_smr* s, const or_sources* src) {
  for (int g = 0; g < s->nseg; ++g) or_tube_set_sources(s->seg[g], src);
}

void or_smr_set_time(or_smr* s, double time) {
  for (int g = 0; g < s->nseg; ++g) s->seg[g]->time = time;
}

void or_smr_output_rows(const or_smr* s, int g, double* rows) { or_output_rows(s->seg[g], rows); }

/* Segment g's conserved columns with its ghosts ((n + 2 lvir) x nequ). */
void or_smr_segment_all(const or_smr* s, int g, double* qc) { or_tube_get_all(s->seg[g], NULL, qc); }

void or_smr_get_interior(const or_smr* s, double* qf, double* qc) {
  size_t off = 0;
  for (int g = 0; g < s->nseg; ++g) {
    const or_tube* t = s->seg[g];
    or_tube_get_interior(t, qf ? qf + off : NULL, qc ? qc + off : NULL);
    off += (size_t)t->n * t->nequ;
  }
}

/* One pass of the time loop over all blocks with one dt = cfl dx_comp /
 * max(|u| + a) (SRC/update.f90:13-59): Euler or TVDRK3 stages with the
 * blocks' ghost exchange after each, the source step, the post-step tail. */
double or_smr_step(or_smr* s, double cfl) {
  double cvel = 0.0;
  for (int g = 0; g < s->nseg; ++g) {
    double c = or_cvel(s->seg[g]);
    if (c > cvel) cvel = c;
  }
  double dt = (cfl * s->dx_comp) / cvel;
  or_tube* t0 = s->seg[0];
  if (t0->select_time == 0) {
    for (int g = 0; g < s->nseg; ++g) euler_update(s->seg[g], dt);
    smr_tail(s);
  } else {
    for (int stage = 1; stage <= 3; ++stage) {
      for (int g = 0; g < s->nseg; ++g) tvdrk3_update(s->seg[g], stage, dt);
      smr_tail(s);
    }
  }
  for (int g = 0; g < s->nseg; ++g) {
    s->seg[g]->time = s->seg[g]->time + dt;
    or_solve_source(s->seg[g], dt);
  }
  smr_tail(s);
  return dt;
}
