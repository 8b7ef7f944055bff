/*
 * Oracle (test infrastructure only): the per-cell chemistry step.
 *
 * The reference calls macks(dt, nspe+1, yiT, rho) (SRC/source.f90:58) from
 * an odes.f90 that is not part of the reference tree, so there is nothing to
 * restate line by line. The contract is kept: a constant-density adiabatic
 * reactor advanced over dt on the state [Y_1..Y_K, T], with the CHEMKIN
 * production rates of CKWYR (GRI/cklib.f:9107) and dT/dt from energy
 * conservation at constant volume:
 *     dY_k/dt = W_k w_k / rho,   dT/dt = -sum_k u_k w_k / (rho cv).
 * The integrator is the project's FP64 reference: the L-stable SDIRK method
 * of order 4 with an embedded order-3 solution (Hairer & Wanner, Solving
 * ODEs II, Table 6.5, gamma = 1/4), simplified Newton with an analytic
 * Jacobian and partially pivoted LU in FP64, error filtered by
 * (I - h gamma J)^-1, standard step-size control.
 */
#include "edyn_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define NMAX (OR_MAXSP + 1)

/* dY/dt and dT/dt in cgs units (rho in g/cm^3). */
void or_chem_rhs(const or_mech* m, double rho, const double* yT, double* f) {
  const int kk = m->kk;
  double wdot[OR_MAXSP], uml[OR_MAXSP], cvml[OR_MAXSP];
  double t = yT[kk];
  or_ckwyr(m, rho, t, yT, wdot);
  or_ckuml(m, t, uml);
  or_ckcvml(m, t, cvml);
  double cv = 0.0, su = 0.0;
  for (int k = 0; k < kk; ++k) {
    cv += yT[k] * cvml[k] / m->wt[k];
    su += uml[k] * wdot[k];
    f[k] = wdot[k] * m->wt[k] / rho;
  }
  f[kk] = -su / (rho * cv);
}

static const double SD_G = 0.25;
static const double SD_A[5][5] = {
    {0.25, 0, 0, 0, 0},
    {0.5, 0.25, 0, 0, 0},
    {17.0 / 50.0, -1.0 / 25.0, 0.25, 0, 0},
    {371.0 / 1360.0, -137.0 / 2720.0, 15.0 / 544.0, 0.25, 0},
    {25.0 / 24.0, -49.0 / 48.0, 125.0 / 16.0, -85.0 / 12.0, 0.25}};
static const double SD_BH[5] = {59.0 / 48.0, -17.0 / 96.0, 225.0 / 32.0, -85.0 / 12.0, 0.0};

static int lu_factor(double* a, int n, int* piv) {
  for (int k = 0; k < n; ++k) {
    int p = k;
    double amax = fabs(a[k * n + k]);
    for (int i = k + 1; i < n; ++i)
      if (fabs(a[i * n + k]) > amax) {
        amax = fabs(a[i * n + k]);
        p = i;
      }
    piv[k] = p;
    if (amax == 0.0) return 1;
    if (p != k)
      for (int j = 0; j < n; ++j) {
        double tmp = a[k * n + j];
        a[k * n + j] = a[p * n + j];
        a[p * n + j] = tmp;
      }
    double inv = 1.0 / a[k * n + k];
    for (int i = k + 1; i < n; ++i) {
      double l = a[i * n + k] * inv;
      a[i * n + k] = l;
      if (l != 0.0)
        for (int j = k + 1; j < n; ++j) a[i * n + j] -= l * a[k * n + j];
    }
  }
  return 0;
}

static void lu_solve(const double* a, int n, const int* piv, double* b) {
  for (int k = 0; k < n; ++k) {
    int p = piv[k];
    if (p != k) {
      double tmp = b[k];
      b[k] = b[p];
      b[p] = tmp;
    }
    for (int i = k + 1; i < n; ++i) b[i] -= a[i * n + k] * b[k];
  }
  for (int i = n - 1; i >= 0; --i) {
    double s = b[i];
    for (int j = i + 1; j < n; ++j) s -= a[i * n + j] * b[j];
    b[i] = s / a[i * n + i];
  }
}

static double wnorm(const double* v, const double* sc, int n) {
  double s = 0.0;
  for (int i = 0; i < n; ++i) {
    double q = v[i] / sc[i];
    s += q * q;
  }
  return sqrt(s / n);
}

/* Jacobian of the reactor right-hand side: analytic mass-action
 * derivatives in concentration space (collider dependence of third-body and
 * fall-off reactions included, the fall-off blending factor held fixed),
 * mapped to mass fractions, with the temperature column by a one-sided
 * difference. Finite differences in the mass fractions are unusable here:
 * the gross reaction fluxes exceed the net rates by orders of magnitude, so
 * the difference quotients of trace species drown in rounding. */
static void chem_jacobian(const or_mech* m, double rho, const double* y, const double* f0, double* jac) {
  const int kk = m->kk, n = kk + 1, ii = m->ii;
  double c[OR_MAXSP], rkf[OR_MAXRX], rkr[OR_MAXRX], kfe[OR_MAXRX], kre[OR_MAXRX], cm[OR_MAXRX], pd[OR_MAXRX];
  double t = y[kk];
  memset(jac, 0, sizeof(double) * n * n);
  /* effective rate constants (third-body and fall-off factors included) */
  or_ckrop_k(m, rho, t, y, rkf, rkr, kfe, kre);
  for (int k = 0; k < kk; ++k) c[k] = rho * y[k] / m->wt[k];
  double ctot = 0.0;
  for (int k = 0; k < kk; ++k) ctot += c[k];
  for (int i = 0; i < ii; ++i) {
    /* collider concentration and d ln(rate) / d ln(C_M) of the pressure factor */
    cm[i] = 1.0;
    pd[i] = 0.0;
    if (m->tb[i] == 1 || (m->tb[i] == 2 && m->kfal[i] < 0)) {
      double v = ctot;
      for (int l = 0; l < m->ntbs[i]; ++l) v += (m->aik[i][l] - 1.0) * c[m->nktb[i][l]];
      cm[i] = v;
      pd[i] = 1.0;
    } else if (m->tb[i] == 2) {
      cm[i] = c[m->kfal[i]];
      pd[i] = 1.0;
    }
    if (m->tb[i] == 2) {
      const double* fp = m->fpar[i];
      double kinf = m->par[i][0] * exp(m->par[i][1] * log(t) - m->par[i][2] / t);
      double pr = fp[0] * exp(fp[1] * log(t) - fp[2] / t) * cm[i] / kinf;
      pd[i] = 1.0 / (1.0 + pr);
    }
  }
  for (int i = 0; i < ii; ++i) {
    int ks[6], nus[6], nk = 0;
    for (int sl = 0; sl < 6; ++sl) {
      int k = m->nunk[i][sl];
      if (k < 0) continue;
      int f = -1;
      for (int z = 0; z < nk; ++z)
        if (ks[z] == k) f = z;
      if (f < 0) { ks[nk] = k; nus[nk] = 0; f = nk++; }
      nus[f] += m->nu[i][sl];
    }
    for (int side = 0; side < 2; ++side) {
      const int base = side == 0 ? 0 : 3;
      const double kk_ = side == 0 ? kfe[i] : -kre[i];
      if (kk_ == 0.0) continue;
      if (m->nu[i][0] == 0) continue;
      for (int s = 0; s < 3; ++s) {
        const int kj = m->nunk[i][base + s];
        if (kj < 0) continue;
        const int nj = abs(m->nu[i][base + s]);
        double d = kk_ * nj;
        for (int s2 = 0; s2 < 3; ++s2) {
          const int k2 = m->nunk[i][base + s2];
          if (k2 < 0) continue;
          const int n2 = abs(m->nu[i][base + s2]);
          for (int q = 0; q < (s2 == s ? n2 - 1 : n2); ++q) d *= c[k2];
        }
        for (int z = 0; z < nk; ++z) jac[ks[z] * n + kj] += nus[z] * d;
      }
    }
    if (pd[i] != 0.0 && cm[i] != 0.0) {
      const double r0 = (rkf[i] - rkr[i]) * pd[i] / cm[i];
      if (m->tb[i] == 2 && m->kfal[i] >= 0) {
        for (int z = 0; z < nk; ++z) jac[ks[z] * n + m->kfal[i]] += nus[z] * r0;
      } else {
        for (int j = 0; j < kk; ++j)
          for (int z = 0; z < nk; ++z) jac[ks[z] * n + j] += nus[z] * r0;
        for (int l = 0; l < m->ntbs[i]; ++l)
          for (int z = 0; z < nk; ++z) jac[ks[z] * n + m->nktb[i][l]] += nus[z] * r0 * (m->aik[i][l] - 1.0);
      }
    }
  }
  /* d f_k/d y_j = (W_k / W_j) d w_k / d C_j;  T row from the energy equation */
  double uml[OR_MAXSP], cvml[OR_MAXSP];
  or_ckuml(m, t, uml);
  or_ckcvml(m, t, cvml);
  double cv = 0.0;
  for (int k = 0; k < kk; ++k) cv += y[k] * cvml[k] / m->wt[k];
  for (int j = 0; j < kk; ++j) {
    double acc = 0.0;
    for (int k = 0; k < kk; ++k) {
      double v = jac[k * n + j] * m->wt[k] / m->wt[j];
      jac[k * n + j] = v;
      acc += uml[k] / m->wt[k] * v;
    }
    jac[kk * n + j] = -(acc + f0[kk] * cvml[j] / m->wt[j]) / cv;
  }
  double yp[OR_MAXSP + 1], fp[OR_MAXSP + 1];
  memcpy(yp, y, sizeof(double) * n);
  double dT = fmax(1e-6 * t, 1e-4);
  yp[kk] = t + dT;
  dT = yp[kk] - t;
  or_chem_rhs(m, rho, yp, fp);
  for (int i = 0; i < n; ++i) jac[i * n + kk] = (fp[i] - f0[i]) / dT;
}

/* One reactor over [0, dt]. rho_si in kg/m^3; yiT = [Y_1..Y_K, T] in/out.
 * Returns 0 on success, nonzero if the step size underflowed or the step
 * budget ran out (the state then holds the last accepted point). */
int or_reactor(const or_mech* m, double rho_si, double dt, double* yiT, double rtol, double atol,
               or_chem_stats* st) {
  const int n = m->kk + 1;
  const double rho = rho_si * 1e-3;
  double y0[NMAX], f0[NMAX], jac[NMAX * NMAX], mm[NMAX * NMAX], sc[NMAX];
  double F[5][NMAX], Y[NMAX], s[NMAX], r[NMAX], d[NMAX], err[NMAX], fy[NMAX];
  int piv[NMAX];
  memcpy(y0, yiT, sizeof(double) * n);
  double t = 0.0, h = dt;
  int rc = 0;
  long nsteps = 0;
  while (t < dt) {
    if (++nsteps > 200000) { rc = 2; break; }
    if (t + h > dt) h = dt - t;
    if (h < dt * 1e-14 && t + h < dt) { rc = 3; break; }
    or_chem_rhs(m, rho, y0, f0);
    st->rhs++;
    if (t == 0.0) {
      /* Inert cell: when the whole window's change predicted by the
       * right-hand side, dt f(y0), is below 1e-3 of the error tolerance, one
       * explicit step is accurate far below the tolerance. */
      double q2 = 0.0;
      for (int i = 0; i < n; ++i) {
        double q = dt * f0[i] / (atol + rtol * fabs(y0[i]));
        q2 += q * q;
      }
      if (sqrt(q2 / n) <= 1e-3) {
        for (int i = 0; i < n; ++i) y0[i] += dt * f0[i];
        st->steps++;
        break;
      }
    }
    chem_jacobian(m, rho, y0, f0, jac);
    st->rhs += 1;
    st->jac++;
    for (int i = 0; i < n; ++i) sc[i] = atol + rtol * fabs(y0[i]);
    int accepted = 0;
    while (!accepted) {
      /* Newton matrix I - h gamma J, equilibrated with the error weights:
       * Ms = D^-1 M D with D = diag(sc). Unscaled, the temperature row
       * (entries in K per unit mass fraction) wins the pivot search and
       * partial pivoting loses all accuracy in the species rows. */
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j)
          mm[i * n + j] = ((i == j ? 1.0 : 0.0) - h * SD_G * jac[i * n + j]) * (sc[j] / sc[i]);
      if (lu_factor(mm, n, piv)) {
        h *= 0.25;
        if (!(h >= dt * 1e-14)) { rc = 3; break; }
        continue;
      }
      int newton_ok = 1;
      for (int stg = 0; stg < 5 && newton_ok; ++stg) {
        for (int i = 0; i < n; ++i) {
          double acc = y0[i];
          for (int j = 0; j < stg; ++j) acc += h * SD_A[stg][j] * F[j][i];
          s[i] = acc;
        }
        const double* fprev = stg == 0 ? f0 : F[stg - 1];
        for (int i = 0; i < n; ++i) Y[i] = s[i] + h * SD_G * fprev[i];
        double nrm_prev = 0.0;
        int conv = 0;
        for (int it = 0; it < 10; ++it) {
          if (!(Y[n - 1] > 100.0 && Y[n - 1] < 8000.0)) break;
          or_chem_rhs(m, rho, Y, fy);
          st->rhs++;
          for (int i = 0; i < n; ++i) {
            r[i] = Y[i] - s[i] - h * SD_G * fy[i];
            d[i] = -r[i] / sc[i];
          }
          lu_solve(mm, n, piv, d);
          for (int i = 0; i < n; ++i) d[i] *= sc[i];
          double nrm = wnorm(d, sc, n);
          /* convergence: weighted correction below 1e-2 of the local
           * tolerance, directly or predicted from the contraction rate;
           * one non-contracting iteration (theta < 2) is tolerated */
          if (nrm <= 1e-2) conv = 1;
          if (!conv && it > 0) {
            double theta = nrm / nrm_prev;
            if (theta >= 2.0 || (theta >= 0.99 && it >= 2)) break;
            if (theta < 0.99 && theta / (1.0 - theta) * nrm <= 1e-2) conv = 1;
          }
          if (conv) {
            /* stage derivative = the FP64 right-hand side at the converged
             * iterate; the stage value is rebuilt from it, so every stage
             * derivative is an exact f value and mass and elements are
             * conserved to rounding */
            for (int i = 0; i < n; ++i) {
              F[stg][i] = fy[i];
              Y[i] = s[i] + h * SD_G * fy[i];
            }
            break;
          }
          for (int i = 0; i < n; ++i) Y[i] += d[i];
          nrm_prev = nrm;
        }
        if (!conv) { newton_ok = 0; break; }
      }
      if (!newton_ok) {
        st->newton_fail++;
        h *= 0.25;
        if (h < dt * 1e-14) { rc = 3; break; }
        continue;
      }
      /* embedded error, filtered through (I - h gamma J)^-1 */
      for (int i = 0; i < n; ++i) {
        double e = 0.0;
        for (int j = 0; j < 5; ++j) e += (SD_A[4][j] - SD_BH[j]) * F[j][i];
        err[i] = h * e / sc[i];
      }
      lu_solve(mm, n, piv, err);
      for (int i = 0; i < n; ++i) err[i] *= sc[i];
      double sc2[NMAX];
      for (int i = 0; i < n; ++i) sc2[i] = atol + rtol * fmax(fabs(y0[i]), fabs(Y[i]));
      double en = wnorm(err, sc2, n);
      double fac = 0.9 * pow(fmax(en, 1e-10), -0.25);
      if (en <= 1.0) {
        accepted = 1;
        t += h;
        memcpy(y0, Y, sizeof(double) * n);
        st->steps++;
        h = h * fmin(5.0, fmax(0.2, fac));
      } else {
        st->rejects++;
        h = h * fmin(1.0, fmax(0.2, fac));
        /* the step size underflowed (or the estimate was not a number) */
        if (!(h >= dt * 1e-14)) { rc = 3; break; }
      }
    }
    if (rc) break;
  }
  memcpy(yiT, y0, sizeof(double) * n);
  return rc;
}

int or_reactor_batch(const or_mech* m, int n, const double* rho_si, const double* dt, double* yiT, double rtol,
                     double atol, int nthreads, long* rhs_total) {
  const int nv = m->kk + 1;
  int fails = 0;
  long rhs = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : fails, rhs) num_threads(nthreads > 0 ? nthreads : or_num_threads())
  for (int c = 0; c < n; ++c) {
    or_chem_stats st = {0, 0, 0, 0, 0};
    fails += or_reactor(m, rho_si[c], dt[c], yiT + (size_t)c * nv, rtol, atol, &st) != 0;
    rhs += st.rhs;
  }
  if (rhs_total) *rhs_total = rhs;
  return fails;
}
