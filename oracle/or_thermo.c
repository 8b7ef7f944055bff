/*
 * Oracle (test infrastructure only): mechanism reader, CHEMKIN-II thermo
 * and kinetics, SRC/thermo.f90 and SRC/eos.f90, restated in plain C FP64
 * with the reference's operation order. Compile with -ffp-contract=off.
 */
#include "edyn_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* CHEMKIN machine constants (GRI/cklib.f:4054-4057). */
static const double CK_SMALL = 1e-300;
static const double CK_BIG = 1e300;

/* libgcc's __powidf2: the integer power gfortran emits for X**N with an
 * integer N (repeated squaring, low bit first). */
static double powi(double x, int m) {
  unsigned n = m < 0 ? (unsigned)(-m) : (unsigned)m;
  double y = (n % 2) ? x : 1.0;
  while (n >>= 1) {
    x = x * x;
    if (n % 2) y = y * x;
  }
  return m < 0 ? 1.0 / y : y;
}

int or_mech_sizeof(void) { return (int)sizeof(or_mech); }

/* Reads the mech.edyn text tables (species NASA-7 data, reaction slots). */
int or_mech_load(const char* path, or_mech* m) {
  memset(m, 0, sizeof(*m));
  FILE* f = fopen(path, "r");
  if (!f) return 1;
  char tag[64];
  int ver, rc = 1;
  if (fscanf(f, "%63s %d", tag, &ver) != 2 || strcmp(tag, "EDYNMECH") || ver != 1) goto done;
  if (fscanf(f, "%63s %d", tag, &m->nelem) != 2 || strcmp(tag, "ELEMENTS") || m->nelem > 8) goto done;
  for (int e = 0; e < m->nelem; ++e)
    if (fscanf(f, "%3s %lf", m->ename[e], &m->awt[e]) != 2) goto done;
  if (fscanf(f, "%63s %d", tag, &m->kk) != 2 || strcmp(tag, "SPECIES") || m->kk > OR_MAXSP) goto done;
  for (int k = 0; k < m->kk; ++k) {
    if (fscanf(f, "%23s %lf %lf %lf %lf", m->kname[k], &m->wt[k], &m->tt[k][0], &m->tt[k][1], &m->tt[k][2]) != 5)
      goto done;
    for (int r = 0; r < 2; ++r)
      for (int j = 0; j < 7; ++j)
        if (fscanf(f, "%lf", &m->aa[k][r][j]) != 1) goto done;
    for (int e = 0; e < m->nelem; ++e)
      if (fscanf(f, "%d", &m->ncf[k][e]) != 1) goto done;
  }
  if (fscanf(f, "%63s %d", tag, &m->ii) != 2 || strcmp(tag, "REACTIONS") || m->ii > OR_MAXRX) goto done;
  for (int i = 0; i < m->ii; ++i) {
    char eq[128];
    int rev, dup;
    if (fscanf(f, "%127s %d", eq, &rev) != 2) goto done;
    m->nspec_sign[i] = rev ? 1 : -1;
    for (int q = 0; q < 6; ++q)
      if (fscanf(f, "%d %d", &m->nunk[i][q], &m->nu[i][q]) != 2) goto done;
    if (fscanf(f, "%lf %lf %lf %d %d %d", &m->par[i][0], &m->par[i][1], &m->par[i][2], &m->tb[i], &m->kfal[i],
               &m->ifop[i]) != 6)
      goto done;
    for (int q = 0; q < 7; ++q)
      if (fscanf(f, "%lf", &m->fpar[i][q]) != 1) goto done;
    if (fscanf(f, "%d %d", &dup, &m->ntbs[i]) != 2 || m->ntbs[i] > 16) goto done;
    for (int q = 0; q < m->ntbs[i]; ++q)
      if (fscanf(f, "%d %lf", &m->nktb[i][q], &m->aik[i][q]) != 2) goto done;
  }
  if (fscanf(f, "%63s", tag) != 1 || strcmp(tag, "END")) goto done;
  /* CKINIT constants (GRI/cklib.f:4040) */
  m->ru = 8.314510e7;
  m->patm = 1.01325e6;
  or_ckhms(m, 298.15, m->hf298);
  rc = 0;
done:
  fclose(f);
  return rc;
}

static inline int range_of(const or_mech* m, int k, double t) {
  /* L = 1, incremented when T > T_mid (GRI/cklib.f:7547-7550) */
  return (t > m->tt[k][1]) ? 1 : 0;
}

/* CKYTX, GRI/cklib.f:9587 */
void or_ckytx(const or_mech* m, const double* y, double* x) {
  double sumyow = 0.0;
  for (int k = 0; k < m->kk; ++k) sumyow = sumyow + y[k] / m->wt[k];
  for (int k = 0; k < m->kk; ++k) x[k] = y[k] / (sumyow * m->wt[k]);
}

/* CKXTY, GRI/cklib.f:9421 */
void or_ckxty(const or_mech* m, const double* x, double* y) {
  double sum = 0.0;
  for (int k = 0; k < m->kk; ++k) sum = sum + x[k] * m->wt[k];
  for (int k = 0; k < m->kk; ++k) y[k] = x[k] * m->wt[k] / sum;
}

/* CKPX, GRI/cklib.f:5708 */
void or_ckpx(const or_mech* m, double rho, double t, const double* x, double* p) {
  double sum = 0.0;
  for (int k = 0; k < m->kk; ++k) sum = sum + x[k] * m->wt[k];
  *p = rho * m->ru * t / sum;
}

/* CKRHOX, GRI/cklib.f:7153 */
void or_ckrhox(const or_mech* m, double p, double t, const double* x, double* rho) {
  double sum = 0.0;
  for (int k = 0; k < m->kk; ++k) sum = sum + x[k] * m->wt[k];
  *rho = sum * p / (m->ru * t);
}

/* CKHML, GRI/cklib.f:3500 */
void or_ckhml(const or_mech* m, double t, double* hml) {
  double rut = t * m->ru, tn[5];
  tn[0] = 1.0;
  for (int n = 2; n <= 5; ++n) tn[n - 1] = powi(t, n - 1) / n;
  for (int k = 0; k < m->kk; ++k) {
    const double* a = m->aa[k][range_of(m, k, t)];
    double sum = 0.0;
    for (int n = 0; n < 5; ++n) sum = sum + tn[n] * a[n];
    hml[k] = rut * (sum + a[5] / t);
  }
}

/* CKHMS, GRI/cklib.f:3562 */
void or_ckhms(const or_mech* m, double t, double* hms) {
  double rut = t * m->ru, tn[5];
  tn[0] = 1.0;
  for (int n = 2; n <= 5; ++n) tn[n - 1] = powi(t, n - 1) / n;
  for (int k = 0; k < m->kk; ++k) {
    const double* a = m->aa[k][range_of(m, k, t)];
    double sum = 0.0;
    for (int n = 0; n < 5; ++n) sum = sum + tn[n] * a[n];
    hms[k] = rut * (sum + a[5] / t) / m->wt[k];
  }
}

/* CKUML, GRI/cklib.f:8409 */
void or_ckuml(const or_mech* m, double t, double* uml) {
  or_ckhml(m, t, uml);
  double rut = t * m->ru;
  for (int k = 0; k < m->kk; ++k) uml[k] = uml[k] - rut;
}

/* CKCPML, GRI/cklib.f:1811 */
void or_ckcpml(const or_mech* m, double t, double* cpml) {
  double tn[5];
  tn[0] = 1.0;
  for (int n = 2; n <= 5; ++n) tn[n - 1] = powi(t, n - 1);
  for (int k = 0; k < m->kk; ++k) {
    const double* a = m->aa[k][range_of(m, k, t)];
    cpml[k] = 0.0;
    for (int n = 0; n < 5; ++n) cpml[k] = cpml[k] + m->ru * tn[n] * a[n];
  }
}

/* CKCVML, GRI/cklib.f:2616 */
void or_ckcvml(const or_mech* m, double t, double* cvml) {
  or_ckcpml(m, t, cvml);
  for (int k = 0; k < m->kk; ++k) cvml[k] = cvml[k] - m->ru;
}

/* CKUBML, GRI/cklib.f:8305 */
void or_ckubml(const or_mech* m, double t, const double* x, double* ubml) {
  double u[OR_MAXSP];
  or_ckuml(m, t, u);
  double s = 0.0;
  for (int k = 0; k < m->kk; ++k) s = s + x[k] * u[k];
  *ubml = s;
}

/* CKCVBL, GRI/cklib.f:2512 */
void or_ckcvbl(const or_mech* m, double t, const double* x, double* cvbml) {
  double c[OR_MAXSP];
  or_ckcvml(m, t, c);
  double s = 0.0;
  for (int k = 0; k < m->kk; ++k) s = s + x[k] * c[k];
  *cvbml = s;
}

/* CKCPBL, GRI/cklib.f:1705 */
void or_ckcpbl(const or_mech* m, double t, const double* x, double* cpbml) {
  double c[OR_MAXSP];
  or_ckcpml(m, t, c);
  double s = 0.0;
  for (int k = 0; k < m->kk; ++k) s = s + x[k] * c[k];
  *cpbml = s;
}

/* CKSMH, GRI/cklib.f:7501 */
void or_cksmh(const or_mech* m, double t, double* smh) {
  double tn[5];
  tn[0] = log(t) - 1.0;
  for (int n = 2; n <= 5; ++n) tn[n - 1] = powi(t, n - 1) / ((n - 1) * n);
  for (int k = 0; k < m->kk; ++k) {
    const double* a = m->aa[k][range_of(m, k, t)];
    double sum = 0.0;
    for (int n = 0; n < 5; ++n) sum = sum + tn[n] * a[n];
    smh[k] = sum + a[6] - a[5] / t;
  }
}

/* CKRATT + CKYTCR + CKRATX (GRI/cklib.f:6630, 9533, 6820): forward and
 * reverse rates of progress [mol/cm^3/s] at (rho [g/cm^3], T, Y). */
void or_ckrop_k(const or_mech* m, double rho, double t, const double* y, double* rkf, double* rkr, double* kf_eff,
                double* kr_eff) {
  const int ii = m->ii, kk = m->kk;
  double rkft[OR_MAXRX], rkrt[OR_MAXRX], eqk[OR_MAXRX], ctb[OR_MAXRX];
  double smh[OR_MAXSP], c[OR_MAXSP];
  const double exparg = log(CK_BIG);
  /* CKRATT */
  double alogt = log(t);
  for (int i = 0; i < ii; ++i) rkft[i] = m->par[i][0] * exp(m->par[i][1] * alogt - m->par[i][2] / t);
  or_cksmh(m, t, smh);
  for (int i = 0; i < ii; ++i) {
    double sumsmh = 0.0;
    for (int n = 0; n < 6; ++n)
      if (m->nunk[i][n] >= 0) sumsmh = sumsmh + (double)m->nu[i][n] * smh[m->nunk[i][n]];
    /* The reference leaves EQK untouched when the sum is exactly zero; the
     * work array it then reads holds a previous value. exp(0) = 1 is used. */
    eqk[i] = (sumsmh != 0.0) ? exp(fmin(sumsmh, exparg)) : 1.0;
  }
  double pfac = m->patm / (m->ru * t);
  for (int i = 0; i < ii; ++i) {
    int nusumk = m->nu[i][0] + m->nu[i][1] + m->nu[i][2] + m->nu[i][3] + m->nu[i][4] + m->nu[i][5];
    eqk[i] = eqk[i] * powi(pfac, nusumk);
  }
  for (int i = 0; i < ii; ++i) {
    rkrt[i] = 0.0;
    if (m->nspec_sign[i] > 0) rkrt[i] = rkft[i] / fmax(eqk[i], CK_SMALL);
  }
  /* CKYTCR */
  for (int k = 0; k < kk; ++k) c[k] = rho * y[k] / m->wt[k];
  /* CKRATX */
  for (int i = 0; i < ii; ++i) {
    ctb[i] = 1.0;
    rkf[i] = 0.0;
    rkr[i] = 0.0;
  }
  double ctot = 0.0;
  for (int k = 0; k < kk; ++k) ctot = ctot + c[k];
  for (int i = 0; i < ii; ++i) {
    int is_tb = (m->tb[i] == 1) || (m->tb[i] == 2 && m->kfal[i] < 0);
    if (!is_tb) continue;
    ctb[i] = ctot;
    for (int l = 0; l < m->ntbs[i]; ++l) ctb[i] = ctb[i] + (m->aik[i][l] - 1.0) * c[m->nktb[i][l]];
  }
  for (int i = 0; i < ii; ++i) {
    if (m->tb[i] != 2) continue;
    const double* fp = m->fpar[i];
    double rklow = fp[0] * exp(fp[1] * alogt - fp[2] / t);
    double pr;
    if (m->kfal[i] < 0) {
      pr = rklow * ctb[i] / rkft[i];
      ctb[i] = 1.0;
    } else {
      pr = rklow * c[m->kfal[i]] / rkft[i];
    }
    double pcor = pr / (1.0 + pr);
    if (m->ifop[i] > 1) {
      double prlog = log10(fmax(pr, CK_SMALL));
      double fc;
      /* (SRI, IFOP = 2, is rejected by the mechanism reader) */
      double fcent = (1.0 - fp[3]) * exp(-t / fp[4]) + fp[3] * exp(-t / fp[5]);
      if (m->ifop[i] == 4) fcent = fcent + exp(-fp[6] / t);
      double fclog = log10(fmax(fcent, CK_SMALL));
      /* single-precision literals of the reference, widened */
      double xn = 0.75 - (double)1.27f * fclog;
      double cprlog = prlog - ((double)0.4f + (double)0.67f * fclog);
      double q = cprlog / (xn - (double)0.14f * cprlog);
      double flog = fclog / (1.0 + q * q);
      fc = pow(10.0, flog);
      pcor = fc * pcor;
    }
    rkft[i] = rkft[i] * pcor;
    rkrt[i] = rkrt[i] * pcor;
  }
  for (int i = 0; i < ii; ++i) {
    rkft[i] = rkft[i] * ctb[i] * 1.0;
    rkrt[i] = rkrt[i] * ctb[i] * 1.0;
    if (kf_eff) kf_eff[i] = rkft[i];
    if (kr_eff) kr_eff[i] = rkrt[i];
    if (m->nu[i][0] != 0) {
      rkf[i] = rkft[i] * powi(c[m->nunk[i][0]], abs(m->nu[i][0]));
      rkr[i] = rkrt[i] * powi(c[m->nunk[i][3]], m->nu[i][3]);
      if (m->nunk[i][1] >= 0) {
        rkf[i] = rkf[i] * powi(c[m->nunk[i][1]], abs(m->nu[i][1]));
        if (m->nunk[i][2] >= 0) rkf[i] = rkf[i] * powi(c[m->nunk[i][2]], abs(m->nu[i][2]));
      }
      if (m->nunk[i][4] >= 0) {
        rkr[i] = rkr[i] * powi(c[m->nunk[i][4]], m->nu[i][4]);
        if (m->nunk[i][5] >= 0) rkr[i] = rkr[i] * powi(c[m->nunk[i][5]], m->nu[i][5]);
      }
    }
  }
}

void or_ckrop(const or_mech* m, double rho, double t, const double* y, double* rkf, double* rkr) {
  or_ckrop_k(m, rho, t, y, rkf, rkr, NULL, NULL);
}

/* CKWYR, GRI/cklib.f:9107: molar production rates [mol/cm^3/s]. */
void or_ckwyr(const or_mech* m, double rho, double t, const double* y, double* wdot) {
  double rkf[OR_MAXRX], rkr[OR_MAXRX];
  or_ckrop(m, rho, t, y, rkf, rkr);
  for (int k = 0; k < m->kk; ++k) wdot[k] = 0.0;
  for (int n = 0; n < 6; ++n)
    for (int i = 0; i < m->ii; ++i) {
      int k = m->nunk[i][n];
      if (k >= 0) {
        double rop = rkf[i] - rkr[i];
        wdot[k] = wdot[k] + rop * (double)m->nu[i][n];
      }
    }
}

/* CKCDYR, GRI/cklib.f:1422: creation and destruction rates. */
void or_ckcdyr(const or_mech* m, double rho, double t, const double* y, double* cdot, double* ddot) {
  double rkf[OR_MAXRX], rkr[OR_MAXRX];
  or_ckrop(m, rho, t, y, rkf, rkr);
  for (int k = 0; k < m->kk; ++k) {
    cdot[k] = 0.0;
    ddot[k] = 0.0;
  }
  for (int i = 0; i < m->ii; ++i)
    for (int n = 0; n < 3; ++n) {
      int nkr = m->nunk[i][n], nkp = m->nunk[i][n + 3];
      if (nkr >= 0) {
        int nur = abs(m->nu[i][n]);
        cdot[nkr] = cdot[nkr] + rkr[i] * nur;
        ddot[nkr] = ddot[nkr] + rkf[i] * nur;
      }
      if (nkp >= 0) {
        int nup = m->nu[i][n + 3];
        cdot[nkp] = cdot[nkp] + rkf[i] * nup;
        ddot[nkp] = ddot[nkp] + rkr[i] * nup;
      }
    }
}

/* ---- SRC/thermo.f90 ---- */

/* adjust_sum, SRC/thermo.f90:136-149 */
void or_adjust_sum(int n, double* v) {
  double s = 0.0;
  for (int i = 0; i < n; ++i) {
    v[i] = fmax(v[i], 0.0);
    s = s + v[i];
  }
  for (int i = 0; i < n; ++i) v[i] = v[i] / s;
}

static double wtm_of(const or_mech* m, const double* x) {
  double w = 0.0;
  for (int i = 0; i < m->kk; ++i) w = w + x[i] * m->wt[i];
  return w;
}

/* pressure, SRC/thermo.f90:166-179 */
double or_pressure(const or_mech* m, double rho, double t, const double* x) {
  double p_cgs;
  or_ckpx(m, rho * 1e-3, t, x, &p_cgs);
  return p_cgs * 0.1;
}

/* density, SRC/thermo.f90:151-164 */
double or_density(const or_mech* m, double p, double t, const double* x) {
  double rho_cgs;
  or_ckrhox(m, p * 10.0, t, x, &rho_cgs);
  return rho_cgs * 1e3;
}

/* temperature_con, SRC/thermo.f90:211-257: Newton on u(T) from 1000 K. */
double or_temperature_con(const or_mech* m, double e, const double* x, int* iters) {
  const double thre_redi = 1e-9, thre_erro = 1e-6, tmin = 20.0, tmax = 6000.0;
  double wtm = wtm_of(m, x);
  double spe = e * 1e4 * wtm;
  double temp = 1000.0, func = 1e30, dtemp = 1e30;
  int it = 0;
  while (fabs(func) >= fabs(spe) * thre_redi && fabs(dtemp) >= temp * thre_erro && it < 10) {
    double ubml, cvbml;
    or_ckubml(m, temp, x, &ubml);
    or_ckcvbl(m, temp, x, &cvbml);
    func = ubml - spe;
    dtemp = -func / cvbml;
    temp = temp + dtemp;
    temp = fmax(tmin, fmin(tmax, temp));
    it = it + 1;
  }
  if (iters) *iters = it;
  return temp;
}

/* Cv, SRC/thermo.f90:304-322 */
double or_cv(const or_mech* m, double t, const double* x) {
  double wtm = wtm_of(m, x), c;
  or_ckcvbl(m, t, x, &c);
  return c * 1e-4 / wtm;
}

/* Cp, SRC/thermo.f90:324-342 */
double or_cp(const or_mech* m, double t, const double* x) {
  double wtm = wtm_of(m, x), c;
  or_ckcpbl(m, t, x, &c);
  return c * 1e-4 / wtm;
}

/* specific_energy, SRC/thermo.f90:356-375 */
double or_specific_energy(const or_mech* m, double t, const double* x) {
  double wtm = wtm_of(m, x), u;
  or_ckubml(m, t, x, &u);
  return u * 1e-4 / wtm;
}

/* sonic_speed, SRC/thermo.f90:408-430 */
double or_sonic_speed(const or_mech* m, double rho, double p, double t, const double* x) {
  double g = or_cp(m, t, x) / or_cv(m, t, x);
  return sqrt(g * p / rho);
}

/* ---- SRC/eos.f90 ---- */

/* qfToQc, SRC/eos.f90:11-46 */
void or_qf_to_qc(const or_mech* m, const double* qf, double* qc) {
  const int ns = m->kk;
  double y[OR_MAXSP], x[OR_MAXSP];
  qc[0] = qf[0];
  qc[1] = qf[0] * qf[1];
  for (int k = 0; k < ns; ++k) y[k] = qf[3 + k];
  or_adjust_sum(ns, y);
  for (int k = 0; k < ns; ++k) qc[3 + k] = qf[0] * y[k];
  or_ckytx(m, qf + 3, x);
  or_adjust_sum(ns, x);
  double pres = or_pressure(m, qf[0], qf[2], x);
  (void)pres;
  double e_int = or_specific_energy(m, qf[2], x);
  qc[2] = qf[0] * (e_int + 0.5 * (qf[1] * qf[1]));
}

/* QcToqf, SRC/eos.f90:49-83 */
void or_qc_to_qf(const or_mech* m, const double* qc, double* qf) {
  const int ns = m->kk;
  double x[OR_MAXSP];
  qf[0] = qc[0];
  qf[1] = qc[1] / qc[0];
  for (int k = 0; k < ns; ++k) qf[3 + k] = qc[3 + k] / qc[0];
  or_adjust_sum(ns, qf + 3);
  or_ckytx(m, qf + 3, x);
  or_adjust_sum(ns, x);
  double e_int = qc[2] / qc[0] - 0.5 * (qf[1] * qf[1]);
  qf[2] = or_temperature_con(m, e_int, x, NULL);
}

/* initialize_variables (SRC/params.f90:305-580, step profiles, no spark)
 * followed by set_block_params (SRC/block.f90:394-431) for one cell. The
 * caller passes the mole fractions after the "other species" fill. */
void or_init_cell(const or_mech* m, double T, double p, double u, const double* x_in, double* qf, double* qc) {
  const int ns = m->kk;
  double x[OR_MAXSP], y[OR_MAXSP];
  for (int k = 0; k < ns; ++k) x[k] = x_in[k];
  or_adjust_sum(ns, x);
  or_ckxty(m, x, y);
  double rho = or_density(m, p, T, x);
  double e_int = or_specific_energy(m, T, x);
  double e_kin = 0.5 * (u * u);
  double e_tot = e_int + e_kin;
  qf[0] = rho;
  qf[1] = u;
  qf[2] = T;
  for (int k = 0; k < ns; ++k) qf[3 + k] = y[k];
  qc[0] = rho;
  qc[1] = rho * u;
  qc[2] = rho * e_tot;
  for (int k = 0; k < ns; ++k) qc[3 + k] = rho * y[k];
}
