/*
 * CPU oracle, transport part -- TEST INFRASTRUCTURE ONLY.
 *
 * Restates the mixture-averaged transport rules of TRANLIB (CHEMKIN-II
 * transport library v3.8, the tranlib.f shipped in every mechanism directory
 * of the reference, e.g. WORK/Examples/CH4_GRI3.0/SOD/GRI3.0_CH4/tranlib.f),
 * the SI wrappers of SRC/trans.f90 and the viscous / conductive / diffusive
 * face flux calc_flux_tran of SRC/flux.f90:18-127, in the reference's
 * operation order (compiled with -ffp-contract=off).
 *
 * The reference's viscosity_ea (SRC/trans.f90:137-151) calls MCAVIS_EA, a
 * routine the shipped tranlib.f does not define; this oracle, like the GPU
 * library, uses TRANLIB's MCAVIS (Wilke's rule in Bird's form) in its place.
 *
 * The fits are read from the library's text form of TRANLIB's linking file
 * (tran.edyn), which holds the reference's tran.bin numbers bit for bit.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "edyn_oracle.h"

int or_tran_sizeof(void) { return (int)sizeof(or_tran); }

int or_tran_load(const char* path, or_tran* t) {
  FILE* f = fopen(path, "r");
  if (!f) return 1;
  memset(t, 0, sizeof(*t));
  char w[64];
  int ver = 0, rc = 1;
  if (fscanf(f, "%63s %d", w, &ver) != 2 || strcmp(w, "EDYNTRAN") || ver != 1) goto done;
  if (fscanf(f, " KK %d NO %d NLITE %d PATMOS %lf", &t->kk, &t->no, &t->nlite, &t->patmos) != 4) goto done;
  if (t->kk < 1 || t->kk > OR_MAXSP || t->no != 4) goto done;
  if (fscanf(f, "%63s", w) != 1 || strcmp(w, "SPECIES")) goto done;
  for (int k = 0; k < t->kk; ++k)
    if (fscanf(f, "%63s %lf %lf %lf %lf %lf %lf %d", w, &t->wt[k], &t->eps[k], &t->sig[k], &t->dip[k], &t->pol[k],
               &t->zrot[k], &t->nlin[k]) != 8)
      goto done;
  if (fscanf(f, "%63s", w) != 1 || strcmp(w, "COFETA")) goto done;
  for (int k = 0; k < t->kk; ++k) {
    int kr;
    if (fscanf(f, "%d %lf %lf %lf %lf", &kr, &t->cofeta[k][0], &t->cofeta[k][1], &t->cofeta[k][2],
               &t->cofeta[k][3]) != 5 || kr != k)
      goto done;
  }
  if (fscanf(f, "%63s", w) != 1 || strcmp(w, "COFLAM")) goto done;
  for (int k = 0; k < t->kk; ++k) {
    int kr;
    if (fscanf(f, "%d %lf %lf %lf %lf", &kr, &t->coflam[k][0], &t->coflam[k][1], &t->coflam[k][2],
               &t->coflam[k][3]) != 5 || kr != k)
      goto done;
  }
  if (fscanf(f, "%63s", w) != 1 || strcmp(w, "COFD")) goto done;
  for (int k = 0; k < t->kk; ++k)
    for (int j = 0; j < t->kk; ++j) {
      int kr, jr;
      double* c = t->cofd[k][j];
      if (fscanf(f, "%d %d %lf %lf %lf %lf", &kr, &jr, &c[0], &c[1], &c[2], &c[3]) != 6 || kr != k || jr != j)
        goto done;
    }
  rc = 0;
done:
  fclose(f);
  return rc;
}

/* MCEVAL4, tranlib.f:1348-1394: ((c4 L + c3) L + c2) L + c1 */
static double eval4(const double* c, double tf) { return (((c[3] * tf) + c[2]) * tf + c[1]) * tf + c[0]; }

/* MCSVIS, tranlib.f:623-679: pure-species viscosities [g/(cm s)] */
void or_mcsvis(const or_tran* t, double T, double* vis) {
  double alogt = log(T);
  for (int k = 0; k < t->kk; ++k) vis[k] = exp(eval4(t->cofeta[k], alogt));
}

/* MCSCON, tranlib.f:769-825: pure-species conductivities [erg/(cm K s)] */
void or_mcscon(const or_tran* t, double T, double* con) {
  double alogt = log(T);
  for (int k = 0; k < t->kk; ++k) con[k] = exp(eval4(t->coflam[k], alogt));
}

/* MCSDIF, tranlib.f:898-971: binary diffusion coefficients at pressure p
 * [dyn/cm^2], djk[k * kk + j] [cm^2/s] */
void or_mcsdif(const or_tran* t, double p, double T, double* djk) {
  double pfac = t->patmos / p, alogt = log(T);
  for (int k = 0; k < t->kk; ++k)
    for (int j = 0; j <= k; ++j) {
      double v = exp(eval4(t->cofd[k][j], alogt)) * pfac;
      djk[k * t->kk + j] = v;
      djk[j * t->kk + k] = v;
    }
}

/* MCAVIS, tranlib.f:681-767: Wilke's mixture rule in Bird's form. */
void or_mcavis(const or_tran* t, double T, const double* x, double* vismix) {
  double vis[OR_MAXSP];
  const double* wt = t->wt;
  or_mcsvis(t, T, vis);
  double sumo = 0.0;
  for (int k = 0; k < t->kk; ++k) {
    double sumi = 0.0;
    for (int j = 0; j < t->kk; ++j) {
      double s = 1.0 + sqrt(vis[k] / vis[j] * sqrt(wt[j] / wt[k]));
      sumi = sumi + x[j] * (s * s) / sqrt(1.0 + wt[k] / wt[j]);
    }
    sumo = sumo + x[k] * vis[k] / sumi;
  }
  *vismix = sumo * sqrt(8.0);
}

/* MCACON, tranlib.f:827-896: half the sum of the arithmetic and harmonic means. */
void or_mcacon(const or_tran* t, double T, const double* x, double* conmix) {
  double con[OR_MAXSP];
  or_mcscon(t, T, con);
  double sum = 0.0, sumr = 0.0;
  for (int k = 0; k < t->kk; ++k) {
    sum = sum + x[k] * con[k];
    sumr = sumr + x[k] / con[k];
  }
  *conmix = 0.5 * (sum + 1.0 / sumr);
}

/* MCADIF + MCEDIF, tranlib.f:973-1153: mixture-averaged diffusion
 * coefficients D_k = sum_{j!=k} X_j W_j / (W sum_{j!=k} X_j / D_jk), with
 * the mole fractions floored at SMALL = 1e-50. */
void or_mcadif(const or_tran* t, double p, double T, const double* x, double* d) {
  const int kk = t->kk;
  const double small = 1.0e-50;
  double alogt = log(T);
  double djk[OR_MAXSP * OR_MAXSP];
  double xx[OR_MAXSP];
  for (int k = 0; k < kk; ++k) {
    for (int j = 0; j < k; ++j) {
      double v = exp(-eval4(t->cofd[k][j], alogt));
      djk[k * kk + j] = v;
      djk[j * kk + k] = v;
    }
    djk[k * kk + k] = 0.0;
  }
  double wtm = 0.0;
  for (int k = 0; k < kk; ++k) {
    wtm = wtm + t->wt[k] * x[k];
    xx[k] = x[k] > small ? x[k] : small;
  }
  for (int k = 0; k < kk; ++k) {
    double sumxw = -xx[k] * t->wt[k];
    double sumxod = 0.0;
    for (int j = 0; j < kk; ++j) {
      sumxw = sumxw + xx[j] * t->wt[j];
      sumxod = sumxod + xx[j] * djk[j * kk + k];
    }
    d[k] = sumxw / (wtm * sumxod);
  }
  for (int k = 0; k < kk; ++k) d[k] = d[k] * t->patmos / p;
}

/* SRC/trans.f90 wrappers in SI: viscosity [Pa s] (viscosity_ea 137-151,
 * with MCAVIS), thermal conductivity [W/(m K)] (63-77), mixture-averaged
 * diffusivities [m^2/s] at pressure p [Pa] (set_diffusivity 80-100). */
double or_viscosity(const or_tran* t, double T, const double* x) {
  double v;
  or_mcavis(t, T, x, &v);
  return v * 0.1;
}

double or_thermal_conductivity(const or_tran* t, double T, const double* x) {
  double c;
  or_mcacon(t, T, x, &c);
  return c * 1.0e-5;
}

void or_diffusivity(const or_tran* t, double p, double T, const double* x, double* di) {
  double d_cgs[OR_MAXSP];
  or_mcadif(t, p * 10.0, T, x, d_cgs);
  for (int k = 0; k < t->kk; ++k) di[k] = d_cgs[k] * 1.0e-4;
}

/* Per-cell transport state of calc_flux_tran (SRC/flux.f90:51-90): from
 * the conserved column qc of a cell, its density, velocity, mass fractions
 * (unnormalised, as the reference divides Qc by rho), temperature,
 * viscosity, conductivity and the diffusivities (1 - X_k)/(1 - Y_k) D_k. */
void or_tran_cell(const or_mech* m, const or_tran* t, const double* qc, double* rho, double* u, double* T, double* y,
                  double* mu, double* kap, double* dif) {
  const int ns = m->kk;
  double x[OR_MAXSP], dm[OR_MAXSP];
  *rho = qc[0];
  *u = qc[1] / *rho;
  for (int k = 0; k < ns; ++k) y[k] = qc[3 + k] / *rho;
  or_ckytx(m, y, x);
  double etot = qc[2] / *rho;
  double ekin = 0.5 * (*u * *u);
  double eint = etot - ekin;
  *T = or_temperature_con(m, eint, x, NULL);
  double p = or_pressure(m, *rho, *T, x);
  *mu = or_viscosity(t, *T, x);
  *kap = or_thermal_conductivity(t, *T, x);
  or_diffusivity(t, p, *T, x, dm);
  for (int k = 0; k < ns; ++k) {
    dif[k] = (1.0 - x[k]) / (1.0 - y[k]) * dm[k];
    if (y[k] == 1.0) dif[k] = 0.0;
  }
}

/* The transport flux of one face from the conserved columns of its two
 * cells (SRC/flux.f90:92-122), added to g[0..nequ). */
void or_face_flux_tran(const or_mech* m, const or_tran* t, const double* qcl, const double* qcr, double dx,
                       double* g) {
  const int ns = m->kk;
  double rho_i, rho_ip, u_i, u_ip, T_i, T_ip, mu_i, mu_ip, kap_i, kap_ip;
  double y_i[OR_MAXSP], y_ip[OR_MAXSP], dif_i[OR_MAXSP], dif_ip[OR_MAXSP], hs[OR_MAXSP];
  or_tran_cell(m, t, qcl, &rho_i, &u_i, &T_i, y_i, &mu_i, &kap_i, dif_i);
  or_tran_cell(m, t, qcr, &rho_ip, &u_ip, &T_ip, y_ip, &mu_ip, &kap_ip, dif_ip);
  double rho_ave = 0.5 * (rho_i + rho_ip);
  double u_ave = 0.5 * (u_i + u_ip);
  double T_ave = 0.5 * (T_i + T_ip);
  double mu_ave = 0.5 * (mu_i + mu_ip);
  double kap_ave = 0.5 * (kap_i + kap_ip);
  double tau_xx = -(2.0 / 3.0 * mu_ave * (2.0 * ((u_ip - u_i) / dx)));
  or_ckhms(m, T_ave, hs);
  for (int k = 0; k < ns; ++k) hs[k] = hs[k] * 1.0e-4;
  double hsum = 0.0;
  for (int k = 0; k < ns; ++k) {
    double dif_ave = 0.5 * (dif_i[k] + dif_ip[k]);
    hsum = hsum - hs[k] * dif_ave * ((y_ip[k] - y_i[k]) / dx);
  }
  g[0] = g[0] + 0.0;
  g[1] = g[1] + tau_xx;
  g[2] = g[2] + tau_xx * u_ave + rho_ave * hsum - kap_ave * ((T_ip - T_i) / dx);
  for (int k = 0; k < ns; ++k) {
    double dif_ave = 0.5 * (dif_i[k] + dif_ip[k]);
    g[3 + k] = g[3 + k] - rho_ave * dif_ave * ((y_ip[k] - y_i[k]) / dx);
  }
}
