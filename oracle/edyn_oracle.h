/*
 * CPU oracle for the EdynCFD per-cell hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * This is a plain-C FP64 restatement of the reference's CPU algorithm
 * (Keisuke043/fortranCFD, the SRC directory, plus the CHEMKIN-II v4.5 routines it
 * calls, GRI/cklib.f). It exists to check the GPU library and to serve as
 * the timed CPU baseline; nothing in the product links, imports or calls it.
 * Every function follows the reference's operation order (compile with
 * -ffp-contract=off) and cites the file:line it restates.
 *
 * Parity status: the reference cannot be compiled in this environment (no
 * Fortran compiler, MPI or HDF5, and its chemistry integrator odes.f90 is not
 * shipped), so the fluid path is "parity unpinned" against a reference run.
 * The thermodynamics and equilibrium constants are pinned against the
 * Cantera TP-equilibrium composition shipped with the reference
 * (WORK/Examples/CH4_GRI3.0/MFR/equilTP_phi1.0_p1.0_T1300.0.txt); the stiff
 * integrator is the project's own FP64 method (the reference's MACKS solver
 * is absent), checked by self-convergence and conservation.
 *
 * Layouts follow the reference: per-cell vectors are AoS, qf(nequ) =
 * (rho, u, T, Y_1..Y_nspe) and Qc(nequ) = (rho, rho*u, rho*e, rho*Y_k),
 * SI units outside the CHEMKIN routines and cgs inside.
 */
#ifndef EDYN_ORACLE_H
#define EDYN_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define OR_MAXSP 64
#define OR_MAXRX 512

typedef struct or_mech {
  int nelem, kk, ii;
  char ename[8][4];
  double awt[8];
  char kname[OR_MAXSP][24];
  double wt[OR_MAXSP];
  double tt[OR_MAXSP][3];         /* T low, T mid, T high */
  double aa[OR_MAXSP][2][7];      /* [k][range 0 low, 1 high][coef] */
  int ncf[OR_MAXSP][8];
  int nspec_sign[OR_MAXRX];       /* +1 reversible, -1 irreversible */
  int nu[OR_MAXRX][6], nunk[OR_MAXRX][6];
  double par[OR_MAXRX][3];        /* A, beta, E/R */
  int tb[OR_MAXRX], kfal[OR_MAXRX], ifop[OR_MAXRX];
  double fpar[OR_MAXRX][7];       /* low A, beta, E/R, troe a, T***, T*, T** */
  int ntbs[OR_MAXRX], nktb[OR_MAXRX][16];
  double aik[OR_MAXRX][16];
  double ru, patm;
  double hf298[OR_MAXSP];         /* CKHMS(298.15) [erg/g] */
} or_mech;

/* Mechanism */
int or_mech_load(const char* path, or_mech* m);
int or_mech_sizeof(void);

/* CHEMKIN-II restatements (cgs) */
void or_ckytx(const or_mech* m, const double* y, double* x);
void or_ckxty(const or_mech* m, const double* x, double* y);
void or_ckpx(const or_mech* m, double rho, double t, const double* x, double* p);
void or_ckrhox(const or_mech* m, double p, double t, const double* x, double* rho);
void or_ckhml(const or_mech* m, double t, double* hml);
void or_ckuml(const or_mech* m, double t, double* uml);
void or_ckcpml(const or_mech* m, double t, double* cpml);
void or_ckcvml(const or_mech* m, double t, double* cvml);
void or_ckubml(const or_mech* m, double t, const double* x, double* ubml);
void or_ckcvbl(const or_mech* m, double t, const double* x, double* cvbml);
void or_ckcpbl(const or_mech* m, double t, const double* x, double* cpbml);
void or_cksmh(const or_mech* m, double t, double* smh);
void or_ckhms(const or_mech* m, double t, double* hms);
void or_ckwyr(const or_mech* m, double rho, double t, const double* y, double* wdot);
void or_ckrop(const or_mech* m, double rho, double t, const double* y, double* qf, double* qr);
/* same, plus the effective rate constants (rate of progress per unit concentration product) */
void or_ckrop_k(const or_mech* m, double rho, double t, const double* y, double* qf, double* qr, double* kf_eff,
                double* kr_eff);
void or_ckcdyr(const or_mech* m, double rho, double t, const double* y, double* cdot, double* ddot);

/* SRC/thermo.f90 restatements (SI) */
void or_adjust_sum(int n, double* v);
double or_pressure(const or_mech* m, double rho, double t, const double* x);
double or_density(const or_mech* m, double p, double t, const double* x);
double or_temperature_con(const or_mech* m, double e, const double* x, int* iters);
double or_cv(const or_mech* m, double t, const double* x);
double or_cp(const or_mech* m, double t, const double* x);
double or_specific_energy(const or_mech* m, double t, const double* x);
double or_sonic_speed(const or_mech* m, double rho, double p, double t, const double* x);

/* SRC/eos.f90 */
void or_qf_to_qc(const or_mech* m, const double* qf, double* qc);
void or_qc_to_qf(const or_mech* m, const double* qc, double* qf);

/* SRC/muscl.f90, SRC/weno.f90 */
void or_muscl3(const double* s, double* sl, double* sr, int flag_muscl);
void or_weno3z(const double* s, double* sl, double* sr);
void or_weno5(const double* s, double* sl, double* sr, int flag_weno);
void or_weno7z(const double* s, double* sl, double* sr);

/* TRANLIB fits (the linking file's tables, cgs) and mixture rules. */
typedef struct or_tran {
  int kk, no, nlite;
  double patmos;
  double wt[OR_MAXSP], eps[OR_MAXSP], sig[OR_MAXSP], dip[OR_MAXSP], pol[OR_MAXSP], zrot[OR_MAXSP];
  int nlin[OR_MAXSP];
  double cofeta[OR_MAXSP][4], coflam[OR_MAXSP][4];
  double cofd[OR_MAXSP][OR_MAXSP][4]; /* [k][j][n]: ln D_jk at patmos */
} or_tran;

int or_tran_load(const char* path, or_tran* t);
int or_tran_sizeof(void);
void or_mcsvis(const or_tran* t, double T, double* vis);
void or_mcscon(const or_tran* t, double T, double* con);
void or_mcsdif(const or_tran* t, double p, double T, double* djk);
void or_mcavis(const or_tran* t, double T, const double* x, double* vismix);
void or_mcacon(const or_tran* t, double T, const double* x, double* conmix);
void or_mcadif(const or_tran* t, double p, double T, const double* x, double* d);
double or_viscosity(const or_tran* t, double T, const double* x);
double or_thermal_conductivity(const or_tran* t, double T, const double* x);
void or_diffusivity(const or_tran* t, double p, double T, const double* x, double* di);
void or_tran_cell(const or_mech* m, const or_tran* t, const double* qc, double* rho, double* u, double* T, double* y,
                  double* mu, double* kap, double* dif);
void or_face_flux_tran(const or_mech* m, const or_tran* t, const double* qcl, const double* qcr, double dx,
                       double* g);

/* Energy sources of solve_source after the chemistry (SRC/update.f90:126-147). */
typedef struct or_sources {
  int nrad;                  /* radiation_heat_loss, SRC/radiation.f90:74-121 */
  int rad_sp[16];
  double rad_coef[16][6];
  int wall;                  /* heat_transfer + Tw, SRC/mfr.f90:41-78 */
  double nu, d_m, tw_min, tw_max, alpha, beta;
  const or_tran* tran;       /* conductivity (MCACON) of the wall heat */
  int ig_type, n_ig;         /* add_igsource(_WZhang), SRC/ignitionsource.f90:150-262 */
  double ig_e[8], ig_r[8], ig_t[8], ig_t0[8];
} or_sources;

/* 1-D tube state with ghost cells (equal-dx blocks collapse to one array). */
typedef struct or_tube {
  const or_mech* m;
  int n, lvir, nequ, nspe;
  int select_time, select_riemann, flag_acu, flag_muscl, flag_weno;
  int flag_lbound, flag_rbound, do_reaction;
  double dx;
  double p_out, t_in, rho_u_in;
  double x_in[OR_MAXSP], y_in[OR_MAXSP];
  double rtol, atol;
  double* qf;   /* (n + 2*lvir) * nequ, cell i at offset (i + lvir) * nequ */
  double* qc;
  double* q0;   /* n * nequ */
  double* fplus;/* (n + 1) * nequ, face i-1/2 of cell i at offset i * nequ */
  double* hrr;  /* n */
  double* hrr_dot;
  double* qrad; /* n: the last radiation loss (eos_obj%Qrad) */
  double* qtw;  /* n: the last wall heat (eos_obj%qTw) */
  long chem_rhs_evals, chem_steps;
  const or_tran* tran; /* do_tran: transport fits (NULL: inviscid) */
  or_sources src;      /* energy sources (all off when zeroed) */
  double time;         /* the time loop's clock: advanced by or_step before the step */
  int is_spherical;    /* spherical geometry, r = (i + 1/2) dx */
  double* pgod;        /* (n + 1): Roe-averaged face pressures (godunov_state) */
  int smr_left, smr_right; /* SMR: this side faces another block (ghosts by interpolation) */
  double x0;           /* coordinate of the tube's left edge: cell i's centre is x0 + (i + 1/2) dx */
} or_tube;

or_tube* or_tube_create(const or_mech* m, int n, int lvir, const int* iflags, const double* rparams,
                        const double* x_in);
void or_tube_destroy(or_tube* t);
void or_tube_set_interior(or_tube* t, const double* qf, const double* qc);
void or_tube_get_interior(const or_tube* t, double* qf, double* qc);
void or_tube_get_all(const or_tube* t, double* qf, double* qc);
/* HRR and HRR_dot of the last source step (eos_obj%HRR, %HRR_dot), n values each. */
void or_tube_get_source(const or_tube* t, double* hrr, double* hrr_dot);
/* The output rows of write_hdf5_b (SRC/write_hdf5.f90:140-162) from
 * set_eos_params (SRC/block.f90:434-470): (15 + nspe) rows of n values --
 * rho, u, T, p, et, ek, ei, HRR, HRR_dot, Qrad, Tw, qTw, x_m, dx, idx, X_k. */
#define OR_OUT_FIXED 15
void or_output_rows(const or_tube* t, double* rows);
void or_update_boundary(or_tube* t);
void or_ghost_qf(or_tube* t);
double or_calc_dt(or_tube* t, double cfl);
void or_calc_flux_advection(or_tube* t);
/* do_tran = 1 with the given fits (NULL switches transport off). */
void or_tube_set_transport(or_tube* t, const or_tran* tr);
/* calc_flux_tran, SRC/flux.f90:18-127: adds the transport flux of every face to fplus. */
void or_calc_flux_tran(or_tube* t);
void or_tube_set_sources(or_tube* t, const or_sources* s);
void or_tube_set_time(or_tube* t, double time);
void or_tube_set_spherical(or_tube* t, int on);
int or_sources_sizeof(void);
void or_solve_fluid(or_tube* t, double dt);
void or_solve_source(or_tube* t, double dt);
void or_post_step(or_tube* t);
double or_step(or_tube* t, double cfl);

/* SMR blocks (SRC/block.f90:91-379, 475-569): segments of equal-dx blocks,
 * left to right, one dt from dx_comp = rparams[0]; Euler or TVDRK3. */
#define OR_MAXSEG 64
typedef struct or_smr or_smr;
or_smr* or_smr_create(const or_mech* m, int nseg, const int* ncell, const double* dx, int lvir, const int* iflags,
                      const double* rparams, const double* x_in);
void or_smr_destroy(or_smr* s);
void or_smr_set_interior(or_smr* s, const double* qf, const double* qc);
void or_smr_get_interior(const or_smr* s, double* qf, double* qc);
double or_smr_step(or_smr* s, double cfl);
void or_smr_segment_all(const or_smr* s, int g, double* qc);
void or_smr_set_transport(or_smr* s, const or_tran* tr);
/* is_spherical and the energy sources on every segment (r and x are each
 * cell's centre x_m, SRC/block.f90:262-304). */
void or_smr_set_spherical(or_smr* s, int on);
void or_smr_set_sources(or_smr* s, const or_sources* src);
void or_smr_set_time(or_smr* s, double time);
/* Segment g's output rows (or_output_rows, with its x_m). */
void or_smr_output_rows(const or_smr* s, int g, double* rows);

/* Initial conditions (SRC/params.f90:305-580 + SRC/block.f90:394-431). */
void or_init_cell(const or_mech* m, double T, double p, double u, const double* x_in, double* qf, double* qc);

/* Chemistry: project FP64 SDIRK4 reference integrator on [Y_1..Y_kk, T]. */
typedef struct or_chem_stats { long steps, rejects, rhs, jac, newton_fail; } or_chem_stats;
int or_reactor(const or_mech* m, double rho_si, double dt, double* yiT, double rtol, double atol,
               or_chem_stats* st);
void or_chem_rhs(const or_mech* m, double rho_cgs, const double* yT, double* f);
int or_reactor_batch(const or_mech* m, int n, const double* rho_si, const double* dt, double* yiT, double rtol,
                     double atol, int nthreads, long* rhs_total);

int or_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif
