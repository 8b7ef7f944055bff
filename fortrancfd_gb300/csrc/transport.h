// Transport fits shared by the host loader and the device kernels.
//
// The layout restates the data model of TRANLIB's linking file (the file
// TRANFIT writes and MCINIT reads, tranlib.f:214-258 in every mechanism
// directory of the reference): per species the molecular weight, the
// Lennard-Jones and polar parameters and the polynomial fits in ln T of
// ln(viscosity) and ln(conductivity); per species pair the fit of
// ln(binary diffusion coefficient at one atmosphere); per light species the
// thermal-diffusion ratio fits. Units are TRANLIB's (cgs).
#pragma once

#include "mechanism.h"

#ifdef __cplusplus
extern "C" {
#endif

#define EDYN_TRAN_NO 4      // fit order (TRANFIT's default, the only one the kernels evaluate)
#define EDYN_TRAN_MAXLITE 8 // light species with thermal-diffusion fits

typedef struct edyn_tran {
  int kk, no, nlite;
  double patmos;                                // dyn/cm^2
  double wt[EDYN_MAX_SPECIES];                  // g/mol
  double eps[EDYN_MAX_SPECIES];                 // epsilon/k_B [K]
  double sig[EDYN_MAX_SPECIES];                 // collision diameter [Angstrom]
  double dip[EDYN_MAX_SPECIES];                 // dipole moment [Debye]
  double pol[EDYN_MAX_SPECIES];                 // polarizability [Angstrom^3]
  double zrot[EDYN_MAX_SPECIES];                // rotational relaxation number at 298 K
  int nlin[EDYN_MAX_SPECIES];                   // 0 atom, 1 linear, 2 nonlinear
  double cofeta[EDYN_MAX_SPECIES][EDYN_TRAN_NO];  // ln eta_k = sum_n cofeta[k][n] (ln T)^n  [g/(cm s)]
  double coflam[EDYN_MAX_SPECIES][EDYN_TRAN_NO];  // ln lambda_k, [erg/(cm K s)]
  // ln D_jk at PATMOS = sum_n cofd[k][j][n] (ln T)^n  [cm^2/s] (TRANLIB's COFD(n, j, k))
  double cofd[EDYN_MAX_SPECIES][EDYN_MAX_SPECIES][EDYN_TRAN_NO];
  int ktdif[EDYN_TRAN_MAXLITE];                 // light species (0-based)
  double coftd[EDYN_TRAN_MAXLITE][EDYN_MAX_SPECIES][EDYN_TRAN_NO];  // thermal-diffusion ratio fits
} edyn_tran;

// Reads a TRANLIB linking file (Fortran unformatted, little-endian record
// markers, double precision, fit order 4) as MCINIT does. 0 on success.
int edyn_tran_read_bin(const char* path, edyn_tran* t, char* err, int errlen);
// Reads / writes the library's text form of the same tables ("tran.edyn").
int edyn_tran_read(const char* path, edyn_tran* t, char* err, int errlen);
int edyn_tran_write(const edyn_tran* t, const edyn_mech* m, const char* path);
// dir/tran.bin (the reference's own file, what set_trans reads) when present,
// else dir/tran.edyn.
int edyn_tran_load_dir(const char* dir, edyn_tran* t, char* err, int errlen);

#ifdef __cplusplus
}
#endif
