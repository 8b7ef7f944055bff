// Mechanism tables shared by the host parser and the device kernels.
//
// The layout restates the data model of CHEMKIN-II's linking file (the
// integer/real work arrays that CKINIT loads, GRI/cklib.f:3972-4300) as a
// plain C struct: NASA-7 two-range polynomials per species, and per reaction
// the six stoichiometric slots (three reactants, three products), Arrhenius
// parameters with the activation energy already divided by R, third-body
// efficiencies and Lindemann/Troe fall-off data.
#pragma once

#ifdef __cplusplus
extern "C" {
#endif

#define EDYN_MAX_SPECIES 64
#define EDYN_MAX_REACTIONS 512
#define EDYN_MAX_ELEMENTS 8
#define EDYN_MAX_EFF 16
#define EDYN_NAME_LEN 24

// Third-body kinds per reaction.
#define EDYN_TB_NONE 0
#define EDYN_TB_M 1        // "+M" with mixture efficiencies
#define EDYN_TB_FALLOFF 2  // "(+M)" or "(+SPECIES)" pressure dependent

// Fall-off functional form (CHEMKIN's IFOP).
#define EDYN_FO_NONE 0
#define EDYN_FO_LINDEMANN 1
#define EDYN_FO_SRI 2
#define EDYN_FO_TROE3 3
#define EDYN_FO_TROE4 4

typedef struct edyn_mech {
  int nelem, nspec, nreac;
  char elem_name[EDYN_MAX_ELEMENTS][4];
  double elem_weight[EDYN_MAX_ELEMENTS];

  char spec_name[EDYN_MAX_SPECIES][EDYN_NAME_LEN];
  double W[EDYN_MAX_SPECIES];                 // g/mol
  double T_lo[EDYN_MAX_SPECIES], T_mid[EDYN_MAX_SPECIES], T_hi[EDYN_MAX_SPECIES];
  double a[EDYN_MAX_SPECIES][2][7];           // [k][0 = low range, 1 = high range][a1..a7]
  int elem_count[EDYN_MAX_SPECIES][EDYN_MAX_ELEMENTS];

  char equation[EDYN_MAX_REACTIONS][64];
  int rev[EDYN_MAX_REACTIONS];                // 1 reversible, 0 irreversible ("=>")
  int nu[EDYN_MAX_REACTIONS][6];              // slots 0-2 reactants (<0), 3-5 products (>0)
  int nunk[EDYN_MAX_REACTIONS][6];            // species index per slot, -1 when empty
  double A[EDYN_MAX_REACTIONS];               // mol-cm-s units
  double beta[EDYN_MAX_REACTIONS];
  double E_R[EDYN_MAX_REACTIONS];             // activation temperature [K]
  int tb[EDYN_MAX_REACTIONS];                 // EDYN_TB_*
  int kfal[EDYN_MAX_REACTIONS];               // fall-off collider species, -1 = mixture
  int ifop[EDYN_MAX_REACTIONS];               // EDYN_FO_*
  double low[EDYN_MAX_REACTIONS][3];          // low-pressure A, beta, E/R
  double troe[EDYN_MAX_REACTIONS][4];         // a, T***, T*, T**
  int dup[EDYN_MAX_REACTIONS];
  int neff[EDYN_MAX_REACTIONS];
  int eff_sp[EDYN_MAX_REACTIONS][EDYN_MAX_EFF];
  double eff_val[EDYN_MAX_REACTIONS][EDYN_MAX_EFF];
} edyn_mech;

#ifdef __cplusplus
}
#endif
