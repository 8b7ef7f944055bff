// Device-side thermodynamics shared by the fluid and chemistry kernels.
//
// GB300's FP64 pipe issues about 1.6 DFMA per clock per SM (1.0 TFLOP/s for
// the chip), 65x below FP32, so every routine here is written to minimise
// FP64 instructions; integer and FP32 work is close to free next to it.
//
// Mixture thermodynamics follow CHEMKIN-II's molar forms (CKUBML, CKCVBL,
// CKCPBL, CKPX as used by SRC/thermo.f90) rewritten in mass-weighted sums:
// with z_k = Y_k / W_k, S_z = sum z_k and S_Y = sum Y_k,
//   mean molar weight   = S_Y / S_z                     (CKPX, CKRHOX)
//   sum X_k u_k(T) / R  = (H(T) - T S_z) / S_z          (CKUBML)
//   sum X_k cv_k / R    = (Cp(T) - S_z) / S_z           (CKCVBL)
// where H(T) = sum z_k h_k(T)/R and Cp(T) = sum z_k cp_k(T)/R are evaluated
// from six "premixed" NASA-7 coefficients A_n = sum_k z_k a_{k,n} of the
// temperature interval that holds T (the range test T > T_mid per species is
// the one of GRI/cklib.f:7547-7550). One premix costs six FMAs per species;
// afterwards each h, u, cv, cp evaluation is a 5-term Horner polynomial.
#pragma once

#include <cstring>

#include <cstdint>

#include "mechanism.h"

#ifndef EDYN_NS_MAX
#define EDYN_NS_MAX 64
#endif

// Status bits a kernel ORs into its context's error word (the values of
// EDYN_E_NEWTON, EDYN_E_CHEM and EDYN_E_STATE of include/edyn_gpu.h).
#define EDYN_STATUS_NEWTON 8u
#define EDYN_STATUS_CHEM 16u
#define EDYN_STATUS_STATE 32u

namespace edyn {

// SI gas constant used by SRC/thermo.f90 (CHEMKIN RU = 8.314510e7 erg/mol/K).
constexpr double RU_CGS = 8.314510e7;
constexpr double R_SI = 8314.510;     // J/(kmol K) = RU_CGS * 1e-4
constexpr double PATM_CGS = 1.01325e6;

struct ThermoTable {
  int ns;
  int nbreak;                       // distinct T_mid values, ascending
  double tbreak[8];
  double invW[EDYN_NS_MAX];
  double W[EDYN_NS_MAX];
  double tmid[EDYN_NS_MAX];
  // [range][coef][species]: coef 0..4 = a1, a2/2, a3/3, a4/4, a5/5 (enthalpy
  // form), coef 5 = a6; range 0 = low, 1 = high.
  double ah[2][6][EDYN_NS_MAX];
  double a7[2][EDYN_NS_MAX];        // entropy constant (Gibbs terms)
};

// Builds the table on the host from a parsed mechanism.
inline void build_thermo_table(const edyn_mech& m, ThermoTable& t) {
  std::memset(&t, 0, sizeof(t));  // tables of one mechanism compare equal byte for byte
  t.ns = m.nspec;
  t.nbreak = 0;
  for (int k = 0; k < m.nspec; ++k) {
    t.W[k] = m.W[k];
    t.invW[k] = 1.0 / m.W[k];
    t.tmid[k] = m.T_mid[k];
    for (int r = 0; r < 2; ++r) {
      t.ah[r][0][k] = m.a[k][r][0];
      t.ah[r][1][k] = m.a[k][r][1] / 2.0;
      t.ah[r][2][k] = m.a[k][r][2] / 3.0;
      t.ah[r][3][k] = m.a[k][r][3] / 4.0;
      t.ah[r][4][k] = m.a[k][r][4] / 5.0;
      t.ah[r][5][k] = m.a[k][r][5];
      t.a7[r][k] = m.a[k][r][6];
    }
    bool seen = false;
    for (int b = 0; b < t.nbreak; ++b) seen |= (t.tbreak[b] == m.T_mid[k]);
    if (!seen && t.nbreak < 8) t.tbreak[t.nbreak++] = m.T_mid[k];
  }
  for (int a = 0; a < t.nbreak; ++a)
    for (int b = a + 1; b < t.nbreak; ++b)
      if (t.tbreak[b] < t.tbreak[a]) {
        double x = t.tbreak[a];
        t.tbreak[a] = t.tbreak[b];
        t.tbreak[b] = x;
      }
  for (int k = m.nspec; k < EDYN_NS_MAX; ++k) {
    t.W[k] = 1.0;
    t.invW[k] = 0.0;
    t.tmid[k] = 1000.0;
  }
}

#ifdef __CUDACC__

// Bit-level helpers: comparisons of non-negative doubles and sign tests as
// integer instructions, which keeps them off the FP64 pipe.
__device__ __forceinline__ long long dbits(double x) { return __double_as_longlong(x); }

// max(x, 0) as the reference's adjust_sum clip; integer select only.
__device__ __forceinline__ double clip0(double x) { return dbits(x) < 0 ? 0.0 : x; }

// minmod(x, y) of SRC/muscl.f90:79-93: sign(x) * max(0, min(|x|, sign(x) y)).
// Same-sign nonzero arguments give the one of smaller magnitude, all other
// cases give zero. Evaluated with 64-bit integer compares.
__device__ __forceinline__ double minmod_i(double x, double y) {
  long long bx = dbits(x), by = dbits(y);
  long long ax = bx & 0x7fffffffffffffffLL, ay = by & 0x7fffffffffffffffLL;
  bool same = ((bx ^ by) >= 0) && ax != 0 && ay != 0;
  return same ? (ax <= ay ? x : y) : 0.0;
}

// Temperature interval of the premix: index of the first breakpoint >= T
// (T inside (tbreak[b-1], tbreak[b]]), matching "T > T_mid -> upper range".
template <class TT>
__device__ __forceinline__ int t_interval(const TT& tb, double T) {
  int b = 0;
  for (int q = 0; q < tb.nbreak; ++q) b += (T > tb.tbreak[q]) ? 1 : 0;
  return b;
}

struct Premix {
  double A[6];  // a1, a2/2, a3/3, a4/4, a5/5, a6 premixed with z_k
  int interval;
  __device__ __forceinline__ void zero(int iv) {
#pragma unroll
    for (int n = 0; n < 6; ++n) A[n] = 0.0;
    interval = iv;
  }
  // H(T) = sum z_k h_k/R  [K]
  __device__ __forceinline__ double H(double T) const {
    double p = fma(A[4], T, A[3]);
    p = fma(p, T, A[2]);
    p = fma(p, T, A[1]);
    p = fma(p, T, A[0]);
    return fma(p, T, A[5]);
  }
  // Cp(T) = sum z_k cp_k/R
  __device__ __forceinline__ double Cp(double T) const {
    double p = fma(5.0 * A[4], T, 4.0 * A[3]);
    p = fma(p, T, 3.0 * A[2]);
    p = fma(p, T, 2.0 * A[1]);
    return fma(p, T, A[0]);
  }
};

// Adds z * coefficients of species k (range chosen from the premix interval).
template <class TT>
__device__ __forceinline__ void premix_add(const TT& tb, Premix& pm, int k, double z, double T) {
  const int r = (T > tb.tmid[k]) ? 1 : 0;
#pragma unroll
  for (int n = 0; n < 6; ++n) pm.A[n] = fma(z, tb.ah[r][n][k], pm.A[n]);
}

// Representative temperature inside an interval (used to pick ranges when
// re-premixing for a Newton iterate).
template <class TT>
__device__ __forceinline__ double interval_probe(const TT& tb, int iv) {
  if (iv <= 0) return tb.nbreak > 0 ? tb.tbreak[0] : 1000.0;
  return tb.tbreak[iv - 1] + 0.5;
}

#endif  // __CUDACC__

}  // namespace edyn
