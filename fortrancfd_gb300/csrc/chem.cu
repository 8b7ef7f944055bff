// Per-cell stiff chemistry on sm_103a: one warp per cell, one persistent
// work-stealing launch for all cells of a tube or batch.
//
// Contract (SRC/source.f90:17-84): for each cell a constant-density
// adiabatic reactor is advanced over dt on [Y_1..Y_K, T] with the CHEMKIN
// production rates of CKWYR (GRI/cklib.f:9107: CKRATT 6630, CKYTCR 9533,
// CKRATX 6820):
//     dY_k/dt = W_k w_k / rho,   dT/dt = -sum_k u_k w_k / (rho cv).
// The reference's integrator (macks, SRC/odes.f90) is not part of its tree;
// this is the project's own method: the L-stable SDIRK4 of Hairer & Wanner
// (gamma = 1/4, embedded order 3) with simplified inexact Newton.
//
// Precision split: every right-hand side that enters a Newton residual, the
// state update, the error estimate and the conservation-bearing quantities
// are FP64 -- including the Arrhenius and equilibrium-constant exponentials.
// The Jacobian (analytic mass-action part, finite differences in T) and its
// LU factorisation are FP32, so the Newton iteration is inexact.
//
// Warp work split: lanes take species for the thermodynamic pass, reactions
// (in an order that groups reactions of one kind into the same 32-wide
// round, so lanes rarely diverge) for the rate pass, and load-balanced
// pieces of the species-major stoichiometry list for the production-rate
// gather. Equilibrium constants use per-species scaled exponentials
// exp(S/R - H/RT) = m 2^n (Cody-Waite reduction), so 53 exponentials replace
// 309 per right-hand side without overflow in the products.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../../include/edyn_gpu.h"
#include "chem.h"
#include "edyn_kernels.h"

namespace edyn {

namespace {

constexpr int NSMAX = 64;
constexpr int NV = 56;      // padded state vector length (54 used for GRI)
constexpr int WARPS = 7;    // warps per CTA (shared memory bound)
constexpr int JS = 55;      // FP32 matrix row stride (odd: conflict-free column walks)

// SDIRK4 (Hairer & Wanner, Solving ODEs II, Table 6.5), gamma = 1/4.
__constant__ double c_sa[5][5] = {{0.25, 0, 0, 0, 0},
                                  {0.5, 0.25, 0, 0, 0},
                                  {17.0 / 50.0, -1.0 / 25.0, 0.25, 0, 0},
                                  {371.0 / 1360.0, -137.0 / 2720.0, 15.0 / 544.0, 0.25, 0},
                                  {25.0 / 24.0, -49.0 / 48.0, 125.0 / 16.0, -85.0 / 12.0, 0.25}};
__constant__ double c_se[5] = {25.0 / 24.0 - 59.0 / 48.0, -49.0 / 48.0 + 17.0 / 96.0, 125.0 / 16.0 - 225.0 / 32.0,
                               0.0, 0.25};

// Packed table header (all offsets in bytes from the blob start).
struct TabHdr {
  int ns, nr, nrp, nsp, npc, ntbl, total_bytes;
  int o_A, o_B, o_E, o_lnA;    // double[nrp]
  int o_w0, o_w1, o_w2, o_w3, o_w4, o_w5;  // uint[nrp]
  int o_sp_aux;               // double[nsp*9]: lowA lowB lowE troe_a T3 T1 T2 ifop ln(lowA)
  int o_sp_i;                 // int[nsp*4]: tb_off, tb_cnt, kfal (-1 mixture), flags
  int o_tb_am1;               // double[ntbl]
  int o_tb_sp;                // int[ntbl]
  int o_W, o_invW, o_tmid, o_hf;   // double[NSMAX]
  int o_cs;                   // double[2][7][NSMAX] smh coefficients
  int o_ch;                   // double[2][6][NSMAX] enthalpy coefficients (a1, a2/2, .., a6)
  int o_pc;                   // int[npc*3]: species, entry begin, entry end
  int o_lane;                 // int[33]: piece range per lane
  int o_spc;                  // int[NSMAX+1]: piece range per species (pieces of a species contiguous in spp)
  int o_spp;                  // int[npc]: piece index list ordered by species
  int o_ent;                  // uint[nent]: (sched reaction index) | (nu + 8) << 16
  int nent;
};

struct Tabs {
  const TabHdr* h;
  const double *A, *B, *E, *lnA, *aux, *tb_am1, *W, *invW, *tmid, *hf, *cs, *ch;
  const unsigned *w0, *w1, *w2, *w3, *w4, *w5, *ent;
  const int *spi, *tb_sp, *pc, *lane, *spc, *spp;
  int ns, nr, nrp, npc;
};

__device__ __forceinline__ Tabs bind_tabs(const char* base) {
  Tabs t;
  t.h = (const TabHdr*)base;
  const TabHdr& h = *t.h;
  t.A = (const double*)(base + h.o_A);
  t.B = (const double*)(base + h.o_B);
  t.E = (const double*)(base + h.o_E);
  t.lnA = (const double*)(base + h.o_lnA);
  t.w0 = (const unsigned*)(base + h.o_w0);
  t.w1 = (const unsigned*)(base + h.o_w1);
  t.w2 = (const unsigned*)(base + h.o_w2);
  t.w3 = (const unsigned*)(base + h.o_w3);
  t.w4 = (const unsigned*)(base + h.o_w4);
  t.w5 = (const unsigned*)(base + h.o_w5);
  t.aux = (const double*)(base + h.o_sp_aux);
  t.spi = (const int*)(base + h.o_sp_i);
  t.tb_am1 = (const double*)(base + h.o_tb_am1);
  t.tb_sp = (const int*)(base + h.o_tb_sp);
  t.W = (const double*)(base + h.o_W);
  t.invW = (const double*)(base + h.o_invW);
  t.tmid = (const double*)(base + h.o_tmid);
  t.hf = (const double*)(base + h.o_hf);
  t.cs = (const double*)(base + h.o_cs);
  t.ch = (const double*)(base + h.o_ch);
  t.pc = (const int*)(base + h.o_pc);
  t.lane = (const int*)(base + h.o_lane);
  t.spc = (const int*)(base + h.o_spc);
  t.spp = (const int*)(base + h.o_spp);
  t.ent = (const unsigned*)(base + h.o_ent);
  t.ns = h.ns;
  t.nr = h.nr;
  t.nrp = h.nrp;
  t.npc = h.npc;
  return t;
}

// reaction flag bits (w0 >> 24)
constexpr unsigned F_REV = 1, F_CM = 2, F_FALL = 4, F_KFAL = 8, F_EXP = 16, F_TB = 32;

// Per-warp shared workspace.
struct alignas(16) WarpWork {
  double y0[NV], Y[NV], sv[NV], fy[NV], F[5][NV], dl[NV];
  double C[NV], m[NV], uR[NV], cvm[NV], wdot[NV];
  double part[128];
  double rop[352];
  int en[NV];
  float J[54 * JS];
  float b32[NV];
  float sc32[NV];  // error weights atol + rtol |y0| of the current step
  int piv[NV];
  float f1[NV], f2[NV];
};

__device__ __forceinline__ double clip0_d(double x) { return __double_as_longlong(x) < 0 ? 0.0 : x; }

template <class R>
__device__ __forceinline__ R warp_sum(R v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
template <class R>
__device__ __forceinline__ R warp_max(R v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

template <class R>
struct Math;
template <>
struct Math<double> {
  static __device__ __forceinline__ double ex(double x) { return exp(x); }
  static __device__ __forceinline__ double lg(double x) { return log(x); }
  static __device__ __forceinline__ double l10(double x) { return log10(x); }
  static __device__ __forceinline__ double p10(double x) { return exp(2.302585092994045684 * x); }
  static __device__ __forceinline__ double ldx(double m, int n) { return ldexp(m, n); }
  static __device__ __forceinline__ double small() { return 1e-300; }
  static __device__ __forceinline__ double big() { return 1e300; }
  static __device__ __forceinline__ double rint_(double x) { return rint(x); }
};
template <>
struct Math<float> {
  static __device__ __forceinline__ float ex(float x) { return __expf(x); }
  static __device__ __forceinline__ float lg(float x) { return __logf(x); }
  static __device__ __forceinline__ float l10(float x) { return __log10f(x); }
  static __device__ __forceinline__ float p10(float x) { return exp2f(3.321928094887362f * x); }
  static __device__ __forceinline__ float ldx(float m, int n) { return ldexpf(m, n); }
  static __device__ __forceinline__ float small() { return 1e-37f; }
  static __device__ __forceinline__ float big() { return 1e37f; }
  static __device__ __forceinline__ float rint_(float x) { return rintf(x); }
};

__device__ __forceinline__ unsigned sp_of(unsigned w, int s) { return (w >> (8 * s)) & 0xffu; }

// Rate constants of one reaction (CKRATT + the third-body/fall-off part of
// CKRATX) and its net rate of progress. Returns qf - qr; also returns the
// forward/reverse parts for the Jacobian. invKc uses the scaled species
// exponentials m[k] 2^en[k] = exp(S_k/R - H_k/RT).
template <class R>
struct RxnEval {
  R kf, kr, qf, qr, cm, pr, pcor_d;  // pcor_d: d ln(pcor)/d ln(CM) (fall-off, F held fixed)
};

template <class R>
__device__ __forceinline__ RxnEval<R> eval_rxn(const Tabs& t, int i, R logT, R invT, R T, R pfac, R ctot,
                                               const R* C, const R* m, const int* en) {
  using M = Math<R>;
  RxnEval<R> o;
  const unsigned w0 = t.w0[i], w1 = t.w1[i], w2 = t.w2[i];
  const unsigned fl = w0 >> 24;
  R kf;
  if (sizeof(R) == sizeof(double)) {
    // CKRATT 6645: A exp(beta ln T - E/T), as the reference evaluates it
    kf = (R)t.A[i];
    if (fl & F_EXP) kf = kf * M::ex((R)t.B[i] * logT - (R)t.E[i] * invT);
  } else {
    // single precision (Jacobian only): pre-exponentials up to 1e74 do not
    // fit in FP32, so the logarithmic form is used
    kf = M::ex((R)t.lnA[i] + (R)t.B[i] * logT - (R)t.E[i] * invT);
  }
  R kr = 0;
  if (fl & F_REV) {
    // 1/Kc = exp(-sum nu (S/R - H/RT)) * pfac^(-sum nu)  (CKRATT, 6647-6667)
    R mant = 1;
    int ex2 = 0;
#pragma unroll
    for (int s = 0; s < 3; ++s) {
      const unsigned kr_ = sp_of(w0, s), kp = sp_of(w1, s);
      const int nr_ = (w2 >> (4 * s)) & 15, np = (w2 >> (12 + 4 * s)) & 15;
      if (kr_ != 255u) {
        R mm = m[kr_];
        mant *= (nr_ == 1) ? mm : (nr_ == 2 ? mm * mm : mm * mm * mm);
        ex2 += nr_ * en[kr_];
      }
      if (kp != 255u) {
        R mm = (R)1 / m[kp];
        mant *= (np == 1) ? mm : (np == 2 ? mm * mm : mm * mm * mm);
        ex2 -= np * en[kp];
      }
    }
    const int dnu = (int)(w1 >> 24) - 8;
    R ikc = M::ldx(mant, ex2);
    if (dnu == 1) ikc = ikc / pfac;
    else if (dnu == -1) ikc = ikc * pfac;
    else if (dnu != 0) ikc = ikc * pow(pfac, (R)(-dnu));
    ikc = fmin(ikc, M::big());  // kr = kf / max(Kc, SMALL)
    kr = kf * ikc;
    if (sizeof(R) != sizeof(double)) kr = fmin(kr, (R)1e30f);
  }
  o.cm = 1;
  o.pr = 0;
  o.pcor_d = 0;
  const int aux = (int)(w2 >> 24);
  if (fl & (F_CM | F_KFAL)) {
    R cm;
    if (fl & F_KFAL) {
      cm = C[t.spi[aux * 4 + 2]];
    } else {
      cm = ctot;
      const int b = t.spi[aux * 4 + 0], c = t.spi[aux * 4 + 1];
      for (int q = b; q < b + c; ++q) cm += (R)t.tb_am1[q] * C[t.tb_sp[q]];
    }
    o.cm = cm;
    if (fl & F_FALL) {
      const double* fp = t.aux + aux * 9;
      const R k0 = (sizeof(R) == sizeof(double)) ? (R)fp[0] * M::ex((R)fp[1] * logT - (R)fp[2] * invT)
                                                 : M::ex((R)fp[8] + (R)fp[1] * logT - (R)fp[2] * invT);
      const R pr = k0 * cm / kf;
      R pcor = pr / (1 + pr);
      const int ifop = (int)fp[7];
      if (ifop > 1) {
        const R prlog = M::l10(fmax(pr, M::small()));
        R fcent = (1 - (R)fp[3]) * M::ex(-T / (R)fp[4]) + (R)fp[3] * M::ex(-T / (R)fp[5]);
        if (ifop == 4) fcent += M::ex(-(R)fp[6] * invT);
        const R fclog = M::l10(fmax(fcent, M::small()));
        const R xn = (R)0.75 - (R)(double)1.27f * fclog;
        const R cprlog = prlog - ((R)(double)0.4f + (R)(double)0.67f * fclog);
        const R q = cprlog / (xn - (R)(double)0.14f * cprlog);
        const R flog = fclog / (1 + q * q);
        pcor = M::p10(flog) * pcor;
      }
      kf *= pcor;
      kr *= pcor;
      o.pr = pr;
      o.pcor_d = 1 / (1 + pr);
    } else {
      kf *= cm;
      kr *= cm;
      o.pcor_d = 1;
    }
  }
  // mass-action products (CKRATX 6900-6915)
  R qf = kf, qr = kr;
#pragma unroll
  for (int s = 0; s < 3; ++s) {
    const unsigned kr_ = sp_of(w0, s), kp = sp_of(w1, s);
    const int nr_ = (w2 >> (4 * s)) & 15, np = (w2 >> (12 + 4 * s)) & 15;
    if (kr_ != 255u) {
      const R c = C[kr_];
      qf *= (nr_ == 1) ? c : (nr_ == 2 ? c * c : c * c * c);
    }
    if (kp != 255u) {
      const R c = C[kp];
      qr *= (np == 1) ? c : (np == 2 ? c * c : c * c * c);
    }
  }
  o.kf = kf;
  o.kr = kr;
  o.qf = qf;
  o.qr = qr;
  return o;
}

// Thermodynamic pass over species (lanes over k): concentrations, scaled
// exp(S/R - H/RT), u_k/R and cv_k/(R W_k).
template <class R>
__device__ __forceinline__ R species_pass(const Tabs& t, const double* y, R rho, R T, R logT, R invT, R* C, R* m,
                                          int* en, R* uR, R* cvm, int lane) {
  using M = Math<R>;
  R csum = 0;
  for (int k = lane; k < t.ns; k += 32) {
    const R c = rho * (R)y[k] * (R)t.invW[k];
    C[k] = c;
    csum += c;
    const int r = (T > (R)t.tmid[k]) ? 1 : 0;
    const double* cs = t.cs + r * 7 * NSMAX;
    // S/R - H/RT = a1 (lnT - 1) + a2/2 T + a3/6 T^2 + a4/12 T^3 + a5/20 T^4 + a7 - a6/T (CKSMH, 7501)
    R p = fma((R)cs[4 * NSMAX + k], T, (R)cs[3 * NSMAX + k]);
    p = fma(p, T, (R)cs[2 * NSMAX + k]);
    p = fma(p, T, (R)cs[1 * NSMAX + k]);
    R smh = fma(p, T, fma((R)cs[0 * NSMAX + k], logT - 1, (R)cs[6 * NSMAX + k])) - (R)cs[5 * NSMAX + k] * invT;
    // Cody-Waite: smh = n ln2 + r
    const R nn = M::rint_(smh * (R)1.4426950408889634);
    const R rr = fma(-nn, (R)6.93147180369123816490e-01, smh) - nn * (R)1.90821492927058770002e-10;
    m[k] = M::ex(rr);
    en[k] = (int)nn;
    const double* ch = t.ch + r * 6 * NSMAX;
    R h = fma((R)ch[4 * NSMAX + k], T, (R)ch[3 * NSMAX + k]);
    h = fma(h, T, (R)ch[2 * NSMAX + k]);
    h = fma(h, T, (R)ch[1 * NSMAX + k]);
    h = fma(h, T, (R)ch[0 * NSMAX + k]);
    uR[k] = fma(h, T, (R)ch[5 * NSMAX + k]) - T;  // u/R = h/R - T
    R cp = fma((R)(5.0 * ch[4 * NSMAX + k]), T, (R)(4.0 * ch[3 * NSMAX + k]));
    cp = fma(cp, T, (R)(3.0 * ch[2 * NSMAX + k]));
    cp = fma(cp, T, (R)(2.0 * ch[1 * NSMAX + k]));
    cp = fma(cp, T, (R)ch[0 * NSMAX + k]);
    cvm[k] = (cp - 1) * (R)t.invW[k];
  }
  return warp_sum(csum);
}

// Full right-hand side in precision R. y (FP64, shared) -> f (shared, R).
// rop buffer in R. Returns nothing; f[ns] is dT/dt.
template <class R>
__device__ void rhs(const Tabs& t, WarpWork& w, const double* y, double rho_cgs, R* f, R* C, R* m, R* uR, R* cvm,
                    R* rop, R* wdot, R* part, int lane) {
  const int ns = t.ns;
  const R T = (R)y[ns];
  const R logT = Math<R>::lg(T);
  const R invT = (R)1 / T;
  const R rho = (R)rho_cgs;
  const R ctot = species_pass<R>(t, y, rho, T, logT, invT, C, m, w.en, uR, cvm, lane);
  const R pfac = (R)(PATM_CGS / RU_CGS) * invT;
  __syncwarp();
  for (int i = lane; i < t.nrp; i += 32) {
    R r = 0;
    if (i < t.nr) {
      RxnEval<R> e = eval_rxn<R>(t, i, logT, invT, T, pfac, ctot, C, m, w.en);
      r = e.qf - e.qr;
    }
    rop[i] = r;
  }
  __syncwarp();
  // production rates: load-balanced pieces of the species-major list
  for (int p = t.lane[lane]; p < t.lane[lane + 1]; ++p) {
    const int e0 = t.pc[p * 3 + 1], e1 = t.pc[p * 3 + 2];
    R s = 0;
    for (int q = e0; q < e1; ++q) {
      const unsigned v = t.ent[q];
      s = fma((R)((int)(v >> 16) - 8), rop[v & 0xffffu], s);
    }
    part[p] = s;
  }
  __syncwarp();
  R su = 0, cv = 0;
  for (int k = lane; k < ns; k += 32) {
    R s = 0;
    for (int q = t.spc[k]; q < t.spc[k + 1]; ++q) s += part[t.spp[q]];
    wdot[k] = s;
    f[k] = s * (R)t.W[k] / rho;
    su = fma(uR[k], s, su);
    cv = fma((R)y[k], cvm[k], cv);
  }
  su = warp_sum(su);
  cv = warp_sum(cv);
  if (lane == 0) f[ns] = -su / (rho * cv);  // RU cancels in u/cv
  __syncwarp();
}

// Analytic FP32 Jacobian of the mass-action species block plus finite
// differences in T. J (row-major, stride JS) receives d f / d y at y.
__device__ void jacobian32(const Tabs& t, WarpWork& w, const double* y, double rho_cgs, int lane) {
  const int ns = t.ns, n = ns + 1;
  float* J = w.J;
  float* Cf = (float*)w.C;
  float* mf = (float*)w.m;
  float* uRf = (float*)w.uR;
  float* cvmf = (float*)w.cvm;
  float* ropf = (float*)w.rop;
  float* wdf = (float*)w.wdot;
  float* partf = (float*)w.part;
  for (int q = lane; q < n * JS; q += 32) J[q] = 0.f;
  // base rates at (y, T) and at (y, T + dT) for the temperature column
  double* yt = w.sv;  // scratch copy with perturbed T
  const float T = (float)y[ns];
  const float dT = fmaxf(1e-3f * T, 0.05f);
  for (int k = lane; k < n; k += 32) yt[k] = y[k];
  __syncwarp();
  if (lane == 0) yt[ns] = y[ns] + (double)dT;
  __syncwarp();
  rhs<float>(t, w, yt, rho_cgs, w.f2, Cf, mf, uRf, cvmf, ropf, wdf, partf, lane);
  rhs<float>(t, w, y, rho_cgs, w.f1, Cf, mf, uRf, cvmf, ropf, wdf, partf, lane);
  // species pass data (C, m, en, uR, cvm) now hold the base state
  const float logT = __logf(T), invT = 1.f / T;
  const float rho = (float)rho_cgs;
  float ctot = 0.f;
  for (int k = lane; k < ns; k += 32) ctot += Cf[k];
  ctot = warp_sum(ctot);
  const float pfac = (float)(PATM_CGS / RU_CGS) * invT;
  // d w_k / d C_j accumulated into J[k][j] (concentration space)
  for (int i = lane; i < t.nr; i += 32) {
    RxnEval<float> e = eval_rxn<float>(t, i, logT, invT, T, pfac, ctot, Cf, mf, w.en);
    const unsigned w0 = t.w0[i], w1 = t.w1[i], w2 = t.w2[i], w3 = t.w3[i], w4 = t.w4[i], w5 = t.w5[i];
    const int nk = (w5 >> 8) & 15;
    int ks[6], nus[6];
    for (int q = 0; q < 6; ++q) {
      ks[q] = q < 4 ? (int)((w3 >> (8 * q)) & 0xff) : (int)((w4 >> (8 * (q - 4))) & 0xff);
      int nu4 = q < 4 ? (int)((w4 >> (16 + 4 * q)) & 15) : (int)((w5 >> (4 * (q - 4))) & 15);
      nus[q] = nu4 - 8;
    }
    // forward: d qf / d C_r ; reverse: d qr / d C_p
    for (int s = 0; s < 3; ++s) {
      const unsigned kr_ = sp_of(w0, s);
      if (kr_ != 255u) {
        const int nr_ = (w2 >> (4 * s)) & 15;
        float d = e.kf * (float)nr_;
        for (int s2 = 0; s2 < 3; ++s2) {
          const unsigned k2 = sp_of(w0, s2);
          if (k2 == 255u) continue;
          const int n2 = (w2 >> (4 * s2)) & 15;
          const float c = Cf[k2];
          const int pw = (s2 == s) ? n2 - 1 : n2;
          for (int q = 0; q < pw; ++q) d *= c;
        }
        for (int q = 0; q < nk; ++q) atomicAdd(&J[ks[q] * JS + kr_], (float)nus[q] * d);
      }
      const unsigned kp = sp_of(w1, s);
      if (kp != 255u) {
        const int np = (w2 >> (12 + 4 * s)) & 15;
        float d = e.kr * (float)np;
        for (int s2 = 0; s2 < 3; ++s2) {
          const unsigned k2 = sp_of(w1, s2);
          if (k2 == 255u) continue;
          const int n2 = (w2 >> (12 + 4 * s2)) & 15;
          const float c = Cf[k2];
          const int pw = (s2 == s) ? n2 - 1 : n2;
          for (int q = 0; q < pw; ++q) d *= c;
        }
        for (int q = 0; q < nk; ++q) atomicAdd(&J[ks[q] * JS + kp], -(float)nus[q] * d);
      }
    }
    // collider dependence (third body / fall-off), fall-off blending held fixed
    const unsigned fl = w0 >> 24;
    if (fl & (F_CM | F_KFAL)) {
      const float r0 = (e.qf - e.qr) * e.pcor_d / e.cm;
      if (isfinite(r0) && r0 != 0.f) {
        const int aux = (int)(w2 >> 24);
        if (fl & F_KFAL) {
          const int kc = t.spi[aux * 4 + 2];
          for (int q = 0; q < nk; ++q) atomicAdd(&J[ks[q] * JS + kc], (float)nus[q] * r0);
        } else {
          for (int j = 0; j < ns; ++j)
            for (int q = 0; q < nk; ++q) atomicAdd(&J[ks[q] * JS + j], (float)nus[q] * r0);
          const int b = t.spi[aux * 4 + 0], c = t.spi[aux * 4 + 1];
          for (int q2 = b; q2 < b + c; ++q2) {
            const int j = t.tb_sp[q2];
            const float a = (float)t.tb_am1[q2] * r0;
            for (int q = 0; q < nk; ++q) atomicAdd(&J[ks[q] * JS + j], (float)nus[q] * a);
          }
        }
      }
    }
  }
  __syncwarp();
  // to mass-fraction space: d f_k / d y_j = (W_k / W_j) d w_k / d C_j; T row
  // d f_T / d y_j = -(sum_k e_k J_kj + f_T cvm_j) / cv with e_k = u_k/W_k.
  float cv = 0.f;
  for (int k = lane; k < ns; k += 32) cv = fmaf((float)y[k], cvmf[k], cv);
  cv = warp_sum(cv);
  const float fT = w.f1[ns];
  for (int j = lane; j < ns; j += 32) {
    const float wj = (float)t.invW[j];
    float acc = 0.f;
    for (int k = 0; k < ns; ++k) {
      const float v = J[k * JS + j] * (float)t.W[k] * wj;
      J[k * JS + j] = v;
      acc = fmaf(uRf[k] * (float)t.invW[k], v, acc);
    }
    J[ns * JS + j] = -(acc + fT * cvmf[j]) / cv;
  }
  const float idT = 1.f / ((float)((double)T + (double)dT - (double)T));
  for (int k = lane; k < n; k += 32) J[k * JS + ns] = (w.f2[k] - w.f1[k]) * idT;
  __syncwarp();
  // an entry that overflowed single precision carries no usable slope
  for (int q = lane; q < n * JS; q += 32)
    if (!isfinite(J[q])) J[q] = 0.f;
  __syncwarp();
}

// In-place LU with partial pivoting of M = I - hg J (FP32, one warp).
__device__ bool lu32(float* A, int* piv, int n, int lane) {
  bool ok = true;
  for (int k = 0; k < n; ++k) {
    float bv = -1.f;
    int bi = k;
    for (int i = k + lane; i < n; i += 32) {
      const float v = fabsf(A[i * JS + k]);
      if (v > bv) { bv = v; bi = i; }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float ov = __shfl_xor_sync(0xffffffffu, bv, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ov > bv || (ov == bv && oi < bi)) { bv = ov; bi = oi; }
    }
    if (!(bv > 0.f)) ok = false;
    if (lane == 0) piv[k] = bi;
    if (bi != k)
      for (int j = lane; j < n; j += 32) {
        const float t0 = A[k * JS + j];
        A[k * JS + j] = A[bi * JS + j];
        A[bi * JS + j] = t0;
      }
    __syncwarp();
    const float inv = 1.f / A[k * JS + k];
    for (int i = k + 1 + lane; i < n; i += 32) A[i * JS + k] *= inv;
    __syncwarp();
    for (int j = k + 1 + lane; j < n; j += 32) {
      const float akj = A[k * JS + j];
      for (int i = k + 1; i < n; ++i) A[i * JS + j] = fmaf(-A[i * JS + k], akj, A[i * JS + j]);
    }
    __syncwarp();
  }
  return ok;
}

__device__ void lusolve32(const float* A, const int* piv, float* b, int n, int lane) {
  for (int k = 0; k < n; ++k) {
    const int p = piv[k];
    if (p != k && lane == 0) {
      const float t0 = b[k];
      b[k] = b[p];
      b[p] = t0;
    }
    __syncwarp();
    const float bk = b[k];
    for (int i = k + 1 + lane; i < n; i += 32) b[i] = fmaf(-A[i * JS + k], bk, b[i]);
    __syncwarp();
  }
  for (int i = n - 1; i >= 0; --i) {
    if (lane == 0) b[i] = b[i] / A[i * JS + i];
    __syncwarp();
    const float bi = b[i];
    for (int j = lane; j < i; j += 32) b[j] = fmaf(-A[j * JS + i], bi, b[j]);
    __syncwarp();
  }
}

struct Cell {
  double rho_cgs, dt, rtol, atol;
};

struct CellStats {
  int rhs, steps, rejects, jac;
  bool failed;
};

// Integrates w.y0 over [0, dt] with SDIRK4. Returns the statistics.
__device__ CellStats integrate(const Tabs& t, WarpWork& w, const Cell& c, int lane) {
  const int n = t.ns + 1;
  CellStats st = {0, 0, 0, 0, false};
  double tcur = 0.0, h = c.dt;
  const int max_steps = 4000;
  bool need_jac = true, need_f0 = true;
  const double g = 0.25;
  while (tcur < c.dt) {
    if (st.steps + st.rejects >= max_steps) { st.failed = true; break; }
    if (tcur + h > c.dt) h = c.dt - tcur;
    // f0 = f(y0) in FP64 (kept across rejections), Jacobian in FP32
    if (need_f0) {
      rhs<double>(t, w, w.y0, c.rho_cgs, w.dl, w.C, w.m, w.uR, w.cvm, w.rop, w.wdot, w.part, lane);
      st.rhs++;
      need_f0 = false;
    }
    if (need_jac) {
      jacobian32(t, w, w.y0, c.rho_cgs, lane);
      st.jac++;
    }
    // Newton matrix I - h g J equilibrated with the error weights,
    // Ms = D^-1 M D, D = diag(atol + rtol |y0|); unscaled, the temperature
    // row (K per unit mass fraction) wins the pivot search and the species
    // rows lose their accuracy. Factorised in place; J is rebuilt after a
    // rejection.
    for (int i = lane; i < n; i += 32) w.sc32[i] = (float)(c.atol + c.rtol * fabs(w.y0[i]));
    __syncwarp();
    for (int q = lane; q < n * JS; q += 32) {
      const int i = q / JS, j = q - i * JS;
      if (j < n) w.J[q] = ((i == j ? 1.f : 0.f) - (float)(h * g) * w.J[q]) * (w.sc32[j] / w.sc32[i]);
    }
    __syncwarp();
    bool lu_ok = lu32(w.J, w.piv, n, lane);
    bool newton_ok = lu_ok;
    for (int s = 0; s < 5 && newton_ok; ++s) {
      for (int i = lane; i < n; i += 32) {
        double acc = w.y0[i];
        for (int j = 0; j < s; ++j) acc = fma(h * c_sa[s][j], w.F[j][i], acc);
        w.sv[i] = acc;
        const double fp = (s == 0) ? w.dl[i] : w.F[s - 1][i];
        w.Y[i] = fma(h * g, fp, acc);
      }
      __syncwarp();
      float nrm_prev = 0.f;
      bool conv = false;
      for (int it = 0; it < 8; ++it) {
        const double Tn = w.Y[n - 1];
        if (!(Tn > 100.0 && Tn < 8000.0)) break;
        rhs<double>(t, w, w.Y, c.rho_cgs, w.fy, w.C, w.m, w.uR, w.cvm, w.rop, w.wdot, w.part, lane);
        st.rhs++;
        for (int i = lane; i < n; i += 32)
          w.b32[i] = (float)(-(w.Y[i] - w.sv[i] - h * g * w.fy[i]) / (double)w.sc32[i]);
        __syncwarp();
        lusolve32(w.J, w.piv, w.b32, n, lane);
        float ss = 0.f;
        for (int i = lane; i < n; i += 32) {
          const float q = w.b32[i];  // scaled correction
          ss = fmaf(q, q, ss);
        }
        const float nrm = sqrtf(warp_sum(ss) / (float)n);
        if (!(nrm == nrm)) break;
        if (nrm <= 1e-3f) conv = true;
        if (!conv && it > 0) {
          const float th = nrm / nrm_prev;
          if (th >= 0.99f) break;
          if (th / (1.f - th) * nrm <= 1e-2f) conv = true;
        }
        if (conv) {
          // stage derivative = the FP64 right-hand side at the converged
          // iterate; the stage value is rebuilt from it, so mass and
          // elements are conserved to rounding
          for (int i = lane; i < n; i += 32) {
            w.F[s][i] = w.fy[i];
            w.Y[i] = fma(h * g, w.fy[i], w.sv[i]);
          }
          __syncwarp();
          break;
        }
        for (int i = lane; i < n; i += 32) w.Y[i] += (double)w.b32[i] * (double)w.sc32[i];
        __syncwarp();
        nrm_prev = nrm;
      }
      if (!conv) { newton_ok = false; break; }
    }
    if (!newton_ok) {
      st.rejects++;
      h *= 0.25;
      need_jac = true;
      if (h < c.dt * 1e-12) { st.failed = true; break; }
      continue;
    }
    // embedded error, filtered through the factorised matrix
    for (int i = lane; i < n; i += 32) {
      double e = 0.0;
      for (int j = 0; j < 5; ++j) e = fma(c_se[j], w.F[j][i], e);
      w.b32[i] = (float)(h * e / (double)w.sc32[i]);
    }
    __syncwarp();
    lusolve32(w.J, w.piv, w.b32, n, lane);
    float ss = 0.f;
    for (int i = lane; i < n; i += 32) {
      const double sc = c.atol + c.rtol * fmax(fabs(w.y0[i]), fabs(w.Y[i]));
      const float q = (float)((double)w.b32[i] * (double)w.sc32[i] / sc);
      ss = fmaf(q, q, ss);
    }
    const float en = sqrtf(warp_sum(ss) / (float)n);
    const float fac = 0.9f * powf(fmaxf(en, 1e-10f), -0.25f);
    if (en <= 1.f) {
      for (int i = lane; i < n; i += 32) w.y0[i] = w.Y[i];
      __syncwarp();
      tcur += h;
      st.steps++;
      need_f0 = true;
      h = h * (double)fminf(5.f, fmaxf(0.2f, fac));
      need_jac = true;
    } else {
      st.rejects++;
      h = h * (double)fminf(1.f, fmaxf(0.2f, fac));
      need_jac = true;
    }
  }
  return st;
}

__device__ __forceinline__ void stage_tables(char* smem_tab, const char* g_tab, int bytes) {
  const int4* src = (const int4*)g_tab;
  int4* dst = (int4*)smem_tab;
  for (int q = threadIdx.x; q < bytes / 16; q += blockDim.x) dst[q] = src[q];
  __syncthreads();
}

__device__ __forceinline__ void add_stats(ChemCounters* cnt, const CellStats& s, int lane) {
  if (lane == 0) {
    atomicAdd(&cnt->rhs, (unsigned long long)s.rhs);
    atomicAdd(&cnt->steps, (unsigned long long)s.steps);
    atomicAdd(&cnt->rejects, (unsigned long long)s.rejects);
    atomicAdd(&cnt->jac, (unsigned long long)s.jac);
    atomicAdd(&cnt->cells, 1ull);
    if (s.failed) atomicAdd(&cnt->failed, 1ull);
  }
}

// Batch of independent reactors (macks contract).
__global__ void __launch_bounds__(WARPS * 32, 1)
    k_reactors(const char* g_tab, int tab_bytes, int n, const double* rho, const double* dt, double* yiT, double rtol,
               double atol, unsigned* next, ChemCounters* cnt, unsigned* err) {
  extern __shared__ __align__(16) char smem[];
  stage_tables(smem, g_tab, tab_bytes);
  const Tabs t = bind_tabs(smem);
  WarpWork& w = ((WarpWork*)(smem + ((tab_bytes + 255) / 256) * 256))[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  const int nv = t.ns + 1;
  for (int guard = 0; guard < (1 << 30); ++guard) {
    unsigned cell = 0;
    if (lane == 0) cell = atomicAdd(next, 1u);
    cell = __shfl_sync(0xffffffffu, cell, 0);
    if (cell >= (unsigned)n) break;
    const double* src = yiT + (size_t)cell * nv;
    for (int i = lane; i < nv; i += 32) w.y0[i] = src[i];
    __syncwarp();
    Cell c{rho[cell] * 1e-3, dt[cell], rtol, atol};
    CellStats s = integrate(t, w, c, lane);
    double* dst = yiT + (size_t)cell * nv;
    for (int i = lane; i < nv; i += 32) dst[i] = w.y0[i];
    add_stats(cnt, s, lane);
    if (s.failed && lane == 0) atomicOr(err, (unsigned)EDYN_E_CHEM);
    __syncwarp();
  }
}

// Tube mode: reaction_macks (SRC/source.f90:17-84) followed by the post-step
// QcToqf (SRC/main.f90:157-161) for every interior cell.
__global__ void __launch_bounds__(WARPS * 32, 1)
    k_tube_chem(const char* g_tab, int tab_bytes, ChemLaunch L, unsigned* next, ChemCounters* cnt) {
  extern __shared__ __align__(16) char smem[];
  if (L.step_active && *L.step_active == 0) return;
  const double dt = L.dt_dev ? *L.dt_dev : L.dt;
  stage_tables(smem, g_tab, tab_bytes);
  const Tabs t = bind_tabs(smem);
  WarpWork& w = ((WarpWork*)(smem + ((tab_bytes + 255) / 256) * 256))[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  const int ns = t.ns;
  const size_t ld = (size_t)L.ld;
  double speed_max = 0.0;
  for (int guard = 0; guard < (1 << 30); ++guard) {
    unsigned cell = 0;
    if (lane == 0) cell = atomicAdd(next, 1u);
    cell = __shfl_sync(0xffffffffu, cell, 0);
    if (cell >= (unsigned)L.n) break;
    double* q = L.qf + cell + GHOST;
    double* Q = L.qc + cell + GHOST;
    const double rho = q[0];
    // reaction_macks: y_sp = adjust_sum(Y), yiT = [y_sp, T] (SRC/source.f90:47-56);
    // the raw Y stay in the qf rows for the heat release rate.
    double s = 0.0;
    for (int k = lane; k < ns; k += 32) {
      const double yp = clip0_d(q[(3 + k) * ld]);
      w.y0[k] = yp;
      s += yp;
    }
    s = warp_sum(s);
    const double inv_s = 1.0 / s;
    for (int k = lane; k < ns; k += 32) w.y0[k] *= inv_s;
    if (lane == 0) w.y0[ns] = q[2 * ld];
    __syncwarp();
    Cell c{rho * 1e-3, dt, L.rtol, L.atol};
    CellStats st = integrate(t, w, c, lane);
    add_stats(cnt, st, lane);
    if (st.failed && lane == 0) atomicOr(L.err, (unsigned)EDYN_E_CHEM);
    // adjust_sum(Y) after the step
    double s2 = 0.0;
    for (int k = lane; k < ns; k += 32) {
      const double y = clip0_d(w.y0[k]);
      w.y0[k] = y;
      s2 += y;
    }
    s2 = warp_sum(s2);
    const double inv2 = 1.0 / s2;
    const double Tn = w.y0[ns];
    // heat release rate, SRC/thermo.f90:83-103 (qf rows still hold Y0 raw)
    const double rho_cgs = rho * 1e-3;
    double hr = 0.0, hs = 0.0, sz = 0.0;
    for (int k = lane; k < ns; k += 32) {
      const double yn = w.y0[k] * inv2;
      w.y0[k] = yn;
      const double y0raw = q[(3 + k) * ld];
      hr = fma(rho_cgs * t.hf[k], yn - y0raw, hr);
      // qfToQc energy: e = R (H(T) - T Sz)/S_Y with the adjusted Y (S_Y = 1)
      const int r = (Tn > t.tmid[k]) ? 1 : 0;
      const double* ch = t.ch + r * 6 * NSMAX;
      double hh = fma(ch[4 * NSMAX + k], Tn, ch[3 * NSMAX + k]);
      hh = fma(hh, Tn, ch[2 * NSMAX + k]);
      hh = fma(hh, Tn, ch[1 * NSMAX + k]);
      hh = fma(hh, Tn, ch[0 * NSMAX + k]);
      hh = fma(hh, Tn, ch[5 * NSMAX + k]);
      const double z = yn * t.invW[k];
      hs = fma(z, hh, hs);
      sz += z;
    }
    hr = warp_sum(hr);
    hs = warp_sum(hs);
    sz = warp_sum(sz);
    const double u = q[ld];
    const double e_int = R_SI * (hs - Tn * sz);
    const double rhoe = rho * (e_int + 0.5 * (u * u));
    // write Qc = qfToQc(qf) and qf (T, Y); the post-step QcToqf then
    // recovers T from rho e with the Newton solve.
    for (int k = lane; k < ns; k += 32) {
      q[(3 + k) * ld] = w.y0[k];
      Q[(3 + k) * ld] = rho * w.y0[k];
    }
    if (lane == 0) {
      Q[2 * ld] = rhoe;
      L.hrr[cell] = -(hr / dt) * 1e-1;
    }
    __syncwarp();
    // post-step QcToqf: Newton on rho e for T (from 1000 K when strict)
    double T = L.strict_newton ? 1000.0 : Tn;
    const double E = (rhoe / rho - 0.5 * (u * u)) / R_SI;
    double gN = 1e30, dTN = 1e30;
    int it = 0;
    double A[6];
    double Sz = 0.0;
    while (fabs(gN) >= fabs(E) * 1e-9 && fabs(dTN) >= T * 1e-6 && it < 10) {
      // premixed NASA coefficients at the current T (lanes over species)
      double a0 = 0, a1 = 0, a2 = 0, a3 = 0, a4 = 0, a5 = 0, sz_ = 0;
      for (int k = lane; k < ns; k += 32) {
        const int r = (T > t.tmid[k]) ? 1 : 0;
        const double* ch = t.ch + r * 6 * NSMAX;
        const double z = w.y0[k] * t.invW[k];
        a0 = fma(z, ch[0 * NSMAX + k], a0);
        a1 = fma(z, ch[1 * NSMAX + k], a1);
        a2 = fma(z, ch[2 * NSMAX + k], a2);
        a3 = fma(z, ch[3 * NSMAX + k], a3);
        a4 = fma(z, ch[4 * NSMAX + k], a4);
        a5 = fma(z, ch[5 * NSMAX + k], a5);
        sz_ += z;
      }
      A[0] = warp_sum(a0);
      A[1] = warp_sum(a1);
      A[2] = warp_sum(a2);
      A[3] = warp_sum(a3);
      A[4] = warp_sum(a4);
      A[5] = warp_sum(a5);
      Sz = warp_sum(sz_);
      double p = fma(A[4], T, A[3]);
      p = fma(p, T, A[2]);
      p = fma(p, T, A[1]);
      p = fma(p, T, A[0]);
      const double H = fma(p, T, A[5]);
      double cp = fma(5.0 * A[4], T, 4.0 * A[3]);
      cp = fma(cp, T, 3.0 * A[2]);
      cp = fma(cp, T, 2.0 * A[1]);
      cp = fma(cp, T, A[0]);
      gN = H - T * Sz - E;
      dTN = -gN / (cp - Sz);
      T = fmax(20.0, fmin(6000.0, T + dTN));
      ++it;
    }
    if (lane == 0) q[2 * ld] = T;
    // signal speed of the new state for the next time step
    if (L.cvel_out) {
      double a0 = 0, a1 = 0, a2 = 0, a3 = 0, a4 = 0, sz_ = 0;
      for (int k = lane; k < ns; k += 32) {
        const int r = (T > t.tmid[k]) ? 1 : 0;
        const double* ch = t.ch + r * 6 * NSMAX;
        const double z = w.y0[k] * t.invW[k];
        a0 = fma(z, ch[0 * NSMAX + k], a0);
        a1 = fma(z, ch[1 * NSMAX + k], a1);
        a2 = fma(z, ch[2 * NSMAX + k], a2);
        a3 = fma(z, ch[3 * NSMAX + k], a3);
        a4 = fma(z, ch[4 * NSMAX + k], a4);
        sz_ += z;
      }
      a0 = warp_sum(a0);
      a1 = warp_sum(a1);
      a2 = warp_sum(a2);
      a3 = warp_sum(a3);
      a4 = warp_sum(a4);
      sz_ = warp_sum(sz_);
      double cp = fma(5.0 * a4, T, 4.0 * a3);
      cp = fma(cp, T, 3.0 * a2);
      cp = fma(cp, T, 2.0 * a1);
      cp = fma(cp, T, a0);
      const double gamma = cp / (cp - sz_);
      const double sp = fabs(u) + sqrt(gamma * R_SI * T * sz_);
      speed_max = fmax(speed_max, sp);
    }
    __syncwarp();
  }
  if (L.cvel_out && lane == 0 && speed_max > 0.0)
    atomicMax(L.cvel_out, (unsigned long long)__double_as_longlong(speed_max));
  if (L.time) {
    // one CTA advances the clock after all warps of the grid have taken
    // their last cell: count finished CTAs.
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      const unsigned done = atomicAdd(next + 1, 1u);
      if (done == gridDim.x - 1) {
        *L.time = *L.time + dt;
        *L.nsteps = *L.nsteps + 1;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Host: table construction
// ---------------------------------------------------------------------------
struct Blob {
  std::vector<char> b;
  int put(const void* p, size_t bytes) {
    size_t off = (b.size() + 15) / 16 * 16;
    b.resize(off + bytes);
    if (p) std::memcpy(b.data() + off, p, bytes);
    return (int)off;
  }
};

}  // namespace

int chem_init(ChemState& s, const edyn_mech& m, const ThermoTable& tb, cudaStream_t st) {
  (void)tb;
  const int ns = m.nspec, nr = m.nreac;
  if (ns + 1 > 54 + 2 || ns > NSMAX - 8 || nr > 352) return (int)cudaErrorInvalidValue;
  // reaction order: group by kind so a 32-wide round rarely diverges
  std::vector<int> order(nr);
  for (int i = 0; i < nr; ++i) order[i] = i;
  auto kind = [&](int i) {
    if (m.tb[i] == EDYN_TB_FALLOFF) return 0;
    if (m.tb[i] == EDYN_TB_M) return 1;
    const bool ex = !(m.beta[i] == 0.0 && m.E_R[i] == 0.0);
    return ex ? 2 : 3;
  };
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return kind(a) < kind(b); });
  const int nrp = (nr + 31) / 32 * 32;
  std::vector<double> A(nrp, 0.0), B(nrp, 0.0), E(nrp, 0.0), lnA(nrp, -700.0);
  std::vector<unsigned> w0(nrp, 0xffffffu), w1(nrp, 0x08ffffffu), w2(nrp, 0u), w3(nrp, 0u), w4(nrp, 0u), w5(nrp, 0u);
  std::vector<double> aux;
  std::vector<int> spi, tb_sp;
  std::vector<double> tb_am1;
  int nsp = 0;
  // species-major stoichiometry entries
  std::vector<std::vector<std::pair<int, int>>> per_sp(ns);
  for (int q = 0; q < nr; ++q) {
    const int i = order[q];
    A[q] = m.A[i];
    lnA[q] = m.A[i] > 0 ? std::log(m.A[i]) : -700.0;
    B[q] = m.beta[i];
    E[q] = m.E_R[i];
    unsigned fl = 0;
    if (m.rev[i]) fl |= F_REV;
    if (!(m.beta[i] == 0.0 && m.E_R[i] == 0.0)) fl |= F_EXP;
    unsigned rs = 0, ps = 0, nn = 0;
    int dnu = 0;
    for (int sl = 0; sl < 3; ++sl) {
      const int kr = m.nunk[i][sl], kp = m.nunk[i][3 + sl];
      rs |= (unsigned)(kr >= 0 ? kr : 255) << (8 * sl);
      ps |= (unsigned)(kp >= 0 ? kp : 255) << (8 * sl);
      if (kr >= 0) {
        const int v = -m.nu[i][sl];
        if (v < 1 || v > 3) return (int)cudaErrorInvalidValue;
        nn |= (unsigned)v << (4 * sl);
        dnu -= v;
      }
      if (kp >= 0) {
        const int v = m.nu[i][3 + sl];
        if (v < 1 || v > 3) return (int)cudaErrorInvalidValue;
        nn |= (unsigned)v << (12 + 4 * sl);
        dnu += v;
      }
    }
    // net stoichiometry per distinct species
    int ks[6], nus[6], nk = 0;
    for (int sl = 0; sl < 6; ++sl) {
      const int k = m.nunk[i][sl];
      if (k < 0) continue;
      int f = -1;
      for (int z = 0; z < nk; ++z)
        if (ks[z] == k) f = z;
      if (f < 0) { ks[nk] = k; nus[nk] = 0; f = nk++; }
      nus[f] += m.nu[i][sl];
    }
    int nk2 = 0;
    for (int z = 0; z < nk; ++z)
      if (nus[z] != 0) { ks[nk2] = ks[z]; nus[nk2] = nus[z]; ++nk2; }
    for (int z = 0; z < nk2; ++z) per_sp[ks[z]].push_back({q, nus[z]});
    unsigned v3 = 0, v4 = 0, v5 = 0;
    for (int z = 0; z < 6; ++z) {
      const unsigned k = z < nk2 ? (unsigned)ks[z] : 255u;
      const unsigned nu = (unsigned)((z < nk2 ? nus[z] : 0) + 8);
      if (z < 4) { v3 |= k << (8 * z); v4 |= nu << (16 + 4 * z); }
      else { v4 |= k << (8 * (z - 4)); v5 |= nu << (4 * (z - 4)); }
    }
    v5 |= (unsigned)nk2 << 8;
    unsigned ax = 0;
    if (m.tb[i] != EDYN_TB_NONE) {
      ax = (unsigned)nsp++;
      if (m.tb[i] == EDYN_TB_FALLOFF) {
        fl |= F_FALL;
        if (m.kfal[i] >= 0) fl |= F_KFAL; else fl |= F_CM;
      } else {
        fl |= F_CM | F_TB;
      }
      double a9[9] = {m.low[i][0], m.low[i][1], m.low[i][2], m.troe[i][0], m.troe[i][1], m.troe[i][2], m.troe[i][3],
                      (double)m.ifop[i], m.low[i][0] > 0 ? std::log(m.low[i][0]) : -700.0};
      aux.insert(aux.end(), a9, a9 + 9);
      spi.push_back((int)tb_sp.size());
      spi.push_back(m.neff[i]);
      spi.push_back(m.kfal[i]);
      spi.push_back(0);
      for (int z = 0; z < m.neff[i]; ++z) {
        tb_sp.push_back(m.eff_sp[i][z]);
        tb_am1.push_back(m.eff_val[i][z] - 1.0);
      }
    }
    w0[q] = rs | (fl << 24);
    w1[q] = ps | ((unsigned)(dnu + 8) << 24);
    w2[q] = nn | (ax << 24);
    w3[q] = v3;
    w4[q] = v4;
    w5[q] = v5;
  }
  // pieces of at most CH entries, greedily balanced over 32 lanes
  int nent = 0;
  for (int k = 0; k < ns; ++k) nent += (int)per_sp[k].size();
  const int CH = std::max(8, (nent + 31) / 32);
  struct Piece { int k, e0, e1; };
  std::vector<unsigned> ent;
  std::vector<Piece> pieces;
  std::vector<int> spc(NSMAX + 1, 0);
  for (int k = 0; k < ns; ++k) {
    const int b = (int)ent.size();
    for (auto& pr : per_sp[k]) ent.push_back((unsigned)pr.first | ((unsigned)(pr.second + 8) << 16));
    const int e = (int)ent.size();
    for (int x = b; x < e; x += CH) pieces.push_back({k, x, std::min(e, x + CH)});
    if (b == e) pieces.push_back({k, b, b});
  }
  const int npc = (int)pieces.size();
  if (npc > 128) return (int)cudaErrorInvalidValue;
  std::vector<int> idx(npc);
  for (int p = 0; p < npc; ++p) idx[p] = p;
  std::sort(idx.begin(), idx.end(), [&](int a, int b) {
    return (pieces[a].e1 - pieces[a].e0) > (pieces[b].e1 - pieces[b].e0);
  });
  std::vector<int> load(32, 0);
  std::vector<std::vector<int>> lane_p(32);
  for (int p : idx) {
    int best = 0;
    for (int l = 1; l < 32; ++l)
      if (load[l] < load[best]) best = l;
    lane_p[best].push_back(p);
    load[best] += pieces[p].e1 - pieces[p].e0;
  }
  // pieces in lane order; part[] slot = position in that order
  std::vector<int> pc, lane(33, 0), slot_of(npc);
  for (int l = 0; l < 32; ++l) {
    lane[l] = (int)pc.size() / 3;
    for (int p : lane_p[l]) {
      slot_of[p] = (int)pc.size() / 3;
      pc.push_back(pieces[p].k);
      pc.push_back(pieces[p].e0);
      pc.push_back(pieces[p].e1);
    }
  }
  lane[32] = (int)pc.size() / 3;
  std::vector<int> spp;
  for (int k = 0; k < ns; ++k) {
    spc[k] = (int)spp.size();
    for (int p = 0; p < npc; ++p)
      if (pieces[p].k == k) spp.push_back(slot_of[p]);
  }
  for (int k = ns; k <= NSMAX; ++k) spc[k] = (int)spp.size();
  // species tables
  std::vector<double> W(NSMAX, 1.0), invW(NSMAX, 0.0), tmid(NSMAX, 1000.0), hf(NSMAX, 0.0);
  std::vector<double> cs(2 * 7 * NSMAX, 0.0), ch(2 * 6 * NSMAX, 0.0);
  for (int k = 0; k < ns; ++k) {
    W[k] = m.W[k];
    invW[k] = 1.0 / m.W[k];
    tmid[k] = m.T_mid[k];
    for (int r = 0; r < 2; ++r) {
      const double* a = m.a[k][r];
      cs[(r * 7 + 0) * NSMAX + k] = a[0];
      cs[(r * 7 + 1) * NSMAX + k] = a[1] / 2.0;
      cs[(r * 7 + 2) * NSMAX + k] = a[2] / 6.0;
      cs[(r * 7 + 3) * NSMAX + k] = a[3] / 12.0;
      cs[(r * 7 + 4) * NSMAX + k] = a[4] / 20.0;
      cs[(r * 7 + 5) * NSMAX + k] = a[5];
      cs[(r * 7 + 6) * NSMAX + k] = a[6];
      ch[(r * 6 + 0) * NSMAX + k] = a[0];
      ch[(r * 6 + 1) * NSMAX + k] = a[1] / 2.0;
      ch[(r * 6 + 2) * NSMAX + k] = a[2] / 3.0;
      ch[(r * 6 + 3) * NSMAX + k] = a[3] / 4.0;
      ch[(r * 6 + 4) * NSMAX + k] = a[4] / 5.0;
      ch[(r * 6 + 5) * NSMAX + k] = a[5];
    }
    // CKHMS(298.15) [erg/g], as set_thermo stores std_heat_formation
    const double T = 298.15;
    const double* a = m.a[k][T > m.T_mid[k] ? 1 : 0];
    double tn[5] = {1.0, T / 2.0, T * T / 3.0, (T * T) * T / 4.0, (T * T) * (T * T) / 5.0};
    double sum = 0.0;
    for (int q = 0; q < 5; ++q) sum += tn[q] * a[q];
    hf[k] = T * RU_CGS * (sum + a[5] / T) / m.W[k];
  }
  TabHdr h;
  std::memset(&h, 0, sizeof(h));
  Blob bl;
  bl.put(&h, sizeof(h));
  h.ns = ns;
  h.nr = nr;
  h.nrp = nrp;
  h.nsp = nsp;
  h.npc = npc;
  h.ntbl = (int)tb_sp.size();
  h.nent = (int)ent.size();
  h.o_A = bl.put(A.data(), A.size() * 8);
  h.o_B = bl.put(B.data(), B.size() * 8);
  h.o_E = bl.put(E.data(), E.size() * 8);
  h.o_lnA = bl.put(lnA.data(), lnA.size() * 8);
  h.o_w0 = bl.put(w0.data(), w0.size() * 4);
  h.o_w1 = bl.put(w1.data(), w1.size() * 4);
  h.o_w2 = bl.put(w2.data(), w2.size() * 4);
  h.o_w3 = bl.put(w3.data(), w3.size() * 4);
  h.o_w4 = bl.put(w4.data(), w4.size() * 4);
  h.o_w5 = bl.put(w5.data(), w5.size() * 4);
  h.o_sp_aux = bl.put(aux.data(), std::max<size_t>(8, aux.size() * 8));
  h.o_sp_i = bl.put(spi.data(), std::max<size_t>(4, spi.size() * 4));
  h.o_tb_am1 = bl.put(tb_am1.data(), std::max<size_t>(8, tb_am1.size() * 8));
  h.o_tb_sp = bl.put(tb_sp.data(), std::max<size_t>(4, tb_sp.size() * 4));
  h.o_W = bl.put(W.data(), NSMAX * 8);
  h.o_invW = bl.put(invW.data(), NSMAX * 8);
  h.o_tmid = bl.put(tmid.data(), NSMAX * 8);
  h.o_hf = bl.put(hf.data(), NSMAX * 8);
  h.o_cs = bl.put(cs.data(), cs.size() * 8);
  h.o_ch = bl.put(ch.data(), ch.size() * 8);
  h.o_pc = bl.put(pc.data(), pc.size() * 4);
  h.o_lane = bl.put(lane.data(), lane.size() * 4);
  h.o_spc = bl.put(spc.data(), spc.size() * 4);
  h.o_spp = bl.put(spp.data(), std::max<size_t>(4, spp.size() * 4));
  h.o_ent = bl.put(ent.data(), std::max<size_t>(4, ent.size() * 4));
  bl.put(nullptr, 16);
  size_t tot = (bl.b.size() + 255) / 256 * 256;
  bl.b.resize(tot, 0);
  h.total_bytes = (int)tot;
  std::memcpy(bl.b.data(), &h, sizeof(h));
  cudaError_t e = cudaMalloc(&s.d_tables, tot);
  if (e != cudaSuccess) return (int)e;
  e = cudaMemcpyAsync(s.d_tables, bl.b.data(), tot, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return (int)e;
  cudaStreamSynchronize(st);
  s.table_bytes = tot;
  s.ns = ns;
  s.nr = nr;
  s.nr_pad = nrp;
  e = cudaMalloc(&s.d_next, 2 * sizeof(unsigned));
  if (e != cudaSuccess) return (int)e;
  e = cudaMalloc(&s.d_count, sizeof(ChemCounters));
  if (e != cudaSuccess) return (int)e;
  cudaMemsetAsync(s.d_count, 0, sizeof(ChemCounters), st);
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  s.warps = WARPS;
  s.smem = tot + sizeof(WarpWork) * WARPS;
  int maxs = 0;
  cudaDeviceGetAttribute(&maxs, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if ((int)s.smem > maxs) return (int)cudaErrorInvalidConfiguration;
  e = cudaFuncSetAttribute(k_reactors, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s.smem);
  if (e != cudaSuccess) return (int)e;
  e = cudaFuncSetAttribute(k_tube_chem, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s.smem);
  if (e != cudaSuccess) return (int)e;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_reactors, WARPS * 32, s.smem);
  s.ctas = nsm * std::max(1, per_sm);
  return 0;
}

cudaError_t chem_launch_batch(ChemState& s, const ChemLaunch& L, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(s.d_next, 0, 2 * sizeof(unsigned), st);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(s.d_count, 0, sizeof(ChemCounters), st);
  if (e != cudaSuccess) return e;
  const int grid = std::min(s.ctas, (L.n + WARPS - 1) / WARPS);
  k_reactors<<<std::max(1, grid), WARPS * 32, s.smem, st>>>((const char*)s.d_tables, (int)s.table_bytes, L.n,
                                                            L.rho_batch, L.dt_batch, L.yiT_batch, L.rtol, L.atol,
                                                            s.d_next, s.d_count, L.err);
  return cudaGetLastError();
}

cudaError_t chem_launch_tube(ChemState& s, const ChemLaunch& L, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(s.d_next, 0, 2 * sizeof(unsigned), st);
  if (e != cudaSuccess) return e;
  const int grid = std::min(s.ctas, (L.n + WARPS - 1) / WARPS);
  k_tube_chem<<<std::max(1, grid), WARPS * 32, s.smem, st>>>((const char*)s.d_tables, (int)s.table_bytes, L,
                                                             s.d_next, s.d_count);
  return cudaGetLastError();
}

cudaError_t chem_read_counters(ChemState& s, ChemCounters* out, cudaStream_t st) {
  cudaError_t e = cudaMemcpyAsync(out, s.d_count, sizeof(ChemCounters), cudaMemcpyDeviceToHost, st);
  if (e != cudaSuccess) return e;
  return cudaStreamSynchronize(st);
}

void chem_free(ChemState& s) {
  cudaFree(s.d_tables);
  cudaFree(s.d_next);
  cudaFree(s.d_count);
  s.d_tables = nullptr;
  s.d_next = nullptr;
  s.d_count = nullptr;
}

}  // namespace edyn
