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
#include "fastmath.cuh"

namespace edyn {

namespace {

constexpr int NSMAX = 64;
constexpr int NV = 56;      // padded state vector length (54 used for GRI)
constexpr int MAXW = 8;     // warps per CTA at most; the launch uses what shared memory allows
constexpr int JS = 55;      // FP32 matrix row stride (odd: conflict-free column walks)
constexpr int AUXW = 11;    // values per third-body / fall-off reaction in the aux table

// SDIRK4 (Hairer & Wanner, Solving ODEs II, Table 6.5), gamma = 1/4.
__constant__ double c_sa[5][5] = {{0.25, 0, 0, 0, 0},
                                  {0.5, 0.25, 0, 0, 0},
                                  {17.0 / 50.0, -1.0 / 25.0, 0.25, 0, 0},
                                  {371.0 / 1360.0, -137.0 / 2720.0, 15.0 / 544.0, 0.25, 0},
                                  {25.0 / 24.0, -49.0 / 48.0, 125.0 / 16.0, -85.0 / 12.0, 0.25}};
__constant__ double c_se[5] = {25.0 / 24.0 - 59.0 / 48.0, -49.0 / 48.0 + 17.0 / 96.0, 125.0 / 16.0 - 225.0 / 32.0,
                               0.0, 0.25};

// Packed table header (all offsets in bytes from the blob start). Every
// real-valued table is stored twice, in FP64 for the residual and in FP32
// for the Jacobian, so neither path converts between precisions.
struct TabHdr {
  int ns, nr, nrp, nsp, npc, ntbl, total_bytes, nent;
  int o_w0, o_w1, o_w2, o_w3, o_w4, o_w5;  // uint[nrp]
  int o_sp_i;                 // int[nsp*4]: tb_off, tb_cnt, kfal (-1 mixture), flags
  int o_tb_sp;                // int[ntbl]
  int o_pc;                   // int[npc*3]: species, entry begin, entry end
  int o_lane;                 // int[33]: piece range per lane
  int o_spc;                  // int[NSMAX+1]: piece range per species
  int o_spp;                  // int[npc]: piece index list ordered by species
  int o_ent;                  // uint[nent]: scheduled reaction index
  // real tables: [0] FP64 offset, [1] FP32 offset
  int o_A[2], o_lnA[2], o_B[2], o_E[2];  // [nrp]
  int o_aux[2];                // [nsp*AUXW]: lowA lowB lowE troe_a T3 T1 T2 ifop ln(lowA) 1/T3 1/T1;
                               // the FP64 copy holds lowA/A, lowB - B, lowE - E in the first three
  int o_tb_am1[2];             // [ntbl]
  int o_W[2], o_invW[2], o_tmid[2], o_hf[2];  // [NSMAX]
  int o_cs[2];                 // [2][7][NSMAX] S/R - H/RT coefficients
  int o_ch[2];                 // [2][6][NSMAX] H/R coefficients (a1, a2/2, .., a6)
  int o_cp[2];                 // [2][5][NSMAX] Cp/R coefficients (a1..a5)
  int o_nu[2];                 // [nent] net stoichiometric coefficient of each entry
  int o_e2;                    // double[64]: 2^(j/64), the table of texp
  int o_lg;                    // double[2][92]: ln(j/128), 128/j for j = 90..181, the tables of tlog
  int fr0, nfr;                // the fall-off reactions fill rounds [fr0, fr0 + nfr) of 32
  int o_grp;                   // int4[TEAM]: per team lane: species (-1 none), entry begin, end, group size
  int gmax;                    // largest species group of the team production rates
  int o_smap;                  // int[NSMAX]: tube row of each species (3 + smap[k]); identity unless a subset
  int nnorm;                   // components counted in the RMS norms: the full mechanism's ns + 1
};

template <class R>
struct RTabs {
  const R *A, *lnA, *B, *E, *aux, *tb_am1, *W, *invW, *tmid, *hf, *cs, *ch, *cp, *nu;
};

struct Tabs {
  const TabHdr* h;
  const unsigned *w0, *w1, *w2, *w3, *w4, *w5, *ent;
  const int *spi, *tb_sp, *pc, *lane, *spc, *spp;
  const int4* grp;
  const int* smap;
  const double* e2;
  const double* lg;
  int ns, nr, nrp, npc;
  RTabs<double> d;
  RTabs<float> f;
  template <class R>
  __device__ __forceinline__ const RTabs<R>& r() const;
};
template <>
__device__ __forceinline__ const RTabs<double>& Tabs::r<double>() const { return d; }
template <>
__device__ __forceinline__ const RTabs<float>& Tabs::r<float>() const { return f; }

template <class R>
__device__ __forceinline__ void bind_real(RTabs<R>& x, const char* base, const TabHdr& h, int p) {
  x.A = (const R*)(base + h.o_A[p]);
  x.lnA = (const R*)(base + h.o_lnA[p]);
  x.B = (const R*)(base + h.o_B[p]);
  x.E = (const R*)(base + h.o_E[p]);
  x.aux = (const R*)(base + h.o_aux[p]);
  x.tb_am1 = (const R*)(base + h.o_tb_am1[p]);
  x.W = (const R*)(base + h.o_W[p]);
  x.invW = (const R*)(base + h.o_invW[p]);
  x.tmid = (const R*)(base + h.o_tmid[p]);
  x.hf = (const R*)(base + h.o_hf[p]);
  x.cs = (const R*)(base + h.o_cs[p]);
  x.ch = (const R*)(base + h.o_ch[p]);
  x.cp = (const R*)(base + h.o_cp[p]);
  x.nu = (const R*)(base + h.o_nu[p]);
}

__device__ __forceinline__ Tabs bind_tabs(const char* base) {
  Tabs t;
  t.h = (const TabHdr*)base;
  const TabHdr& h = *t.h;
  t.w0 = (const unsigned*)(base + h.o_w0);
  t.w1 = (const unsigned*)(base + h.o_w1);
  t.w2 = (const unsigned*)(base + h.o_w2);
  t.w3 = (const unsigned*)(base + h.o_w3);
  t.w4 = (const unsigned*)(base + h.o_w4);
  t.w5 = (const unsigned*)(base + h.o_w5);
  t.spi = (const int*)(base + h.o_sp_i);
  t.tb_sp = (const int*)(base + h.o_tb_sp);
  t.pc = (const int*)(base + h.o_pc);
  t.lane = (const int*)(base + h.o_lane);
  t.spc = (const int*)(base + h.o_spc);
  t.spp = (const int*)(base + h.o_spp);
  t.grp = (const int4*)(base + h.o_grp);
  t.smap = (const int*)(base + h.o_smap);
  t.ent = (const unsigned*)(base + h.o_ent);
  t.e2 = (const double*)(base + h.o_e2);
  t.lg = (const double*)(base + h.o_lg);
  t.ns = h.ns;
  t.nr = h.nr;
  t.nrp = h.nrp;
  t.npc = h.npc;
  bind_real(t.d, base, h, 0);
  bind_real(t.f, base, h, 1);
  return t;
}

// reaction flag bits (w0 >> 24)
// F_GEN: a side of order above 3, kept as (species, nu) slots; every other
// reaction lists each side as up to three species slots with nu = 1 (2 OH is
// OH, OH), so its concentration products are three plain factors.
constexpr unsigned F_REV = 1, F_CM = 2, F_FALL = 4, F_KFAL = 8, F_EXP = 16, F_TB = 32, F_GEN = 64;

// Per-team shared workspace. A team is the group of threads that works on
// one cell: one warp, or four warps of a CTA (one per SM sub-partition, each
// with its own FP64 unit) for the cells that cost the most.
struct alignas(16) WarpWork {
  double y0[NV], Y[NV], sv[NV], fy[NV], F[5][NV], dl[NV];
  double C[NV], m[NV], uR[NV], cvm[NV], wdot[NV];
  double part[100];
  double rop[352];
  int en[NV];
  float J[54 * JS];   // Jacobian, then the inverse of the scaled Newton matrix
  float b32[NV];
  float sc32[NV];     // error weights atol + rtol |y0| of the current Newton matrix
  float isc32[NV];    // their reciprocals
  float col[NV];      // pivot column during the inversion
  int piv[NV];
  float f1[NV], f2[NV];
  float yf[NV];       // FP32 copy of the state for the Jacobian
};

constexpr int TEAM = 128;        // threads of a four-warp team
constexpr int TEAM_PIECES = 128; // gather pieces per warp row of a team's partial sums
constexpr int HOT_MIN_RHS = 32;  // right-hand sides in the last call that make a cell hot

__device__ __forceinline__ double clip0_d(double x) { return __double_as_longlong(x) < 0 ? 0.0 : x; }

template <class R>
__device__ __forceinline__ R warp_sum(R v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
// Lane that holds value i of N after warp_sumv's halving levels.
__host__ __device__ constexpr int sumv_lane(int i, int n) {
  int lane = 0;
  for (int o = 16; o > 0 && n > 1; o >>= 1) {
    const int h = (n + 1) / 2;
    if (i >= h) {
      lane |= o;
      i -= h;
    }
    n = h;
  }
  return lane;
}

// N warp sums at once, bit for bit the sums of warp_sum (the same pairs are
// added at each level), with fewer additions: at each butterfly level a lane
// keeps half of the values and adds its partner's copies of them, so N = 7
// takes 9 additions per lane instead of 35. Every lane receives all N sums.
template <class R, int N>
__device__ __forceinline__ void warp_sumv(R (&v)[N]) {
  const int lane = threadIdx.x & 31;
  R a[N];
#pragma unroll
  for (int j = 0; j < N; ++j) a[j] = v[j];
  int m = N;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    if (m > 1) {
      const int h = (m + 1) / 2;
      const bool low = (lane & o) == 0;
#pragma unroll
      for (int j = 0; j < N; ++j) {
        if (j < h) {
          const R hi = (h + j < m) ? a[h + j] : (R)0;
          const R mine = low ? a[j] : hi;
          const R send = low ? hi : a[j];
          a[j] = mine + __shfl_xor_sync(0xffffffffu, send, o);
        }
      }
      m = h;
    } else {
      a[0] += __shfl_xor_sync(0xffffffffu, a[0], o);
    }
  }
#pragma unroll
  for (int j = 0; j < N; ++j) v[j] = __shfl_sync(0xffffffffu, a[0], sumv_lane(j, N));
}

template <class R>
__device__ __forceinline__ R warp_max(R v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Team primitives. TW = 32: one warp, warp-synchronous. TW = 128: four warps
// of one CTA synchronised by a named barrier; cross-warp reductions go
// through `red` in a fixed order, so results do not depend on timing.
template <int TW>
struct Team {
  int tid;        // thread index within the team
  int bar;        // named barrier id (four-warp teams)
  double* red;    // cross-warp scratch, 256 doubles (four-warp teams)
  double* part4;  // gather partial sums, [4][TEAM_PIECES] (four-warp teams)
  double* pre;    // temperature-only rate parts, 480 doubles (four-warp teams)
  float* jsave;   // the Jacobian kept across steps (four-warp teams; warps rebuild it)
  // per-warp partial Jacobians and collider rows of warps 1-3 (four-warp
  // teams): each warp accumulates its reactions' terms in its own buffers,
  // which are then added in warp order, so the result does not depend on
  // how the warps' shared-memory atomics interleave
  float* jp[3];
  float* rp[3];
  __device__ __forceinline__ void sync() const {
    if constexpr (TW == 32) {
      __syncwarp();
    } else {
      asm volatile("bar.sync %0, %1;" ::"r"(bar), "n"(TW) : "memory");
    }
  }
  template <class R>
  __device__ __forceinline__ R sum(R v) const {
    v = warp_sum(v);
    if constexpr (TW == 32) {
      return v;
    } else {
      R* r = reinterpret_cast<R*>(red);
      if ((tid & 31) == 0) r[tid >> 5] = v;
      sync();
      R s = r[0];
#pragma unroll
      for (int q = 1; q < TW / 32; ++q) s += r[q];
      sync();
      return s;
    }
  }
  template <class R, int N>
  __device__ __forceinline__ void sumv(R (&v)[N]) const {
    if constexpr (N == 1) {
      v[0] = warp_sum(v[0]);
    } else {
      warp_sumv(v);
    }
    if constexpr (TW > 32) {
      R* r = reinterpret_cast<R*>(red);
      if ((tid & 31) == 0) {
#pragma unroll
        for (int j = 0; j < N; ++j) r[j * 4 + (tid >> 5)] = v[j];
      }
      sync();
#pragma unroll
      for (int j = 0; j < N; ++j) {
        R s = r[j * 4];
#pragma unroll
        for (int q = 1; q < TW / 32; ++q) s += r[j * 4 + q];
        v[j] = s;
      }
      sync();
    }
  }
};

// A producer / consumer named barrier between two warps of a four-warp team
// (id 2; the team itself uses id 1): the producer arrives without
// waiting, the consumer waits until the producer's earlier shared-memory
// writes are visible.
constexpr int BAR_FALL_MA = 2;  // warp 1 -> warp 3: the fall-off concentration products
__device__ __forceinline__ void pair_arrive(int id) {
  __syncwarp();
  asm volatile("bar.arrive %0, 64;" ::"r"(id) : "memory");
}
__device__ __forceinline__ void pair_wait(int id) {
  __syncwarp();
  asm volatile("bar.sync %0, 64;" ::"r"(id) : "memory");
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

// exp in the rate evaluation: the table method in FP64, the SFU in FP32
template <class R>
__device__ __forceinline__ R ex_t(R x, const Tabs& t);
template <>
__device__ __forceinline__ double ex_t<double>(double x, const Tabs& t) { return texp(x, t.e2); }
template <>
__device__ __forceinline__ float ex_t<float>(float x, const Tabs& t) { return __expf(x); }

// ln and log10 in the rate evaluation: the table method in FP64, the SFU in FP32
template <class R>
__device__ __forceinline__ R lg_t(R x, const Tabs& t);
template <>
__device__ __forceinline__ double lg_t<double>(double x, const Tabs& t) { return tlog(x, t.lg); }
template <>
__device__ __forceinline__ float lg_t<float>(float x, const Tabs& t) { return __logf(x); }
template <class R>
__device__ __forceinline__ R l10_t(R x, const Tabs& t) {
  if constexpr (sizeof(R) == sizeof(double)) return tlog(x, t.lg) * 0.43429448190325182765;
  else return __log10f(x);
}

__device__ __forceinline__ unsigned sp_of(unsigned w, int s) { return (w >> (8 * s)) & 0xffu; }

// Rate constants of one reaction (CKRATT + the third-body/fall-off part of
// CKRATX) and its net rate of progress, in pieces that the four-warp FP64
// right-hand side also uses with precomputed temperature-only parts. invKc
// uses the scaled species exponentials m[k] 2^en[k] = exp(S_k/R - H_k/RT).
template <class R>
struct RxnEval {
  R kf, kr, qf, qr, cm, pr, pcor_d;  // pcor_d: d ln(pcor)/d ln(CM) (fall-off, F held fixed)
};

// Arrhenius k = A exp(beta ln T - E/T) (CKRATT 6645), as the reference
// evaluates it in FP64; FP32 (Jacobian only) uses the logarithmic form since
// pre-exponentials up to 1e74 do not fit in single precision.
template <class R>
__device__ __forceinline__ R arrhenius(const Tabs& t, int i, unsigned fl, R logT, R invT) {
  const RTabs<R>& x = t.r<R>();
  if constexpr (sizeof(R) == sizeof(double)) {
    R kf = x.A[i];
    if (fl & F_EXP) kf = kf * texp_a(x.B[i] * logT - x.E[i] * invT, t.e2);
    return kf;
  } else {
    return Math<R>::ex(x.lnA[i] + x.B[i] * logT - x.E[i] * invT);
  }
}

// 1/Kc = exp(-sum nu (S/R - H/RT)) * pfac^(-sum nu)  (CKRATT, 6647-6667),
// from the scaled species exponentials m 2^en and their reciprocals
template <class R>
__device__ __forceinline__ R inv_kc(unsigned w0, unsigned w1, unsigned w2, R pfac, R ipfac, const R* m, const R* mi,
                                    const int* en) {
  using M = Math<R>;
  R mant = 1;
  int ex2 = 0;
#pragma unroll
  for (int s = 0; s < 3; ++s) {
    const unsigned kr_ = sp_of(w0, s), kp = sp_of(w1, s);
    const int nr_ = (w2 >> (4 * s)) & 15, np = (w2 >> (12 + 4 * s)) & 15;
    if (kr_ != 255u) {
      const R mm = m[kr_];
      mant *= (nr_ == 1) ? mm : (nr_ == 2 ? mm * mm : mm * mm * mm);
      ex2 += nr_ * en[kr_];
    }
    if (kp != 255u) {
      const R mm = mi[kp];
      mant *= (np == 1) ? mm : (np == 2 ? mm * mm : mm * mm * mm);
      ex2 -= np * en[kp];
    }
  }
  const int dnu = (int)(w1 >> 24) - 8;
  R ikc;
  if constexpr (sizeof(R) == sizeof(double)) {
    // mant (a product of at most six factors in [0.7, 1.42]) times 2^ex2
    // from its exponent bits. From 2^900 on, the result with up to three
    // factors ipfac <= 7e5 could pass the cap kr = kf / max(Kc, SMALL), and
    // the cap stands for it; 2^-1000 and below are zero.
    if (ex2 >= 900) return M::big();
    ikc = (ex2 <= -1000) ? 0.0 : mant * __hiloint2double((ex2 + 1023) << 20, 0);
  } else {
    ikc = M::ldx(mant, ex2);
  }
  // pfac^(-dnu); |dnu| <= 3 for three-slot reactions
  const R pm = dnu > 0 ? ipfac : pfac;
  for (int q = dnu > 0 ? dnu : -dnu; q > 0; --q) ikc = ikc * pm;
  if constexpr (sizeof(R) != sizeof(double)) ikc = fmin(ikc, M::big());
  return ikc;
}

// third-body concentration: a named collider (fall-off "(+X)") or the mixture
// with efficiencies (CKRATX 6860-6890)
template <class R>
__device__ __forceinline__ R collider(const Tabs& t, unsigned fl, int aux, R ctot, const R* C) {
  const RTabs<R>& x = t.r<R>();
  if (fl & F_KFAL) return C[t.spi[aux * 4 + 2]];
  R cm = ctot;
  const int b = t.spi[aux * 4 + 0], c = t.spi[aux * 4 + 1];
  for (int q = b; q < b + c; ++q) cm += x.tb_am1[q] * C[t.tb_sp[q]];
  return cm;
}

// log10 of the Troe centering factor (temperature only; CKRATX 6895-6905)
template <class R>
__device__ __forceinline__ R troe_fclog(const Tabs& t, const R* fp, int ifop, R T, R invT) {
  using M = Math<R>;
  // -T/T*** and -T/T* with reciprocals precomputed on the host
  R fcent, f3 = 0;
  if constexpr (sizeof(R) == sizeof(double)) {
    fcent = (1 - fp[3]) * texp_a(-T * fp[9], t.e2) + fp[3] * texp_a(-T * fp[10], t.e2);
    if (ifop == 4) f3 = texp_a(-fp[6] * invT, t.e2);
  } else {
    fcent = (1 - fp[3]) * ex_t<R>(-T * fp[9], t) + fp[3] * ex_t<R>(-T * fp[10], t);
    if (ifop == 4) f3 = ex_t<R>(-fp[6] * invT, t);
  }
  fcent += f3;
  return l10_t<R>(fmax(fcent, M::small()), t);
}

// fall-off blending factor pr/(1+pr) F from the reduced pressure and, for
// Troe, log10 Fcent (the CHEMKIN-II single-precision constants widened)
template <class R>
__device__ __forceinline__ R falloff_pcor(const Tabs& t, R pr, int ifop, R fclog) {
  using M = Math<R>;
  R pcor = pr / (1 + pr);
  if (ifop > 1) {
    const R prlog = l10_t<R>(fmax(pr, M::small()), t);
    const R xn = (R)0.75 - (R)(double)1.27f * fclog;
    const R cprlog = prlog - ((R)(double)0.4f + (R)(double)0.67f * fclog);
    const R q = cprlog / (xn - (R)(double)0.14f * cprlog);
    const R flog = fclog / (1 + q * q);
    if constexpr (sizeof(R) == sizeof(double)) pcor = texp_a(2.302585092994045684 * flog, t.e2) * pcor;  // 10^flog
    else pcor = Math<R>::ex((R)2.302585092994045684 * flog) * pcor;
  }
  return pcor;
}

// FP64 form of falloff_pcor with one reciprocal: with c = log10 Pr -
// (0.4 + 0.67 log10 Fc) and d = 0.75 - 1.27 log10 Fc - 0.14 c, Troe's
// 1 + (c/d)^2 is e/d^2 for e = d^2 + c^2, and 1/((1 + Pr) e) gives both
// 1/(1 + Pr) and 1/e. The same quantities as falloff_pcor<double> up to
// rounding; beyond Pr = 1e150 the two reciprocals are taken apart.
__device__ __forceinline__ double log10_pr(const Tabs& t, double pr) {
  return tlog(fmax(pr, Math<double>::small()), t.lg) * 0.43429448190325182765;
}

// The Troe branch of falloff_pcor_d from Pr and log10 Pr.
__device__ __forceinline__ double troe_pcor_d(const Tabs& t, double pr, double prlog, double fclog) {
  const double p1 = 1.0 + pr;
  const double c = prlog - ((double)0.4f + (double)0.67f * fclog);
  const double d = (0.75 - (double)1.27f * fclog) - (double)0.14f * c;
  const double d2 = d * d;
  const double e = fma(c, c, d2);
  double inv_p1, inv_e;
  if (pr < 1e150) {
    const double r = 1.0 / (p1 * e);
    inv_p1 = r * e;
    inv_e = r * p1;
  } else {
    inv_p1 = 1.0 / p1;
    inv_e = 1.0 / e;
  }
  const double flog = (fclog * d2) * inv_e;
  return texp_a(2.302585092994045684 * flog, t.e2) * (pr * inv_p1);  // 10^flog Pr/(1+Pr)
}

__device__ __forceinline__ double falloff_pcor_d(const Tabs& t, double pr, int ifop, double fclog) {
  if (ifop <= 1) return pr / (1.0 + pr);
  return troe_pcor_d(t, pr, log10_pr(t, pr), fclog);
}

// mass-action products (CKRATX 6900-6915)
template <class R>
__device__ __forceinline__ void mass_action(unsigned w0, unsigned w1, unsigned w2, const R* C, R& qf, R& qr) {
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
}

template <class R>
__device__ __forceinline__ RxnEval<R> eval_rxn(const Tabs& t, int i, R logT, R invT, R T, R pfac, R ipfac, R ctot,
                                               const R* C, const R* m, const R* mi, const int* en) {
  const RTabs<R>& x = t.r<R>();
  RxnEval<R> o;
  const unsigned w0 = t.w0[i], w1 = t.w1[i], w2 = t.w2[i];
  const unsigned fl = w0 >> 24;
  R kf = arrhenius<R>(t, i, fl, logT, invT);
  R kr = 0;
  if (fl & F_REV) {
    kr = kf * inv_kc<R>(w0, w1, w2, pfac, ipfac, m, mi, en);
    if (sizeof(R) != sizeof(double)) kr = fmin(kr, (R)1e30f);
  }
  o.cm = 1;
  o.pr = 0;
  o.pcor_d = 0;
  const int aux = (int)(w2 >> 24);
  if (fl & (F_CM | F_KFAL)) {
    const R cm = collider<R>(t, fl, aux, ctot, C);
    o.cm = cm;
    if (fl & F_FALL) {
      const R* fp = x.aux + aux * AUXW;
      R pr;
      if constexpr (sizeof(R) == sizeof(double)) pr = fp[0] * texp_a(fp[1] * logT - fp[2] * invT, t.e2) * cm;
      else pr = Math<R>::ex(fp[8] + fp[1] * logT - fp[2] * invT) * cm / kf;
      const int ifop = (int)fp[7];
      const R fclog = (ifop > 1) ? troe_fclog<R>(t, fp, ifop, T, invT) : (R)0;
      const R pcor = falloff_pcor<R>(t, pr, ifop, fclog);
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
  R qf = kf, qr = kr;
  mass_action<R>(w0, w1, w2, C, qf, qr);
  o.kf = kf;
  o.kr = kr;
  o.qf = qf;
  o.qr = qr;
  return o;
}

// Net rate of progress in FP64 from the effective forward constant kfe (kf
// times the collider or fall-off factor) and the species factors of the FP64
// species pass, a_k = m_k pfac and b_k = C_k ipfac / m_k with m_k 2^en_k =
// exp(S_k/R - H_k/RT): qf = kfe prod C_r^nu and, when reversible,
// qr = kfe 2^ex2 prod a_r^nu prod b_p^nu, which is kf / Kc times the
// collider factor and prod C_p^nu of CKRATT/CKRATX with the pressure power
// and the product concentrations folded into b. From 2^900 on, 1/Kc stands
// at the cap kr = kf / max(Kc, SMALL) as in inv_kc.
__device__ __forceinline__ double net_rate_gen(unsigned w0, unsigned w1, unsigned w2, bool rev, double kfe,
                                               const double* C, const double* a, const double* b, const int* en) {
  double qf = kfe, qr = kfe;
  int ex2 = 0;
#pragma unroll
  for (int s = 0; s < 3; ++s) {
    const unsigned kr_ = sp_of(w0, s), kp = sp_of(w1, s);
    const int nr_ = (w2 >> (4 * s)) & 15, np = (w2 >> (12 + 4 * s)) & 15;
    if (kr_ != 255u) {
      const double c = C[kr_], x = a[kr_];
      qf *= (nr_ == 1) ? c : (nr_ == 2 ? c * c : c * c * c);
      qr *= (nr_ == 1) ? x : (nr_ == 2 ? x * x : x * x * x);
      ex2 += nr_ * en[kr_];
    }
    if (kp != 255u) {
      const double x = b[kp];
      qr *= (np == 1) ? x : (np == 2 ? x * x : x * x * x);
      ex2 -= np * en[kp];
    }
  }
  if (!rev) return qf;
  if (ex2 >= 900) {
    qr = kfe * 1e300;
#pragma unroll
    for (int s = 0; s < 3; ++s) {
      const unsigned kp = sp_of(w1, s);
      const int np = (w2 >> (12 + 4 * s)) & 15;
      if (kp != 255u) {
        const double c = C[kp];
        qr *= (np == 1) ? c : (np == 2 ? c * c : c * c * c);
      }
    }
  } else {
    qr = (ex2 <= -1000) ? 0.0 : qr * __hiloint2double((ex2 + 1023) << 20, 0);
  }
  return qf - qr;
}

// Slot form: three factors per side, absent slots (255) count as 1 (selected
// on the integer pipe, so every lane issues the same 11 FP64 instructions).
__device__ __forceinline__ double slot(const double* v, unsigned k) { return k != 255u ? v[k] : 1.0; }
__device__ __forceinline__ int slot_en(const int* en, unsigned k) { return k != 255u ? en[k] : 0; }

__device__ __forceinline__ double net_rate(unsigned w0, unsigned w1, unsigned w2, bool rev, double kfe,
                                           const double* C, const double* a, const double* b, const int* en) {
  if ((w0 >> 24) & F_GEN) return net_rate_gen(w0, w1, w2, rev, kfe, C, a, b, en);
  const unsigned r0 = sp_of(w0, 0), r1 = sp_of(w0, 1), r2 = sp_of(w0, 2);
  const unsigned p0 = sp_of(w1, 0), p1 = sp_of(w1, 1), p2 = sp_of(w1, 2);
  const double qf = (kfe * slot(C, r0)) * (slot(C, r1) * slot(C, r2));
  if (!rev) return qf;
  const int ex2 = slot_en(en, r0) + slot_en(en, r1) + slot_en(en, r2) - slot_en(en, p0) - slot_en(en, p1) -
                  slot_en(en, p2);
  double qr;
  if (ex2 >= 900) {
    // the cap of net_rate_gen: 1/Kc beyond 2^900 stands at 1e300 (pfac powers folded out)
    qr = ((kfe * 1e300) * slot(C, p0)) * (slot(C, p1) * slot(C, p2));
  } else {
    const double fa = slot(a, r0) * (slot(a, r1) * slot(a, r2));
    const double fb = slot(b, p0) * (slot(b, p1) * slot(b, p2));
    qr = (ex2 <= -1000) ? 0.0 : (kfe * __hiloint2double((ex2 + 1023) << 20, 0)) * (fa * fb);
  }
  return qf - qr;
}

// The FP64 net rate of reaction i evaluated from scratch (warp path).
__device__ __forceinline__ double rop_d(const Tabs& t, int i, double logT, double invT, double T, double ctot,
                                       const double* C, const double* a, const double* b, const int* en) {
  const RTabs<double>& x = t.d;
  const unsigned w0 = t.w0[i], w1 = t.w1[i], w2 = t.w2[i];
  const unsigned fl = w0 >> 24;
  // the concentration products with a unit rate constant first: they do not
  // depend on the fall-off chain below, which overlaps their latency
  const double ma = net_rate(w0, w1, w2, (fl & F_REV) != 0, 1.0, C, a, b, en);
  double kf = arrhenius<double>(t, i, fl, logT, invT);
  if (fl & (F_CM | F_KFAL)) {
    const int aux = (int)(w2 >> 24);
    const double cm = collider<double>(t, fl, aux, ctot, C);
    if (fl & F_FALL) {
      const double* fp = x.aux + aux * AUXW;
      const double k0kf = fp[0] * texp_a(fp[1] * logT - fp[2] * invT, t.e2);  // k0 / kinf
      const int ifop = (int)fp[7];
      const double fclog = (ifop > 1) ? troe_fclog<double>(t, fp, ifop, T, invT) : 0.0;
      kf *= falloff_pcor_d(t, k0kf * cm, ifop, fclog);
    } else {
      kf *= cm;
    }
  }
  return kf * ma;
}

// Net rate of progress of reaction i in FP64 from its precomputed Arrhenius
// constant kf and, for fall-off, k0/kinf [aux] and log10 Fcent fcl[aux]: the
// concentration-dependent rest of eval_rxn, with the same arithmetic.
__device__ __forceinline__ double rop_pre(const Tabs& t, int i, double kf, const double* k0a, const double* fcl,
                                          double pfac, double ipfac, double ctot, const double* C, const double* m,
                                          const double* mi, const int* en) {
  (void)pfac;
  (void)ipfac;
  const unsigned w0 = t.w0[i], w1 = t.w1[i], w2 = t.w2[i];
  const unsigned fl = w0 >> 24;
  const int aux = (int)(w2 >> 24);
  const double ma = net_rate(w0, w1, w2, (fl & F_REV) != 0, 1.0, C, m, mi, en);
  if (fl & (F_CM | F_KFAL)) {
    const double cm = collider<double>(t, fl, aux, ctot, C);
    if (fl & F_FALL) {
      kf *= falloff_pcor_d(t, k0a[aux] * cm, (int)t.d.aux[aux * AUXW + 7], fcl[aux]);
    } else {
      kf *= cm;
    }
  }
  return kf * ma;
}

// Thermodynamics of species k: its concentration (returned), scaled
// exp(S/R - H/RT) and its reciprocal, u_k/R and cv_k/(R W_k).
template <class R, bool STORE_C = true>
__device__ __forceinline__ R species_one(const Tabs& t, int k, const R* y, R rho, R T, R logT, R invT, R pfac,
                                         R ipfac, R* C, R* m, R* mi, int* en, R* uR, R* cvm) {
  using M = Math<R>;
  const RTabs<R>& x = t.r<R>();
  const R c = rho * y[k] * x.invW[k];
  if constexpr (STORE_C) C[k] = c;
  const int r = (T > x.tmid[k]) ? 1 : 0;
  const R* cs = x.cs + r * 7 * NSMAX;
  // S/R - H/RT = a1 (lnT - 1) + a2/2 T + a3/6 T^2 + a4/12 T^3 + a5/20 T^4 + a7 - a6/T (CKSMH, 7501)
  R p = fma(cs[4 * NSMAX + k], T, cs[3 * NSMAX + k]);
  p = fma(p, T, cs[2 * NSMAX + k]);
  p = fma(p, T, cs[1 * NSMAX + k]);
  const R smh = fma(p, T, fma(cs[0 * NSMAX + k], logT - 1, cs[6 * NSMAX + k])) - cs[5 * NSMAX + k] * invT;
  // Cody-Waite: smh = n ln2 + r, exp(smh) = exp(r) 2^n
  const R nn = M::rint_(smh * (R)1.4426950408889634);
  const R rr = fma(-nn, (R)6.93147180369123816490e-01, smh) - nn * (R)1.90821492927058770002e-10;
  if constexpr (sizeof(R) == sizeof(double)) {
    // the FP64 rates take the species factors of net_rate: a_k = m_k pfac
    // for reactants, b_k = C_k ipfac / m_k for products
    const double e = texp_r(rr, t.e2);
    m[k] = e * pfac;
    mi[k] = (c * ipfac) * __drcp_rn(e);
  } else {
    m[k] = M::ex(rr);
    mi[k] = M::ex(-rr);
  }
  en[k] = (int)nn;
  const R* ch = x.ch + r * 6 * NSMAX;
  R h = fma(ch[4 * NSMAX + k], T, ch[3 * NSMAX + k]);
  h = fma(h, T, ch[2 * NSMAX + k]);
  h = fma(h, T, ch[1 * NSMAX + k]);
  h = fma(h, T, ch[0 * NSMAX + k]);
  uR[k] = fma(h, T, ch[5 * NSMAX + k]) - T;  // u/R = h/R - T
  const R* cc = x.cp + r * 5 * NSMAX;
  R cp = fma(cc[4 * NSMAX + k], T, cc[3 * NSMAX + k]);
  cp = fma(cp, T, cc[2 * NSMAX + k]);
  cp = fma(cp, T, cc[1 * NSMAX + k]);
  cp = fma(cp, T, cc[0 * NSMAX + k]);
  cvm[k] = (cp - 1) * x.invW[k];
  return c;
}

// Thermodynamic pass over species (threads over k); returns sum of C_k.
template <class R, int TW>
__device__ __forceinline__ R species_pass(const Tabs& t, const Team<TW>& tm, const R* y, R rho, R T, R logT, R invT,
                                          R pfac, R ipfac, R* C, R* m, R* mi, int* en, R* uR, R* cvm) {
  R csum = 0;
  for (int k = tm.tid; k < t.ns; k += TW)
    csum += species_one<R>(t, k, y, rho, T, logT, invT, pfac, ipfac, C, m, mi, en, uR, cvm);
  return tm.sum(csum);
}

// Full right-hand side in precision R. y (shared, R) -> f (shared, R). Wk is
// the team's workspace (only its species exponent slots en are used here).
template <class R, int TW, class Wk>
__device__ void rhs(const Tabs& t, const Team<TW>& tm, Wk& w, const R* y, R rho, R* f, R* C, R* m, R* mi, R* uR,
                    R* cvm, R* rop, R* part) {
  const RTabs<R>& x = t.r<R>();
  const int ns = t.ns;
  const R T = y[ns];
  const R logT = lg_t<R>(T, t);
  const R invT = (R)1 / T;
  const R pfac = (R)(PATM_CGS / RU_CGS) * invT;
  const R ipfac = T * (R)(RU_CGS / PATM_CGS);
  const R ctot = species_pass<R, TW>(t, tm, y, rho, T, logT, invT, pfac, ipfac, C, m, mi, w.en, uR, cvm);
  tm.sync();
  for (int i = tm.tid; i < t.nrp; i += TW) {
    R r = 0;
    if (i < t.nr) {
      if constexpr (sizeof(R) == sizeof(double)) {
        r = rop_d(t, i, logT, invT, T, ctot, C, m, mi, w.en);
      } else {
        RxnEval<R> e = eval_rxn<R>(t, i, logT, invT, T, pfac, ipfac, ctot, C, m, mi, w.en);
        r = e.qf - e.qr;
      }
    }
    rop[i] = r;
  }
  tm.sync();
  // production rates: load-balanced pieces of the species-major list; a
  // four-warp team splits each piece's entries over its warps
  R su = 0, cv = 0;
  if constexpr (TW == 32) {
    for (int p = t.lane[tm.tid]; p < t.lane[tm.tid + 1]; ++p) {
      const int e0 = t.pc[p * 3 + 1], e1 = t.pc[p * 3 + 2];
      R s = 0;
      for (int q = e0; q < e1; ++q) s = fma(x.nu[q], rop[t.ent[q]], s);
      part[p] = s;
    }
    tm.sync();
    for (int k = tm.tid; k < ns; k += TW) {
      R s = 0;
      for (int q = t.spc[k]; q < t.spc[k + 1]; ++q) s += part[t.spp[q]];
      f[k] = s * x.W[k] / rho;
      su = fma(uR[k], s, su);
      cv = fma(y[k], cvm[k], cv);
    }
  } else {
    R* p4 = reinterpret_cast<R*>(tm.part4);
    const int l = tm.tid & 31, wq = tm.tid >> 5;
    for (int p = t.lane[l]; p < t.lane[l + 1]; ++p) {
      const int e0 = t.pc[p * 3 + 1], e1 = t.pc[p * 3 + 2];
      R s = 0;
      for (int q = e0 + wq; q < e1; q += 4) s = fma(x.nu[q], rop[t.ent[q]], s);
      p4[wq * TEAM_PIECES + p] = s;
    }
    tm.sync();
    for (int k = tm.tid; k < ns; k += TW) {
      R s = 0;
      for (int q = t.spc[k]; q < t.spc[k + 1]; ++q) {
        const int pp = t.spp[q];
        s += ((p4[pp] + p4[TEAM_PIECES + pp]) + p4[2 * TEAM_PIECES + pp]) + p4[3 * TEAM_PIECES + pp];
      }
      f[k] = s * x.W[k] / rho;
      su = fma(uR[k], s, su);
      cv = fma(y[k], cvm[k], cv);
    }
  }
  R sc[2] = {su, cv};
  tm.sumv(sc);
  if (tm.tid == 0) f[ns] = -sc[0] / (rho * sc[1]);  // RU cancels in u/cv
  tm.sync();
}

// Species k's FP64 thermodynamics for the rates, as values (species_one's
// FP64 branch without its stores, so that a caller can interleave it with
// independent work and store under a predicate).
struct SpeciesVals {
  double m, mi, uR, cvm;
  int en;
};
__device__ __forceinline__ SpeciesVals species_vals(const Tabs& t, int k, double c, double T, double logT,
                                                    double invT, double pfac, double ipfac) {
  const RTabs<double>& x = t.d;
  SpeciesVals o;
  const int r = (T > x.tmid[k]) ? 1 : 0;
  const double* cs = x.cs + r * 7 * NSMAX;
  double p = fma(cs[4 * NSMAX + k], T, cs[3 * NSMAX + k]);
  p = fma(p, T, cs[2 * NSMAX + k]);
  p = fma(p, T, cs[1 * NSMAX + k]);
  const double smh = fma(p, T, fma(cs[0 * NSMAX + k], logT - 1, cs[6 * NSMAX + k])) - cs[5 * NSMAX + k] * invT;
  const double nn = Math<double>::rint_(smh * 1.4426950408889634);
  const double rr = fma(-nn, 6.93147180369123816490e-01, smh) - nn * 1.90821492927058770002e-10;
  const double e = texp_r(rr, t.e2);
  o.m = e * pfac;
  o.mi = (c * ipfac) * __drcp_rn(e);
  o.en = (int)nn;
  const double* ch = x.ch + r * 6 * NSMAX;
  double h = fma(ch[4 * NSMAX + k], T, ch[3 * NSMAX + k]);
  h = fma(h, T, ch[2 * NSMAX + k]);
  h = fma(h, T, ch[1 * NSMAX + k]);
  h = fma(h, T, ch[0 * NSMAX + k]);
  o.uR = fma(h, T, ch[5 * NSMAX + k]) - T;
  const double* cc = x.cp + r * 5 * NSMAX;
  double cp = fma(cc[4 * NSMAX + k], T, cc[3 * NSMAX + k]);
  cp = fma(cp, T, cc[2 * NSMAX + k]);
  cp = fma(cp, T, cc[1 * NSMAX + k]);
  cp = fma(cp, T, cc[0 * NSMAX + k]);
  o.cvm = (cp - 1) * x.invW[k];
  return o;
}

// arrhenius<double> without a branch: a reaction without an exponential
// factor takes texp_a(0) = 1 exactly, so the value is the same.
__device__ __forceinline__ double arrhenius_bl(const Tabs& t, int i, double logT, double invT) {
  const RTabs<double>& x = t.d;
  const bool ex = ((t.w0[i] >> 24) & F_EXP) != 0;
  return x.A[i] * texp_a(ex ? x.B[i] * logT - x.E[i] * invT : 0.0, t.e2);
}

// The FP64 right-hand side by a four-warp team, balanced over its warps.
// Phase 1: warps 0-1 run the species pass while warp 2 evaluates the
// temperature-only parts of the fall-off reactions (k_inf, k0, log10 Fcent:
// the transcendental-heavy part) and warp 3 the Arrhenius constants of all
// other reactions. Phase 2: warp 3 takes the fall-off rounds, warps 0-2 the
// others. Phase 3: production rates from the species-major entry list.
__device__ void rhs64_team(const Tabs& t, const Team<TEAM>& tm, WarpWork& w, const double* y, double rho,
                           double* f) {
  const RTabs<double>& x = t.d;
  const int ns = t.ns, tid = tm.tid, wq = tid >> 5, lane = tid & 31;
  double* kfe = tm.pre;       // [352] Arrhenius constants
  double* k0a = tm.pre + 352; // [64] k0 / kinf, by special-reaction index
  double* fcl = k0a + 64;     // [64] log10 Fcent
  const double T = y[ns];
  const double logT = tlog(T, t.lg);
  const double invT = 1.0 / T;
  const int fr0 = t.h->fr0, nfr = t.h->nfr;
  const int nround = t.nrp >> 5;
  const double pfac = (PATM_CGS / RU_CGS) * invT;
  const double ipfac = T * (RU_CGS / PATM_CGS);
  // Non-fall-off rounds e = 0..nE-1 sit at round re(e). Phase 0: the
  // concentrations and their sum, by all four warps. Phase 1 gives the
  // Arrhenius constants of rounds e to warps 0 (e < 2), 1 (e < 4), 2 (e < 6)
  // and 3 (the rest), after each warp's own part: the species pass (warps
  // 0-1), log10 Fcent of the fall-off reactions (warp 2), and k_inf, k0/k_inf,
  // the collider sum, Pr and log10 Pr of every slot of the fall-off rounds
  // (warp 3, which keeps Pr and log10 Pr for its phase 2).
  const int nE = nround - nfr;
  auto re = [&](int e) { return (nfr > 0 && e >= fr0) ? e + nfr : e; };
  auto prep_round = [&](int rr) {
    const int i = rr * 32 + lane;
    if (i < t.nr) kfe[i] = arrhenius<double>(t, i, t.w0[i] >> 24, logT, invT);
  };
  {
    double cs = 0.0;
    for (int k = tid; k < ns; k += TEAM) {
      const double c = rho * y[k] * x.invW[k];
      w.C[k] = c;
      cs += c;
    }
    cs = warp_sum(cs);
    if (lane == 0) tm.red[24 + wq] = cs;
    // 1/rho for the production rates, kept in the last cross-warp slot
    if (tid == 0) tm.red[255] = 1.0 / rho;
  }
  tm.sync();
  const double ctot = ((tm.red[24] + tm.red[25]) + tm.red[26]) + tm.red[27];
  double* fpr = tm.part4;  // [nfr][64]: Pr, log10 Pr of the fall-off slots (warp 3's own)
  double ycv = 0.0;        // sum Y_k cv_k
  int e0 = 0, e1 = 0;
  if (wq < 2) {
    // the species pass (one species per lane: ns <= 64) and this warp's two
    // Arrhenius rounds as one straight block: three independent chains that
    // the compiler interleaves (a lone warp issues an FP64 instruction per
    // 64 cycles at best, and a single chain also waits on each result);
    // loads stay in range and stores go under predicates
    const bool sp = tid < ns;
    const int k = sp ? tid : ns - 1;
    const int ea = 2 * wq, eb = 2 * wq + 1;
    const int ia = re(ea < nE ? ea : 0) * 32 + lane, ib = re(eb < nE ? eb : 0) * 32 + lane;
    const double c = w.C[k];
    const SpeciesVals v = species_vals(t, k, c, T, logT, invT, pfac, ipfac);
    const double kfa = arrhenius_bl(t, ia, logT, invT);
    const double kfb = arrhenius_bl(t, ib, logT, invT);
    if (sp) {
      w.m[k] = v.m;
      w.wdot[k] = v.mi;
      w.en[k] = v.en;
      w.uR[k] = v.uR;
      w.cvm[k] = v.cvm;
      ycv = y[k] * v.cvm;
    }
    if (ea < nE && ia < t.nr) kfe[ia] = kfa;
    if (eb < nE && ib < t.nr) kfe[ib] = kfb;
    e0 = e1 = 0;
  } else if (wq == 2) {
    for (int r = 0; r < nfr; ++r) {
      const int i = (fr0 + r) * 32 + lane;
      if (i < t.nr && ((t.w0[i] >> 24) & F_FALL)) {
        const int aux = (int)(t.w2[i] >> 24);
        const double* fp = x.aux + aux * AUXW;
        const int ifop = (int)fp[7];
        fcl[aux] = (ifop > 1) ? troe_fclog<double>(t, fp, ifop, T, invT) : 0.0;
      }
    }
    e0 = 4;
    e1 = 6;
  } else {
    for (int r = 0; r < nfr; ++r) {
      const int i = (fr0 + r) * 32 + lane;
      if (i < t.nr) {
        const unsigned fl = t.w0[i] >> 24;
        kfe[i] = arrhenius<double>(t, i, fl, logT, invT);
        if (fl & F_FALL) {
          const int aux = (int)(t.w2[i] >> 24);
          const double* fp = x.aux + aux * AUXW;
          const double pr = fp[0] * texp_a(fp[1] * logT - fp[2] * invT, t.e2) *  // k0 / kinf
                            collider<double>(t, fl, aux, ctot, w.C);
          fpr[r * 64 + lane] = pr;
          fpr[r * 64 + 32 + lane] = log10_pr(t, pr);
        }
      }
    }
    e0 = 6;
    e1 = nE;
  }
  for (int e = min(e0, nE); e < min(e1, nE); ++e) prep_round(re(e));
  ycv = tm.sum(ycv);  // its barriers close phase 1
  // 1/(rho cv) for dT/dt, on the thread that writes it (warp 0 has time to
  // spare in phase 2)
  const double inv_rhocv = tid == 0 ? 1.0 / (rho * ycv) : 0.0;
  // phase 2: warp 3 turns its Pr and log10 Pr into the fall-off rate
  // constants (the Troe factor, with its reciprocal and exponential) and,
  // when there are more than seven other rounds, takes the last one; warp 1
  // forms the fall-off concentration products and hands them over through a
  // named barrier; warps 0-2 take the other rounds in turn (all four without
  // fall-off)
  auto rate_round = [&](int rr) {
    const int i = rr * 32 + lane;
    w.rop[i] = (i < t.nr) ? rop_pre(t, i, kfe[i], k0a, fcl, pfac, ipfac, ctot, w.C, w.m, w.wdot, w.en) : 0.0;
  };
  if (nfr > 0) {
    if (wq == 1) {
      for (int r = 0; r < nfr; ++r) {
        const int i = (fr0 + r) * 32 + lane;
        if (i < t.nr) {
          const unsigned w0 = t.w0[i];
          w.rop[i] = net_rate(w0, t.w1[i], t.w2[i], ((w0 >> 24) & F_REV) != 0, 1.0, w.C, w.m, w.wdot, w.en);
        } else {
          w.rop[i] = 0.0;
        }
      }
      pair_arrive(BAR_FALL_MA);
    }
    const int nE3 = nE > 7 ? nE - 1 : nE;  // rounds for warps 0-2
    if (wq < 3) {
      for (int e = wq; e < nE3; e += 3) rate_round(re(e));
    } else {
      for (int r = 0; r < nfr; ++r) {
        const int i = (fr0 + r) * 32 + lane;
        double kp = 0.0;
        if (i < t.nr) {
          const unsigned fl = t.w0[i] >> 24;
          const int aux = (int)(t.w2[i] >> 24);
          kp = kfe[i];
          if (fl & F_FALL) {
            const double pr = fpr[r * 64 + lane];
            kp *= ((int)t.d.aux[aux * AUXW + 7] > 1) ? troe_pcor_d(t, pr, fpr[r * 64 + 32 + lane], fcl[aux])
                                                     : pr / (1.0 + pr);
          } else if (fl & (F_CM | F_KFAL)) {
            kp *= collider<double>(t, fl, aux, ctot, w.C);
          }
        }
        fpr[r * 64 + lane] = kp;
      }
      if (nE3 < nE) rate_round(re(nE - 1));
      pair_wait(BAR_FALL_MA);
      for (int r = 0; r < nfr; ++r) {
        const int i = (fr0 + r) * 32 + lane;
        w.rop[i] = fpr[r * 64 + lane] * w.rop[i];
      }
    }
  } else {
    for (int e = wq; e < nE; e += 4) rate_round(e);
  }
  tm.sync();
  // production rates: species k's entries split over an aligned group of
  // lanes of one warp (a power of two; one lane for most species), the
  // group's sums added by a shuffle tree, so no cross-warp partials
  const int4 gl = t.grp[tid];
  double s0 = 0.0, s1 = 0.0;
  int q = gl.y;
  for (; q + 1 < gl.z; q += 2) {
    s0 = fma(x.nu[q], w.rop[t.ent[q]], s0);
    s1 = fma(x.nu[q + 1], w.rop[t.ent[q + 1]], s1);
  }
  if (q < gl.z) s0 = fma(x.nu[q], w.rop[t.ent[q]], s0);
  double s = s0 + s1;
  for (int o = 1; o < t.h->gmax; o <<= 1) {
    const double v = __shfl_xor_sync(0xffffffffu, s, o);
    if (o < gl.w) s += v;
  }
  double su = 0.0;  // u_k/R w_k of the group's species, on its first lane
  if (gl.x >= 0 && (lane & (gl.w - 1)) == 0) {
    f[gl.x] = s * x.W[gl.x] * tm.red[255];
    su = w.uR[gl.x] * s;
  }
  su = warp_sum(su);
  if (lane == 0) tm.red[wq] = su;
  tm.sync();
  if (tid == 0) f[ns] = -(((tm.red[0] + tm.red[1]) + tm.red[2]) + tm.red[3]) * inv_rhocv;  // RU cancels in u/cv
  tm.sync();
}

template <int TW>
__device__ __forceinline__ void rhs64(const Tabs& t, const Team<TW>& tm, WarpWork& w, const double* y,
                                      double rho_cgs, double* f) {
  if constexpr (TW == 32) rhs<double, TW>(t, tm, w, y, rho_cgs, f, w.C, w.m, w.wdot, w.uR, w.cvm, w.rop, w.part);
  else rhs64_team(t, tm, w, y, rho_cgs, f);
}

// Analytic FP32 Jacobian of the mass-action species block plus finite
// differences in T. J (row-major, stride JS) receives d f / d y at y.
template <int TW>
__device__ void jacobian32(const Tabs& t, const Team<TW>& tm, WarpWork& w, const double* y, double rho_cgs, float* J) {
  const RTabs<float>& x = t.f;
  const int ns = t.ns, n = ns + 1;
  const int tid = tm.tid;
  float* Cf = (float*)w.C;
  float* mf = (float*)w.m;
  float* mif = (float*)w.wdot;
  float* uRf = (float*)w.uR;
  float* cvmf = (float*)w.cvm;
  float* ropf = (float*)w.rop;
  float* partf = (float*)w.part;
  float* rowc = (float*)w.sv;  // per-species collider coefficients
  for (int q = tid; q < n * JS; q += TW) J[q] = 0.f;
  float* Jw = J;      // this thread's accumulation target
  float* rw = rowc;
  if constexpr (TW > 32) {
    for (int b = 0; b < 3; ++b) {
      for (int q = tid; q < n * JS; q += TW) tm.jp[b][q] = 0.f;
      for (int q = tid; q < n; q += TW) tm.rp[b][q] = 0.f;
    }
    const int wq = tid >> 5;
    if (wq > 0) {
      Jw = wq == 1 ? tm.jp[0] : (wq == 2 ? tm.jp[1] : tm.jp[2]);
      rw = wq == 1 ? tm.rp[0] : (wq == 2 ? tm.rp[1] : tm.rp[2]);
    }
  }
  const float T = (float)y[ns];
  const float dT = fmaxf(1e-3f * T, 0.05f);
  const float rho = (float)rho_cgs;
  // perturbed-T state first, base state second: the species-pass arrays
  // then hold the base state for the analytic part
  for (int k = tid; k < n; k += TW) w.yf[k] = (float)y[k];
  tm.sync();
  if (tid == 0) w.yf[ns] = T + dT;
  tm.sync();
  rhs<float, TW>(t, tm, w, w.yf, rho, w.f2, Cf, mf, mif, uRf, cvmf, ropf, partf);
  if (tid == 0) w.yf[ns] = T;
  tm.sync();
  rhs<float, TW>(t, tm, w, w.yf, rho, w.f1, Cf, mf, mif, uRf, cvmf, ropf, partf);
  for (int k = tid; k < n; k += TW) rowc[k] = 0.f;
  const float logT = __logf(T), invT = 1.f / T;
  float ctot = 0.f;
  for (int k = tid; k < ns; k += TW) ctot += Cf[k];
  ctot = tm.sum(ctot);
  const float pfac = (float)(PATM_CGS / RU_CGS) * invT;
  const float ipfac = T * (float)(RU_CGS / PATM_CGS);
  tm.sync();
  // d w_k / d C_j accumulated into J[k][j] (concentration space)
  for (int i = tid; i < t.nr; i += TW) {
    RxnEval<float> e = eval_rxn<float>(t, i, logT, invT, T, pfac, ipfac, ctot, Cf, mf, mif, w.en);
    const unsigned w0 = t.w0[i], w1 = t.w1[i], w2 = t.w2[i], w3 = t.w3[i], w4 = t.w4[i], w5 = t.w5[i];
    const int nk = (w5 >> 8) & 15;
    // forward: d qf / d C_r ; reverse: d qr / d C_p
#pragma unroll
    for (int side = 0; side < 2; ++side) {
      const unsigned ws = side == 0 ? w0 : w1;
      const float kk = side == 0 ? e.kf : -e.kr;
      if (kk == 0.f) continue;
#pragma unroll
      for (int s = 0; s < 3; ++s) {
        const unsigned kj = sp_of(ws, s);
        if (kj == 255u) continue;
        const int nj = (w2 >> (12 * side + 4 * s)) & 15;
        float d = kk * (float)nj;
#pragma unroll
        for (int s2 = 0; s2 < 3; ++s2) {
          const unsigned k2 = sp_of(ws, s2);
          if (k2 == 255u) continue;
          const int n2 = (w2 >> (12 * side + 4 * s2)) & 15;
          const float c = Cf[k2];
          const int pw = (s2 == s) ? n2 - 1 : n2;
          d *= (pw == 0) ? 1.f : (pw == 1 ? c : (pw == 2 ? c * c : c * c * c));
        }
#pragma unroll
        for (int q = 0; q < 6; ++q) {
          if (q >= nk) break;
          const unsigned kq = q < 4 ? ((w3 >> (8 * q)) & 0xff) : ((w4 >> (8 * (q - 4))) & 0xff);
          const int nuq = (int)(q < 4 ? ((w4 >> (16 + 4 * q)) & 15) : ((w5 >> (4 * (q - 4))) & 15)) - 8;
          atomicAdd(&Jw[kq * JS + kj], (float)nuq * d);
        }
      }
    }
    // collider dependence (third body / fall-off), fall-off blending held
    // fixed: a rank-one part (efficiency 1 for every species, added row-wise
    // below) plus the sparse efficiency corrections
    const unsigned fl = w0 >> 24;
    if (fl & (F_CM | F_KFAL)) {
      const float r0 = (e.qf - e.qr) * e.pcor_d / e.cm;
      if (isfinite(r0) && r0 != 0.f) {
        const int aux = (int)(w2 >> 24);
        for (int q = 0; q < nk; ++q) {
          const unsigned kq = q < 4 ? ((w3 >> (8 * q)) & 0xff) : ((w4 >> (8 * (q - 4))) & 0xff);
          const int nuq = (int)(q < 4 ? ((w4 >> (16 + 4 * q)) & 15) : ((w5 >> (4 * (q - 4))) & 15)) - 8;
          if (fl & F_KFAL) {
            atomicAdd(&Jw[kq * JS + t.spi[aux * 4 + 2]], (float)nuq * r0);
          } else {
            atomicAdd(&rw[kq], (float)nuq * r0);
            const int b = t.spi[aux * 4 + 0], c = t.spi[aux * 4 + 1];
            for (int q2 = b; q2 < b + c; ++q2)
              atomicAdd(&Jw[kq * JS + t.tb_sp[q2]], (float)nuq * r0 * x.tb_am1[q2]);
          }
        }
      }
    }
  }
  __syncwarp();
  if constexpr (TW > 32) {
    // the warps' partial sums in warp order
    tm.sync();
    for (int q = tid; q < n * JS; q += TW) J[q] = ((J[q] + tm.jp[0][q]) + tm.jp[1][q]) + tm.jp[2][q];
    for (int q = tid; q < n; q += TW) rowc[q] = ((rowc[q] + tm.rp[0][q]) + tm.rp[1][q]) + tm.rp[2][q];
    tm.sync();
  }
  // to mass-fraction space: d f_k / d y_j = (W_k / W_j) (d w_k / d C_j + rowc_k);
  // T row d f_T / d y_j = -(sum_k e_k J_kj + f_T cvm_j) / cv with e_k = u_k/W_k.
  float cv = 0.f;
  for (int k = tid; k < ns; k += TW) cv = fmaf(w.yf[k], cvmf[k], cv);
  cv = tm.sum(cv);
  const float fT = w.f1[ns];
  if constexpr (TW == 32) {
    for (int j = tid; j < ns; j += TW) {
      const float wj = x.invW[j];
      float acc = 0.f;
      for (int k = 0; k < ns; ++k) {
        const float v = (J[k * JS + j] + rowc[k]) * x.W[k] * wj;
        J[k * JS + j] = v;
        acc = fmaf(uRf[k] * x.invW[k], v, acc);
      }
      J[ns * JS + j] = -(acc + fT * cvmf[j]) / cv;
    }
  } else {
    // columns over threads, the rows of each column in two halves; the
    // halves' T-row partial sums meet in the team scratch
    float* accp = reinterpret_cast<float*>(tm.red + 64);  // [2][64]
    const int kh = (ns + 1) / 2;
    for (int it = tid; it < 2 * ns; it += TW) {
      const int j = it % ns, hf = it / ns;
      const float wj = x.invW[j];
      float acc = 0.f;
      const int k1 = hf == 0 ? kh : ns;
      for (int k = hf * kh; k < k1; ++k) {
        const float v = (J[k * JS + j] + rowc[k]) * x.W[k] * wj;
        J[k * JS + j] = v;
        acc = fmaf(uRf[k] * x.invW[k], v, acc);
      }
      accp[hf * 64 + j] = acc;
    }
    tm.sync();
    for (int j = tid; j < ns; j += TW) J[ns * JS + j] = -((accp[j] + accp[64 + j]) + fT * cvmf[j]) / cv;
  }
  const float idT = 1.f / ((T + dT) - T);
  for (int k = tid; k < n; k += TW) J[k * JS + ns] = (w.f2[k] - w.f1[k]) * idT;
  tm.sync();
  // an entry that overflowed single precision carries no usable slope
  for (int q = tid; q < n * JS; q += TW)
    if (!isfinite(J[q])) J[q] = 0.f;
  tm.sync();
}

// In-place Gauss-Jordan inversion with partial pivoting (FP32, one warp).
// Each Newton solve is then a matrix-vector product without the serial
// dependence chain of triangular substitution.
__device__ bool gj_invert_warp(float* A, int* perm, float* col, int n, int lane) {
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
    if (lane == 0) perm[k] = bi;
    if (bi != k)
      for (int j = lane; j < n; j += 32) {
        const float t0 = A[k * JS + j];
        A[k * JS + j] = A[bi * JS + j];
        A[bi * JS + j] = t0;
      }
    __syncwarp();
    const float inv = 1.f / A[k * JS + k];
    for (int i = lane; i < n; i += 32) col[i] = (i == k) ? 0.f : A[i * JS + k];
    __syncwarp();
    for (int j = lane; j < n; j += 32) A[k * JS + j] = (j == k) ? inv : A[k * JS + j] * inv;
    __syncwarp();
    for (int j = lane; j < n; j += 32) {
      const float rk = A[k * JS + j];
      if (j != k) {
        int i = 0;
        for (; i + 6 <= n; i += 6) {
          float a0 = A[(i + 0) * JS + j], a1 = A[(i + 1) * JS + j], a2 = A[(i + 2) * JS + j];
          float a3 = A[(i + 3) * JS + j], a4 = A[(i + 4) * JS + j], a5 = A[(i + 5) * JS + j];
          a0 = fmaf(-col[i + 0], rk, a0);
          a1 = fmaf(-col[i + 1], rk, a1);
          a2 = fmaf(-col[i + 2], rk, a2);
          a3 = fmaf(-col[i + 3], rk, a3);
          a4 = fmaf(-col[i + 4], rk, a4);
          a5 = fmaf(-col[i + 5], rk, a5);
          A[(i + 0) * JS + j] = a0;
          A[(i + 1) * JS + j] = a1;
          A[(i + 2) * JS + j] = a2;
          A[(i + 3) * JS + j] = a3;
          A[(i + 4) * JS + j] = a4;
          A[(i + 5) * JS + j] = a5;
        }
        for (; i < n; ++i) A[i * JS + j] = fmaf(-col[i], rk, A[i * JS + j]);
      }
    }
    // the pivot column, in parallel over rows (row k already holds inv)
    for (int i = lane; i < n; i += 32)
      if (i != k) A[i * JS + k] = -col[i] * inv;
    __syncwarp();
  }
  // row interchanges of the elimination become column interchanges of the inverse
  for (int k = n - 1; k >= 0; --k) {
    const int p = perm[k];
    if (p != k)
      for (int i = lane; i < n; i += 32) {
        const float t0 = A[i * JS + k];
        A[i * JS + k] = A[i * JS + p];
        A[i * JS + p] = t0;
      }
    __syncwarp();
  }
  return ok;
}

// The same inversion by a four-warp team, column by column: lanes 2j and
// 2j+1 hold column j of the working matrix in registers, rows h*GJ_HALF + q
// (h = lane parity, q < GJ_HALF). Pivoting is implicit: the pivot of column
// k is the largest remaining entry among the rows not yet used (lowest row
// on ties), and no rows move. At step k the owner pair of column k finds the
// pivot (one shuffle) and publishes the column through double-buffered
// shared memory, so a step costs one barrier; every pair then takes its
// pivot-row entry from its own registers and updates its column. With pivot
// rows p_k the result B satisfies inv(A)[k][p_j] = B[p_k][j], which the
// write-back applies.
constexpr int GJ_HALF = 28;  // rows per lane: columns of up to 56 rows
__device__ bool gj_invert_team(const Team<TEAM>& tm, float* A, int* perm, float* col, int n) {
  (void)col;
  const int tid = tm.tid, j = tid >> 1, h = tid & 1, r0 = h * GJ_HALF;
  const unsigned pair = 3u << (tid & 30);
  float* colk = reinterpret_cast<float*>(tm.red);       // [2][64]: column k of step k
  int* pinfo = reinterpret_cast<int*>(colk + 128);      // [2][2]: pivot row, nonsingular flag
  float c[GJ_HALF];
  unsigned usedl = 0u;  // bit q: row r0 + q is a pivot row already, or beyond n
#pragma unroll
  for (int q = 0; q < GJ_HALF; ++q) {
    const bool in = j < n && r0 + q < n;
    c[q] = in ? A[(r0 + q) * JS + j] : 0.f;
    usedl |= (r0 + q < n) ? 0u : (1u << q);
  }
  bool ok = true;
  // the owner pair of column k publishes it and the pivot among the unused
  // rows: a pairwise tree over the lane's rows (the left half of every pair
  // holds the lower rows, so ties keep the lowest row), then the pair
  auto publish = [&](int k) {
    const int buf = k & 1;
    float4* dst = reinterpret_cast<float4*>(colk + buf * 64 + r0);
#pragma unroll
    for (int v = 0; v < GJ_HALF / 4; ++v) dst[v] = make_float4(c[4 * v], c[4 * v + 1], c[4 * v + 2], c[4 * v + 3]);
    float bv[32];
    int bi[32];
#pragma unroll
    for (int q = 0; q < 32; ++q) {
      bv[q] = (q < GJ_HALF && !((usedl >> q) & 1u)) ? fabsf(c[q < GJ_HALF ? q : 0]) : -1.f;
      bi[q] = q;
    }
#pragma unroll
    for (int st = 1; st < 32; st <<= 1)
#pragma unroll
      for (int q = 0; q + st < 32; q += 2 * st) {
        const bool take = bv[q + st] > bv[q];
        bv[q] = take ? bv[q + st] : bv[q];
        bi[q] = take ? bi[q + st] : bi[q];
      }
    float b = bv[0];
    int i = (b >= 0.f) ? r0 + bi[0] : n;
    const float ov = __shfl_xor_sync(pair, b, 1);
    const int oi = __shfl_xor_sync(pair, i, 1);
    if (ov > b || (ov == b && oi < i)) { b = ov; i = oi; }
    if (h == 0) {
      pinfo[buf * 2] = i;
      pinfo[buf * 2 + 1] = (b > 0.f && i < n) ? 1 : 0;
    }
  };
  if (j == 0) publish(0);
  for (int k = 0; k < n; ++k) {
    const int buf = k & 1;
    tm.sync();
    int p = pinfo[buf * 2];
    if (!pinfo[buf * 2 + 1]) { ok = false; p = (p >= n) ? k : p; }
    if (tid == 0) perm[k] = p;
    const float inv = 1.f / colk[buf * 64 + p];
    // this column's entry in the pivot row: a binary select on the bits of
    // qs in the lane that holds row p, zero in the other, then the pair
    const int qs = p - r0;
    const bool here = qs >= 0 && qs < GJ_HALF;
    float t16[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) t16[q] = (qs & 16) ? c[q + 16 < GJ_HALF ? q + 16 : 0] : c[q];
#pragma unroll
    for (int q = 0; q < 8; ++q) t16[q] = (qs & 8) ? t16[q + 8] : t16[q];
#pragma unroll
    for (int q = 0; q < 4; ++q) t16[q] = (qs & 4) ? t16[q + 4] : t16[q];
#pragma unroll
    for (int q = 0; q < 2; ++q) t16[q] = (qs & 2) ? t16[q + 2] : t16[q];
    const float mine = here ? ((qs & 1) ? t16[1] : t16[0]) : 0.f;
    const float rp = mine + __shfl_xor_sync(0xffffffffu, mine, 1);  // every lane of the warp is here
    const bool isk = (j == k);
    const float rj = isk ? inv : rp * inv;
    if (isk) {
#pragma unroll
      for (int q = 0; q < GJ_HALF; ++q) c[q] = 0.f;
    }
    const float4* cb = reinterpret_cast<const float4*>(colk + buf * 64 + r0);
#pragma unroll
    for (int v = 0; v < GJ_HALF / 4; ++v) {
      const float4 ck = cb[v];
      const float cv[4] = {ck.x, ck.y, ck.z, ck.w};
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int q = 4 * v + u;
        c[q] = (q == qs) ? rj : fmaf(-cv[u], rj, c[q]);
      }
    }
    usedl |= here ? (1u << qs) : 0u;
    if (j == k + 1 && k + 1 < n) publish(k + 1);
  }
  // write back the inverse: inv(A)[k][p_j] = B[p_k][j], through A in the
  // natural layout
  tm.sync();
#pragma unroll
  for (int q = 0; q < GJ_HALF; ++q)
    if (j < n && r0 + q < n) A[(r0 + q) * JS + j] = c[q];
  tm.sync();
#pragma unroll
  for (int q = 0; q < GJ_HALF; ++q) {
    const int k = r0 + q;
    c[q] = (j < n && k < n) ? A[perm[k] * JS + j] : 0.f;
  }
  tm.sync();
  if (j < n) {
    const int pj = perm[j];
#pragma unroll
    for (int q = 0; q < GJ_HALF; ++q)
      if (r0 + q < n) A[(r0 + q) * JS + pj] = c[q];
  }
  tm.sync();
  return ok;
}

template <int TW>
__device__ __forceinline__ bool gj_invert(const Team<TW>& tm, float* A, int* perm, float* col, int n) {
  if constexpr (TW == 32) return gj_invert_warp(A, perm, col, n, tm.tid);
  else return gj_invert_team(tm, A, perm, col, n);
}

// b <- A b for the n x n inverse in A (lanes over rows).
__device__ __forceinline__ void gemv_solve_warp(const float* A, float* b, int n, int lane) {
  float r0 = 0.f, r1 = 0.f;
  const int i0 = lane, i1 = lane + 32;
  float a0 = 0.f, a1 = 0.f, c0 = 0.f, c1 = 0.f;
  for (int j = 0; j + 1 < n; j += 2) {
    const float bj = b[j], bj1 = b[j + 1];
    if (i0 < n) {
      a0 = fmaf(A[i0 * JS + j], bj, a0);
      c0 = fmaf(A[i0 * JS + j + 1], bj1, c0);
    }
    if (i1 < n) {
      a1 = fmaf(A[i1 * JS + j], bj, a1);
      c1 = fmaf(A[i1 * JS + j + 1], bj1, c1);
    }
  }
  if (n & 1) {
    const float bj = b[n - 1];
    if (i0 < n) a0 = fmaf(A[i0 * JS + n - 1], bj, a0);
    if (i1 < n) a1 = fmaf(A[i1 * JS + n - 1], bj, a1);
  }
  r0 = a0 + c0;
  r1 = a1 + c1;
  __syncwarp();
  if (i0 < n) b[i0] = r0;
  if (i1 < n) b[i1] = r1;
  __syncwarp();
}

// b <- A b by a four-warp team: two threads per row, even and odd columns.
template <int TW>
__device__ __forceinline__ void gemv_solve(const Team<TW>& tm, const float* A, float* b, int n) {
  if constexpr (TW == 32) {
    gemv_solve_warp(A, b, n, tm.tid);
  } else {
    const int i = tm.tid >> 1, h = tm.tid & 1;
    float a = 0.f;
    if (i < n)
      for (int j = h; j < n; j += 2) a = fmaf(A[i * JS + j], b[j], a);
    a += __shfl_xor_sync(0xffffffffu, a, 1);
    tm.sync();
    if (i < n && h == 0) b[i] = a;
    tm.sync();
  }
}

// One simplified-Newton correction at the iterate Y with f(Y) in fy: the
// scaled residual b = -(Y - sv - hg f) / sc, b <- M^-1 b, Y += b sc; returns
// the RMS of the scaled correction b. A four-warp team updates Y and forms
// the norm where the product lands, inside the product's two barriers.
template <int TW>
__device__ __forceinline__ float newton_correct(const Team<TW>& tm, WarpWork& w, double hg, int n, float nn) {
  for (int i = tm.tid; i < n; i += TW) w.b32[i] = (float)(hg * w.fy[i] - (w.Y[i] - w.sv[i])) * w.isc32[i];
  tm.sync();
  float ss = 0.f;
  if constexpr (TW == 32) {
    gemv_solve_warp(w.J, w.b32, n, tm.tid);
    for (int i = tm.tid; i < n; i += 32) {
      const float q = w.b32[i];
      ss = fmaf(q, q, ss);
      w.Y[i] += (double)q * (double)w.sc32[i];
    }
    __syncwarp();
    return sqrtf(tm.sum(ss) / nn);
  } else {
    const int i = tm.tid >> 1, hh = tm.tid & 1;
    float a = 0.f;
    if (i < n)
      for (int j = hh; j < n; j += 2) a = fmaf(w.J[i * JS + j], w.b32[j], a);
    a += __shfl_xor_sync(0xffffffffu, a, 1);
    ss = warp_sum((i < n && hh == 0) ? a * a : 0.f);
    tm.sync();
    if (i < n && hh == 0) {
      w.b32[i] = a;
      w.Y[i] += (double)a * (double)w.sc32[i];
    }
    if ((tm.tid & 31) == 0) tm.red[16 + (tm.tid >> 5)] = (double)ss;
    tm.sync();
    return sqrtf((float)(((tm.red[16] + tm.red[17]) + tm.red[18]) + tm.red[19]) / nn);
  }
}

struct Cell {
  double rho_cgs, dt, rtol, atol;
  double h0;      // first step size to try (<= dt)
  int max_steps;  // accepted + rejected steps after which the cell fails (<= 0: 4000)
  bool screen;    // stop after the inert-cell test: a cell that is not inert is deferred
};

struct CellStats {
  int rhs, steps, rejects, jac;
  bool failed;
  double hnext;   // step size the cell's next window starts with
  bool deferred;  // screen mode: not inert; w.y0 = y0 and w.dl = f(y0) are left for the caller
};

constexpr float THETA_JAC = 0.1f;  // Newton contraction above which a kept Jacobian is rebuilt
constexpr int JAC_MAX_AGE = 20;    // accepted steps a kept Jacobian serves at most
constexpr double M_REUSE = 0.5;    // a kept inverse serves while |h / h_m - 1| stays within this

// Integrates w.y0 over [0, dt] with SDIRK4. Returns the statistics.
template <int TW>
__device__ CellStats integrate(const Tabs& t, const Team<TW>& tm, WarpWork& w, const Cell& c) {
  const int lane = tm.tid;
  const int n = t.ns + 1;
  const float nn = (float)t.h->nnorm;  // RMS over the full mechanism's components (a subset's others are zero)
  CellStats st = {0, 0, 0, 0, false, c.dt, false};
  double tcur = 0.0, h = c.h0;
  const int max_steps = c.max_steps > 0 ? c.max_steps : 4000;
  bool need_jac = true, need_f0 = true;
  // A four-warp team keeps its Jacobian in a separate buffer and reuses it
  // across steps while the Newton iterations contract fast (the iteration is
  // inexact anyway); a warp forms the Newton matrix over its Jacobian.
  constexpr bool keep_jac = TW > 32;
  float* Jd = keep_jac ? tm.jsave : w.J;
  bool jac_fresh = false;  // Jacobian evaluated at the current y0
  int jac_age = 0;         // accepted steps since it was evaluated
  // The inverted Newton matrix I - g h_m J (in w.J) keeps serving the
  // simplified Newton iteration, and the error filter, while the Jacobian is
  // kept and h stays within 50 % of h_m: the iteration is inexact anyway and
  // converges slightly slower, for far fewer inversions (Hairer and Wanner,
  // Solving ODEs II, IV.8). A Newton failure rebuilds it.
  bool m_ok = false;
  double h_m = 0.0;
  // The first accepted step of the window starts the next one: a cell at a
  // reaction front opens each window with the fast transient the fluid step
  // sets off, which the step size the window ended with overshoots.
  double hfirst = 0.0;
  const double g = 0.25;
  while (tcur < c.dt) {
    if (st.steps + st.rejects >= max_steps) { st.failed = true; break; }
    if (tcur + h > c.dt) h = c.dt - tcur;
    // f0 = f(y0) in FP64 at the window start; later the last stage
    // derivative of the accepted step (kept across rejections)
    if (need_f0) {
      rhs64<TW>(t, tm, w, w.y0, c.rho_cgs, w.dl);
      st.rhs++;
      need_f0 = false;
      if (tcur == 0.0) {
        // Inert cell: when the whole window's change predicted by the FP64
        // right-hand side, dt f(y0), is below 1e-3 of the error tolerance,
        // one explicit step is accurate far below the tolerance and the
        // implicit machinery is skipped.
        float ss = 0.f;
        for (int i = lane; i < n; i += TW) {
          const float q = (float)(c.dt * w.dl[i] / (c.atol + c.rtol * fabs(w.y0[i])));
          ss = fmaf(q, q, ss);
        }
        const float nrm = sqrtf(tm.sum(ss) / nn);
        if (nrm <= 1e-3f) {
          for (int i = lane; i < n; i += TW) w.y0[i] = fma(c.dt, w.dl[i], w.y0[i]);
          tm.sync();
          st.steps++;
          st.hnext = c.dt;
          break;
        }
        if (c.screen) {
          st.deferred = true;
          break;
        }
      }
    }
    const bool form_m = need_jac || !m_ok || fabs(h - h_m) > M_REUSE * h_m;
    if (need_jac) {
      jacobian32<TW>(t, tm, w, w.y0, c.rho_cgs, Jd);
      st.jac++;
      jac_fresh = true;
      jac_age = 0;
    }
    // Newton matrix I - h g J equilibrated with the error weights,
    // Ms = D^-1 M D, D = diag(atol + rtol |y0|); unscaled, the temperature
    // row (K per unit mass fraction) wins the pivot search and the species
    // rows lose their accuracy. Inverted in place (J is rebuilt after a
    // rejection).
    bool newton_ok = true;
    if (form_m) {
      for (int i = lane; i < n; i += TW) {
        w.sc32[i] = (float)(c.atol + c.rtol * fabs(w.y0[i]));
        w.isc32[i] = 1.f / w.sc32[i];
      }
      tm.sync();
      for (int q = lane; q < n * JS; q += TW) {
        const int i = q / JS, j = q - i * JS;
        if (j < n) w.J[q] = ((i == j ? 1.f : 0.f) - (float)(h * g) * Jd[q]) * (w.sc32[j] / w.sc32[i]);
      }
      tm.sync();
      newton_ok = gj_invert<TW>(tm, w.J, w.piv, w.col, n);
      m_ok = newton_ok;
      h_m = h;
    }
    float theta_max = 0.f;  // largest Newton contraction of this step
    for (int s = 0; s < 5 && newton_ok; ++s) {
      for (int i = lane; i < n; i += TW) {
        double acc = w.y0[i];
        for (int j = 0; j < s; ++j) acc = fma(h * c_sa[s][j], w.F[j][i], acc);
        w.sv[i] = acc;
        // starting value: the stage derivative interpolated or extrapolated
        // linearly in the stage abscissa c = (1/4, 3/4, 11/20, 1/2, 1) from
        // two earlier derivatives (f0 at c = 0; stage 4 between 1/4 and
        // 11/20, stage 5 from the pair at 3/4 and 1/2)
        double fp;
        switch (s) {
          case 0: fp = w.dl[i]; break;
          case 1: fp = fma(3.0, w.F[0][i], -2.0 * w.dl[i]); break;
          case 2: fp = fma(0.6, w.F[1][i], 0.4 * w.F[0][i]); break;
          case 3: fp = fma(5.0 / 6.0, w.F[2][i], (1.0 / 6.0) * w.F[0][i]); break;
          default: fp = fma(2.0, w.F[1][i], -w.F[3][i]); break;
        }
        w.Y[i] = fma(h * g, fp, acc);
      }
      tm.sync();
      float nrm_prev = 0.f;
      bool conv = false;
      for (int it = 0; it < 8; ++it) {
        const double Tn = w.Y[n - 1];
        if (!(Tn > 100.0 && Tn < 8000.0)) break;
        rhs64<TW>(t, tm, w, w.Y, c.rho_cgs, w.fy);
        st.rhs++;
        // the correction is applied to Y at once: on convergence Y is rebuilt
        // from f below, on failure the step is redone
        const float nrm = newton_correct<TW>(tm, w, h * g, n, nn);
        if (!(nrm == nrm)) break;
        // convergence: weighted correction below 1e-2 of the local
        // tolerance, directly or predicted from the contraction rate; one
        // non-contracting iteration (theta < 2) is tolerated
        if (nrm <= 1e-2f) conv = true;
        if (it > 0) theta_max = fmaxf(theta_max, nrm / nrm_prev);
        if (!conv && it > 0) {
          const float th = nrm / nrm_prev;
          if (th >= 2.f || (th >= 0.99f && it >= 2)) break;
          if (th < 0.99f && th / (1.f - th) * nrm <= 1e-2f) conv = true;
        }
        if (conv) {
          // stage derivative = the FP64 right-hand side at the converged
          // iterate; the stage value is rebuilt from it, so mass and
          // elements are conserved to rounding
          for (int i = lane; i < n; i += TW) {
            w.F[s][i] = w.fy[i];
            w.Y[i] = fma(h * g, w.fy[i], w.sv[i]);
          }
          tm.sync();
          break;
        }
        nrm_prev = nrm;
      }
      if (!conv) { newton_ok = false; break; }
    }
    if (!newton_ok) {
      st.rejects++;
      m_ok = false;
      h *= 0.25;
      need_jac = !(keep_jac && jac_fresh);
      if (h < c.dt * 1e-12) { st.failed = true; break; }
      continue;
    }
    // embedded error, filtered through the inverted matrix
    for (int i = lane; i < n; i += TW) {
      double e = 0.0;
      for (int j = 0; j < 5; ++j) e = fma(c_se[j], w.F[j][i], e);
      w.b32[i] = (float)(h * e) * w.isc32[i];
    }
    tm.sync();
    gemv_solve<TW>(tm, w.J, w.b32, n);
    float ss = 0.f;
    for (int i = lane; i < n; i += TW) {
      const float sc = (float)(c.atol + c.rtol * fmax(fabs(w.y0[i]), fabs(w.Y[i])));
      const float q = w.b32[i] * w.sc32[i] / sc;
      ss = fmaf(q, q, ss);
    }
    const float en = sqrtf(tm.sum(ss) / nn);
    const float fac = 0.9f * powf(fmaxf(en, 1e-10f), -0.25f);
    if (en <= 1.f) {
      // SDIRK4 is stiffly accurate (y1 = Y5), so the last stage derivative is
      // f at the new y0 up to the Newton tolerance: it serves as the next
      // step's f0, which only predicts the first stage (Hairer and Wanner,
      // Solving ODEs II, IV.8, starting values)
      for (int i = lane; i < n; i += TW) {
        w.y0[i] = w.Y[i];
        w.dl[i] = w.F[4][i];
      }
      tm.sync();
      if (hfirst == 0.0) hfirst = h;
      tcur += h;
      st.steps++;
      const float q = fminf(5.f, fmaxf(0.2f, fac));
      const double hprop = h * (double)q;
      // the proposal after a step cut short by the window end is measured
      // on the shorter step; the step size wanted before the cut stands too
      jac_fresh = false;
      ++jac_age;
      h = hprop;
      need_jac = !keep_jac || theta_max > THETA_JAC || jac_age >= JAC_MAX_AGE;
    } else {
      st.rejects++;
      h = h * (double)fminf(1.f, fmaxf(0.2f, fac));
      need_jac = !keep_jac;
    }
  }
  if (hfirst > 0.0) st.hnext = hfirst;
  return st;
}

__device__ __forceinline__ void stage_tables(char* smem_tab, const char* g_tab, int bytes) {
  const int4* src = (const int4*)g_tab;
  int4* dst = (int4*)smem_tab;
  for (int q = threadIdx.x; q < bytes / 16; q += blockDim.x) dst[q] = src[q];
  __syncthreads();
}

__device__ __forceinline__ void add_stats(ChemCounters* cnt, const CellStats& s, bool team) {
  atomicAdd(&cnt->rhs, (unsigned long long)s.rhs);
  atomicAdd(&cnt->steps, (unsigned long long)s.steps);
  atomicAdd(&cnt->rejects, (unsigned long long)s.rejects);
  atomicAdd(&cnt->jac, (unsigned long long)s.jac);
  atomicAdd(&cnt->cells, 1ull);
  if (team) atomicAdd(&cnt->team_cells, 1ull);
  if (s.failed) atomicAdd(&cnt->failed, 1ull);
}

__device__ __forceinline__ WarpWork* work_slots(char* smem, int tab_bytes) {
  return (WarpWork*)(smem + ((tab_bytes + 255) / 256) * 256);
}

// Batch of independent reactors (macks contract).
__global__ void __launch_bounds__(MAXW * 32, 1)
    k_reactors(const char* g_tab, int tab_bytes, int n, const double* rho, const double* dt, double* yiT, double rtol,
               double atol, int max_steps, unsigned* next, ChemCounters* cnt, unsigned* err) {
  extern __shared__ __align__(16) char smem[];
  stage_tables(smem, g_tab, tab_bytes);
  const Tabs t = bind_tabs(smem);
  WarpWork& w = work_slots(smem, tab_bytes)[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  const Team<32> tm{lane, 0, nullptr, nullptr, nullptr, nullptr};
  // rows hold the full mechanism's species and T (nnorm values); a species
  // subset's tables read and write the kept species through smap
  const int ns = t.ns, nrow = t.h->nnorm;
  for (int guard = 0; guard < (1 << 30); ++guard) {
    unsigned cell = 0;
    if (lane == 0) cell = atomicAdd(next, 1u);
    cell = __shfl_sync(0xffffffffu, cell, 0);
    if (cell >= (unsigned)n) break;
    const double* src = yiT + (size_t)cell * nrow;
    for (int k = lane; k < ns; k += 32) w.y0[k] = src[t.smap[k]];
    if (lane == 0) w.y0[ns] = src[nrow - 1];
    __syncwarp();
    Cell c{rho[cell] * 1e-3, dt[cell], rtol, atol, dt[cell], max_steps, false};
    CellStats s = integrate<32>(t, tm, w, c);
    double* dst = yiT + (size_t)cell * nrow;
    for (int k = lane; k < ns; k += 32) dst[t.smap[k]] = w.y0[k];
    if (lane == 0) dst[nrow - 1] = w.y0[ns];
    if (lane == 0) {
      add_stats(cnt, s, false);
      if (s.failed) atomicOr(err, EDYN_STATUS_CHEM);
    }
    __syncwarp();
  }
}

// FP64 right-hand side f = d(Y_1..Y_ns, T)/dt of a batch of reactors (the
// function integrate() advances), one warp per cell. Rows hold the full
// mechanism's species and T (nnorm values); with a species subset's tables
// the kept species are read through smap, and the rows of the others get 0
// (their concentrations and rates are zero).
__global__ void __launch_bounds__(MAXW * 32, 1)
    k_reactor_rhs(const char* g_tab, int tab_bytes, int n, const double* rho, const double* yiT, double* f) {
  extern __shared__ __align__(16) char smem[];
  stage_tables(smem, g_tab, tab_bytes);
  const Tabs t = bind_tabs(smem);
  WarpWork& w = work_slots(smem, tab_bytes)[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  const Team<32> tm{lane, 0, nullptr, nullptr, nullptr, nullptr};
  const int ns = t.ns;
  const int nrow = t.h->nnorm;  // full species + T
  const int nw = blockDim.x >> 5;
  for (int cell = blockIdx.x * nw + (threadIdx.x >> 5); cell < n; cell += gridDim.x * nw) {
    const double* src = yiT + (size_t)cell * nrow;
    for (int k = lane; k < ns; k += 32) w.y0[k] = src[t.smap[k]];
    if (lane == 0) w.y0[ns] = src[nrow - 1];
    __syncwarp();
    rhs64<32>(t, tm, w, w.y0, rho[cell] * 1e-3, w.fy);
    __syncwarp();
    double* dst = f + (size_t)cell * nrow;
    if (ns + 1 < nrow)
      for (int i = lane; i < nrow; i += 32) dst[i] = 0.0;
    __syncwarp();
    for (int k = lane; k < ns; k += 32) dst[t.smap[k]] = w.fy[k];
    if (lane == 0) dst[nrow - 1] = w.fy[ns];
    __syncwarp();
  }
}

// HRR_dot of the tube cells (heat_release_rate_omegadot, SRC/thermo.f90:
// 105-134, called at SRC/source.f90:72-73): -sum_k W_k h_f,k (cdot_k -
// ddot_k) with the production rates at the state the chemistry step left
// (rho, Y after adjust_sum, T of the integration), converted to W/m^3. With
// the molar production rates w_k = cdot_k - ddot_k and f_k = dY_k/dt =
// w_k W_k / rho (the integrator's right-hand side), the sum is rho sum_k
// h_f,k f_k. One warp per cell. The reference evaluates it every step for
// output only; here it is evaluated when the host downloads it.
__global__ void __launch_bounds__(MAXW * 32, 1)
    k_hrr_dot(const char* g_tab, int tab_bytes, int n, int ld, const double* qf, const double* tchem, double* out,
              const int* colmap) {
  extern __shared__ __align__(16) char smem[];
  stage_tables(smem, g_tab, tab_bytes);
  const Tabs t = bind_tabs(smem);
  WarpWork& w = work_slots(smem, tab_bytes)[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  const Team<32> tm{lane, 0, nullptr, nullptr, nullptr, nullptr};
  const int ns = t.ns;
  const int nw = blockDim.x >> 5;
  for (int cell = blockIdx.x * nw + (threadIdx.x >> 5); cell < n; cell += gridDim.x * nw) {
    const double* q = qf + (colmap ? (size_t)colmap[cell] : (size_t)cell) + GHOST;
    for (int k = lane; k < ns; k += 32) w.y0[k] = q[(3 + t.smap[k]) * (size_t)ld];
    if (lane == 0) w.y0[ns] = tchem[cell];
    __syncwarp();
    const double rho_cgs = q[0] * 1e-3;
    rhs64<32>(t, tm, w, w.y0, rho_cgs, w.fy);
    __syncwarp();
    double sum = 0.0;
    for (int k = lane; k < ns; k += 32) sum = fma(t.d.hf[k], w.fy[k], sum);
    sum = warp_sum(sum);
    if (lane == 0) out[cell] = -(rho_cgs * sum) * 1e-1;
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------
// Single-precision pre-check of the inert-cell test.
//
// The inert-cell test of integrate() needs f(y0) in FP64: one full right-hand
// side per cell, the bulk of a source step on a tube whose cells are mostly
// cold or burnt out. The pre-check evaluates f in FP32 together with the
// gross rates g_k = (W_k / rho) sum_r |nu_kr| (qf_r + qr_r) (and their image
// sum_k |u_k/R| G_k / (rho cv) for T). Every FP32 rate of progress is within
// a relative DELTA of its FP64 value: its logarithm is a sum of terms below
// ~300 in magnitude (ln A, beta ln T, E/RT and the S/R - H/RT of at most six
// species), each good to a few units in the last place of FP32. A worst-case
// count of those roundings over GRI-Mech 3.0 from 300 to 3500 K gives DELTA
// = 8.2e-4, largest for a reverse constant at 300 K (tests/
// test_precheck_bound.py); products that underflow FP32 lose at most EPS_ABS
// per second of mass fraction. Then
//     |f64_i - f32_i| <= DELTA g_i + EPS_ABS,
// and with KAPPA = 1e-2 (over 12 x DELTA) a cell whose bound
//     sqrt(mean_i (dt (|f32_i| + KAPPA g_i + EPS_ABS) / (atol + rtol |y_i|))^2) <= 1e-3
// passes the FP64 test as well. It takes the explicit step with f32, which
// differs from the FP64 explicit step by at most DELTA / KAPPA x 1e-3 x
// sqrt(n) ~ 6e-4 error-weight units per component. A cell with a reaction
// the FP32 form does not cover (a general-order reaction, or a reverse
// constant held at the FP32 cap while its products are present), or whose
// bound is not finite, goes to the FP64 test unchanged.
// ---------------------------------------------------------------------------
constexpr float PRE_KAPPA = 1e-2f;
constexpr float PRE_EPS = 1e-12f;  // per second, mass fraction (and K for T)

// FP32 workspace of the pre-check; it overlays a warp's FP64 right-hand-side
// arrays (C .. rop of WarpWork and ScreenWork), which it finishes with
// before an FP64 right-hand side reuses them.
struct Pre32 {
  float y[NV], C[NV], m[NV], mi[NV], uR[NV], cvm[NV], f[NV], g[NV];
  float rop[352], rg[352];
  float part[100], pg[100];
};

// One reaction's forward and reverse rates of progress in FP32. Returns
// true when the FP32 value is not covered by the DELTA bound.
__device__ __forceinline__ bool rxn32(const Tabs& t, int i, float logT, float invT, float T, float pfac,
                                      float ipfac, float ctot, const float* C, const float* m, const float* mi,
                                      const int* en, float& qf, float& qr) {
  const RTabs<float>& x = t.f;
  const unsigned w0 = t.w0[i], w1 = t.w1[i], w2 = t.w2[i];
  const unsigned fl = w0 >> 24;
  qf = qr = 0.f;
  if (fl & F_GEN) return true;
  const float lkf = x.lnA[i] + x.B[i] * logT - x.E[i] * invT;  // ln kf
  float kf = __expf(lkf), kr = 0.f;
  bool capped = false;
  if (fl & F_REV) {
    const float k0 = kf * inv_kc<float>(w0, w1, w2, pfac, ipfac, m, mi, en);
    capped = !(k0 < 1e30f);
    kr = capped ? 1e30f : k0;
  }
  if (fl & (F_CM | F_KFAL)) {
    const int aux = (int)(w2 >> 24);
    const float cm = collider<float>(t, fl, aux, ctot, C);
    if (fl & F_FALL) {
      const float* fp = x.aux + aux * AUXW;
      // Pr = k0 [M] / kinf with k0 / kinf taken in logarithms (no 0/0 when
      // both underflow)
      const float pr = __expf(fp[8] + fp[1] * logT - fp[2] * invT - lkf) * cm;
      const int ifop = (int)fp[7];
      const float fclog = (ifop > 1) ? troe_fclog<float>(t, fp, ifop, T, invT) : 0.f;
      const float pcor = falloff_pcor<float>(t, pr, ifop, fclog);
      kf *= pcor;
      kr *= pcor;
    } else {
      kf *= cm;
      kr *= cm;
    }
  }
  qf = kf;
  qr = kr;
  mass_action<float>(w0, w1, w2, C, qf, qr);
  return capped && qr > 0.f;
}

// FP32 right-hand side of s.y (one warp) into s.f and its gross rates into
// s.g. Returns true (on every lane) when a reaction is not covered.
__device__ bool rhs32_bound(const Tabs& t, int lane, Pre32& s, int* en, float rho) {
  const RTabs<float>& x = t.f;
  const Team<32> tm{lane, 0, nullptr, nullptr, nullptr, nullptr};
  const int ns = t.ns;
  const float T = s.y[ns];
  const float logT = __logf(T), invT = 1.f / T;
  const float pfac = (float)(PATM_CGS / RU_CGS) * invT;
  const float ipfac = T * (float)(RU_CGS / PATM_CGS);
  const float ctot =
      species_pass<float, 32>(t, tm, s.y, rho, T, logT, invT, pfac, ipfac, s.C, s.m, s.mi, en, s.uR, s.cvm);
  __syncwarp();
  bool bad = false;
  for (int i = lane; i < t.nrp; i += 32) {
    float qf = 0.f, qr = 0.f;
    if (i < t.nr) bad |= rxn32(t, i, logT, invT, T, pfac, ipfac, ctot, s.C, s.m, s.mi, en, qf, qr);
    s.rop[i] = qf - qr;
    s.rg[i] = qf + qr;
  }
  __syncwarp();
  for (int p = t.lane[lane]; p < t.lane[lane + 1]; ++p) {
    const int e0 = t.pc[p * 3 + 1], e1 = t.pc[p * 3 + 2];
    float a = 0.f, b = 0.f;
    for (int q = e0; q < e1; ++q) {
      const float nu = x.nu[q];
      const unsigned r = t.ent[q];
      a = fmaf(nu, s.rop[r], a);
      b = fmaf(fabsf(nu), s.rg[r], b);
    }
    s.part[p] = a;
    s.pg[p] = b;
  }
  __syncwarp();
  float v[3] = {0.f, 0.f, 0.f};  // sum u/R w, sum |u/R| G, cv / R
  for (int k = lane; k < ns; k += 32) {
    float a = 0.f, b = 0.f;
    for (int q = t.spc[k]; q < t.spc[k + 1]; ++q) {
      const int pp = t.spp[q];
      a += s.part[pp];
      b += s.pg[pp];
    }
    const float wr = x.W[k] / rho;
    s.f[k] = a * wr;
    s.g[k] = b * wr;
    v[0] = fmaf(s.uR[k], a, v[0]);
    v[1] = fmaf(fabsf(s.uR[k]), b, v[1]);
    v[2] = fmaf(s.y[k], s.cvm[k], v[2]);
  }
  tm.sumv(v);
  if (lane == 0) {
    s.f[ns] = -v[0] / (rho * v[2]);
    s.g[ns] = v[1] / (rho * v[2]);
  }
  __syncwarp();
  return __any_sync(0xffffffffu, bad);
}

// The pre-check on one cell (one warp): y0 holds the adjusted [Y, T] in
// FP64. When the bound passes, y0 takes the explicit step y0 + dt f32 and
// the call returns true; otherwise y0 is left as it was.
__device__ bool precheck_inert(const Tabs& t, int lane, Pre32& s, int* en, double* y0, double rho_cgs, double dt,
                               double rtol, double atol, float nn) {
  const int n = t.ns + 1;
  for (int i = lane; i < n; i += 32) s.y[i] = (float)y0[i];
  __syncwarp();
  const bool bad = rhs32_bound(t, lane, s, en, (float)rho_cgs);
  const float dtf = (float)dt;
  float ss = 0.f;
  for (int i = lane; i < n; i += 32) {
    const float tol = (float)(atol + rtol * fabs(y0[i]));
    const float z = dtf * (fabsf(s.f[i]) + fmaf(PRE_KAPPA, s.g[i], PRE_EPS)) / tol;
    ss = fmaf(z, z, ss);
  }
  const float nrm = sqrtf(warp_sum(ss) / nn);
  // the norm is itself rounded in FP32: a 1 % margin below the test's 1e-3
  if (bad || !(nrm <= 0.99e-3f)) return false;
  for (int i = lane; i < n; i += 32) y0[i] = fma(dt, (double)s.f[i], y0[i]);
  __syncwarp();
  return true;
}

// Packed tubes: a cell's column in the rows (its tube's block offset + its
// index) and its tube's dt; a single tube: the cell index and the launch's dt.
__device__ __forceinline__ size_t cell_col(const ChemLaunch& L, unsigned cell) {
  return L.colmap ? (size_t)L.colmap[cell] : (size_t)cell;
}
__device__ __forceinline__ double cell_dt(const ChemLaunch& L, unsigned cell, double dt) {
  return L.dt_tube ? L.dt_tube[L.tube_of[cell]] : dt;
}
__device__ __forceinline__ bool cell_active(const ChemLaunch& L, unsigned cell) {
  return !L.active_tube || L.active_tube[L.tube_of[cell]] != 0;
}

template <int TW, class Wk>
__device__ void finish_cell(const Tabs& t, const Team<TW>& tm, Wk& w, const ChemLaunch& L, unsigned cell, double dt,
                            double& speed_max);

// One tube cell: reaction_macks (SRC/source.f90:17-84) followed by the
// post-step QcToqf (SRC/main.f90:157-161). Returns the right-hand sides the
// cell took (its cost, which picks the cells that get a team next time).
template <int TW>
__device__ int tube_cell(const Tabs& t, const Team<TW>& tm, WarpWork& w, const ChemLaunch& L, unsigned cell,
                         double dt_launch, double& speed_max, ChemCounters* cnt) {
  const int tid = tm.tid;
  const int ns = t.ns;
  const size_t ld = (size_t)L.ld;
  if (!cell_active(L, cell)) return 0;
  const double dt = cell_dt(L, cell, dt_launch);
  double* q = L.qf + cell_col(L, cell) + GHOST;
  const double rho = q[0];
  // reaction_macks: y_sp = adjust_sum(Y), yiT = [y_sp, T] (SRC/source.f90:47-56);
  // the raw Y stay in the qf rows for the heat release rate.
  double s = 0.0;
  for (int k = tid; k < ns; k += TW) {
    const double yp = clip0_d(q[(3 + t.smap[k]) * ld]);
    w.y0[k] = yp;
    s += yp;
  }
  s = tm.sum(s);
  const double inv_s = 1.0 / s;
  for (int k = tid; k < ns; k += TW) w.y0[k] *= inv_s;
  if (tid == 0) w.y0[ns] = q[2 * ld];
  tm.sync();
  if constexpr (TW == 32) {
    // the single-precision pre-check: an inert cell without the FP64 f(y0)
    static_assert(sizeof(Pre32) <= offsetof(WarpWork, en) - offsetof(WarpWork, C), "Pre32 overlay");
    if (L.precheck &&
        precheck_inert(t, tid, *reinterpret_cast<Pre32*>(w.C), w.en, w.y0, rho * 1e-3, dt, L.rtol, L.atol,
                       (float)t.h->nnorm)) {
      if (tid == 0) {
        if (L.hlast) L.hlast[cell] = dt;
        atomicAdd(&cnt->steps, 1ull);
        atomicAdd(&cnt->cells, 1ull);
        atomicAdd(&cnt->cells32, 1ull);
      }
      finish_cell<TW, WarpWork>(t, tm, w, L, cell, dt, speed_max);
      return 1;
    }
  }
  // start from the first accepted step of this cell's last window
  const double hl = L.hlast ? L.hlast[cell] : 0.0;
  Cell c{rho * 1e-3, dt, L.rtol, L.atol, (hl > 0.0 && hl < dt) ? hl : dt, L.max_steps, L.screen != 0};
  CellStats st = integrate<TW>(t, tm, w, c);
  if (tid == 0 && L.hlast && !st.deferred) L.hlast[cell] = st.hnext;
  if (tid == 0) {
    add_stats(cnt, st, TW > 32);
    if (st.failed) atomicOr(L.err, EDYN_STATUS_CHEM);
  }
  if (st.deferred) {
    // screen mode (single warps only): the cell is not inert; its adjusted
    // state and f(y0) go to the next free packed row, in the full
    // mechanism's layout, for the surrogate and its gate
    if constexpr (TW == 32) {
      unsigned j = 0;
      if (tid == 0) j = atomicAdd(L.pk_count, 1u);
      j = __shfl_sync(0xffffffffu, j, 0);
      const int nrow = t.h->nnorm;
      double* y0p = L.pk_y0 + (size_t)j * nrow;
      double* f0p = L.pk_f0 + (size_t)j * nrow;
      if (ns + 1 < nrow)
        for (int i = tid; i < nrow; i += TW) y0p[i] = f0p[i] = 0.0;
      __syncwarp();
      for (int k = tid; k < ns; k += TW) {
        y0p[t.smap[k]] = w.y0[k];
        f0p[t.smap[k]] = w.dl[k];
      }
      if (tid == 0) {
        y0p[nrow - 1] = w.y0[ns];
        f0p[nrow - 1] = w.dl[ns];
        L.pk_idx[j] = cell;
        L.pk_rho[j] = rho;
        L.pk_dt[j] = dt;
      }
      __syncwarp();
    }
    return st.rhs;
  }
  finish_cell<TW, WarpWork>(t, tm, w, L, cell, dt, speed_max);
  return st.rhs;
}

// The tail of reaction_macks for one tube cell whose integration over dt left
// [Y, T] in w.y0 (the qf rows still hold the cell's Y before the step):
// adjust_sum, the heat release rate, qfToQc, then the post-step QcToqf of
// SRC/main.f90:157-161 and the cell's signal speed for the next time step.
template <int TW, class Wk>
__device__ void finish_cell(const Tabs& t, const Team<TW>& tm, Wk& w, const ChemLaunch& L, unsigned cell, double dt,
                            double& speed_max) {
  const int tid = tm.tid;
  const int ns = t.ns;
  const size_t ld = (size_t)L.ld;
  double* q = L.qf + cell_col(L, cell) + GHOST;
  double* Q = L.qc + cell_col(L, cell) + GHOST;
  const double rho = q[0];
  // the temperature the integration ended with: HRR_dot is evaluated at it
  // (SRC/source.f90:72-73 passes qf(iqtemp) = macks' T)
  if (tid == 0 && L.tchem) L.tchem[cell] = w.y0[ns];
  // adjust_sum(Y) after the step
  double s2 = 0.0;
  for (int k = tid; k < ns; k += TW) {
    const double y = clip0_d(w.y0[k]);
    w.y0[k] = y;
    s2 += y;
  }
  s2 = tm.sum(s2);
  const double inv2 = 1.0 / s2;
  const double Tn = w.y0[ns];
  // heat release rate, SRC/thermo.f90:83-103 (qf rows still hold Y0 raw)
  const double rho_cgs = rho * 1e-3;
  const bool warm = !L.strict_newton;
  double hsum[4] = {0.0, 0.0, 0.0, 0.0};  // hr / rho, hs, sz and (warm start) cp
  for (int k = tid; k < ns; k += TW) {
    const double yn = w.y0[k] * inv2;
    w.y0[k] = yn;
    const double y0raw = q[(3 + t.smap[k]) * ld];
    hsum[0] = fma(t.d.hf[k], yn - y0raw, hsum[0]);
    // qfToQc energy: e = R (H(T) - T Sz)/S_Y with the adjusted Y (S_Y = 1)
    const int r = (Tn > t.d.tmid[k]) ? 1 : 0;
    const double* ch = t.d.ch + r * 6 * NSMAX;
    double hh = fma(ch[4 * NSMAX + k], Tn, ch[3 * NSMAX + k]);
    hh = fma(hh, Tn, ch[2 * NSMAX + k]);
    hh = fma(hh, Tn, ch[1 * NSMAX + k]);
    hh = fma(hh, Tn, ch[0 * NSMAX + k]);
    hh = fma(hh, Tn, ch[5 * NSMAX + k]);
    const double z = yn * t.d.invW[k];
    hsum[1] = fma(z, hh, hsum[1]);
    hsum[2] += z;
    if (warm) {
      const double* cc = t.d.cp + r * 5 * NSMAX;
      double cp = fma(cc[4 * NSMAX + k], Tn, cc[3 * NSMAX + k]);
      cp = fma(cp, Tn, cc[2 * NSMAX + k]);
      cp = fma(cp, Tn, cc[1 * NSMAX + k]);
      cp = fma(cp, Tn, cc[0 * NSMAX + k]);
      hsum[3] = fma(z, cp, hsum[3]);
    }
  }
  tm.sumv(hsum);
  const double u = q[ld];
  // e/R of the adjusted state at the integration's final T
  const double E = hsum[1] - Tn * hsum[2];
  const double rhoe = rho * fma(R_SI, E, 0.5 * (u * u));
  // write Qc = qfToQc(qf) and qf (T, Y); the post-step QcToqf then
  // recovers T from rho e with the Newton solve.
  tm.sync();  // every thread has read the raw Y rows
  for (int k = tid; k < ns; k += TW) {
    q[(3 + t.smap[k]) * ld] = w.y0[k];
    Q[(3 + t.smap[k]) * ld] = rho * w.y0[k];
  }
  if (tid == 0) {
    Q[2 * ld] = rhoe;
    L.hrr[cell] = -((rho_cgs * hsum[0]) / dt) * 1e-1;
  }
  tm.sync();
  // post-step QcToqf: T from rho e (E = e/R). From 1000 K (strict) Newton
  // iterates as the reference does. Warm-started at Tn, its first residual
  // H(Tn) - Tn Sz - E is zero by construction (rho e was just formed from
  // the same sums at Tn), so T = Tn and the loop does not run.
  double T = L.strict_newton ? 1000.0 : Tn;
  double gN = 1e30, dTN = 1e30;
  int it = 0;
  if (warm) gN = dTN = 0.0;
  while (fabs(gN) >= fabs(E) * 1e-9 && fabs(dTN) >= T * 1e-6 && it < 10) {
    // premixed NASA coefficients at the current T (threads over species)
    double A[7] = {0, 0, 0, 0, 0, 0, 0};
    for (int k = tid; k < ns; k += TW) {
      const int r = (T > t.d.tmid[k]) ? 1 : 0;
      const double* ch = t.d.ch + r * 6 * NSMAX;
      const double z = w.y0[k] * t.d.invW[k];
      A[0] = fma(z, ch[0 * NSMAX + k], A[0]);
      A[1] = fma(z, ch[1 * NSMAX + k], A[1]);
      A[2] = fma(z, ch[2 * NSMAX + k], A[2]);
      A[3] = fma(z, ch[3 * NSMAX + k], A[3]);
      A[4] = fma(z, ch[4 * NSMAX + k], A[4]);
      A[5] = fma(z, ch[5 * NSMAX + k], A[5]);
      A[6] += z;
    }
    tm.sumv(A);
    const double Sz = A[6];
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
  if (tid == 0) {
    q[2 * ld] = T;
    // the reference's silent cap and clamps (SRC/thermo.f90:244-255) made
    // loud: Newton at its cap with both stopping tests failing, or a state
    // that is non-finite, non-positive or pinned at a clamp bound
    unsigned bad = 0;
    if (fabs(gN) >= fabs(E) * 1e-9 && fabs(dTN) >= T * 1e-6) bad |= EDYN_STATUS_NEWTON;
    if (!(rho > 0.0) || !isfinite(rhoe) || !(T > 20.0 && T < 6000.0) || !(s2 > 0.0) || !isfinite(s2))
      bad |= EDYN_STATUS_STATE;
    if (bad) atomicOr(L.err, bad);
  }
  // signal speed of the new state for the next time step (warm: T = Tn,
  // whose cp/R and S_z the sums above hold)
  if (L.cvel_out || L.cvel_tube) {
    double cp = hsum[3], Sz = hsum[2];
    if (!warm) {
      double a[6] = {0, 0, 0, 0, 0, 0};
      for (int k = tid; k < ns; k += TW) {
        const int r = (T > t.d.tmid[k]) ? 1 : 0;
        const double* ch = t.d.ch + r * 6 * NSMAX;
        const double z = w.y0[k] * t.d.invW[k];
        a[0] = fma(z, ch[0 * NSMAX + k], a[0]);
        a[1] = fma(z, ch[1 * NSMAX + k], a[1]);
        a[2] = fma(z, ch[2 * NSMAX + k], a[2]);
        a[3] = fma(z, ch[3 * NSMAX + k], a[3]);
        a[4] = fma(z, ch[4 * NSMAX + k], a[4]);
        a[5] += z;
      }
      tm.sumv(a);
      cp = fma(5.0 * a[4], T, 4.0 * a[3]);
      cp = fma(cp, T, 3.0 * a[2]);
      cp = fma(cp, T, 2.0 * a[1]);
      cp = fma(cp, T, a[0]);
      Sz = a[5];
    }
    const double gamma = cp / (cp - Sz);
    const double sp = fabs(u) + sqrt(gamma * R_SI * T * Sz);
    if (L.cvel_tube) {
      if (tid == 0) atomicMax(L.cvel_tube + L.tube_of[cell], (unsigned long long)__double_as_longlong(sp));
    } else {
      speed_max = fmax(speed_max, sp);
    }
  }
  tm.sync();
}

// Picks the cells that get a four-warp team in the next launch: those whose
// neighbourhood [i-2, i+2] took at least HOT_MIN_RHS right-hand sides in
// this launch (the reaction front moves under a cell per step), the costliest
// power-of-two classes first, at most HOT_MAX, listed in cell order. Run by
// the last CTA of a launch, after every cell's cost is written.
__device__ void select_hot(const int* cost, int n, unsigned* hot, unsigned* scratch, int scratch_words) {
  unsigned* hist = scratch;        // [33]
  unsigned* cnt = scratch + 40;    // [blockDim]
  const int nt = blockDim.x, tid = threadIdx.x;
  for (int b = tid; b < 33; b += nt) hist[b] = 0;
  // the costs staged in shared memory when they fit (independent loads, many
  // in flight), so the passes below do not wait on L2 cell by cell
  int* sc = reinterpret_cast<int*>(scratch + 512);
  const bool staged = n <= scratch_words - 512;
  if (staged) {
#pragma unroll 8
    for (int i = tid; i < n; i += nt) sc[i] = __ldcg(cost + i);
  }
  __syncthreads();
  const int chunk = (n + nt - 1) / nt;
  const int c0 = min(n, tid * chunk), c1 = min(n, c0 + chunk);
  auto nmax = [&](int i) {
    int m = 0;
    for (int j = max(0, i - 2); j <= min(n - 1, i + 2); ++j) m = max(m, staged ? sc[j] : __ldcg(cost + j));
    return m;
  };
  for (int i = c0; i < c1; ++i) {
    const int m = nmax(i);
    if (m >= HOT_MIN_RHS) atomicAdd(&hist[31 - __clz(m)], 1u);
  }
  __syncthreads();
  if (tid == 0) {
    // smallest class threshold whose cumulative count fits; if the top
    // class alone overflows, it is taken and capped in cell order
    int B = 32;
    unsigned cum = 0;
    for (int b = 30; b >= 0 && (1 << b) >= HOT_MIN_RHS; --b) {
      if (hist[b] == 0) continue;
      if (cum + hist[b] > (unsigned)HOT_MAX) {
        if (B == 32) B = b;
        break;
      }
      cum += hist[b];
      B = b;
    }
    hist[32] = (unsigned)B;
  }
  __syncthreads();
  const int B = (int)hist[32];
  unsigned mine = 0;
  if (B < 32)
    for (int i = c0; i < c1; ++i) mine += (nmax(i) >= (1 << B)) ? 1u : 0u;
  cnt[tid] = mine;
  __syncthreads();
  if (tid == 0) {
    unsigned run = 0;
    for (int q = 0; q < nt; ++q) {
      const unsigned v = cnt[q];
      cnt[q] = run;
      run += v;
    }
    hot[0] = min(run, (unsigned)HOT_MAX);
  }
  __syncthreads();
  if (B < 32) {
    unsigned pos = cnt[tid];
    for (int i = c0; i < c1 && pos < (unsigned)HOT_MAX; ++i)
      if (nmax(i) >= (1 << B)) hot[1 + pos++] = (unsigned)i;
  }
}

// Tube mode: every interior cell of the tube. The cells listed as hot by the
// previous launch go first, one per CTA, each to a four-warp team (warps
// 0-3, one per SM sub-partition; the CTA's other warps wait); then all warps
// take the remaining cells one per warp from the work counter.
__global__ void __launch_bounds__(MAXW * 32, 1)
    k_tube_chem(const char* g_tab, int tab_bytes, ChemLaunch L, unsigned* next, ChemCounters* cnt) {
  extern __shared__ __align__(16) char smem[];
  __shared__ unsigned s_hot[HOT_MAX + 1];
  __shared__ int s_last;
  if (L.step_active && *L.step_active == 0) return;
  const double dt = L.dt_dev ? *L.dt_dev : L.dt;
  for (int i = threadIdx.x; i <= HOT_MAX; i += blockDim.x) s_hot[i] = L.hot ? L.hot[i] : 0u;
  stage_tables(smem, g_tab, tab_bytes);
  const Tabs t = bind_tabs(smem);
  WarpWork* ww = work_slots(smem, tab_bytes);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double speed_max = 0.0;
  const int nwarps = blockDim.x >> 5;
  const unsigned nteam =
      (nwarps >= TEAM / 32 && !L.screen) ? min(min(s_hot[0], (unsigned)HOT_MAX), gridDim.x) : 0u;
  if (blockIdx.x < nteam) {
    const unsigned cell = s_hot[1 + blockIdx.x];
    // list mode: the screening pass finished the cell if it marked it
    // inert (cost 1); the team works only on a cell it listed (cost -1)
    const bool work = !L.list || L.cost[cell] == -1;
    if (warp < TEAM / 32 && work) {
      // team scratch: the second work slot, unused while the team runs
      double* spare = reinterpret_cast<double*>(&ww[1]);
      // the Jacobian partials of warps 1-3 go to work slots the team does not
      // otherwise use while it evaluates one (slot 0's matrix is rebuilt
      // from the Jacobian afterwards)
      const Team<TEAM> tm{(int)threadIdx.x, 1, spare, spare + 256, spare + 768, ww[2].J,
                          {ww[0].J, ww[1].J, ww[3].J}, {ww[0].b32, ww[1].b32, ww[3].b32}};
      const int c = tube_cell<TEAM>(t, tm, ww[0], L, cell, dt, speed_max, cnt);
      if (threadIdx.x == 0 && L.cost) L.cost[cell] = c;
    }
    __syncthreads();
  }
  const Team<32> tw{lane, 0, nullptr, nullptr, nullptr, nullptr};
  WarpWork& w = ww[warp];
  // every cell of the tube, or (list mode) the cells the screening pass listed
  const unsigned nwork = L.list ? *L.list_count : (unsigned)L.n;
  for (int guard = 0; guard < (1 << 30); ++guard) {
    unsigned item = 0;
    if (lane == 0) item = atomicAdd(next, 1u);
    item = __shfl_sync(0xffffffffu, item, 0);
    if (item >= nwork) break;
    const unsigned cell = L.list ? (unsigned)L.list[item] : item;
    // cells taken by a team in this launch
    bool taken = false;
    for (unsigned j = lane; j < nteam; j += 32) taken |= (s_hot[1 + j] == cell);
    if (__any_sync(0xffffffffu, taken)) continue;
    const int c = tube_cell<32>(t, tw, w, L, cell, dt, speed_max, cnt);
    if (lane == 0 && L.cost) L.cost[cell] = c;
  }
  if (L.cvel_out && lane == 0 && speed_max > 0.0)
    atomicMax(L.cvel_out, (unsigned long long)__double_as_longlong(speed_max));
  // the last CTA to finish advances the clock (device loop) and picks the
  // next launch's team cells
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned done = atomicAdd(next + 1, 1u);
    s_last = (done == gridDim.x - 1) ? 1 : 0;
  }
  __syncthreads();
  if (s_last) {
    __threadfence();
    if (L.time_tube) {
      // packed tubes: every stepping tube's clock by its own dt
      for (int q = threadIdx.x; q < L.ntube; q += blockDim.x)
        if (L.active_tube[q]) L.time_tube[q] = L.time_tube[q] + L.dt_tube[q];
      if (threadIdx.x == 0) *L.nsteps = *L.nsteps + 1;
    } else if (threadIdx.x == 0 && L.time) {
      *L.time = *L.time + dt;
      *L.nsteps = *L.nsteps + 1;
    }
    if (L.cost && L.hot && !L.screen && !L.list)
      select_hot(L.cost, L.n, L.hot, reinterpret_cast<unsigned*>(ww), (int)(nwarps * sizeof(WarpWork) / 4));
  }
}

// The packed rows' tail of a screened launch: each row's state after the
// step (pk_y1, full-mechanism layout: the surrogate's accepted candidate or
// the implicit integrator's result) goes through the same tail as a cell of
// k_tube_chem (finish_cell). One warp per row; *pk_count rows.
__global__ void __launch_bounds__(MAXW * 32, 1)
    k_tube_finish(const char* g_tab, int tab_bytes, ChemLaunch L, const double* pk_y1) {
  extern __shared__ __align__(16) char smem[];
  stage_tables(smem, g_tab, tab_bytes);
  const Tabs t = bind_tabs(smem);
  WarpWork& w = work_slots(smem, tab_bytes)[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  const Team<32> tm{lane, 0, nullptr, nullptr, nullptr, nullptr};
  const int ns = t.ns, nrow = t.h->nnorm;
  const int nw = blockDim.x >> 5;
  const unsigned m = *L.pk_count;
  double speed_max = 0.0;
  for (unsigned j = blockIdx.x * nw + (threadIdx.x >> 5); j < m; j += gridDim.x * nw) {
    const double* y = pk_y1 + (size_t)j * nrow;
    for (int k = lane; k < ns; k += 32) w.y0[k] = y[t.smap[k]];
    if (lane == 0) w.y0[ns] = y[nrow - 1];
    __syncwarp();
    finish_cell<32, WarpWork>(t, tm, w, L, (unsigned)L.pk_idx[j], L.pk_dt[j], speed_max);
    if (lane == 0 && L.cost) L.cost[L.pk_idx[j]] = 1;
  }
  if (L.cvel_out && lane == 0 && speed_max > 0.0)
    atomicMax(L.cvel_out, (unsigned long long)__double_as_longlong(speed_max));
}

// Per-warp workspace of the screening pass: one FP64 right-hand side and the
// cell's tail, no Jacobian or stage storage (7 KB against 24 KB), so a CTA
// holds 16 warps next to the tables and each SM sub-partition has four warps
// to hide the FP64 unit's latency.
struct alignas(16) ScreenWork {
  double y0[NV], fy[NV];
  double C[NV], m[NV], mi[NV], uR[NV], cvm[NV];
  double part[100];
  double rop[352];
  int en[NV];
};
static_assert(sizeof(Pre32) <= offsetof(ScreenWork, en) - offsetof(ScreenWork, C), "Pre32 overlay");
constexpr int SCREEN_WARPS = 16;

// Screening pass of a tube's source step. Every cell: y0 = adjust_sum(Y),
// f(y0) in FP64 and the integrator's inert-cell test (the first step of
// integrate()); an inert cell takes its explicit step and finishes here
// (cost 1). Any other cell is either listed (cost -1) for k_tube_chem in
// list mode, which integrates it from the same y0, or -- on the surrogate
// path (L.pk_count set) -- packed with y0 and f(y0) for the network and its
// gate. Cells are dealt in a fixed grid-stride order (their costs are
// alike); counters are summed per warp.
__global__ void __launch_bounds__(SCREEN_WARPS * 32, 1)
    k_tube_screen(const char* g_tab, int tab_bytes, ChemLaunch L, ChemCounters* cnt) {
  extern __shared__ __align__(16) char smem[];
  __shared__ int s_last;
  if (L.step_active && *L.step_active == 0) return;
  // over run heads, a CTA with none exits before staging the tables
  if (L.heads && !L.pk_count && blockIdx.x * (blockDim.x >> 5) >= *L.head_count) return;
  const double dt_launch = L.dt_dev ? *L.dt_dev : L.dt;
  stage_tables(smem, g_tab, tab_bytes);
  const Tabs t = bind_tabs(smem);
  ScreenWork& w = reinterpret_cast<ScreenWork*>(smem + ((tab_bytes + 255) / 256) * 256)[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  const Team<32> tm{lane, 0, nullptr, nullptr, nullptr, nullptr};
  const int ns = t.ns, n = ns + 1;
  const size_t ld = (size_t)L.ld;
  const float nn = (float)t.h->nnorm;
  const int nw = blockDim.x >> 5;
  double speed_max = 0.0;
  unsigned long long done = 0, listed = 0, done32 = 0, rhs64n = 0;
  // every cell, or the first cell of each run of identical cells (k_runs)
  const unsigned nwork = L.heads ? *L.head_count : (unsigned)L.n;
  for (unsigned item = blockIdx.x * nw + (threadIdx.x >> 5); item < nwork; item += gridDim.x * nw) {
    const unsigned cell = L.heads ? (unsigned)L.heads[item] : item;
    if (!cell_active(L, cell)) continue;
    const double dt = cell_dt(L, cell, dt_launch);
    const double* q = L.qf + cell_col(L, cell) + GHOST;
    const double rho = q[0];
    double s = 0.0;
    for (int k = lane; k < ns; k += 32) {
      const double yp = clip0_d(q[(3 + t.smap[k]) * ld]);
      w.y0[k] = yp;
      s += yp;
    }
    s = warp_sum(s);
    const double inv_s = 1.0 / s;
    for (int k = lane; k < ns; k += 32) w.y0[k] *= inv_s;
    if (lane == 0) w.y0[ns] = q[2 * ld];
    __syncwarp();
    // the single-precision pre-check first; the FP64 f(y0) and test where it
    // does not decide
    bool inert = L.precheck && precheck_inert(t, lane, *reinterpret_cast<Pre32*>(w.C), w.en, w.y0, rho * 1e-3, dt,
                                              L.rtol, L.atol, nn);
    if (inert) {
      ++done32;
    } else {
      rhs<double, 32>(t, tm, w, w.y0, rho * 1e-3, w.fy, w.C, w.m, w.mi, w.uR, w.cvm, w.rop, w.part);
      ++rhs64n;
      float ss = 0.f;
      for (int i = lane; i < n; i += 32) {
        const float z = (float)(dt * w.fy[i] / (L.atol + L.rtol * fabs(w.y0[i])));
        ss = fmaf(z, z, ss);
      }
      const float nrm = sqrtf(warp_sum(ss) / nn);
      if (nrm <= 1e-3f) {
        for (int i = lane; i < n; i += 32) w.y0[i] = fma(dt, w.fy[i], w.y0[i]);
        __syncwarp();
        inert = true;
      }
    }
    if (inert) {
      finish_cell<32, ScreenWork>(t, tm, w, L, cell, dt, speed_max);
      if (lane == 0) {
        if (L.cost) L.cost[cell] = 1;
        if (L.hlast) L.hlast[cell] = dt;
      }
      ++done;
    } else if (L.pk_count) {
      // surrogate path: y0 and f(y0) to the next packed row (full
      // mechanism layout), as tube_cell's screen mode does
      unsigned j = 0;
      if (lane == 0) j = atomicAdd(L.pk_count, 1u);
      j = __shfl_sync(0xffffffffu, j, 0);
      const int nrow = t.h->nnorm;
      double* y0p = L.pk_y0 + (size_t)j * nrow;
      double* f0p = L.pk_f0 + (size_t)j * nrow;
      if (ns + 1 < nrow)
        for (int i = lane; i < nrow; i += 32) y0p[i] = f0p[i] = 0.0;
      __syncwarp();
      for (int k = lane; k < ns; k += 32) {
        y0p[t.smap[k]] = w.y0[k];
        f0p[t.smap[k]] = w.fy[k];
      }
      if (lane == 0) {
        y0p[nrow - 1] = w.y0[ns];
        f0p[nrow - 1] = w.fy[ns];
        L.pk_idx[j] = (int)cell;
        L.pk_rho[j] = rho;
        L.pk_dt[j] = dt;
        // over run heads: -3 until the surrogate path's finish, which the
        // head's followers wait for (k_follow)
        if (L.cost) L.cost[cell] = L.heads ? -3 : 1;
      }
      ++listed;
    } else {
      if (lane == 0) {
        L.list[atomicAdd(L.list_count, 1u)] = (int)cell;
        if (L.cost) L.cost[cell] = -1;
      }
      ++listed;
    }
    __syncwarp();
  }
  if (lane == 0) {
    // FP64 right-hand sides: every cell the pre-check did not decide
    if (rhs64n) atomicAdd(&cnt->rhs, rhs64n);
    if (done) {
      atomicAdd(&cnt->steps, done);
      atomicAdd(&cnt->cells, done);
    }
    if (done32) atomicAdd(&cnt->cells32, done32);
    if (L.cvel_out && speed_max > 0.0)
      atomicMax(L.cvel_out, (unsigned long long)__double_as_longlong(speed_max));
  }
  // the surrogate path's screen is its step's last pass over every cell: its
  // last CTA advances the device clock (a listed launch leaves that to the
  // integrator pass that follows)
  if (L.pk_count && L.time) {
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      s_last = atomicAdd(L.pk_count + 3, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (s_last && threadIdx.x == 0) {
      __threadfence();
      *L.time = *L.time + dt_launch;
      *L.nsteps = *L.nsteps + 1;
    }
  }
}


// ---------------------------------------------------------------------------
// Runs of identical cells. A cell's source step is a function of its qf
// column (rho, u, T, Y), its tube's dt and -- when it needs the integrator --
// the step size its last window ended with (hlast) and whether a four-warp
// team or a warp integrates it. Cells whose columns are equal bit for bit
// therefore get equal results, and k_runs marks each stepping cell as the
// head of a run (its column differs from its left neighbour's, the
// neighbour is in another tube, or either is on the team list) or a
// follower, and lists the heads for the screening pass. k_follow then gives
// each follower its head's result where it is known: the head's finished
// column when the screening pass finished the head. When the head was
// listed for the integrator, a follower with the head's hlast waits for the
// head's integrated column (k_follow_integrated, after the integrator
// pass); one with another hlast is listed itself. Blocks of RUN_BLOCK cells;
// run_last[b] = the last head of block b, run_head[c] = the head of c.
// ---------------------------------------------------------------------------
constexpr int RUN_BLOCK = CHEM_RUN_BLOCK;
constexpr int RUN_THREADS = 256;

__device__ __forceinline__ bool on_hot_list(const unsigned* s_hot, int c) {
  const unsigned nh = s_hot[0];
  for (unsigned j = 0; j < nh; ++j)
    if (s_hot[1 + j] == (unsigned)c) return true;
  return false;
}

// The result of cell h is also cell c's: the finished column from T on (rho
// and u are not changed by a source step), heat release, final T, step size
// and cost.
__device__ __forceinline__ void copy_result(const ChemLaunch& L, int h, int c) {
  const size_t ld = (size_t)L.ld;
  const size_t ch = cell_col(L, h) + GHOST, cc = cell_col(L, c) + GHOST;
  int row = 2;
  // eight rows of both arrays in flight, then their stores
  for (; row + 8 <= L.nrow; row += 8) {
    double a[8], b[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      a[k] = L.qf[(row + k) * ld + ch];
      b[k] = L.qc[(row + k) * ld + ch];
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      L.qf[(row + k) * ld + cc] = a[k];
      L.qc[(row + k) * ld + cc] = b[k];
    }
  }
  for (; row < L.nrow; ++row) {
    L.qf[row * ld + cc] = L.qf[row * ld + ch];
    L.qc[row * ld + cc] = L.qc[row * ld + ch];
  }
  L.hrr[c] = L.hrr[h];
  if (L.tchem) L.tchem[c] = L.tchem[h];
  if (L.hlast) L.hlast[c] = L.hlast[h];
  L.cost[c] = L.cost[h];
}

__global__ void __launch_bounds__(RUN_THREADS) k_runs(ChemLaunch L) {
  __shared__ int s_max[RUN_THREADS / 32];
  __shared__ unsigned s_hot[HOT_MAX + 1];
  if (L.step_active && *L.step_active == 0) return;
  const int b = blockIdx.x, tid = threadIdx.x, lane = tid & 31;
  for (int j = tid; j <= HOT_MAX; j += RUN_THREADS) s_hot[j] = L.hot ? L.hot[j] : 0u;
  if (tid == 0) s_hot[0] = min(s_hot[0], (unsigned)HOT_MAX);
  __syncthreads();
  const size_t ld = (size_t)L.ld;
  int last = -1;
  for (int j = 0; j < RUN_BLOCK / RUN_THREADS; ++j) {
    const int c = b * RUN_BLOCK + j * RUN_THREADS + tid;
    unsigned char fl = 0;  // 0 not stepping, 1 head, 2 follower
    if (c < L.n && cell_active(L, c)) {
      bool same = c > 0 && (!L.tube_of || L.tube_of[c] == L.tube_of[c - 1]);
      if (same) same = !on_hot_list(s_hot, c) && !on_hot_list(s_hot, c - 1);
      if (same) {
        const double* q = L.qf + cell_col(L, c) + GHOST;
        const double* r = L.qf + cell_col(L, c - 1) + GHOST;
        // eight rows' loads in flight at a time
        for (int row = 0; row < L.nrow && same; row += 8) {
          long long x[8], y[8];
#pragma unroll
          for (int k = 0; k < 8; ++k) {
            const int rr = min(row + k, L.nrow - 1);
            x[k] = __double_as_longlong(q[rr * ld]);
            y[k] = __double_as_longlong(r[rr * ld]);
          }
#pragma unroll
          for (int k = 0; k < 8; ++k) same = same && x[k] == y[k];
        }
      }
      fl = same ? 2 : 1;
    }
    if (c < L.n) L.run_flag[c] = fl;
    const bool head = fl == 1;
    const unsigned m = __ballot_sync(0xffffffffu, head);
    if (m) {
      unsigned base = 0;
      if (lane == 0) base = atomicAdd(L.head_count, (unsigned)__popc(m));
      base = __shfl_sync(0xffffffffu, base, 0);
      if (head) L.heads[base + __popc(m & ((1u << lane) - 1u))] = c;
    }
    if (head) last = c;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) last = max(last, __shfl_xor_sync(0xffffffffu, last, o));
  if (lane == 0) s_max[tid >> 5] = last;
  __syncthreads();
  if (tid == 0) {
    int m = -1;
    for (int q = 0; q < RUN_THREADS / 32; ++q) m = max(m, s_max[q]);
    L.run_last[b] = m;
  }
}

__global__ void __launch_bounds__(RUN_THREADS) k_follow(ChemLaunch L, ChemCounters* cnt) {
  constexpr int PER = RUN_BLOCK / RUN_THREADS;  // consecutive cells of a thread in the scan
  __shared__ int s_w[RUN_THREADS / 32];
  __shared__ int s_head[RUN_BLOCK];
  __shared__ int s_carry;
  __shared__ unsigned s_copied;
  if (L.step_active && *L.step_active == 0) return;
  const int b = blockIdx.x, tid = threadIdx.x, lane = tid & 31, wq = tid >> 5;
  // the last head before this block
  int cm = -1;
  for (int q = tid; q < b; q += RUN_THREADS) cm = max(cm, L.run_last[q]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) cm = max(cm, __shfl_xor_sync(0xffffffffu, cm, o));
  if (lane == 0) s_w[wq] = cm;
  if (tid == 0) s_copied = 0u;
  __syncthreads();
  if (tid == 0) {
    int m = -1;
    for (int q = 0; q < RUN_THREADS / 32; ++q) m = max(m, s_w[q]);
    s_carry = m;
  }
  __syncthreads();
  // the head of each cell: the last head at or before it (an inclusive max
  // scan of head positions over the block, started from the carry)
  const int c0 = b * RUN_BLOCK + tid * PER;
  int hp[PER];
  int run = -1;
#pragma unroll
  for (int k = 0; k < PER; ++k) {
    const int c = c0 + k;
    if (c < L.n && L.run_flag[c] == 1) run = c;
    hp[k] = run;
  }
  int v = run;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v = max(v, t);
  }
  __syncthreads();  // s_w is reused
  if (lane == 31) s_w[wq] = v;
  __syncthreads();
  int prev = __shfl_up_sync(0xffffffffu, v, 1);
  if (lane == 0) prev = -1;
  prev = max(prev, s_carry);
  for (int q = 0; q < wq; ++q) prev = max(prev, s_w[q]);
#pragma unroll
  for (int k = 0; k < PER; ++k) s_head[tid * PER + k] = max(prev, hp[k]);
  __syncthreads();
  // the followers, one cell per thread in turn (coalesced rows)
  unsigned copied = 0;
  for (int j = 0; j < RUN_BLOCK / RUN_THREADS; ++j) {
    const int c = b * RUN_BLOCK + j * RUN_THREADS + tid;
    bool listed = false;
    if (c < L.n && L.run_flag[c] == 2) {
      const int h = s_head[c - b * RUN_BLOCK];
      if (L.cost[h] == 1) {
        copy_result(L, h, c);  // finished by the screening pass
        ++copied;
      } else if (L.cost[h] == -3 || !L.hlast ||
                 __double_as_longlong(L.hlast[c]) == __double_as_longlong(L.hlast[h])) {
        // the head's result comes from the surrogate path (a function of the
        // state alone) or from an integration that starts like this cell's
        L.run_flag[c] = 3;  // takes the head's integrated result
        L.run_head[c] = h;
        L.cost[c] = -2;
      } else {
        listed = true;
        L.cost[c] = -1;
      }
    }
    const unsigned m = __ballot_sync(0xffffffffu, listed);
    if (m) {
      unsigned base = 0;
      if (lane == 0) base = atomicAdd(L.list_count, (unsigned)__popc(m));
      base = __shfl_sync(0xffffffffu, base, 0);
      if (listed) L.list[base + __popc(m & ((1u << lane) - 1u))] = c;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) copied += __shfl_xor_sync(0xffffffffu, copied, o);
  if (lane == 0 && copied) atomicAdd(&s_copied, copied);
  __syncthreads();
  if (tid == 0 && s_copied) {
    atomicAdd(&cnt->cells, (unsigned long long)s_copied);
    atomicAdd(&cnt->steps, (unsigned long long)s_copied);
    atomicAdd(&cnt->cells_same, (unsigned long long)s_copied);
  }
}

// The followers of integrated heads (run_flag 3) take their head's result.
__global__ void __launch_bounds__(RUN_THREADS) k_follow_integrated(ChemLaunch L, ChemCounters* cnt) {
  __shared__ unsigned s_copied;
  if (L.step_active && *L.step_active == 0) return;
  if (threadIdx.x == 0) s_copied = 0u;
  __syncthreads();
  unsigned copied = 0;
  for (int j = 0; j < RUN_BLOCK / RUN_THREADS; ++j) {
    const int c = blockIdx.x * RUN_BLOCK + j * RUN_THREADS + threadIdx.x;
    if (c < L.n && L.run_flag[c] == 3) {
      copy_result(L, L.run_head[c], c);
      ++copied;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) copied += __shfl_xor_sync(0xffffffffu, copied, o);
  if ((threadIdx.x & 31) == 0 && copied) atomicAdd(&s_copied, copied);
  __syncthreads();
  if (threadIdx.x == 0 && s_copied) {
    atomicAdd(&cnt->cells, (unsigned long long)s_copied);
    atomicAdd(&cnt->cells_same, (unsigned long long)s_copied);
  }
}

// Hot-cell selection over the whole tube in parallel (the selection rule of
// select_hot): class of each cell = floor(log2) of the largest cost in
// [i-2, i+2] when at least HOT_MIN_RHS, else 0; histogram of the classes.
__global__ void k_hot_classes(const int* cost, int n, unsigned char* cls, unsigned* hist) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int m = 0;
  for (int j = max(0, i - 2); j <= min(n - 1, i + 2); ++j) m = max(m, cost[j]);
  const int c = m >= HOT_MIN_RHS ? 31 - __clz(m) : 0;
  cls[i] = (unsigned char)c;
  if (c) {
    atomicAdd(&hist[c], 1u);
    // the candidates' range: first = n - hist[33], last = hist[34] - 1
    atomicMax(&hist[33], (unsigned)(n - i));
    atomicMax(&hist[34], (unsigned)(i + 1));
  }
}

// One CTA: the smallest class threshold whose cells fit in HOT_MAX (the top
// class capped in cell order if it alone overflows), then the cells at or
// above it in cell order, by a block-wide ballot scan that stops at HOT_MAX.
__global__ void __launch_bounds__(1024) k_hot_pick(const unsigned char* cls, int n, const unsigned* hist,
                                                   unsigned* hot) {
  __shared__ int s_B;
  __shared__ unsigned warp_tot[32];
  __shared__ unsigned carry;
  if (threadIdx.x == 0) {
    int B = 32;
    unsigned cum = 0;
    for (int b = 30; b >= 0 && (1 << b) >= HOT_MIN_RHS; --b) {
      if (hist[b] == 0) continue;
      if (cum + hist[b] > (unsigned)HOT_MAX) {
        if (B == 32) B = b;
        break;
      }
      cum += hist[b];
      B = b;
    }
    s_B = B;
    carry = 0;
  }
  __syncthreads();
  const int B = s_B;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // four consecutive cells a thread per round (4096 a round): a warp-shuffle
  // scan of the per-thread counts and a scan of the warp totals; the rounds
  // span the candidates' range only
  const int first = hist[33] ? n - (int)hist[33] : n, last = (int)hist[34];
  for (int c0 = first & ~3; c0 < last && B < 32; c0 += 4 * (int)blockDim.x) {
    const int base = c0 + 4 * threadIdx.x;
    int f[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) f[j] = (base + j < n && cls[base + j] >= B) ? 1 : 0;
    const int mine = f[0] + f[1] + f[2] + f[3];
    int incl = mine;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += v;
    }
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    unsigned off = carry;
    for (int w2 = 0; w2 < warp; ++w2) off += warp_tot[w2];
    off += incl - mine;
#pragma unroll
    for (int j = 0; j < 4; ++j)
      if (f[j]) {
        if (off < (unsigned)HOT_MAX) hot[1 + off] = (unsigned)(base + j);
        ++off;
      }
    __syncthreads();
    if (threadIdx.x == 0) {
      unsigned tot = 0;
      for (int w2 = 0; w2 < (int)(blockDim.x >> 5); ++w2) tot += warp_tot[w2];
      carry += tot;
    }
    __syncthreads();
    if (carry >= (unsigned)HOT_MAX) break;
  }
  if (threadIdx.x == 0) hot[0] = B < 32 ? min(carry, (unsigned)HOT_MAX) : 0u;
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

int chem_init(ChemState& s, const edyn_mech& m, const ThermoTable& tb, cudaStream_t st, const int* smap, int nnorm) {
  (void)tb;
  const int ns = m.nspec, nr = m.nreac;
  if (ns + 1 > 54 + 2 || ns > NSMAX - 8 || nr > 352) return (int)cudaErrorInvalidValue;
  // reaction order: the fall-off reactions fill the rounds of 32 from round
  // fr0 = 3 on (a four-warp team gives those rounds to one warp); the others
  // are grouped by kind so that a 32-wide round rarely diverges: third-body,
  // Arrhenius with an exponential, constant.
  std::vector<int> fall, rest;
  for (int i = 0; i < nr; ++i) (m.tb[i] == EDYN_TB_FALLOFF ? fall : rest).push_back(i);
  auto kind = [&](int i) {
    if (m.tb[i] == EDYN_TB_M) return 1;
    const bool ex = !(m.beta[i] == 0.0 && m.E_R[i] == 0.0);
    return ex ? 2 : 3;
  };
  std::stable_sort(rest.begin(), rest.end(), [&](int a, int b) { return kind(a) < kind(b); });
  const int nfr = ((int)fall.size() + 31) / 32;
  const int fr0 = nfr > 0 ? std::min(3, (int)rest.size() / 32) : 0;
  std::vector<int> order;
  size_t ri = 0;
  while ((int)order.size() < fr0 * 32) order.push_back(rest[ri++]);
  for (int i : fall) order.push_back(i);
  while ((int)order.size() < (fr0 + nfr) * 32 && ri < rest.size()) order.push_back(rest[ri++]);
  while (ri < rest.size()) order.push_back(rest[ri++]);
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
    int dnu = 0, rord = 0, pord = 0;
    for (int sl = 0; sl < 3; ++sl) {
      const int kr = m.nunk[i][sl], kp = m.nunk[i][3 + sl];
      rs |= (unsigned)(kr >= 0 ? kr : 255) << (8 * sl);
      ps |= (unsigned)(kp >= 0 ? kp : 255) << (8 * sl);
      if (kr >= 0) {
        const int v = -m.nu[i][sl];
        if (v < 1 || v > 3) return (int)cudaErrorInvalidValue;
        nn |= (unsigned)v << (4 * sl);
        dnu -= v;
        rord += v;
      }
      if (kp >= 0) {
        const int v = m.nu[i][3 + sl];
        if (v < 1 || v > 3) return (int)cudaErrorInvalidValue;
        nn |= (unsigned)v << (12 + 4 * sl);
        dnu += v;
        pord += v;
      }
    }
    if (rord <= 3 && pord <= 3) {
      // each side as species slots with nu = 1
      rs = ps = 0xffffffu;
      nn = 0;
      int ri = 0, pi = 0;
      for (int sl = 0; sl < 3; ++sl) {
        const int kr = m.nunk[i][sl], kp = m.nunk[i][3 + sl];
        for (int v = kr >= 0 ? -m.nu[i][sl] : 0; v > 0; --v, ++ri) {
          rs = (rs & ~(0xffu << (8 * ri))) | ((unsigned)kr << (8 * ri));
          nn |= 1u << (4 * ri);
        }
        for (int v = kp >= 0 ? m.nu[i][3 + sl] : 0; v > 0; --v, ++pi) {
          ps = (ps & ~(0xffu << (8 * pi))) | ((unsigned)kp << (8 * pi));
          nn |= 1u << (12 + 4 * pi);
        }
      }
    } else {
      fl |= F_GEN;
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
      double a9[AUXW] = {m.low[i][0], m.low[i][1], m.low[i][2], m.troe[i][0], m.troe[i][1], m.troe[i][2], m.troe[i][3],
                      (double)m.ifop[i], m.low[i][0] > 0 ? std::log(m.low[i][0]) : -700.0,
                      // 1/T*** and 1/T*, capped at 1e4: beyond, exp(-T/T) is below 1e-400 at
                      // T >= 100 K, and the capped argument stays in the table exponential's range
                      std::min(1e4, 1.0 / m.troe[i][1]), std::min(1e4, 1.0 / m.troe[i][2])};
      aux.insert(aux.end(), a9, a9 + AUXW);
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
  if (npc > 100 || nsp > 64) return (int)cudaErrorInvalidValue;
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
  // four-warp teams: species k's entries over an aligned group of g_k lanes
  // (a power of two, within one warp); the group of the species with the
  // most entries per lane doubles while the 128 lanes allow
  std::vector<int> eb(ns), en_(ns), gk(ns, 1);
  {
    int b = 0;
    for (int k = 0; k < ns; ++k) {
      eb[k] = b;
      en_[k] = (int)per_sp[k].size();
      b += en_[k];
    }
  }
  if (ns > TEAM) return (int)cudaErrorInvalidValue;
  for (int used = ns;;) {
    int kb = 0;
    for (int k = 1; k < ns; ++k)
      if ((en_[k] + gk[k] - 1) / gk[k] > (en_[kb] + gk[kb] - 1) / gk[kb]) kb = k;
    if (gk[kb] >= 32 || used + gk[kb] > TEAM) break;
    used += gk[kb];
    gk[kb] *= 2;
  }
  std::vector<int> byg(ns);
  for (int k = 0; k < ns; ++k) byg[k] = k;
  std::stable_sort(byg.begin(), byg.end(), [&](int a, int b) { return gk[a] > gk[b]; });
  std::vector<int> grp(4 * TEAM, 0);
  for (int l = 0; l < TEAM; ++l) { grp[4 * l] = -1; grp[4 * l + 3] = 1; }
  int gmax = 1;
  for (int off = 0, z = 0; z < ns; ++z) {
    const int k = byg[z], g = gk[k], per = (en_[k] + g - 1) / g;
    for (int j = 0; j < g; ++j) {
      const int l = off + j;
      grp[4 * l] = k;
      grp[4 * l + 1] = eb[k] + std::min(en_[k], j * per);
      grp[4 * l + 2] = eb[k] + std::min(en_[k], (j + 1) * per);
      grp[4 * l + 3] = g;
    }
    off += g;  // sizes descending: every offset is a multiple of the group size
    gmax = std::max(gmax, g);
  }
  // species tables
  std::vector<double> W(NSMAX, 1.0), invW(NSMAX, 0.0), tmid(NSMAX, 1000.0), hf(NSMAX, 0.0);
  std::vector<double> cs(2 * 7 * NSMAX, 0.0), ch(2 * 6 * NSMAX, 0.0), cpt(2 * 5 * NSMAX, 0.0);
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
      for (int q = 0; q < 5; ++q) cpt[(r * 5 + q) * NSMAX + k] = a[q];
    }
    // CKHMS(298.15) [erg/g], as set_thermo stores std_heat_formation
    const double T = 298.15;
    const double* a = m.a[k][T > m.T_mid[k] ? 1 : 0];
    double tn[5] = {1.0, T / 2.0, T * T / 3.0, (T * T) * T / 4.0, (T * T) * (T * T) / 5.0};
    double sum = 0.0;
    for (int q = 0; q < 5; ++q) sum += tn[q] * a[q];
    hf[k] = T * RU_CGS * (sum + a[5] / T) / m.W[k];
  }
  std::vector<unsigned> ent_idx(ent.size());
  std::vector<double> ent_nu(ent.size());
  for (size_t q = 0; q < ent.size(); ++q) {
    ent_idx[q] = ent[q] & 0xffffu;
    ent_nu[q] = (double)((int)(ent[q] >> 16) - 8);
  }
  TabHdr h;
  std::memset(&h, 0, sizeof(h));
  Blob bl;
  bl.put(&h, sizeof(h));
  h.ns = ns;
  h.nr = nr;
  h.nrp = nrp;
  h.fr0 = fr0;
  h.nfr = nfr;
  h.nsp = nsp;
  h.npc = npc;
  h.ntbl = (int)tb_sp.size();
  h.nent = (int)ent.size();
  h.o_w0 = bl.put(w0.data(), w0.size() * 4);
  h.o_w1 = bl.put(w1.data(), w1.size() * 4);
  h.o_w2 = bl.put(w2.data(), w2.size() * 4);
  h.o_w3 = bl.put(w3.data(), w3.size() * 4);
  h.o_w4 = bl.put(w4.data(), w4.size() * 4);
  h.o_w5 = bl.put(w5.data(), w5.size() * 4);
  h.o_sp_i = bl.put(spi.data(), std::max<size_t>(4, spi.size() * 4));
  h.o_tb_sp = bl.put(tb_sp.data(), std::max<size_t>(4, tb_sp.size() * 4));
  h.o_pc = bl.put(pc.data(), pc.size() * 4);
  h.o_lane = bl.put(lane.data(), lane.size() * 4);
  h.o_spc = bl.put(spc.data(), spc.size() * 4);
  h.o_spp = bl.put(spp.data(), std::max<size_t>(4, spp.size() * 4));
  h.o_grp = bl.put(grp.data(), grp.size() * 4);
  h.gmax = gmax;
  {
    std::vector<int> sm(NSMAX, 0);
    for (int k = 0; k < ns; ++k) sm[k] = smap ? smap[k] : k;
    h.o_smap = bl.put(sm.data(), sm.size() * 4);
    h.nnorm = nnorm > 0 ? nnorm : ns + 1;
  }
  h.o_ent = bl.put(ent_idx.data(), std::max<size_t>(4, ent_idx.size() * 4));
  auto put2 = [&](int* off, const std::vector<double>& v) {
    std::vector<double> d(v);
    if (d.empty()) d.push_back(0.0);
    std::vector<float> f(d.size());
    for (size_t q = 0; q < d.size(); ++q) f[q] = (float)d[q];
    off[0] = bl.put(d.data(), d.size() * 8);
    off[1] = bl.put(f.data(), f.size() * 4);
  };
  put2(h.o_A, A);
  put2(h.o_lnA, lnA);  // FP32 path uses ln A, FP64 path uses A
  put2(h.o_B, B);
  put2(h.o_E, E);
  {
    // FP64 fall-off rows: k0/kinf = (lowA/A) exp((lowB - B) ln T - (lowE - E)/T),
    // so the reduced pressure needs no division
    std::vector<double> d(aux);
    if (d.empty()) d.push_back(0.0);
    std::vector<float> f(d.size());
    for (size_t q = 0; q < d.size(); ++q) f[q] = (float)d[q];
    for (int q = 0; q < nr; ++q) {
      const int i = order[q];
      if (m.tb[i] != EDYN_TB_FALLOFF) continue;
      double* fp = d.data() + (size_t)(w2[q] >> 24) * AUXW;
      fp[0] = m.A[i] > 0.0 ? m.low[i][0] / m.A[i] : 0.0;
      fp[1] = m.low[i][1] - m.beta[i];
      fp[2] = m.low[i][2] - m.E_R[i];
    }
    h.o_aux[0] = bl.put(d.data(), d.size() * 8);
    h.o_aux[1] = bl.put(f.data(), f.size() * 4);
  }
  put2(h.o_tb_am1, tb_am1);
  put2(h.o_W, W);
  put2(h.o_invW, invW);
  put2(h.o_tmid, tmid);
  put2(h.o_hf, hf);
  put2(h.o_cs, cs);
  put2(h.o_ch, ch);
  put2(h.o_cp, cpt);
  put2(h.o_nu, ent_nu);
  {
    double e2[64];
    fill_exp_table(e2);
    h.o_e2 = bl.put(e2, sizeof(e2));
    double lgt[2 * 92];
    fill_log_table(lgt);
    h.o_lg = bl.put(lgt, sizeof(lgt));
  }
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
  int maxs = 0;
  cudaDeviceGetAttribute(&maxs, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  cudaFuncAttributes fa;
  e = cudaFuncGetAttributes(&fa, k_tube_chem);
  if (e != cudaSuccess) return (int)e;
  const long room = (long)maxs - (long)tot - (long)fa.sharedSizeBytes;
  s.warps = (int)std::min<long>(MAXW, room / (long)sizeof(WarpWork));
  if (s.warps < 1) return (int)cudaErrorInvalidConfiguration;
  s.smem = tot + sizeof(WarpWork) * (size_t)s.warps;
  // the attribute serves every table set of the process: it only grows
  int cur = 0;
  {
    cudaFuncAttributes fr;
    e = cudaFuncGetAttributes(&fr, k_reactors);
    if (e != cudaSuccess) return (int)e;
    cur = std::max(fa.maxDynamicSharedSizeBytes, fr.maxDynamicSharedSizeBytes);
  }
  const int want = std::max(cur, (int)s.smem);
  e = cudaFuncSetAttribute(k_reactors, cudaFuncAttributeMaxDynamicSharedMemorySize, want);
  if (e != cudaSuccess) return (int)e;
  e = cudaFuncSetAttribute(k_tube_chem, cudaFuncAttributeMaxDynamicSharedMemorySize, want);
  if (e != cudaSuccess) return (int)e;
  e = cudaFuncSetAttribute(k_reactor_rhs, cudaFuncAttributeMaxDynamicSharedMemorySize, want);
  if (e != cudaSuccess) return (int)e;
  e = cudaFuncSetAttribute(k_hrr_dot, cudaFuncAttributeMaxDynamicSharedMemorySize, want);
  if (e != cudaSuccess) return (int)e;
  e = cudaFuncSetAttribute(k_tube_finish, cudaFuncAttributeMaxDynamicSharedMemorySize, want);
  if (e != cudaSuccess) return (int)e;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_reactors, s.warps * 32, s.smem);
  s.ctas = nsm * std::max(1, per_sm);
  // the screening pass: as many light warps as fit beside the tables
  {
    cudaFuncAttributes fs;
    e = cudaFuncGetAttributes(&fs, k_tube_screen);
    if (e != cudaSuccess) return (int)e;
    const long room_s = (long)maxs - (long)((tot + 255) / 256 * 256) - (long)fs.sharedSizeBytes;
    s.screen_warps = (int)std::min<long>(SCREEN_WARPS, room_s / (long)sizeof(ScreenWork));
    if (s.screen_warps < 1) return (int)cudaErrorInvalidConfiguration;
    s.screen_smem = (tot + 255) / 256 * 256 + sizeof(ScreenWork) * (size_t)s.screen_warps;
    const int want_s = std::max(fs.maxDynamicSharedSizeBytes, (int)s.screen_smem);
    e = cudaFuncSetAttribute(k_tube_screen, cudaFuncAttributeMaxDynamicSharedMemorySize, want_s);
    if (e != cudaSuccess) return (int)e;
    int per_sm_s = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_s, k_tube_screen, s.screen_warps * 32, s.screen_smem);
    s.screen_ctas = nsm * std::max(1, per_sm_s);
  }
  return 0;
}

cudaError_t chem_launch_batch(ChemState& s, const ChemLaunch& L, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(s.d_next, 0, 2 * sizeof(unsigned), st);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(s.d_count, 0, sizeof(ChemCounters), st);
  if (e != cudaSuccess) return e;
  const int grid = std::min(s.ctas, (L.n + s.warps - 1) / s.warps);
  k_reactors<<<std::max(1, grid), s.warps * 32, s.smem, st>>>((const char*)s.d_tables, (int)s.table_bytes, L.n,
                                                            L.rho_batch, L.dt_batch, L.yiT_batch, L.rtol, L.atol,
                                                            L.max_steps, s.d_next, s.d_count, L.err);
  return cudaGetLastError();
}

cudaError_t chem_rhs_batch(ChemState& s, int n, const double* rho, const double* yiT, double* f, cudaStream_t st) {
  const int grid = std::min(s.ctas, (n + s.warps - 1) / s.warps);
  k_reactor_rhs<<<std::max(1, grid), s.warps * 32, s.smem, st>>>((const char*)s.d_tables, (int)s.table_bytes, n, rho,
                                                                yiT, f);
  return cudaGetLastError();
}

cudaError_t chem_hrr_dot(ChemState& s, int n, int ld, const double* qf, const double* tchem, double* out,
                         const int* colmap, cudaStream_t st) {
  const int grid = std::min(s.ctas, (n + s.warps - 1) / s.warps);
  k_hrr_dot<<<std::max(1, grid), s.warps * 32, s.smem, st>>>((const char*)s.d_tables, (int)s.table_bytes, n, ld, qf,
                                                            tchem, out, colmap);
  return cudaGetLastError();
}

cudaError_t chem_finish_packed(ChemState& s, const ChemLaunch& L, int m, const double* pk_y1, cudaStream_t st) {
  if (m <= 0) return cudaSuccess;
  const int grid = std::min(s.ctas, (m + s.warps - 1) / s.warps);
  k_tube_finish<<<std::max(1, grid), s.warps * 32, s.smem, st>>>((const char*)s.d_tables, (int)s.table_bytes, L,
                                                               pk_y1);
  return cudaGetLastError();
}

namespace {
// Clears a launch's counters unless the device loop skips this step (the
// counters then keep the last step that ran).
__global__ void k_clear_counters(const int* step_active, ChemCounters* cnt) {
  if (step_active && *step_active == 0) return;
  *cnt = ChemCounters{0, 0, 0, 0, 0, 0, 0};
}
}  // namespace

cudaError_t chem_launch_tube_listed(ChemState& s, const ChemLaunch& L0, int* list, unsigned* list_count,
                                    unsigned char* cls, unsigned* hist, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(s.d_next, 0, 2 * sizeof(unsigned), st);
  if (e != cudaSuccess) return e;
  k_clear_counters<<<1, 1, 0, st>>>(L0.step_active, s.d_count);
  e = cudaMemsetAsync(list_count, 0, sizeof(unsigned), st);
  if (e != cudaSuccess) return e;
  ChemLaunch L = L0;
  L.list = list;
  L.list_count = list_count;
  const int nblk = (L.n + RUN_BLOCK - 1) / RUN_BLOCK;
  if (L.heads) {
    e = cudaMemsetAsync(L.head_count, 0, sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    k_runs<<<nblk, RUN_THREADS, 0, st>>>(L);
  }
  const int sgrid = std::min(s.screen_ctas, (L.n + s.screen_warps - 1) / s.screen_warps);
  k_tube_screen<<<std::max(1, sgrid), s.screen_warps * 32, s.screen_smem, st>>>((const char*)s.d_tables,
                                                                              (int)s.table_bytes, L, s.d_count);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if (L.heads) k_follow<<<nblk, RUN_THREADS, 0, st>>>(L, s.d_count);
  k_tube_chem<<<s.ctas, s.warps * 32, s.smem, st>>>((const char*)s.d_tables, (int)s.table_bytes, L, s.d_next,
                                                    s.d_count);
  if (L.heads) k_follow_integrated<<<nblk, RUN_THREADS, 0, st>>>(L, s.d_count);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if (L.cost && L.hot) {
    e = cudaMemsetAsync(hist, 0, 35 * sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    k_hot_classes<<<(L.n + 255) / 256, 256, 0, st>>>(L.cost, L.n, cls, hist);
    k_hot_pick<<<1, 1024, 0, st>>>(cls, L.n, hist, L.hot);
    e = cudaGetLastError();
  }
  return e;
}

cudaError_t chem_launch_screen_packed(ChemState& s, const ChemLaunch& L, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(s.d_count, 0, sizeof(ChemCounters), st);
  if (e != cudaSuccess) return e;
  const int nblk = (L.n + RUN_BLOCK - 1) / RUN_BLOCK;
  if (L.heads) {
    e = cudaMemsetAsync(L.head_count, 0, sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    k_runs<<<nblk, RUN_THREADS, 0, st>>>(L);
  }
  const int sgrid = std::min(s.screen_ctas, (L.n + s.screen_warps - 1) / s.screen_warps);
  k_tube_screen<<<std::max(1, sgrid), s.screen_warps * 32, s.screen_smem, st>>>((const char*)s.d_tables,
                                                                              (int)s.table_bytes, L, s.d_count);
  e = cudaGetLastError();
  if (e == cudaSuccess && L.heads) k_follow<<<nblk, RUN_THREADS, 0, st>>>(L, s.d_count);
  return cudaGetLastError();
}

cudaError_t chem_follow_packed(ChemState& s, const ChemLaunch& L, cudaStream_t st) {
  if (!L.heads) return cudaSuccess;
  k_follow_integrated<<<(L.n + RUN_BLOCK - 1) / RUN_BLOCK, RUN_THREADS, 0, st>>>(L, s.d_count);
  return cudaGetLastError();
}

cudaError_t chem_launch_tube(ChemState& s, const ChemLaunch& L, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(s.d_next, 0, 2 * sizeof(unsigned), st);
  if (e != cudaSuccess) return e;
  k_clear_counters<<<1, 1, 0, st>>>(L.step_active, s.d_count);
  const int grid = std::min(s.ctas, (L.n + s.warps - 1) / s.warps);
  k_tube_chem<<<std::max(1, grid), s.warps * 32, s.smem, st>>>((const char*)s.d_tables, (int)s.table_bytes, L,
                                                             s.d_next, s.d_count);
  return cudaGetLastError();
}

namespace {
// texp against CUDA's exp on the same arguments: the largest difference in
// units in the last place of CUDA's result (device-wide max via the bit
// pattern of a non-negative double).
__global__ void k_check_exp(const char* g_tab, int n, const double* x, unsigned long long* maxulp) {
  __shared__ double e2[64];
  const TabHdr* h = (const TabHdr*)g_tab;
  if (threadIdx.x < 64) e2[threadIdx.x] = ((const double*)(g_tab + h->o_e2))[threadIdx.x];
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double a = exp(x[i]), b = texp(x[i], e2);
  const double ulp = __longlong_as_double(__double_as_longlong(fabs(a)) + 1) - fabs(a);
  const double u = fabs(a - b) / ulp;
  atomicMax(maxulp, (unsigned long long)__double_as_longlong(u));
}
// tlog against CUDA's log, as k_check_exp.
__global__ void k_check_log(const char* g_tab, int n, const double* x, unsigned long long* maxulp) {
  __shared__ double lg[184];
  const TabHdr* h = (const TabHdr*)g_tab;
  for (int q = threadIdx.x; q < 184; q += blockDim.x) lg[q] = ((const double*)(g_tab + h->o_lg))[q];
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double a = log(x[i]), b = tlog(x[i], lg);
  const double ulp = __longlong_as_double(__double_as_longlong(fabs(a)) + 1) - fabs(a);
  const double u = fabs(a - b) / ulp;
  atomicMax(maxulp, (unsigned long long)__double_as_longlong(u));
}
}  // namespace

cudaError_t chem_check_log(ChemState& s, int n, const double* x_d, unsigned long long* maxulp_d, cudaStream_t st) {
  k_check_log<<<(n + 255) / 256, 256, 0, st>>>((const char*)s.d_tables, n, x_d, maxulp_d);
  return cudaGetLastError();
}

cudaError_t chem_check_exp(ChemState& s, int n, const double* x_d, unsigned long long* maxulp_d, cudaStream_t st) {
  k_check_exp<<<(n + 255) / 256, 256, 0, st>>>((const char*)s.d_tables, n, x_d, maxulp_d);
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
