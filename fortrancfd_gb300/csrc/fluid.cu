// Fused fluid stage kernel and its helpers (sm_103a).
//
// One launch performs one stage of the reference's explicit time integrator
// for a whole tube (SRC/timeintegration.f90: explicit_euler 12-96, TVDRK3
// 99-219): face reconstruction (SRC/muscl.f90, SRC/weno.f90), the face
// equation of state (qfToQc, SRC/eos.f90:11-46, plus pressure and sound
// speed), the LxF / HLL / HLLC flux (SRC/flux.f90:130-373), the conservative
// Runge-Kutta update, and QcToqf with the temperature Newton solve
// (SRC/eos.f90:49-83, SRC/thermo.f90:211-257) for every owned cell. Ghost
// cells at the tube ends are produced in the consuming kernel from the
// boundary rule (SRC/boundary.f90:12-199), so no separate boundary pass or
// ghost-copy launch exists. The stage that finishes a step also reduces the
// maximum signal speed for the next CFL time step (SRC/update.f90:13-59).
//
// Layout in HBM: structure of arrays, one row of ld = n + 2*GHOST doubles
// per variable; cell i lives at column i + GHOST. qf rows are (rho, u, T,
// Y_1..Y_K), Qc rows are (rho, rho u, rho e, rho Y_1..rho Y_K).
//
// Work split: one thread per face and per cell (team size 1); a CTA of NT
// threads owns NT-1 cells and the NT faces that bound them, stages the
// primitive state of its cells plus lvir halo cells in shared memory with
// coalesced row loads, writes face fluxes to shared memory and then updates
// its cells. Every per-species quantity is a streaming loop over constant
// memory tables, so the kernel is bound by the FP64 pipe, not by HBM.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "edyn_dev.cuh"
#include "edyn_kernels.h"
#include "fastmath.cuh"
#include "recon.cuh"

namespace edyn {

__constant__ ThermoTable c_thermo;

static_assert(sizeof(ThermoTable) < 60000, "constant tables too large");

// ---------------------------------------------------------------------------
// Cell equation of state: QcToqf (SRC/eos.f90:49-83).
// ys: per-thread strided species scratch holding rho*Y_k on entry; on exit it
// holds the clipped, renormalised mass fractions (the qf species entries).
// Returns T; writes u. strict = Newton starts at 1000 K as the reference.
// ---------------------------------------------------------------------------
struct CellEOS {
  double T, u, Sz, cpR;  // cpR = Cp(T) of the final premix, for the sound speed
  unsigned status;       // EDYN_E_NEWTON / EDYN_E_STATE bits of this cell (0: sound)
};

// Status bits of one cell's QcToqf, which the reference leaves silent
// (temperature_con stops at its iteration cap and clamps T to [20, 6000] K,
// SRC/thermo.f90:244-255): EDYN_E_NEWTON when the Newton ended at the cap
// with neither stopping test met, EDYN_E_STATE for a non-positive or
// non-finite density, energy or mass-fraction sum, or a temperature pinned
// at a clamp bound.
__device__ __forceinline__ unsigned cell_status(double rho, double E, double sy, double T, int iters) {
  unsigned st = 0;
  if (iters < 0) st |= EDYN_STATUS_NEWTON;
  if (!(rho > 0.0) || !isfinite(rho) || !isfinite(E) || !(sy > 0.0) || !isfinite(sy) || !(T > 20.0 && T < 6000.0))
    st |= EDYN_STATUS_STATE;
  return st;
}

// Sum of v over an aligned group of S lanes (a power of two) that split a
// cell's species between them (identity for S = 1), by an xor tree: every
// lane of the group gets the same bits (each level adds the same two
// partial sums, in either order, and addition commutes).
template <int S>
__device__ __forceinline__ double pair_sum(double v, unsigned mask) {
#pragma unroll
  for (int o = 1; o < S; o <<= 1) v += __shfl_xor_sync(mask, v, o);
  return v;
}

template <int S>
__device__ __forceinline__ void pair_sum(Premix& pm, unsigned mask) {
#pragma unroll
  for (int n = 0; n < 6; ++n) pm.A[n] = pair_sum<S>(pm.A[n], mask);
}

// Premixed NASA-7 coefficients of a cell; with S > 1 the thread takes the
// species k = h, h + S, ... and the group sums its parts.
template <int S = 1>
__device__ __forceinline__ void premix_cell(const double* ys, int st, double T, Premix& pm, double& Sz, int h = 0,
                                            unsigned mask = 0u) {
  const ThermoTable& tb = c_thermo;
  pm.zero(t_interval(tb, T));
  double sz = 0.0;
  for (int k = h; k < tb.ns; k += S) {
    double z = ys[k * st] * tb.invW[k];
    sz += z;
    premix_add(tb, pm, k, z, T);
  }
  Sz = pair_sum<S>(sz, mask);
  pair_sum<S>(pm, mask);
}

// Newton on sum z_k u_k(T) = e for T (temperature_con, SRC/thermo.f90:211-257)
// in the premixed variables: g(T) = H(T) - T Sz - E, dg/dT = Cp(T) - Sz.
// The threads of a group iterate alike (same sums, same iterates).
template <int S = 1>
__device__ __forceinline__ double t_newton(const double* ys, int st, double E, double T0, Premix& pm, double& Sz,
                                           int& iters, int h = 0, unsigned mask = 0u) {
  const ThermoTable& tb = c_thermo;
  double T = T0, g = 1e30, dT = 1e30;
  int it = 0;
  premix_cell<S>(ys, st, T, pm, Sz, h, mask);
  while (fabs(g) >= fabs(E) * 1e-9 && fabs(dT) >= T * 1e-6 && it < 10) {
    if (t_interval(tb, T) != pm.interval) premix_cell<S>(ys, st, T, pm, Sz, h, mask);
    g = pm.H(T) - T * Sz - E;
    double cvR = pm.Cp(T) - Sz;
    dT = -g / cvR;
    T = fmax(20.0, fmin(6000.0, T + dT));
    ++it;
  }
  if (t_interval(tb, T) != pm.interval) premix_cell<S>(ys, st, T, pm, Sz, h, mask);
  // the cap ended the loop while both stopping tests still failed: -it
  iters = (fabs(g) >= fabs(E) * 1e-9 && fabs(dT) >= T * 1e-6) ? -it : it;
  return T;
}

// Full QcToqf. On entry ys[k*st] = rho*Y_k. Writes the normalised Y_k back
// (with S > 1, the species k = h, h + S, ... of this thread).
template <int S = 1>
__device__ __forceinline__ CellEOS qc_to_qf_cell(double rho, double rhou, double rhoe, double* ys, int st,
                                                 double Tguess, bool strict, int& iters, int h = 0,
                                                 unsigned mask = 0u) {
  const ThermoTable& tb = c_thermo;
  CellEOS r;
  const double inv_rho = 1.0 / rho;
  r.u = rhou * inv_rho;
  double s = 0.0;
  for (int k = h; k < tb.ns; k += S) {
    double y = clip0(ys[k * st] * inv_rho);
    ys[k * st] = y;
    s += y;
  }
  s = pair_sum<S>(s, mask);
  const double inv_s = 1.0 / s;
  for (int k = h; k < tb.ns; k += S) ys[k * st] *= inv_s;
  const double e_int = rhoe * inv_rho - 0.5 * (r.u * r.u);
  const double E = e_int * (1.0 / R_SI);
  Premix pm;
  double Sz;
  r.T = t_newton<S>(ys, st, E, strict ? 1000.0 : Tguess, pm, Sz, iters, h, mask);
  r.Sz = Sz;
  r.cpR = pm.Cp(r.T);
  r.status = cell_status(rho, E, s, r.T, iters);
  return r;
}

// Signal speed max(|u-a|,|u|,|u+a|) = |u| + a of calc_dt (SRC/update.f90:33-41)
// from a cell's primitive state: a^2 = gamma p / rho = gamma R T Sz / S_Y.
__device__ __forceinline__ double cell_speed(double u, double T, double Sz, double cpR) {
  double gamma = cpR / (cpR - Sz);
  double a = sqrt(gamma * R_SI * T * Sz);
  return fabs(u) + a;
}

__device__ __forceinline__ void atomic_max_pos(unsigned long long* addr, double v) {
  atomicMax(addr, (unsigned long long)__double_as_longlong(v));
}

// ---------------------------------------------------------------------------
// Face equation of state for a reconstructed state (qfToQc + pressure +
// sonic_speed, SRC/eos.f90:11-46, SRC/thermo.f90:166-179, 421-430).
// ---------------------------------------------------------------------------
struct FaceState {
  double rho, u, T, p, a, E;     // E = rho e (total)
  double inv_SY;                 // 1 / sum max(Y,0)
};

__device__ __forceinline__ void face_finish(FaceState& f, const Premix& pm, double SY, double Sz) {
  f.inv_SY = 1.0 / SY;
  const double rt = f.rho * f.T;
  const double zr = Sz * f.inv_SY;              // S_z / S_Y = 1 / mean molar weight
  f.p = R_SI * rt * zr;
  const double e_int = R_SI * (pm.H(f.T) - f.T * Sz) * f.inv_SY;
  f.E = f.rho * (e_int + 0.5 * (f.u * f.u));
  const double cpR = pm.Cp(f.T);
  const double gamma = cpR / (cpR - Sz);
  f.a = sqrt(gamma * R_SI * f.T * zr);
}

// The tube a stage CTA works on: the context's one tube, or one tube of a
// packed set (its block's columns, cell size, outlet pressure, clock).
struct TubeView {
  int n;
  const double* qf_in;
  double *qf_out, *qc, *q0, *acc;
  double dx, p_out;
  unsigned long long* cvel;  // signal-speed maximum of this tube (or null)
  int tube = 0;              // index among packed tubes
  long long off = 0;         // column offset of the tube's block among packed tubes
  double x0 = 0.0;           // SMR segments: the coordinate of the segment's left edge
};

// minmod slope of interpolation_block: 0.5 (sign(1, m) + sign(1, p)) min(|m|, |p|)
__device__ __forceinline__ double smr_slope(double m, double p) {
  return 0.5 * (copysign(1.0, m) + copysign(1.0, p)) * fmin(fabs(m), fabs(p));
}

// Conserved column of the ghost l (1..lvir) that segment t takes from its
// neighbour across interface j (SRC/block.f90:488-567), from the snapshot:
// a plain copy between equal cell sizes; on the coarse side the mean of two
// fine cells; on the fine side the coarse cell -+ 1/4 of its minmod slope,
// the coarse side's first ghost (a mean of two fine cells) serving as its
// neighbour across the interface.
__device__ __noinline__ void smr_ghost_qc(const StageArgs& a, int t, int g, int n, double& q0, double& q1, double& q2,
                                          double* ys, int st) {
  const TubeTab& T = a.tubes;
  const int S = 2 * a.lvir;
  const int ne = a.ns + 3;
  const bool left = g < 0;  // a left ghost of segment t: interface t-1
  const int j = left ? t - 1 : t;
  const int l = left ? -g : g - n + 1;
  const double dxl = T.dx[j], dxr = T.dx[j + 1];
  const double* base = T.smr_snap + (size_t)j * 2 * ne * S;
  for (int v = 0; v < ne; ++v) {
    const double* sl = base + (size_t)v * S;         // segment j: cell iend + idx at S - 1 + idx (idx <= 0)
    const double* sr = base + (size_t)(ne + v) * S;  // segment j+1: cell idx at idx (idx >= 0)
    auto lx = [&](int idx) {  // segment j's cells and, past its end, its restricted ghosts
      return idx <= 0 ? sl[S - 1 + idx] : (sr[2 * (idx - 1)] + sr[2 * (idx - 1) + 1]) / 2.0;
    };
    auto rx = [&](int idx) {  // segment j+1's cells and, before its start, its restricted ghosts
      return idx >= 0 ? sr[idx] : (sl[S - 1 - 2 * (-idx - 1)] + sl[S - 1 - 2 * (-idx - 1) - 1]) / 2.0;
    };
    double q;
    if (dxl == dxr) {
      q = left ? lx(-(l - 1)) : rx(l - 1);
    } else if (dxl > dxr) {  // coarse | fine
      if (!left) {
        q = lx(l);
      } else {
        const int ic = -((l - 1) / 2);
        const double c = lx(ic);
        const double d = smr_slope(c - lx(ic - 1), lx(ic + 1) - c);
        q = (l % 2 == 1) ? c + 0.25 * d : c - 0.25 * d;
      }
    } else {  // fine | coarse
      if (left) {
        q = rx(-l);
      } else {
        const int ic = (l - 1) / 2;
        const double c = rx(ic);
        const double d = smr_slope(c - rx(ic - 1), rx(ic + 1) - c);
        q = (l % 2 == 1) ? c - 0.25 * d : c + 0.25 * d;
      }
    }
    if (v == 0) q0 = q;
    else if (v == 1) q1 = q;
    else if (v == 2) q2 = q;
    else ys[(v - 3) * st] = q;
  }
}

// ---------------------------------------------------------------------------
// Boundary ghost cells (SRC/boundary.f90). ghost_qc computes the conserved
// column of the ghost cell g (g < 0 left, g >= n right) from the interior
// conserved state in global memory: q0, q1, q2 and ys[k*st] = rho Y_k.
// ghost_cell adds its QcToqf and stores the primitive state into the shared
// stencil.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void ghost_qc(const StageArgs& a, const TubeView& v, int g, double& q0, double& q1,
                                         double& q2, double* ys, int st) {
  const ThermoTable& tb = c_thermo;
  const int ns = tb.ns;
  const int ld = a.ld;
  int iters;
  if (a.tubes.smr_snap && (g < 0 ? v.tube > 0 : v.tube < a.tubes.ntube - 1)) {
    smr_ghost_qc(a, v.tube, g, v.n, q0, q1, q2, ys, st);
    return;
  }
  if (g < 0) {
    const int l = -g;  // 1..lvir
    const int src = l - 1;
    const double* Q = v.qc + src + GHOST;
    if (a.lbound == 0) {  // lbound_wall 152-174
      q0 = Q[0];
      q1 = -Q[ld];
      q2 = Q[2 * ld];
      for (int k = 0; k < ns; ++k) ys[k * st] = Q[(3 + k) * ld];
    } else {  // lbound_inlet 70-103
      const double rho_in = Q[0];
      const double u_in = a.bc.rho_u_in / rho_in;
      q0 = rho_in;
      q1 = a.bc.rho_u_in;
      q2 = rho_in * (a.bc.e_in + 0.5 * (u_in * u_in));
      for (int k = 0; k < ns; ++k) ys[k * st] = rho_in * a.bc.y_in[k];
    }
  } else {
    const int l = g - v.n + 1;  // 1..lvir
    const int src = v.n - l;
    const double* Q = v.qc + src + GHOST;
    if (a.rbound == 0) {  // rbound_wall 177-199
      q0 = Q[0];
      q1 = -Q[ld];
      q2 = Q[2 * ld];
      for (int k = 0; k < ns; ++k) ys[k * st] = Q[(3 + k) * ld];
    } else {  // rbound_outlet 106-149: fixed p_out, T from the interior energy
      const double rho_i = Q[0], inv = 1.0 / rho_i;
      const double u_out = Q[ld] * inv;
      const double e_out = Q[2 * ld] * inv - 0.5 * (u_out * u_out);
      double sy = 0.0, sz = 0.0;
      for (int k = 0; k < ns; ++k) {
        double y = Q[(3 + k) * ld] * inv;  // no clipping in the reference here
        ys[k * st] = y;
        sy += y;
        sz += y * tb.invW[k];
      }
      // temperature_con with the unclipped mole fractions: E scaled by S_Y.
      Premix pm;
      double Sz;
      const double E = e_out * sy * (1.0 / R_SI);
      double T_out = t_newton(ys, st, E, 1000.0, pm, Sz, iters);
      (void)sz;
      const double rho_out = v.p_out * sy / (R_SI * T_out * Sz);
      const double e2 = R_SI * (pm.H(T_out) - T_out * Sz) / sy;
      q0 = rho_out;
      q1 = rho_out * u_out;
      q2 = rho_out * (e2 + 0.5 * (u_out * u_out));
      for (int k = 0; k < ns; ++k) ys[k * st] = rho_out * ys[k * st];
    }
  }
}

__device__ void ghost_cell(const StageArgs& a, const TubeView& v, int g, double* dst, int dst_st, double* ys, int st) {
  const int ns = c_thermo.ns;
  double q0, q1, q2;
  int iters;
  ghost_qc(a, v, g, q0, q1, q2, ys, st);
  CellEOS e = qc_to_qf_cell(q0, q1, q2, ys, st, 1000.0, true, iters);
  if (e.status && a.err) atomicOr(a.err, e.status);
  dst[0] = q0;
  dst[dst_st] = e.u;
  dst[2 * dst_st] = e.T;
  for (int k = 0; k < ns; ++k) dst[(3 + k) * dst_st] = ys[k * st];
}

// ---------------------------------------------------------------------------
// The stage kernel.
// ---------------------------------------------------------------------------
// SPH = 1: spherical geometry (is_spherical, SRC/flux.f90:272-278,
// SRC/timeintegration.f90:58-75, 177-198): the momentum flux carries no
// pressure, the update weighs the face fluxes by the face areas r^2 over
// the cell volume, and the momentum takes the gradient of the faces' Roe-
// averaged pressures separately, after the stage combination, as written.
template <int ACU, int LIM, int WFLAG, int RIEMANN, int SPH = 0>
__global__ void __launch_bounds__(STAGE_MAX_THREADS) k_stage(StageArgs a) {
  constexpr int LV = acu_lvir(ACU);
  extern __shared__ double sm[];
  const int TC = a.tc;        // cells of a tile
  const int P = TC + 2;       // positions: the cells c0-1..c0+TC, or the faces c0..c0+TC
  constexpr int SP = STAGE_SPLIT;
  const int NT = blockDim.x;  // whole warps, at least SP threads per position
  const int tid = threadIdx.x;
  // Tile of this CTA: cells [c0, c1), TC wide. The right-end ghost cells are
  // built from the conserved state of the last LV cells, which the stage
  // updates in place, so those cells and every window that holds a ghost
  // built from them must belong to one CTA: when the last tile would hold
  // fewer than LV cells, the boundary between the last two tiles moves to
  // n - LV. (The first tile always holds the first LV cells.)
  // The CTA's tube: the context's one tube, or (packed tubes) the tube of
  // this tile, with that tube's own dt.
  TubeView tv{a.n, a.qf_in, a.qf_out, a.qc, a.q0, a.acc, a.dx, a.p_out, a.cvel_out};
  int tile = blockIdx.x, nb = gridDim.x, tube = 0;
  double dt = a.dt;
  if (a.step_active) {
    if (*a.step_active == 0) return;
    dt = *a.dt_dev;
  }
  if (a.tubes.tiles) {
    const int4 tl = a.tubes.tiles[blockIdx.x];
    tube = tl.x;
    tile = tl.y;
    nb = tl.z;
    if (a.tubes.active && a.tubes.active[tube] == 0) return;
    const long long off = a.tubes.off[tube];
    tv.n = a.tubes.n[tube];
    tv.qf_in = a.qf_in + off;
    tv.qf_out = a.qf_out + off;
    tv.qc = a.qc + off;
    tv.q0 = a.q0 + off;
    tv.acc = a.acc ? a.acc + off : nullptr;
    tv.dx = a.tubes.dx[tube];
    tv.p_out = a.tubes.p_out[tube];
    tv.cvel = a.cvel_out ? a.cvel_out + tube : nullptr;
    tv.tube = tube;
    if constexpr (SPH != 0) tv.x0 = a.tubes.x0 ? a.tubes.x0[tube] : 0.0;
    dt = a.tubes.dt[tube];
  }
  int c0 = tile * TC;
  int c1 = min(c0 + TC, tv.n);
  if (nb >= 2 && tv.n - (nb - 1) * TC < LV) {
    if (tile == nb - 1) c0 = tv.n - LV;
    if (tile == nb - 2) c1 = tv.n - LV;
  }
  // stencil window [c0 - LW, c0 + TC + LW): the cells c0-1..c1 whose face
  // values the tile needs, each with its reconstruction radius LV - 1, and
  // one more cell on each side, which decides whether the tile's end faces
  // are needed (1b)
  constexpr int LW = LV + 1;
  const int Wd = TC + 2 * LW;
  const ThermoTable& tb = c_thermo;
  const int ns = a.ns, ne = ns + 3;
  double* s_q = sm;             // [ne][Wd] primitive window
  double* s_l = s_q + ne * Wd;  // [ne][P] value at the right face of cell c0-1+p (left state of face c0+p);
                                //         then the flux of face c0+p
  double* s_r = s_l + ne * P;   // [ne][P] value at the left face of cell c0-1+p (right state of face c0-1+p);
                                //         then per-thread species scratch
  // s_diff[w]: window cells w and w + 1 differ in some primitive (bitwise)
  __shared__ unsigned char s_diff[STAGE_MAX_CELLS + 2 * 5];
  // SPH: Roe-averaged pressure of each face (the reference's godunov_state)
  __shared__ double s_pg[SPH ? STAGE_MAX_CELLS + 2 : 1];
  const bool skip_uniform = a.skip_uniform != 0;
  if (skip_uniform)
    for (int w = tid; w < Wd; w += NT) s_diff[w] = 0;

  // 1. stage the primitive state window (coalesced row loads)
#pragma unroll 4
  for (int idx = tid; idx < ne * Wd; idx += NT) {
    const int v = idx / Wd, j = idx - v * Wd;
    const int cell = c0 - LW + j;
    if (cell >= 0 && cell < tv.n) s_q[idx] = tv.qf_in[(size_t)v * a.ld + cell + GHOST];
  }
  // ghost cells of the tube ends inside the window: thread t < LV takes the
  // left ghost -1-t, thread LV <= t < 2 LV the right ghost n + t - LV.
  if (tid < 2 * LV) {
    const int g = (tid < LV) ? -1 - tid : tv.n + (tid - LV);
    // (the ghosts of the stencils only: a ghost is built from the conserved
    // state of the tube's end cells, which only their own tile may read
    // while this stage updates them)
    if (g >= c0 - LV && g < c1 + LV) ghost_cell(a, tv, g, s_q + (g - (c0 - LW)), Wd, s_r + tid, P);
  }
  __syncthreads();

  // 1b. Uniform neighbourhoods. A tube cell c whose cells c-LV..c+LV hold
  //     one state bit for bit has two faces with identical inputs, hence
  //     identical fluxes and dF = 0 exactly ("frozen"); a face between two
  //     frozen cells is needed by neither, and a reconstruction only by a
  //     needed face. An owned cell's test reads tube cells and stencil
  //     ghosts only; the outer window positions (unloaded where they fall
  //     on a ghost) enter only the tests of the cells next to the tile,
  //     which decide nothing but whether the tile's end faces are skipped,
  //     and an end face is skipped only next to a frozen owned cell, whose
  //     dF is zero without it.
  if (skip_uniform) {
    for (int idx = tid; idx < ne * (Wd - 1); idx += NT) {
      const int v = idx / (Wd - 1), w = idx - v * (Wd - 1);
      if (__double_as_longlong(s_q[v * Wd + w]) != __double_as_longlong(s_q[v * Wd + w + 1])) s_diff[w] = 1;
    }
    __syncthreads();
  }
  auto frozen = [&](int c) -> bool {
    if (!skip_uniform || c < 0 || c >= tv.n) return false;
    const int wc = c - (c0 - LW);
    if (wc - LV < 0 || wc + LV - 1 > Wd - 2) return false;
    for (int w = wc - LV; w < wc + LV; ++w)
      if (s_diff[w]) return false;
    return true;
  };
  // face c0+f (between cells c0-1+f and c0+f) is computed
  auto need_face = [&](int f) -> bool {
    return f >= 0 && c0 + f <= c1 && !(frozen(c0 - 1 + f) && frozen(c0 + f));
  };

  // 2. face values of the cells c0-1..c1: position p = tid % P, rows split
  //    between the SP parts of the CTA
  if (tid < SP * P) {
    const int p = tid % P, part = tid / P;
    // position p's right-face value serves face p, its left-face value face p - 1
    if (need_face(p) || need_face(p - 1)) {
      const int c = p + LW - 1;  // window index of cell c0-1+p
      for (int v = part; v < ne; v += SP) {
        double vr, vl;
        recon_cell<ACU, LIM, WFLAG>(s_q + v * Wd, c, vr, vl);
        s_l[v * P + p] = vr;
        s_r[v * P + p] = vl;
      }
    }
  }
  __syncthreads();

  // 3. one face per group of SP lanes: face c0+f between cells c0-1+f and
  //    c0+f; lane h of the group takes the species k = h, h + SP, ...
  const int f = tid / SP, h = tid % SP;
  const unsigned pair = ((1u << SP) - 1u) << (tid & 31 & ~(SP - 1));
  if (f < P && need_face(f)) {
    FaceState L, R;
    L.rho = s_l[0 * P + f];
    L.u = s_l[1 * P + f];
    L.T = s_l[2 * P + f];
    R.rho = s_r[0 * P + f + 1];
    R.u = s_r[1 * P + f + 1];
    R.T = s_r[2 * P + f + 1];
    Premix pl, pr;
    pl.zero(t_interval(tb, L.T));
    pr.zero(t_interval(tb, R.T));
    double syl = 0.0, syr = 0.0, szl = 0.0, szr = 0.0;
    for (int k = h; k < ns; k += SP) {
      const double yl = s_l[(3 + k) * P + f], yr = s_r[(3 + k) * P + f + 1];
      const double pl_ = clip0(yl), pr_ = clip0(yr);
      syl += pl_;
      syr += pr_;
      const double zl = pl_ * tb.invW[k], zr = pr_ * tb.invW[k];
      szl += zl;
      szr += zr;
      premix_add(tb, pl, k, zl, L.T);
      premix_add(tb, pr, k, zr, R.T);
    }
    syl = pair_sum<SP>(syl, pair);
    syr = pair_sum<SP>(syr, pair);
    szl = pair_sum<SP>(szl, pair);
    szr = pair_sum<SP>(szr, pair);
    pair_sum<SP>(pl, pair);
    pair_sum<SP>(pr, pair);
    face_finish(L, pl, syl, szl);
    face_finish(R, pr, syr, szr);
    const double ml = L.rho * L.u, mr = R.rho * R.u;
    // physical fluxes of the three bulk rows
    const double fl0 = ml, fr0 = mr;
    const double fl1 = SPH ? ml * L.u : ml * L.u + L.p, fr1 = SPH ? mr * R.u : mr * R.u + R.p;
    if constexpr (SPH != 0) {
      // godunov_state(iqpres) of the face, SRC/flux.f90:360-367
      const double rt = sqrt(R.rho / L.rho);
      if (h == 0) s_pg[f] = (L.p + rt * R.p) / (1.0 + rt);
    }
    const double fl2 = (L.E + L.p) * L.u, fr2 = (R.E + R.p) * R.u;
    double F0, F1, F2;
    // species row k: flux = aL * YL + bL * max(YL,0) + aR * YR + bR * max(YR,0)
    double aL = 0.0, bL = 0.0, aR = 0.0, bR = 0.0;
    if (RIEMANN == 0) {  // LxF, SRC/flux.f90:287-294
      const double lamL = fabs(L.u) + L.a, lamR = fabs(R.u) + R.a;
      const double alpha = fmax(lamL, lamR);
      F0 = 0.5 * (fl0 + fr0 - alpha * (R.rho - L.rho));
      F1 = 0.5 * (fl1 + fr1 - alpha * (mr - ml));
      F2 = 0.5 * (fl2 + fr2 - alpha * (R.E - L.E));
      aL = 0.5 * ml;
      aR = 0.5 * mr;
      bR = -0.5 * alpha * R.rho * R.inv_SY;
      bL = 0.5 * alpha * L.rho * L.inv_SY;
    } else {
      const double rt = sqrt(R.rho / L.rho);
      const double inv1 = 1.0 / (1.0 + rt);
      const double u_roe = (L.u + rt * R.u) * inv1;
      const double a_roe = (L.a + rt * R.a) * inv1;
      const double sL = fmin(L.u - L.a, u_roe - a_roe);
      const double sR = fmax(R.u + R.a, u_roe + a_roe);
      if (RIEMANN == 1) {  // HLL, SRC/flux.f90:296-315
        if (0.0 <= sL) {
          F0 = fl0; F1 = fl1; F2 = fl2;
          aL = ml;
        } else if (0.0 <= sR) {
          const double inv = 1.0 / (sR - sL), ss = sL * sR;
          F0 = (sR * fl0 - sL * fr0 + ss * (R.rho - L.rho)) * inv;
          F1 = (sR * fl1 - sL * fr1 + ss * (mr - ml)) * inv;
          F2 = (sR * fl2 - sL * fr2 + ss * (R.E - L.E)) * inv;
          aL = sR * ml * inv;
          aR = -sL * mr * inv;
          bR = ss * R.rho * R.inv_SY * inv;
          bL = -ss * L.rho * L.inv_SY * inv;
        } else {
          F0 = fr0; F1 = fr1; F2 = fr2;
          aR = mr;
        }
      } else {  // HLLC, SRC/flux.f90:317-354
        const double sM = (L.p - R.p + mr * (sR - R.u) - ml * (sL - L.u)) /
                          (R.rho * (sR - R.u) - L.rho * (sL - L.u));
        if (0.0 <= sL) {
          F0 = fl0; F1 = fl1; F2 = fl2;
          aL = ml;
        } else if (0.0 <= sM) {
          const double fac = L.rho * (sL - L.u) / (sL - sM);
          const double ve = L.E / L.rho + (sM - L.u) * (sM + L.p / (L.rho * (sL - L.u)));
          F0 = fl0 + sL * (fac - L.rho);
          F1 = fl1 + sL * (fac * sM - ml);
          F2 = fl2 + sL * (fac * ve - L.E);
          aL = ml;
          bL = sL * (fac - L.rho) * L.inv_SY;
        } else if (0.0 <= sR) {
          const double fac = R.rho * (sR - R.u) / (sR - sM);
          const double ve = R.E / R.rho + (sM - R.u) * (sM + R.p / (R.rho * (sR - R.u)));
          F0 = fr0 + sR * (fac - R.rho);
          F1 = fr1 + sR * (fac * sM - mr);
          F2 = fr2 + sR * (fac * ve - R.E);
          aR = mr;
          bR = sR * (fac - R.rho) * R.inv_SY;
        } else {
          F0 = fr0; F1 = fr1; F2 = fr2;
          aR = mr;
        }
      }
    }
    // The fluxes replace the left states of this face, which no other group
    // reads: the bulk rows by lane 0, species row k by the lane that owns k.
    double* F = s_l + f;
    if (h == 0) {
      F[0] = F0;
      F[P] = F1;
      F[2 * P] = F2;
    }
    for (int k = h; k < ns; k += SP) {
      const double yl = s_l[(3 + k) * P + f], yr = s_r[(3 + k) * P + f + 1];
      double v = aL * yl;
      v = fma(bL, clip0(yl), v);
      v = fma(aR, yr, v);
      v = fma(bR, clip0(yr), v);
      F[(3 + k) * P] = v;
    }
  }
  __syncthreads();

  // 3b. transport (one tube only): the transport flux of each computed face
  //     comes first, as in the reference's Fplus (transport, then +
  //     advection): F = G + F_adv, row by row with coalesced G loads
  if (a.tran.flux) {
    const size_t gld = (size_t)a.ld;
    // the tube's block (packed tubes), read here rather than kept live
    const double* G = a.tran.flux + (a.tubes.tiles ? a.tubes.off[tube] : 0ll) + c0 + GHOST;
    for (int idx = tid; idx < ne * P; idx += NT) {
      const int v = idx / P, fp = idx - v * P;
      if (need_face(fp)) s_l[idx] = G[v * gld + fp] + s_l[idx];
    }
    __syncthreads();
  }

  // 4. one cell per group of SP lanes: conservative update + QcToqf,
  //    species split as in phase 3 (the bulk rows are computed by every lane)
  const int i = c0 + f;
  double speed = 0.0;
  // RK4 (kind 2) keeps the interior primitive state of the step's start
  // through its stages, as the reference does (its stages update only Qc and
  // the boundary ghosts): only the last stage runs QcToqf.
  const bool rk4_mid = a.kind == 2 && a.rk4_stage < 3;
  // a frozen cell's faces were not computed: its dF is exactly zero
  const bool fz = f < P && i < c1 && frozen(i);
  if (f < P && i < c1 && rk4_mid) {
    const double c = dt / tv.dx;
    const double cq = 0.5 * ((0.5 * dt) / tv.dx);  // 0.5 (0.5 dt / dx) of stages 1 and 2
    const size_t ld = (size_t)a.ld;
    double* Q = tv.qc + i + GHOST;
    double* Q0 = tv.q0 + i + GHOST;
    double* A = tv.acc + i + GHOST;
    for (int v = h; v < ne; v += SP) {
      const double dF = fz ? 0.0 : s_l[v * P + f + 1] - s_l[v * P + f];
      const double k = -(c * dF);
      const double qs = Q[v * ld];
      if (a.rk4_stage == 0) {
        Q0[v * ld] = qs;
        A[v * ld] = k;
      } else {
        A[v * ld] = A[v * ld] + 2.0 * k;
      }
      Q[v * ld] = qs - (a.rk4_stage < 2 ? cq : c) * dF;
    }
  }
  // the other stages: the update, then QcToqf, which with the uniform-region
  // shortcuts on is left to k_qc_to_qf_runs (one QcToqf per run of equal
  // conserved columns in a block of the tube, after every tile is updated).
  const bool own = f < P && i < c1 && !rk4_mid;
  const bool defer = skip_uniform && !rk4_mid;
  const size_t ld = (size_t)a.ld;
  const double Tg = own ? s_q[2 * Wd + f + LW] : 0.0;
  double q[3] = {0.0, 0.0, 0.0};
  if (own) {
    const double c = dt / tv.dx;
    double* Q = tv.qc + i + GHOST;
    double* Q0 = tv.q0 + i + GHOST;
    double* ys = s_r + f;  // strided by P
    // Euler or first TVDRK3 stage: Q - c dF; later stages h1 Q0 + h2 (Q - c dF);
    // last RK4 stage: Q0 + (k1 + 2 k2 + 2 k3 + k4) / 6
    auto update = [&](int v, double qv) {
      if constexpr (SPH != 0) {
        // cell centre r = x_m (x0 + (i + 1/2) dx), face areas (r -+ dx/2)^2, volume r^2 dx
        const double rm = tv.x0 + (i + 0.5) * tv.dx, hd = tv.dx / 2.0;
        const double Al = (rm - hd) * (rm - hd), Ar = (rm + hd) * (rm + hd), dV = rm * rm * tv.dx;
        const double cdF = (dt / dV) * (Ar * s_l[v * P + f + 1] - Al * s_l[v * P + f]);
        double r = a.kind == 0 ? qv - cdF : fma(a.h1, Q0[v * ld], a.h2 * (qv - cdF));
        if (v == 1) r = r - (dt / tv.dx) * (s_pg[f + 1] - s_pg[f]);
        return r;
      }
      const double dF = fz ? 0.0 : s_l[v * P + f + 1] - s_l[v * P + f];
      if (a.kind == 2) return Q0[v * ld] + (1.0 / 6.0) * (tv.acc[v * ld + i + GHOST] + -(c * dF));
      return a.kind == 0 ? qv - c * dF : fma(a.h1, Q0[v * ld], a.h2 * (qv - c * dF));
    };
    double qv[3];
#pragma unroll
    for (int v = 0; v < 3; ++v) qv[v] = Q[v * ld];
    __syncwarp(pair);  // every lane has read the bulk rows before lane v % SP rewrites row v
#pragma unroll
    for (int v = 0; v < 3; ++v) {
      q[v] = update(v, qv[v]);
      if (v % SP == h) {
        if (a.save_q0) Q0[v * ld] = qv[v];
        Q[v * ld] = q[v];
      }
    }
    for (int v = 3 + h; v < ne; v += SP) {
      const double qs = Q[v * ld];
      const double qn = update(v, qs);
      if (a.save_q0) Q0[v * ld] = qs;
      Q[v * ld] = qn;
      ys[(v - 3) * P] = qn;
    }
  }
  if (own && !defer) {
    double* ys = s_r + f;
    int iters;
    CellEOS e = qc_to_qf_cell<SP>(q[0], q[1], q[2], ys, P, Tg, a.strict_newton != 0, iters, h, pair);
    double* out = tv.qf_out + i + GHOST;
    if (h == 0) {
      out[0] = q[0];
      out[ld] = e.u;
      out[2 * ld] = e.T;
      if (tv.cvel) speed = cell_speed(e.u, e.T, e.Sz, e.cpR);
      if (e.status && a.err) atomicOr(a.err, e.status);
    }
    for (int k = h; k < ns; k += SP) out[(3 + k) * ld] = ys[k * P];
  }
  if (tv.cvel) {
    double m = speed;
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((tid & 31) == 0 && m > 0.0) atomic_max_pos(tv.cvel, m);
  }
  if (a.tubes.tiles) {
    // packed tubes: the first tile of each tube advances that tube's clock,
    // tube 0's the step count
    if (a.time && tile == 0 && tid == 0) {
      a.tubes.time[tube] = a.tubes.time[tube] + dt;
      if (tube == 0) *a.nsteps = *a.nsteps + 1;
    }
  } else if (a.time && blockIdx.x == 0 && tid == 0) {
    // No CTA of this kernel reads the clock; k_step_begin of the next step does.
    *a.time = *a.time + dt;
    *a.nsteps = *a.nsteps + 1;
  }
}


// ---------------------------------------------------------------------------
// QcToqf of a stage with the uniform-region shortcuts: one CTA per block of
// QR_BLOCK cells. A cell whose new conserved column and Newton start (its
// input T) equal its left neighbour's bit for bit, in the same tube and
// block, takes that neighbour's primitives; each run's first cell computes
// them (one group of STAGE_SPLIT lanes per cell, the stage kernel's own
// qc_to_qf_cell, so the results are bit for bit the stage's), then the
// others copy its column. Cells of tubes that do not step are left alone.
// ---------------------------------------------------------------------------
constexpr int QR_BLOCK = 1024;
constexpr int QR_THREADS = 256;

__global__ void __launch_bounds__(QR_THREADS) k_qc_to_qf_runs(StageArgs a) {
  constexpr int SP = STAGE_SPLIT, PER = QR_BLOCK / QR_THREADS, NG = QR_THREADS / SP;
  extern __shared__ double s_ys[];  // [NG][ne]: each group's species scratch
  __shared__ unsigned char s_fl[QR_BLOCK];
  __shared__ int s_hd[QR_BLOCK];
  __shared__ int s_list[QR_BLOCK];
  __shared__ int s_w[QR_THREADS / 32];
  __shared__ int s_nh;
  if (a.step_active && *a.step_active == 0) return;
  const int ns = a.ns, ne = ns + 3;
  const size_t ld = (size_t)a.ld;
  const int b0 = blockIdx.x * QR_BLOCK, tid = threadIdx.x, lane = tid & 31, wq = tid >> 5;
  const int* cm = a.tubes.colmap;
  const int* to = a.tubes.tube_of;
  auto col = [&](int c) { return (size_t)(cm ? cm[c] : c) + GHOST; };
  auto tube = [&](int c) { return to ? to[c] : 0; };
  if (tid == 0) s_nh = 0;
  // 1. flags (0: not stepping, 1: head, 2: follower), four consecutive cells
  //    a thread, and the last head at or before each cell (a max scan)
  const int j0 = tid * PER;
  int hp[PER];
  int run = -1;
#pragma unroll
  for (int k = 0; k < PER; ++k) {
    const int j = j0 + k, c = b0 + j;
    unsigned char fl = 0;
    if (c < a.n && (!a.tubes.active || !to || a.tubes.active[tube(c)] != 0)) {
      bool same = j > 0 && tube(c) == tube(c - 1);
      if (same) {
        const size_t qc = col(c), qr = col(c - 1);
        same = __double_as_longlong(a.qf_in[2 * ld + qc]) == __double_as_longlong(a.qf_in[2 * ld + qr]);
        for (int row = 0; row < ne && same; row += 8) {
          long long x[8], y[8];
#pragma unroll
          for (int m = 0; m < 8; ++m) {
            const int rr = min(row + m, ne - 1);
            x[m] = __double_as_longlong(a.qc[rr * ld + qc]);
            y[m] = __double_as_longlong(a.qc[rr * ld + qr]);
          }
#pragma unroll
          for (int m = 0; m < 8; ++m) same = same && x[m] == y[m];
        }
      }
      fl = same ? 2 : 1;
    }
    s_fl[j] = fl;
    if (fl == 1) run = j;
    hp[k] = run;
  }
  int v = run;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v = max(v, t);
  }
  if (lane == 31) s_w[wq] = v;
  __syncthreads();
  int prev = __shfl_up_sync(0xffffffffu, v, 1);
  if (lane == 0) prev = -1;
  for (int q = 0; q < wq; ++q) prev = max(prev, s_w[q]);
#pragma unroll
  for (int k = 0; k < PER; ++k) {
    s_hd[j0 + k] = max(prev, hp[k]);
    if (s_fl[j0 + k] == 1) s_list[atomicAdd(&s_nh, 1)] = j0 + k;
  }
  __syncthreads();
  // 2. the heads: QcToqf by groups of SP lanes
  const int g = tid / SP, h = tid % SP;
  const unsigned pair = ((1u << SP) - 1u) << (tid & 31 & ~(SP - 1));
  double* ys = s_ys + (size_t)g * ne;
  const int nh = s_nh;
  double speed = 0.0;
  for (int q = g; q < nh; q += NG) {
    const int c = b0 + s_list[q];
    const size_t cc = col(c);
    const double q0 = a.qc[cc], q1 = a.qc[ld + cc], q2 = a.qc[2 * ld + cc];
    for (int k = h; k < ns; k += SP) ys[k] = a.qc[(3 + k) * ld + cc];
    __syncwarp(pair);
    int iters;
    const CellEOS e = qc_to_qf_cell<SP>(q0, q1, q2, ys, 1, a.qf_in[2 * ld + cc], a.strict_newton != 0, iters, h, pair);
    double* out = a.qf_out + cc;
    if (h == 0) {
      out[0] = q0;
      out[ld] = e.u;
      out[2 * ld] = e.T;
      if (e.status && a.err) atomicOr(a.err, e.status);
      if (a.cvel_out) {
        const double sp = cell_speed(e.u, e.T, e.Sz, e.cpR);
        if (to) atomic_max_pos(a.cvel_out + tube(c), sp);
        else speed = fmax(speed, sp);
      }
    }
    for (int k = h; k < ns; k += SP) out[(3 + k) * ld] = ys[k];
    __syncwarp(pair);
  }
  if (a.cvel_out && !to) {
    double m = speed;
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0 && m > 0.0) atomic_max_pos(a.cvel_out, m);
  }
  __syncthreads();  // every head's column is written
  // 3. the followers copy their head's column (eight rows in flight)
  for (int j = tid; j < QR_BLOCK; j += QR_THREADS) {
    if (s_fl[j] != 2) continue;
    const size_t cc = col(b0 + j), ch = col(b0 + s_hd[j]);
    for (int row = 0; row < ne; row += 8) {
      double x[8];
#pragma unroll
      for (int m = 0; m < 8; ++m)
        if (row + m < ne) x[m] = a.qf_out[(row + m) * ld + ch];
#pragma unroll
      for (int m = 0; m < 8; ++m)
        if (row + m < ne) a.qf_out[(row + m) * ld + cc] = x[m];
    }
  }
}

// One thread: decides whether the step runs (time < tend, the loop test of
// SRC/main.f90:130), computes dt = cfl dx / max speed (SRC/update.f90:50)
// from the maximum left by the previous step, and clears the accumulator.
// The loop test and time steps of packed tubes, one CTA: tube t steps while
// its time < tend (and the call's step budget lasts), with dt_t = cfl dx_t /
// (its maximum signal speed); step_active = any tube steps.
// ---------------------------------------------------------------------------
// Transport (do_tran = 1): calc_flux_tran, SRC/flux.f90:18-127, with the
// mixture rules of TRANLIB (MCAVIS, MCACON, MCADIF; SRC/trans.f90 wrappers).
//
// k_tran_props: one thread per cell c = -1..n (the two ghosts included),
// from the stage's input conserved column, as the reference recomputes it
// for every face: rho, u = rho u / rho, Y_k = rho Y_k / rho (unnormalised),
// T from temperature_con with the 1000 K start, p, and
//   mu    = MCAVIS (Wilke's rule; the reference names MCAVIS_EA, which its
//           tranlib.f does not define) x 0.1,
//   kappa = MCACON (half the arithmetic plus harmonic mean) x 1e-5,
//   D'_k  = (1 - X_k) / (1 - Y_k) MCADIF_k x 1e-4 (0 where Y_k = 1).
// A thread walks the species and species pairs of its cell alone, so every
// pair's binary coefficient is evaluated once (ns (ns - 1) / 2 exponentials
// per cell) and the table reads are the same address across the warp. The
// Wilke sum sum_j X_j (1 + sqrt(eta_k / eta_j) q_kj)^2 g_kj is expanded into
// three matrix-vector products with constant matrices (wa, wb, wc): all its
// terms are positive, so the expansion moves the result by rounding only.
//
// k_tran_flux: one thread per face j = 0..n between cells j-1 and j: the
// viscous stress, heat conduction, species diffusion and the enthalpy they
// carry (hs_k at the face-average temperature, CKHMS), in the reference's
// order; the stage kernel adds the result to the advective flux
// (SRC/timeintegration.f90:31-47: Fplus = transport, then + advection).
// ---------------------------------------------------------------------------
constexpr int TRAN_PROPS_THREADS = 128;
constexpr int TRAN_FLUX_THREADS = 128;

__global__ void __launch_bounds__(TRAN_PROPS_THREADS) k_tran_props(StageArgs a) {
  if (a.step_active && *a.step_active == 0) return;
  const int gid = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  // the cell: c of the one tube, or of the packed tube whose block holds column gid
  TubeView tv{a.n, a.qf_in, a.qf_out, a.qc, a.q0, a.acc, a.dx, a.p_out, nullptr};
  int c = gid - 1;
  if (a.tubes.tiles) {
    if (gid >= a.ld) return;
    const int tt = a.tran.col_tube[gid];
    const long long off = a.tubes.off[tt];
    tv.n = a.tubes.n[tt];
    tv.qf_in = a.qf_in + off;
    tv.qc = a.qc + off;
    tv.dx = a.tubes.dx[tt];
    tv.p_out = a.tubes.p_out[tt];
    tv.tube = tt;
    tv.off = off;
    c = (int)(gid - off - GHOST);
  }
  if (c < -1 || c > tv.n) return;
  const ThermoTable& tb = c_thermo;
  const TranDev& t = a.tran;
  const int ns = a.ns;
  const size_t ld = (size_t)a.ld;
  double y[EDYN_NS_MAX], x[EDYN_NS_MAX], eta[EDYN_NS_MAX], v1[EDYN_NS_MAX], v2[EDYN_NS_MAX];
  double q0, q1, q2;
  if (c < 0 || c == tv.n) {
    ghost_qc(a, tv, c < 0 ? -1 : tv.n, q0, q1, q2, y, 1);
  } else {
    const double* Q = tv.qc + c + GHOST;
    q0 = Q[0];
    q1 = Q[ld];
    q2 = Q[2 * ld];
    for (int k = 0; k < ns; ++k) y[k] = Q[(3 + k) * ld];
  }
  const double rho = q0;
  const double u = q1 / rho;
  double sy = 0.0, sumyow = 0.0;
  for (int k = 0; k < ns; ++k) {
    const double yk = y[k] / rho;
    y[k] = yk;
    sy += yk;
    sumyow = fma(yk, tb.invW[k], sumyow);
  }
  const double isw = 1.0 / sumyow;  // CKYTX: X_k = Y_k / (W_k sum_j Y_j / W_j)
  for (int k = 0; k < ns; ++k) x[k] = y[k] * tb.invW[k] * isw;
  // temperature_con (SRC/thermo.f90:211-257) with these mole fractions: the
  // premixed Newton on the unnormalised Y with E scaled by S_Y
  const double eint = q2 / rho - 0.5 * (u * u);
  Premix pm;
  double Sz;
  int iters;
  const double T = t_newton(y, 1, eint * sy * (1.0 / R_SI), 1000.0, pm, Sz, iters);
  if (iters < 0 && a.err) atomicOr(a.err, EDYN_STATUS_NEWTON);
  const double p_cgs = 10.0 * (R_SI * rho * T * Sz / sy);  // CKPX: rho R T / W, W = S_Y / S_z
  const double L = tlog(T, t.lg);

  // pure-species viscosities and conductivities; MCACON's two means
  double sl = 0.0, sr = 0.0;
  for (int k = 0; k < ns; ++k) {
    const double* ce = t.eta + 4 * k;
    const double* cl = t.lam + 4 * k;
    const double ek = texp_r(fma(fma(fma(ce[3], L, ce[2]), L, ce[1]), L, ce[0]), t.e2);
    const double lk = texp_r(fma(fma(fma(cl[3], L, cl[2]), L, cl[1]), L, cl[0]), t.e2);
    eta[k] = ek;
    const double r = rsqrt(ek);
    v1[k] = x[k] * r;
    v2[k] = x[k] / ek;
    sl = fma(x[k], lk, sl);
    sr += x[k] / lk;
  }
  const double kap = 0.5 * (sl + 1.0 / sr) * 1.0e-5;
  // MCAVIS: sum_k X_k eta_k / sum_j X_j (1 + sqrt(eta_k/eta_j) q_kj)^2 g_kj, times sqrt(8)
  double vm = 0.0;
  for (int k = 0; k < ns; ++k) {
    const double* pa = t.wa + (size_t)k * ns;
    const double* pb = t.wb + (size_t)k * ns;
    const double* pc = t.wc + (size_t)k * ns;
    double A = 0.0, B = 0.0, C = 0.0;
    for (int j = 0; j < ns; ++j) {
      A = fma(pa[j], x[j], A);
      B = fma(pb[j], v1[j], B);
      C = fma(pc[j], v2[j], C);
    }
    const double sumi = fma(eta[k], C, fma(2.0 * sqrt(eta[k]), B, A));
    vm += x[k] * eta[k] / sumi;
  }
  const double mu = vm * 2.8284271247461903 * 0.1;

  // MCADIF (MCEDIF): S_k = sum_{j != k} XX_j / D_jk over the pairs j < k,
  // each exponential shared by both sums; the sums take their terms in the
  // order j = 0, 1, ... as MCEDIF's loop does. XX = max(X, 1e-50).
  double* S = v1;
  double* xx = v2;
  for (int k = 0; k < ns; ++k) {
    S[k] = 0.0;
    xx[k] = fmax(x[k], 1.0e-50);
  }
  const double* cd = t.dif;
  for (int k = 1; k < ns; ++k) {
    const double xk = xx[k];
    double sk = 0.0;
    for (int j = 0; j < k; ++j, cd += 4) {
      const double v = texp_r(-fma(fma(fma(cd[3], L, cd[2]), L, cd[1]), L, cd[0]), t.e2);
      sk = fma(xx[j], v, sk);
      S[j] = fma(xk, v, S[j]);
    }
    S[k] = sk;
  }
  // sum_{j != k} XX_j W_j as a prefix plus a suffix sum (eta[] holds the suffixes)
  double wtm = 0.0, suf = 0.0;
  for (int k = ns - 1; k >= 0; --k) {
    eta[k] = suf;
    suf = fma(xx[k], t.W[k], suf);
    wtm = fma(t.W[k], x[k], wtm);
  }
  double* out = t.tp + tv.off + c + GHOST;
  out[0] = rho;
  out[ld] = u;
  out[2 * ld] = T;
  out[3 * ld] = mu;
  out[4 * ld] = kap;
  double pre = 0.0;
  for (int k = 0; k < ns; ++k) {
    const double sumxw = pre + eta[k];
    pre = fma(xx[k], t.W[k], pre);
    const double dk = sumxw / (wtm * S[k]) * t.patmos / p_cgs * 1.0e-4;
    const double dif = (y[k] == 1.0) ? 0.0 : (1.0 - x[k]) / (1.0 - y[k]) * dk;
    out[(TRAN_ROWS_FIXED + k) * ld] = y[k];
    out[(TRAN_ROWS_FIXED + ns + k) * ld] = dif;
  }
}

__global__ void __launch_bounds__(TRAN_FLUX_THREADS) k_tran_flux(StageArgs a) {
  if (a.step_active && *a.step_active == 0) return;
  const int gid = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  // the face: j of the one tube, or of the packed tube whose block holds column gid
  int j = gid, n = a.n;
  long long off = 0;
  double dx = a.dx;
  if (a.tubes.tiles) {
    if (gid >= a.ld) return;
    const int tt = a.tran.col_tube[gid];
    off = a.tubes.off[tt];
    n = a.tubes.n[tt];
    dx = a.tubes.dx[tt];
    j = (int)(gid - off - GHOST);
    if (j < 0) return;
  }
  if (j > n) return;
  const ThermoTable& tb = c_thermo;
  const TranDev& t = a.tran;
  const int ns = a.ns;
  const size_t ld = (size_t)a.ld;
  const double* L = t.tp + off + (j - 1) + GHOST;  // cell j-1
  const double* R = L + 1;                         // cell j
  const double rho_ave = 0.5 * (L[0] + R[0]);
  const double u_ave = 0.5 * (L[ld] + R[ld]);
  const double T_ave = 0.5 * (L[2 * ld] + R[2 * ld]);
  const double mu_ave = 0.5 * (L[3 * ld] + R[3 * ld]);
  const double kap_ave = 0.5 * (L[4 * ld] + R[4 * ld]);
  const double tau = -(2.0 / 3.0 * mu_ave * (2.0 * ((R[ld] - L[ld]) / dx)));
  double* G = t.flux + off + j + GHOST;
  double hsum = 0.0;
  for (int k = 0; k < ns; ++k) {
    // CKHMS at the face temperature, J/kg: R T (a1 + a2 T/2 + ... + a6/T) / W
    const int r = (T_ave > tb.tmid[k]) ? 1 : 0;
    double h = fma(tb.ah[r][4][k], T_ave, tb.ah[r][3][k]);
    h = fma(h, T_ave, tb.ah[r][2][k]);
    h = fma(h, T_ave, tb.ah[r][1][k]);
    h = fma(h, T_ave, tb.ah[r][0][k]);
    h = fma(h, T_ave, tb.ah[r][5][k]);
    const double hs = R_SI * h * tb.invW[k];
    const double dif_ave = 0.5 * (L[(TRAN_ROWS_FIXED + ns + k) * ld] + R[(TRAN_ROWS_FIXED + ns + k) * ld]);
    const double dy = (R[(TRAN_ROWS_FIXED + k) * ld] - L[(TRAN_ROWS_FIXED + k) * ld]) / dx;
    hsum = hsum - hs * dif_ave * dy;
    G[(3 + k) * ld] = -(rho_ave * dif_ave * dy);
  }
  G[0] = 0.0;
  G[ld] = tau;
  G[2 * ld] = tau * u_ave + rho_ave * hsum - kap_ave * ((R[2 * ld] - L[2 * ld]) / dx);
}

// k_tran_props_warp: the same properties with one warp per cell, for tubes
// too short to fill the GPU with one thread per cell (there the launch
// lasts one thread's chain of ~32,000 FP64 instructions). Lane 0 does the
// cell's sequential part (mass and mole fractions, the temperature Newton,
// the sums of MCACON and MCAVIS over species, in the thread kernel's
// order); lane l takes species k = l, l + 32: its pure-species fits, its
// Wilke denominator and its MCADIF sum over the other species, whose
// binary coefficients it evaluates itself (each pair twice per cell, once
// per lane). Every operation and every summation order are the thread
// kernel's, so the results are the same bits.
constexpr int TRAN_WARP_CELLS = 4;        // cells (warps) per CTA
constexpr int TRAN_WARP_MAX_CELLS = 40000;  // up to this many cells per launch the warp form runs

__global__ void __launch_bounds__(32 * TRAN_WARP_CELLS) k_tran_props_warp(StageArgs a) {
  if (a.step_active && *a.step_active == 0) return;
  __shared__ double s_y[TRAN_WARP_CELLS][EDYN_NS_MAX], s_x[TRAN_WARP_CELLS][EDYN_NS_MAX];
  __shared__ double s_v1[TRAN_WARP_CELLS][EDYN_NS_MAX], s_v2[TRAN_WARP_CELLS][EDYN_NS_MAX];
  __shared__ double s_eta[TRAN_WARP_CELLS][EDYN_NS_MAX], s_aux[TRAN_WARP_CELLS][EDYN_NS_MAX];
  __shared__ double s_term[TRAN_WARP_CELLS][EDYN_NS_MAX], s_sc[TRAN_WARP_CELLS][8];
  const int lane = (int)(threadIdx.x & 31), w = (int)(threadIdx.x >> 5);
  const int gid = (int)(blockIdx.x * TRAN_WARP_CELLS) + w;
  // the cell, as in k_tran_props (warp-uniform)
  TubeView tv{a.n, a.qf_in, a.qf_out, a.qc, a.q0, a.acc, a.dx, a.p_out, nullptr};
  int c = gid - 1;
  if (a.tubes.tiles) {
    if (gid >= a.ld) return;
    const int tt = a.tran.col_tube[gid];
    const long long off = a.tubes.off[tt];
    tv.n = a.tubes.n[tt];
    tv.qf_in = a.qf_in + off;
    tv.qc = a.qc + off;
    tv.dx = a.tubes.dx[tt];
    tv.p_out = a.tubes.p_out[tt];
    tv.tube = tt;
    tv.off = off;
    c = (int)(gid - off - GHOST);
  }
  if (c < -1 || c > tv.n) return;
  const ThermoTable& tb = c_thermo;
  const TranDev& t = a.tran;
  const int ns = a.ns;
  const size_t ld = (size_t)a.ld;
  double* y = s_y[w];
  double* x = s_x[w];
  double* v1 = s_v1[w];
  double* v2 = s_v2[w];
  double* eta = s_eta[w];
  double* aux = s_aux[w];
  double* sc = s_sc[w];
  // 1. the conserved column (rho Y_k into y)
  if (c < 0 || c == tv.n) {
    if (lane == 0) ghost_qc(a, tv, c < 0 ? -1 : tv.n, sc[0], sc[1], sc[2], y, 1);
  } else {
    const double* Q = tv.qc + c + GHOST;
    for (int k = lane; k < ns; k += 32) y[k] = Q[(3 + k) * ld];
    if (lane == 0) {
      sc[0] = Q[0];
      sc[1] = Q[ld];
      sc[2] = Q[2 * ld];
    }
  }
  __syncwarp();
  // 2. lane 0: Y, X, T (temperature_con from 1000 K), p, ln T
  if (lane == 0) {
    const double rho = sc[0];
    const double u = sc[1] / rho;
    double sy = 0.0, sumyow = 0.0;
    for (int k = 0; k < ns; ++k) {
      const double yk = y[k] / rho;
      y[k] = yk;
      sy += yk;
      sumyow = fma(yk, tb.invW[k], sumyow);
    }
    const double isw = 1.0 / sumyow;
    for (int k = 0; k < ns; ++k) x[k] = y[k] * tb.invW[k] * isw;
    const double eint = sc[2] / rho - 0.5 * (u * u);
    Premix pm;
    double Sz;
    int iters;
    const double T = t_newton(y, 1, eint * sy * (1.0 / R_SI), 1000.0, pm, Sz, iters);
    if (iters < 0 && a.err) atomicOr(a.err, EDYN_STATUS_NEWTON);
    sc[3] = rho;
    sc[4] = u;
    sc[5] = T;
    sc[6] = tlog(T, t.lg);
    sc[7] = 10.0 * (R_SI * rho * T * Sz / sy);
  }
  __syncwarp();
  const double L = sc[6], p_cgs = sc[7];
  // 3. pure-species viscosity and conductivity (conductivities into aux)
  for (int k = lane; k < ns; k += 32) {
    const double* ce = t.eta + 4 * k;
    const double* cl = t.lam + 4 * k;
    const double ek = texp_r(fma(fma(fma(ce[3], L, ce[2]), L, ce[1]), L, ce[0]), t.e2);
    const double lk = texp_r(fma(fma(fma(cl[3], L, cl[2]), L, cl[1]), L, cl[0]), t.e2);
    eta[k] = ek;
    aux[k] = lk;
    const double r = rsqrt(ek);
    v1[k] = x[k] * r;
    v2[k] = x[k] / ek;
  }
  __syncwarp();
  // 4. Wilke's denominator of species k; lane 0 then sums the terms and
  //    MCACON's two means in species order
  for (int k = lane; k < ns; k += 32) {
    const double* pa = t.wa + (size_t)k * ns;
    const double* pb = t.wb + (size_t)k * ns;
    const double* pc = t.wc + (size_t)k * ns;
    double A = 0.0, B = 0.0, C = 0.0;
    for (int j = 0; j < ns; ++j) {
      A = fma(pa[j], x[j], A);
      B = fma(pb[j], v1[j], B);
      C = fma(pc[j], v2[j], C);
    }
    const double sumi = fma(eta[k], C, fma(2.0 * sqrt(eta[k]), B, A));
    s_term[w][k] = x[k] * eta[k] / sumi;
  }
  __syncwarp();
  if (lane == 0) {
    double sl = 0.0, sr = 0.0, vm = 0.0;
    for (int k = 0; k < ns; ++k) {
      sl = fma(x[k], aux[k], sl);
      sr += x[k] / aux[k];
    }
    for (int k = 0; k < ns; ++k) vm += s_term[w][k];
    sc[0] = vm * 2.8284271247461903 * 0.1;
    sc[1] = 0.5 * (sl + 1.0 / sr) * 1.0e-5;
  }
  __syncwarp();
  // 5. XX = max(X, 1e-50) (into aux)
  for (int k = lane; k < ns; k += 32) aux[k] = fmax(x[k], 1.0e-50);
  __syncwarp();
  // 6. MCADIF for species k: S_k = sum_{j != k} XX_j / D_jk in increasing j,
  //    sum_{j != k} XX_j W_j as the prefix plus the suffix, D'_k
  double* out = t.tp + tv.off + c + GHOST;
  for (int k = lane; k < ns; k += 32) {
    double S = 0.0;
    for (int j = 0; j < ns; ++j) {
      if (j == k) continue;
      const double* cd = t.dif + 4 * (j < k ? (size_t)k * (k - 1) / 2 + j : (size_t)j * (j - 1) / 2 + k);
      const double v = texp_r(-fma(fma(fma(cd[3], L, cd[2]), L, cd[1]), L, cd[0]), t.e2);
      S = fma(aux[j], v, S);
    }
    double suf = 0.0, sufk = 0.0, wtm = 0.0;
    for (int j = ns - 1; j >= 0; --j) {
      if (j == k) sufk = suf;
      suf = fma(aux[j], t.W[j], suf);
      wtm = fma(t.W[j], x[j], wtm);
    }
    double pre = 0.0;
    for (int j = 0; j < k; ++j) pre = fma(aux[j], t.W[j], pre);
    const double sumxw = pre + sufk;
    const double dk = sumxw / (wtm * S) * t.patmos / p_cgs * 1.0e-4;
    const double dif = (y[k] == 1.0) ? 0.0 : (1.0 - x[k]) / (1.0 - y[k]) * dk;
    out[(TRAN_ROWS_FIXED + k) * ld] = y[k];
    out[(TRAN_ROWS_FIXED + ns + k) * ld] = dif;
  }
  if (lane == 0) {
    out[0] = sc[3];
    out[ld] = sc[4];
    out[2 * ld] = sc[5];
    out[3 * ld] = sc[0];
    out[4 * ld] = sc[1];
  }
}

cudaError_t launch_tran(const StageArgs& a, cudaStream_t s) {
  // one thread per cell (-1..n) and per face (0..n); packed tubes: per column
  const int np = a.tubes.tiles ? a.ld : a.n + 2, nf = a.tubes.tiles ? a.ld : a.n + 1;
  if (np <= TRAN_WARP_MAX_CELLS)
    k_tran_props_warp<<<(np + TRAN_WARP_CELLS - 1) / TRAN_WARP_CELLS, 32 * TRAN_WARP_CELLS, 0, s>>>(a);
  else
    k_tran_props<<<(np + TRAN_PROPS_THREADS - 1) / TRAN_PROPS_THREADS, TRAN_PROPS_THREADS, 0, s>>>(a);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_tran_flux<<<(nf + TRAN_FLUX_THREADS - 1) / TRAN_FLUX_THREADS, TRAN_FLUX_THREADS, 0, s>>>(a);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Energy sources of solve_source after the chemistry (SRC/update.f90:126-147),
// one thread per cell, in the reference's order, each followed by QcToqf of
// the cell (the reference recomputes every interior cell's qf after each):
//   radiation   heat_transfer_radiation (SRC/source.f90:88-137) with
//               radiation_heat_loss (SRC/radiation.f90:74-121): optically
//               thin, Q = -4 Kp sigma (T^4 - 300^4), Kp = sum_r kp_r(T) X_r p/atm;
//   wall heat   heat_transfer_mfr (SRC/source.f90:140-189) with heat_transfer
//               and Tw (SRC/mfr.f90:41-78): Q = -4 lambda Nu (T - Tw(x)) / d^2,
//               lambda from MCACON;
//   ignition    energy_source (SRC/source.f90:192-239) with add_igsource /
//               add_igsource_WZhang (SRC/ignitionsource.f90:150-262).
// rho E += dt Q each time. The new state's signal speed feeds the next
// step's dt in the device loop (the chemistry then publishes none).
// ---------------------------------------------------------------------------
constexpr int SRC_THREADS = 128;

__global__ void __launch_bounds__(SRC_THREADS) k_energy_sources(SourceArgs s) {
  if (s.step_active && *s.step_active == 0) return;
  const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  double speed = 0.0;
  if (i < s.n) {
    const ThermoTable& tb = c_thermo;
    const int ns = s.ns;
    const size_t ld = (size_t)s.ld;
    const double dt = s.dt_dev ? *s.dt_dev : s.dt;
    const double time = s.time_dev ? *s.time_dev : s.time;
    const size_t col = (size_t)(s.colmap ? s.colmap[i] : i) + GHOST;
    double* Q = s.qc + col;
    double* F = s.qf + col;
    const double q0 = Q[0], q1 = Q[ld];
    double q2 = Q[2 * ld];
    double rho = F[0], u = F[ld], T = F[2 * ld];
    double y[EDYN_NS_MAX], ys[EDYN_NS_MAX];
    for (int k = 0; k < ns; ++k) y[k] = F[(3 + k) * ld];
    const double xm = s.xm ? s.xm[i] : (i + 0.5) * s.dx;
    CellEOS e{};
    for (int src = 0; src < 3; ++src) {
      double add = 0.0;
      if (src == 0 || src == 1) {
        if (src == 0 ? s.nrad == 0 : s.wall == 0) continue;
        // mole fractions (CKYTX) and pressure (CKPX) of the cell's qf
        double sumyow = 0.0;
        for (int k = 0; k < ns; ++k) sumyow = fma(y[k], tb.invW[k], sumyow);
        const double isw = 1.0 / sumyow;
        double sy = 0.0;
        for (int k = 0; k < ns; ++k) sy += y[k];
        if (src == 0) {
          const double p = R_SI * rho * T * sumyow / sy;
          const double T1 = T, T2 = T1 * T1, T3 = T2 * T1, T4 = T3 * T1, T5 = T4 * T1;
          const double T04 = 300.0 * 300.0 * 300.0 * 300.0;
          double kp = 0.0;
          for (int r = 0; r < s.nrad; ++r) {
            const double* c = s.rad_coef[r];
            const double kpi = c[0] + c[1] * T1 + c[2] * T2 + c[3] * T3 + c[4] * T4 + c[5] * T5;
            const int k = s.rad_sp[r];
            kp = kp + kpi * (y[k] * tb.invW[k] * isw) * (p / 101325.0);
          }
          add = -4.0 * kp * 5.6703744191844294e-08 * (T4 - T04);
          if (s.q_rad) s.q_rad[i] = add;
        } else {
          const double L = tlog(T, s.lg);
          double sl = 0.0, sr = 0.0;
          for (int k = 0; k < ns; ++k) {
            const double* cl = s.lam + 4 * k;
            const double lk = texp_r(fma(fma(fma(cl[3], L, cl[2]), L, cl[1]), L, cl[0]), s.e2);
            const double xk = y[k] * tb.invW[k] * isw;
            sl = fma(xk, lk, sl);
            sr += xk / lk;
          }
          const double lambda = 0.5 * (sl + 1.0 / sr) * 1.0e-5;
          const double A = 0.5 * (s.tw_max - s.tw_min), B = 0.5 * (s.tw_max + s.tw_min);
          const double tw = A * tanh(s.alpha * (xm - s.beta)) + B;
          add = -4.0 * lambda * s.nu * (T - tw) / (s.d_m * s.d_m);
          if (s.q_tw) s.q_tw[i] = add;
        }
      } else {
        if (s.ig_type == 0) continue;
        const double pi = 3.14159265359;  // the reference's constant
        for (int g = 0; g < s.n_ig; ++g) {
          const double r = s.ig_r[g], tg = s.ig_t[g], t0 = s.ig_t0[g];
          if (!(t0 < time && time < t0 + tg)) continue;
          const double w = xm / r;
          if (s.ig_type == 1) {  // Frendi et al.: top-hat-like exp(-(pi/4) (r/r_ig)^6) over a sphere's volume
            const double vol = 4.0 * pi * (r * r * r) / 3.0;
            const double w2 = w * w;
            add = s.ig_e[g] / (vol * tg) * exp(-(pi / 4.0) * (w2 * w2 * w2));
          } else {               // Zhang et al.: Gaussian
            add = s.ig_e[g] / (pow(pi, 1.5) * (r * r * r) * tg) * exp(-(w * w));
          }
        }
      }
      q2 = q2 + dt * add;
      for (int k = 0; k < ns; ++k) ys[k] = Q[(3 + k) * ld];
      int it;
      e = qc_to_qf_cell(q0, q1, q2, ys, 1, T, s.strict_newton != 0, it);
      if (e.status && s.err) atomicOr(s.err, e.status);
      rho = q0;
      u = e.u;
      T = e.T;
      for (int k = 0; k < ns; ++k) y[k] = ys[k];
    }
    Q[2 * ld] = q2;
    F[0] = rho;
    F[ld] = u;
    F[2 * ld] = T;
    for (int k = 0; k < ns; ++k) F[(3 + k) * ld] = y[k];
    if (s.cvel) speed = cell_speed(u, T, e.Sz, e.cpR);
    // SMR segments: the maximum of each segment (calc_dt takes the largest)
    if (s.cvel && s.tube_of) atomic_max_pos(s.cvel + s.tube_of[i], speed);
  }
  if (s.cvel && !s.tube_of) {
    double m = speed;
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m > 0.0) atomic_max_pos(s.cvel, m);
  }
}

cudaError_t launch_energy_sources(const SourceArgs& a, cudaStream_t s) {
  k_energy_sources<<<(a.n + SRC_THREADS - 1) / SRC_THREADS, SRC_THREADS, 0, s>>>(a);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Output fields (set_eos_params, SRC/block.f90:434-470, in write_hdf5_b's row
// order, SRC/write_hdf5.f90:140-162), one thread per cell:
//   X = CKYTX(Y), p = CKPX(rho, T, X), ek = u^2 / 2,
//   ei = CKUBML(T, X) / W (specific_energy, SRC/thermo.f90:356-375),
//   et = rho E / rho, and the per-cell source outputs as the last source
//   step left them (HRR, HRR_dot, Qrad, qTw; Tw from the wall profile).
// Each row is written contiguously, as the file's datasets hold them.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_output_rows(OutputArgs a) {
  const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  if (i >= a.n) return;
  const ThermoTable& tb = c_thermo;
  const int ns = a.ns;
  const size_t ld = (size_t)a.ld, n = (size_t)a.n;
  const size_t col = (size_t)(a.colmap ? a.colmap[i] : i) + GHOST;
  const double rho = a.qf[col], u = a.qf[ld + col], T = a.qf[2 * ld + col];
  double* o = a.out + i;
  double sumyow = 0.0;
  for (int k = 0; k < ns; ++k) sumyow = fma(a.qf[(3 + k) * ld + col], tb.invW[k], sumyow);
  const double isw = 1.0 / sumyow;
  double wtm = 0.0, ubml = 0.0;
  for (int k = 0; k < ns; ++k) {
    const double xk = a.qf[(3 + k) * ld + col] * tb.invW[k] * isw;
    o[(EDYN_OUT_FIXED + k) * n] = xk;
    wtm = fma(xk, tb.W[k], wtm);
    // U_k / R = H_k / R - T (NASA-7, the range of T)
    const int r = (T > tb.tmid[k]) ? 1 : 0;
    double h = fma(tb.ah[r][4][k], T, tb.ah[r][3][k]);
    h = fma(h, T, tb.ah[r][2][k]);
    h = fma(h, T, tb.ah[r][1][k]);
    h = fma(h, T, tb.ah[r][0][k]);
    h = fma(h, T, tb.ah[r][5][k]);
    ubml = fma(xk, h - T, ubml);
  }
  o[0] = rho;
  o[n] = u;
  o[2 * n] = T;
  o[3 * n] = rho * R_SI * T / wtm;
  o[4 * n] = a.qc[2 * ld + col] / rho;
  o[5 * n] = 0.5 * (u * u);
  o[6 * n] = R_SI * ubml / wtm;
  o[7 * n] = a.hrr ? a.hrr[i] : 0.0;
  o[8 * n] = a.hrr_dot ? a.hrr_dot[i] : 0.0;
  o[9 * n] = a.q_rad ? a.q_rad[i] : 0.0;
  const double xm = a.xm[i];
  o[10 * n] = a.wall ? 0.5 * (a.tw_max - a.tw_min) * tanh(a.alpha * (xm - a.beta)) + 0.5 * (a.tw_max + a.tw_min) : 0.0;
  o[11 * n] = a.q_tw ? a.q_tw[i] : 0.0;
  o[12 * n] = xm;
  o[13 * n] = a.xm[n + i];
  o[14 * n] = (double)(i + 1);
}

cudaError_t launch_output_rows(const OutputArgs& a, cudaStream_t s) {
  if (a.n <= 0) return cudaSuccess;
  k_output_rows<<<(a.n + 127) / 128, 128, 0, s>>>(a);
  return cudaGetLastError();
}

// SMR: the end columns of every segment next to an interface, before a
// stage updates them in place (one thread per copied value).
__global__ void k_smr_snapshot(TubeTab T, const double* qc, int ld, int ne, int lvir) {
  const int S = 2 * lvir;
  const long long tot = (long long)(T.ntube - 1) * 2 * ne * S;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot; e += (long long)gridDim.x * blockDim.x) {
    const int col = (int)(e % S);
    const long long r = e / S;
    const int v = (int)(r % ne);
    const long long js = r / ne;
    const int side = (int)(js % 2), j = (int)(js / 2);
    const int t = j + side;
    const int cell = side == 0 ? T.n[t] - S + col : col;
    T.smr_snap[e] = qc[(size_t)v * ld + T.off[t] + GHOST + cell];
  }
}

cudaError_t launch_smr_snapshot(const StageArgs& a, cudaStream_t s) {
  const long long tot = (long long)(a.tubes.ntube - 1) * 2 * (a.ns + 3) * 2 * a.lvir;
  if (tot <= 0) return cudaSuccess;
  const int blocks = (int)std::min<long long>((tot + 255) / 256, 1024);
  k_smr_snapshot<<<blocks, 256, 0, s>>>(a.tubes, a.qc, a.ld, a.ns + 3, a.lvir);
  return cudaGetLastError();
}

// SMR: one dt for every segment, cfl dx_comp / max(|u| + a) over all of
// them (calc_dt, SRC/update.f90:13-59); every segment steps while the
// (common) clock is below tend.
__global__ void k_step_begin_blocks(int ntube, const double* time, double tend, const long long* nsteps,
                                    const long long* max_steps, double cfl, double dx_comp, unsigned long long* cvel,
                                    int* active, double* dt, int* step_active) {
  __shared__ unsigned long long s_max;
  if (threadIdx.x == 0) s_max = 0ull;
  __syncthreads();
  unsigned long long m = 0ull;
  for (int t = threadIdx.x; t < ntube; t += blockDim.x) m = max(m, cvel[t]);
  atomicMax(&s_max, m);
  __syncthreads();
  const int on = (*nsteps < *max_steps && time[0] < tend) ? 1 : 0;
  const double d = (cfl * dx_comp) / __longlong_as_double((long long)s_max);
  for (int t = threadIdx.x; t < ntube; t += blockDim.x) {
    active[t] = on;
    if (on) {
      dt[t] = d;
      cvel[t] = 0ull;
    }
  }
  if (threadIdx.x == 0) *step_active = on;
}

cudaError_t launch_step_begin_blocks(int ntube, const double* time, double tend, const long long* nsteps,
                                     const long long* max_steps, double cfl, double dx_comp, unsigned long long* cvel,
                                     int* active, double* dt, int* step_active, cudaStream_t s) {
  k_step_begin_blocks<<<1, 256, 0, s>>>(ntube, time, tend, nsteps, max_steps, cfl, dx_comp, cvel, active, dt,
                                        step_active);
  return cudaGetLastError();
}

__global__ void k_step_begin_tubes(int ntube, const double* time, double tend, const long long* nsteps,
                                   const long long* max_steps, double cfl, const double* dx, unsigned long long* cvel,
                                   int* active, double* dt, int* step_active) {
  const bool budget = *nsteps < *max_steps;
  int any = 0;
  for (int t = threadIdx.x; t < ntube; t += blockDim.x) {
    const int on = (budget && time[t] < tend) ? 1 : 0;
    active[t] = on;
    any |= on;
    if (!on) continue;  // an idle tube keeps its last dt and speed
    const double cv = __longlong_as_double((long long)cvel[t]);
    dt[t] = (cfl * dx[t]) / cv;
    cvel[t] = 0ull;
  }
  any = __syncthreads_or(any);
  if (threadIdx.x == 0) *step_active = any;
}

__global__ void k_step_begin(const double* time, double tend, const long long* nsteps, const long long* max_steps,
                             double cfl, double dx, unsigned long long* cvel, int* step_active, double* dt_dev) {
  // the step budget of this call (edyn_advance's max_steps) ends the loop as
  // the end time does, so a call runs exactly the steps it was given
  if (!(*time < tend) || *nsteps >= *max_steps) {
    *step_active = 0;
    return;
  }
  const double cv = __longlong_as_double((long long)*cvel);
  *dt_dev = (cfl * dx) / cv;
  *step_active = 1;
  *cvel = 0ull;
}

// Signal-speed maximum of the current primitive state (calc_dt); with
// packed tubes (colmap, tube_of) one maximum per tube.
__global__ void k_cvel(const double* qf, int n, int ld, unsigned long long* cvel, const int* colmap,
                       const int* tube_of) {
  const ThermoTable& tb = c_thermo;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double sp = 0.0;
  // a cell whose column (u, T, Y) equals its left neighbour's in the same
  // tube bit for bit has the same signal speed, which the neighbour brings
  bool same = false;
  if (i > 0 && i < n && (!tube_of || tube_of[i] == tube_of[i - 1])) {
    const double* q = qf + (colmap ? colmap[i] : i) + GHOST;
    const double* r = qf + (colmap ? colmap[i - 1] : i - 1) + GHOST;
    same = true;
    for (int row = 1; row < 3 + tb.ns && same; row += 8) {
      long long x[8], y[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const int rr = min(row + k, 2 + tb.ns);
        x[k] = __double_as_longlong(q[rr * (size_t)ld]);
        y[k] = __double_as_longlong(r[rr * (size_t)ld]);
      }
#pragma unroll
      for (int k = 0; k < 8; ++k) same = same && x[k] == y[k];
    }
  }
  if (i < n && !same) {
    const double* q = qf + (colmap ? colmap[i] : i) + GHOST;
    const double T = q[2 * (size_t)ld];
    Premix pm;
    pm.zero(t_interval(tb, T));
    double sz = 0.0, sy = 0.0;
    for (int k = 0; k < tb.ns; ++k) {
      const double y = q[(3 + k) * (size_t)ld];
      const double z = y * tb.invW[k];
      sy += y;
      sz += z;
      premix_add(tb, pm, k, z, T);
    }
    // calc_dt uses CKYTX without the clip; the stored Y are non-negative.
    const double cpR = pm.Cp(T);
    const double gamma = cpR / (cpR - sz);
    const double a = sqrt(gamma * R_SI * T * sz / sy);
    sp = fabs(q[ld]) + a;
  }
  if (tube_of) {
    if (i < n && !same) atomic_max_pos(cvel + tube_of[i], sp);
    return;
  }
  double m = sp;
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomic_max_pos(cvel, m);
}

// ---------------------------------------------------------------------------
// Layout conversion between the reference's AoS (nequ, ncell) arrays and
// the device SoA rows.
// ---------------------------------------------------------------------------
__global__ void k_aos_to_soa(const double* aos, int ne, int n, double* soa, int ld) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)ne * n) return;
  const int i = (int)(idx / ne), v = (int)(idx - (size_t)i * ne);
  soa[(size_t)v * ld + i + GHOST] = aos[idx];
}

__global__ void k_soa_to_aos(const double* soa, int ne, int n, int ld, double* aos) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)ne * n) return;
  const int i = (int)(idx / ne), v = (int)(idx - (size_t)i * ne);
  aos[idx] = soa[(size_t)v * ld + i + GHOST];
}

// QcToqf for every interior cell (used after chemistry and when only Qc is
// uploaded). Tguess from the current qf when warm.
__global__ void k_qc_to_qf(StageArgs a) {
  extern __shared__ double sm[];
  const int ns = c_thermo.ns;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const size_t ld = (size_t)a.ld;
  double* ys = sm + threadIdx.x;
  const double* Q = a.qc + i + GHOST;
  for (int k = 0; k < ns; ++k) ys[k * blockDim.x] = Q[(3 + k) * ld];
  int iters;
  double* out = a.qf_out + i + GHOST;
  const double Tg = a.qf_in ? a.qf_in[2 * ld + i + GHOST] : 1000.0;
  CellEOS e = qc_to_qf_cell(Q[0], Q[ld], Q[2 * ld], ys, blockDim.x, Tg, a.strict_newton != 0 || !a.qf_in, iters);
  if (e.status && a.err) atomicOr(a.err, e.status);
  out[0] = Q[0];
  out[ld] = e.u;
  out[2 * ld] = e.T;
  for (int k = 0; k < ns; ++k) out[(3 + k) * ld] = ys[k * blockDim.x];
}

// Checks an uploaded interior state: per cell a positive, finite density and
// total energy, a temperature strictly inside the clamp bounds (20, 6000) K,
// finite mass fractions none below -1e-6 (adjust_sum clips round-off
// negatives; larger ones mean a broken state) and finite conserved rows.
// ORs EDYN_E_STATE into err for any cell that fails.
__global__ void k_check_state(const double* qf, const double* qc, int n, int ns, int ld, unsigned* err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* q = qf + i + GHOST;
  const double* Q = qc + i + GHOST;
  const size_t l = (size_t)ld;
  bool ok = q[0] > 0.0 && isfinite(q[0]) && isfinite(q[l]) && q[2 * l] > 20.0 && q[2 * l] < 6000.0 && Q[0] > 0.0 &&
            isfinite(Q[0]) && isfinite(Q[l]) && isfinite(Q[2 * l]);
  for (int k = 0; k < ns && ok; ++k) {
    const double y = q[(3 + k) * l];
    ok = isfinite(y) && y >= -1e-6 && isfinite(Q[(3 + k) * l]);
  }
  if (!ok) atomicOr(err, EDYN_STATUS_STATE);
}

cudaError_t launch_check_state(const double* qf, const double* qc, int n, int ns, int ld, unsigned* err,
                               cudaStream_t s) {
  k_check_state<<<(n + 127) / 128, 128, 0, s>>>(qf, qc, n, ns, ld, err);
  return cudaGetLastError();
}

// Initial state of one cell from (T, p, u, X): initialize_variables
// (SRC/params.f90:305-580, step profiles) and set_block_params
// (SRC/block.f90:394-431).
__global__ void k_init_cells(int n, const double* T, const double* p, const double* u, const double* X, int ldx,
                             double* qf, double* qc, int ld) {
  extern __shared__ double sm[];
  const ThermoTable& tb = c_thermo;
  const int ns = tb.ns;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double* xs = sm + threadIdx.x;
  const int st = blockDim.x;
  double s = 0.0;
  for (int k = 0; k < ns; ++k) {
    double x = clip0(X[(size_t)i * ldx + k]);
    xs[k * st] = x;
    s += x;
  }
  const double inv_s = 1.0 / s;
  double wsum = 0.0;
  for (int k = 0; k < ns; ++k) {
    const double x = xs[k * st] * inv_s;
    xs[k * st] = x;
    wsum += x * tb.W[k];
  }
  const double Ti = T[i];
  Premix pm;
  pm.zero(t_interval(tb, Ti));
  double sz = 0.0;
  const double inv_w = 1.0 / wsum;
  for (int k = 0; k < ns; ++k) {
    const double y = xs[k * st] * tb.W[k] * inv_w;  // CKXTY
    xs[k * st] = y;
    const double z = y * tb.invW[k];
    sz += z;
    premix_add(tb, pm, k, z, Ti);
  }
  const double rho = p[i] * wsum / (R_SI * Ti);  // density(): sum X W p / (R T)
  const double e_int = R_SI * (pm.H(Ti) - Ti * sz);
  const double ui = u[i];
  double* F = qf + i + GHOST;
  double* C = qc + i + GHOST;
  const size_t L = (size_t)ld;
  F[0] = rho;
  F[L] = ui;
  F[2 * L] = Ti;
  C[0] = rho;
  C[L] = rho * ui;
  C[2 * L] = rho * (e_int + 0.5 * (ui * ui));
  for (int k = 0; k < ns; ++k) {
    const double y = xs[k * st];
    F[(3 + k) * L] = y;
    C[(3 + k) * L] = rho * y;
  }
}

// ---------------------------------------------------------------------------
// Host side launchers
// ---------------------------------------------------------------------------
// The thermodynamic table lives in constant memory, once per device: every
// context on a device must use the same mechanism (checked against the
// table uploaded first on that device).
int fluid_upload_tables(const ThermoTable& tb, cudaStream_t s) {
  static std::mutex mu;
  static bool loaded[64];
  static ThermoTable first[64];
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return (int)e;
  if (dev < 0 || dev >= 64) return (int)cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(mu);
  if (loaded[dev]) return std::memcmp(&first[dev], &tb, sizeof(tb)) == 0 ? (int)cudaSuccess : -1;
  e = cudaMemcpyToSymbolAsync(c_thermo, &tb, sizeof(tb), 0, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return (int)e;
  e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return (int)e;
  first[dev] = tb;
  loaded[dev] = true;
  return (int)cudaSuccess;
}

size_t stage_smem_bytes(int acu, int ns, int tc) {
  const int lv = acu_lvir(acu);
  const int ne = ns + 3;
  const int p = tc + 2;
  return sizeof(double) * ((size_t)ne * (tc + 2 * (lv + 1)) + (size_t)2 * ne * p);
}

namespace {

using StageFn = void (*)(StageArgs);

template <int ACU, int LIM, int WF, int SPH = 0>
StageFn stage_fn_rm(int rm) {
  if (rm == 0) return k_stage<ACU, LIM, WF, 0, SPH>;
  if (rm == 1) return k_stage<ACU, LIM, WF, 1, SPH>;
  return k_stage<ACU, LIM, WF, 2, SPH>;
}

// spherical geometry: first order and MUSCL (the schemes of the reference's
// spherical examples); null for the others
StageFn stage_fn_sph(int acu, int lim, int rm) {
  if (acu == ACU_FIRST) return stage_fn_rm<ACU_FIRST, 2, 3, 1>(rm);
  if (acu != ACU_MUSCL) return nullptr;
  if (lim == 1) return stage_fn_rm<ACU_MUSCL, 1, 3, 1>(rm);
  if (lim == 3) return stage_fn_rm<ACU_MUSCL, 3, 3, 1>(rm);
  if (lim == 4) return stage_fn_rm<ACU_MUSCL, 4, 3, 1>(rm);
  return stage_fn_rm<ACU_MUSCL, 2, 3, 1>(rm);
}

StageFn stage_fn(int acu, int lim, int wflag, int rm, int sph = 0) {
  if (sph) return stage_fn_sph(acu, lim, rm);
  switch (acu) {
    case ACU_FIRST: return stage_fn_rm<ACU_FIRST, 2, 3>(rm);
    case ACU_MUSCL:
      if (lim == 1) return stage_fn_rm<ACU_MUSCL, 1, 3>(rm);
      if (lim == 3) return stage_fn_rm<ACU_MUSCL, 3, 3>(rm);
      if (lim == 4) return stage_fn_rm<ACU_MUSCL, 4, 3>(rm);
      return stage_fn_rm<ACU_MUSCL, 2, 3>(rm);
    case ACU_WENO3: return stage_fn_rm<ACU_WENO3, 2, 3>(rm);
    case ACU_WENO5:
      if (wflag == 2) return stage_fn_rm<ACU_WENO5, 2, 2>(rm);
      return stage_fn_rm<ACU_WENO5, 2, 3>(rm);
    default: return stage_fn_rm<ACU_WENO7, 2, 3>(rm);
  }
}

}  // namespace

// Cells per stage tile for a tube of n cells. A CTA's time hardly depends on
// its tile (each thread reconstructs part of one position, then helps with
// one face and one cell, so the CTA is as long as one thread's chain of FP64
// latencies), so
// the launch lasts about one CTA time per wave of resident CTAs. The choice:
// the fewest waves over the thread counts 64..STAGE_MAX_THREADS (their
// occupancy, limited by the shared-memory window, from the runtime), then
// the smallest tile that keeps that number of waves, so that the CTAs spread
// over all resident slots. 20,000 cells with WENO5 and GRI-3.0: 66-cell tiles,
// 304 CTAs, two per SM, one wave (62-cell tiles would need 323 CTAs, and the
// 19 of a second wave would double the launch).
cudaError_t stage_tiling(int acu, int lim, int wflag, int rm, int ns, int n, int* tc_out, int sph) {
  int dev = 0, nsm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  const StageFn kern = stage_fn(acu, lim, wflag, rm, sph);
  if (!kern) return cudaErrorInvalidValue;
  long best_waves = -1, best_slots = 0;
  int best_tcmax = 0;
  for (int nt = 64; nt <= STAGE_MAX_THREADS; nt += 32) {
    const int tcmax = nt / STAGE_SPLIT - 2;
    const size_t smem = stage_smem_bytes(acu, ns, tcmax);
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) {
      (void)cudaGetLastError();
      continue;  // window larger than a CTA may hold
    }
    int occ = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, nt, smem);
    if (e != cudaSuccess) return e;
    if (occ < 1) continue;
    const long slots = (long)occ * nsm;
    const long nb = (n + tcmax - 1) / tcmax;
    const long waves = (nb + slots - 1) / slots;
    if (best_waves < 0 || waves < best_waves) {
      best_waves = waves;
      best_slots = slots;
      best_tcmax = tcmax;
    }
  }
  if (best_waves < 0) return cudaErrorInvalidConfiguration;
  long tc = (n + best_waves * best_slots - 1) / (best_waves * best_slots);
  tc = std::max<long>(tc, 16);
  tc = std::min<long>(tc, best_tcmax);
  *tc_out = (int)tc;
  return cudaSuccess;
}

cudaError_t launch_stage(const StageArgs& a, int acu, int lim, int wflag, int rm, cudaStream_t s) {
  const StageFn kern = stage_fn(acu, lim, wflag, rm, a.spherical);
  if (!kern || (a.spherical && (a.kind == 2 || a.skip_uniform))) return cudaErrorInvalidValue;
  const size_t smem = stage_smem_bytes(acu, a.ns, a.tc);
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  // SMR: the segments' end columns, before the stage updates them in place
  if (a.tubes.smr_snap) {
    e = launch_smr_snapshot(a, s);
    if (e != cudaSuccess) return e;
  }
  // transport fluxes of the stage input, before the stage updates it in place
  if (a.tran.flux) {
    if (a.skip_uniform || (a.tubes.tiles && !a.tran.col_tube)) return cudaErrorInvalidValue;
    e = launch_tran(a, s);
    if (e != cudaSuccess) return e;
  }
  const int grid = a.tubes.tiles ? a.tubes.ntiles : (a.n + a.tc - 1) / a.tc;
  kern<<<grid, stage_threads(a.tc), smem, s>>>(a);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  // with the uniform-region shortcuts, QcToqf runs after every tile's update
  if (a.skip_uniform && !(a.kind == 2 && a.rk4_stage < 3)) {
    const size_t qsm = sizeof(double) * (size_t)(QR_THREADS / STAGE_SPLIT) * (size_t)(a.ns + 3);
    k_qc_to_qf_runs<<<(a.n + QR_BLOCK - 1) / QR_BLOCK, QR_THREADS, qsm, s>>>(a);
    e = cudaGetLastError();
  }
  return e;
}

// flags[k] = 1 when species row k of the conserved state is nonzero in some
// interior cell (one CTA per row).
// flags[k] |= 1 when species row k holds a non-zero entry; blockIdx.y takes
// one chunk of the row (flags cleared by the caller)
__global__ void k_species_present(const double* qc, int ld, int n, int* flags) {
  const double* row = qc + (size_t)(3 + blockIdx.x) * ld + GHOST;
  const int chunk = (n + gridDim.y - 1) / gridDim.y;
  const int i0 = blockIdx.y * chunk, i1 = min(n, i0 + chunk);
  int any = 0;
  for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) any |= (row[i] != 0.0) ? 1 : 0;
  any = __syncthreads_or(any);
  if (threadIdx.x == 0 && any) atomicOr(flags + blockIdx.x, 1);
}

cudaError_t launch_species_present(const double* qc, int ld, int n, int ns, int* flags, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(flags, 0, (size_t)ns * sizeof(int), s);
  if (e != cudaSuccess) return e;
  const int chunks = std::max(1, std::min(64, (n + 4095) / 4096));
  k_species_present<<<dim3(ns, chunks), 256, 0, s>>>(qc, ld, n, flags);
  return cudaGetLastError();
}

cudaError_t launch_cvel(const double* qf, int n, int ld, unsigned long long* cvel, cudaStream_t s,
                        const int* colmap, const int* tube_of) {
  k_cvel<<<(n + 127) / 128, 128, 0, s>>>(qf, n, ld, cvel, colmap, tube_of);
  return cudaGetLastError();
}

cudaError_t launch_step_begin_tubes(int ntube, const double* time, double tend, const long long* nsteps,
                                    const long long* max_steps, double cfl, const double* dx, unsigned long long* cvel,
                                    int* active, double* dt, int* step_active, cudaStream_t s) {
  k_step_begin_tubes<<<1, 256, 0, s>>>(ntube, time, tend, nsteps, max_steps, cfl, dx, cvel, active, dt, step_active);
  return cudaGetLastError();
}

cudaError_t launch_aos_to_soa(const double* aos, int ne, int n, double* soa, int ld, cudaStream_t s) {
  const size_t tot = (size_t)ne * n;
  k_aos_to_soa<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(aos, ne, n, soa, ld);
  return cudaGetLastError();
}

cudaError_t launch_soa_to_aos(const double* soa, int ne, int n, int ld, double* aos, cudaStream_t s) {
  const size_t tot = (size_t)ne * n;
  k_soa_to_aos<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(soa, ne, n, ld, aos);
  return cudaGetLastError();
}

cudaError_t launch_step_begin(const double* time, double tend, const long long* nsteps, const long long* max_steps,
                              double cfl, double dx, unsigned long long* cvel, int* step_active, double* dt_dev,
                              cudaStream_t s) {
  k_step_begin<<<1, 1, 0, s>>>(time, tend, nsteps, max_steps, cfl, dx, cvel, step_active, dt_dev);
  return cudaGetLastError();
}

cudaError_t launch_qc_to_qf(const StageArgs& a, cudaStream_t s) {
  const int nt = 64;
  const size_t smem = sizeof(double) * (size_t)a.ns * nt;
  k_qc_to_qf<<<(a.n + nt - 1) / nt, nt, smem, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_init_cells(int n, int ns, const double* T, const double* p, const double* u, const double* X,
                              int ldx, double* qf, double* qc, int ld, cudaStream_t s) {
  const int nt = 64;
  const size_t smem = sizeof(double) * (size_t)ns * nt;
  k_init_cells<<<(n + nt - 1) / nt, nt, smem, s>>>(n, T, p, u, X, ldx, qf, qc, ld);
  return cudaGetLastError();
}

}  // namespace edyn
