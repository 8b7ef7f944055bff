// The kernels and launchers of fortrancfd_gb300/csrc/fluid.cu, translated
// for the host (tests/emu/host_source.py) and run through the CTA
// emulation of cta_emu.h, behind a small C ABI for the tests (test
// infrastructure: the product library never contains this). Entry points
// mirror the library's host code for one step of a tube: the stage
// launches of fluid_step (launch_stage, which runs the transport kernels
// first), the energy-source kernel and the output rows.
#include <memory>
#include <string>

#include <cuda_runtime.h>

#include "cta_emu.h"
#define __CUDACC__ 1
#include "edyn_dev.cuh"
#include "fastmath.cuh"
#include "recon.cuh"
#undef __CUDACC__
#include "edyn_kernels.h"
#include "transport.h"
using std::isfinite;
#include "fluid_host.inc"

using namespace edyn;
// only the entry points below leave the library: the runtime stubs and the
// translated kernels bind to their own definitions, whatever CUDA runtime
// or solver library the process has loaded before
#define EMU_EXPORT __attribute__((visibility("default")))
extern "C" int edyn_mech_load_dir(const char* dir, edyn_mech* m, char* err, int errlen);

namespace {
edyn_mech g_mech;
std::vector<double> g_tables;
TranDev g_tr;
int g_ns = 0;

struct Rows {
  int n, ld, ne;
  std::vector<double> qf[2], qc, q0, tp, fl;
  int cur = 0;
  Rows(int ld_, int ne_) : n(0), ld(ld_), ne(ne_) {
    for (auto* v : {&qf[0], &qf[1], &qc, &q0, &fl}) v->assign((size_t)ne * ld, 0.0);
    tp.assign((size_t)(TRAN_ROWS_FIXED + 2 * (ne - 3)) * ld, 0.0);
  }
};

// scheme flags -> (acu, lim, wflag) as edyn_init sets them
void scheme(const int* fl, int& acu, int& lim, int& wflag) {
  acu = ACU_MUSCL;
  lim = fl[3];
  wflag = 3;
  if (fl[2] == 0) {
    acu = ACU_FIRST;
  } else if (fl[2] == 2) {
    if (fl[4] == 1) acu = ACU_WENO3;
    else if (fl[4] == 2 || fl[4] == 3) {
      acu = ACU_WENO5;
      wflag = fl[4];
    } else {
      acu = ACU_WENO7;
    }
  }
}

// the stages of one fluid_step (host mode)
int stages(Rows& r, StageArgs a, const int* fl, int acu, int lim, int wflag) {
  const int nst = fl[0] == 0 ? 1 : 3;
  for (int s = 0; s < nst; ++s) {
    a.qf_in = r.qf[r.cur].data();
    a.qf_out = r.qf[r.cur ^ 1].data();
    if (fl[0] == 0) {
      a.kind = 0;
      a.save_q0 = 0;
    } else if (s == 0) {
      a.kind = 0;
      a.save_q0 = 1;
    } else if (s == 1) {
      a.kind = 1;
      a.save_q0 = 0;
      a.h1 = 3.0 / 4.0;
      a.h2 = 1.0 / 4.0;
    } else {
      a.kind = 1;
      a.save_q0 = 0;
      a.h1 = 1.0 / 3.0;
      a.h2 = 2.0 / 3.0;
    }
    if (launch_stage(a, acu, lim, wflag, fl[1], 0) != cudaSuccess) return 11;
    r.cur ^= 1;
  }
  return 0;
}
}  // namespace

extern "C" {

EMU_EXPORT int emu_setup(const char* dir) {
  char err[512];
  if (edyn_mech_load_dir(dir, &g_mech, err, 512)) return 1;
  ThermoTable tb;
  build_thermo_table(g_mech, tb);
  if (fluid_upload_tables(tb, 0)) return 2;
  g_ns = g_mech.nspec;
  std::unique_ptr<edyn_tran> t(new edyn_tran);
  if (edyn_tran_load_dir(dir, t.get(), err, 512)) return 3;
  // the device tables of load_tran_tables, in host memory
  const int ns = g_ns, npair = ns * (ns - 1) / 2;
  std::vector<double>& h = g_tables;
  h.clear();
  auto put = [&](size_t n) {
    const size_t o = h.size();
    h.resize(o + n, 0.0);
    return o;
  };
  const size_t o_eta = put(4 * ns), o_lam = put(4 * ns), o_dif = put(4 * (size_t)npair);
  const size_t o_wa = put((size_t)ns * ns), o_wb = put((size_t)ns * ns), o_wc = put((size_t)ns * ns);
  const size_t o_w = put(ns), o_e2 = put(64), o_lg = put(184);
  for (int k = 0; k < ns; ++k)
    for (int n = 0; n < 4; ++n) {
      h[o_eta + 4 * k + n] = t->cofeta[k][n];
      h[o_lam + 4 * k + n] = t->coflam[k][n];
    }
  size_t q = o_dif;
  for (int k = 1; k < ns; ++k)
    for (int j = 0; j < k; ++j)
      for (int n = 0; n < 4; ++n) h[q++] = t->cofd[k][j][n];
  for (int k = 0; k < ns; ++k) {
    h[o_w + k] = t->wt[k];
    for (int j = 0; j < ns; ++j) {
      const double g = 1.0 / std::sqrt(1.0 + t->wt[k] / t->wt[j]);
      h[o_wa + (size_t)k * ns + j] = g;
      h[o_wb + (size_t)k * ns + j] = std::sqrt(std::sqrt(t->wt[j] / t->wt[k])) * g;
      h[o_wc + (size_t)k * ns + j] = std::sqrt(t->wt[j] / t->wt[k]) * g;
    }
  }
  fill_exp_table(&h[o_e2]);
  fill_log_table(&h[o_lg]);
  g_tr = TranDev{};
  g_tr.eta = &h[o_eta];
  g_tr.lam = &h[o_lam];
  g_tr.dif = &h[o_dif];
  g_tr.wa = &h[o_wa];
  g_tr.wb = &h[o_wb];
  g_tr.wc = &h[o_wc];
  g_tr.W = &h[o_w];
  g_tr.e2 = &h[o_e2];
  g_tr.lg = &h[o_lg];
  g_tr.patmos = t->patmos;
  return 0;
}

// Packed tubes (one tube: ntube = 1 and the single-tube launch when
// packed == 0; packed == 2: the segments of an SMR domain, left to right,
// with the interface ghosts of interpolation_block and x = 0 where the
// leading segments coarser than dx_comp = dx_comp end) stepped nsteps times
// with their own dt (dts[step * ntube + t]) by the stages of fluid_step. flags: select_time, select_riemann,
// flag_acu, flag_muscl, flag_weno, flag_rbound, do_tran, is_spherical;
// p_out; walls on the left. qf, qc: AoS rows of all cells, tube after tube;
// qc is updated, qf_out receives the new primitive rows.
EMU_EXPORT int emu_fluid(int ntube, const int* ncell, const double* dx, int packed, double dx_comp, const int* fl,
                         double p_out, const double* qf_aos, double* qc_io, double* qf_out, int nsteps,
                         const double* dts, unsigned* err) {
  const int ns = g_ns, ne = ns + 3;
  std::vector<long long> off(ntube), first(ntube);
  long long cols = 0, ntot = 0;
  for (int t = 0; t < ntube; ++t) {
    off[t] = cols;
    first[t] = ntot;
    cols += ncell[t] + 2 * GHOST;
    ntot += ncell[t];
  }
  if (!packed && ntube != 1) return 1;
  Rows r((int)cols, ne);
  for (int t = 0; t < ntube; ++t)
    for (int i = 0; i < ncell[t]; ++i)
      for (int v = 0; v < ne; ++v) {
        const size_t src = (size_t)(first[t] + i) * ne + v, dst = (size_t)v * cols + off[t] + i + GHOST;
        r.qf[0][dst] = qf_aos[src];
        r.qc[dst] = qc_io[src];
      }
  int acu, lim, wflag;
  scheme(fl, acu, lim, wflag);
  int tc = 0;
  if (stage_tiling(acu, lim, wflag, fl[1], ns, (int)ntot, &tc, fl[7]) != cudaSuccess) return 10;
  std::vector<int4> tiles;
  std::vector<int> n(ncell, ncell + ntube), active(ntube, 1), col_tube(cols, 0);
  std::vector<double> dxs(dx, dx + ntube), pout(ntube, p_out), dtt(ntube, 0.0), x0(ntube, 0.0);
  {
    double x = 0.0;
    for (int t = 0; t < ntube && dx[t] != dx_comp; ++t) x -= ncell[t] * dx[t];
    for (int t = 0; t < ntube; ++t) {
      x0[t] = x;
      x += ncell[t] * dx[t];
    }
  }
  std::vector<double> snap(ntube > 1 ? (size_t)(ntube - 1) * 2 * ne * 2 * acu_lvir(acu) : 1, 0.0);
  for (int t = 0; t < ntube; ++t) {
    const int nb = (ncell[t] + tc - 1) / tc;
    for (int b = 0; b < nb; ++b) tiles.push_back(make_int4(t, b, nb, 0));
    for (long long j = 0; j < ncell[t] + 2 * GHOST; ++j) col_tube[off[t] + j] = t;
  }
  unsigned e = 0;
  for (int step = 0; step < nsteps; ++step) {
    StageArgs a;
    std::memset(&a, 0, sizeof(a));
    a.n = packed ? (int)ntot : ncell[0];
    a.ld = (int)cols;
    a.lvir = acu_lvir(acu);
    a.ns = ns;
    a.tc = tc;
    a.qc = r.qc.data();
    a.q0 = r.q0.data();
    a.dx = dx[0];
    a.dt = dts[(size_t)step * ntube];
    a.rbound = fl[5];
    a.p_out = p_out;
    a.strict_newton = 1;
    a.err = &e;
    if (fl[6]) {
      a.tran = g_tr;
      a.tran.tp = r.tp.data();
      a.tran.flux = r.fl.data();
      a.tran.col_tube = packed ? col_tube.data() : nullptr;
    }
    a.spherical = fl[7];
    if (packed) {
      for (int t = 0; t < ntube; ++t) dtt[t] = dts[(size_t)step * ntube + t];
      a.tubes.tiles = tiles.data();
      a.tubes.n = n.data();
      a.tubes.off = off.data();
      a.tubes.dx = dxs.data();
      a.tubes.p_out = pout.data();
      a.tubes.dt = dtt.data();
      a.tubes.active = active.data();
      a.tubes.ntiles = (int)tiles.size();
      a.tubes.ntube = ntube;
      if (packed == 2) {
        a.tubes.smr_snap = ntube > 1 ? snap.data() : nullptr;
        a.tubes.x0 = x0.data();
      }
    }
    const int rc = stages(r, a, fl, acu, lim, wflag);
    if (rc) return rc;
  }
  for (int t = 0; t < ntube; ++t)
    for (int i = 0; i < ncell[t]; ++i)
      for (int v = 0; v < ne; ++v) {
        const size_t dst = (size_t)(first[t] + i) * ne + v, src = (size_t)v * cols + off[t] + i + GHOST;
        qf_out[dst] = r.qf[r.cur][src];
        qc_io[dst] = r.qc[src];
      }
  if (err) *err = e;
  return 0;
}

// k_energy_sources on one tube: radiation (nrad species, their fit rows),
// wall heat (wall, params: Nu, d, Tw_min, Tw_max, alpha, beta), ignition
// (type, nig sources of E, r, duration, start). qrad, qtw: the per-cell
// source outputs.
// With nseg > 0 the cells are the segments seg_n[] (cell size seg_dx[]) of
// an SMR domain laid out as the library packs them, each cell at its x_m
// (x = 0 at the left edge: no coarser leading segments here).
EMU_EXPORT int emu_sources(int n, double dx, int nseg, const int* seg_n, const double* seg_dx, const double* qf_aos,
                           double* qc_io, double* qf_out, double dt, double time, int nrad, const int* rsp,
                           const double* rcoef, int wall, const double* wp, int igt, int nig, const double* ig,
                           double* qrad, double* qtw, unsigned* err) {
  const int ns = g_ns, ne = ns + 3;
  std::vector<int> colmap(n), tube_of(n);
  std::vector<double> xm(2 * (size_t)n);
  int ld = n + 2 * GHOST;
  if (nseg > 0) {
    int i = 0;
    long long off = 0;
    double x = 0.0;
    for (int t = 0; t < nseg; ++t) {
      for (int j = 0; j < seg_n[t]; ++j, ++i) {
        colmap[i] = (int)(off + j);
        tube_of[i] = t;
        xm[i] = x + (j + 0.5) * seg_dx[t];
      }
      off += seg_n[t] + 2 * GHOST;
      x += seg_n[t] * seg_dx[t];
    }
    ld = (int)off;
  } else {
    for (int i = 0; i < n; ++i) colmap[i] = i;
  }
  Rows r(ld, ne);
  for (int i = 0; i < n; ++i)
    for (int v = 0; v < ne; ++v) {
      r.qf[0][(size_t)v * ld + colmap[i] + GHOST] = qf_aos[(size_t)i * ne + v];
      r.qc[(size_t)v * ld + colmap[i] + GHOST] = qc_io[(size_t)i * ne + v];
    }
  SourceArgs s;
  std::memset(&s, 0, sizeof(s));
  unsigned e = 0;
  s.n = n;
  s.ld = ld;
  s.ns = ns;
  s.qf = r.qf[0].data();
  s.qc = r.qc.data();
  s.dt = dt;
  s.time = time;
  s.dx = dx;
  s.strict_newton = 1;
  s.err = &e;
  s.nrad = nrad;
  for (int k = 0; k < nrad; ++k) {
    s.rad_sp[k] = rsp[k];
    for (int j = 0; j < 6; ++j) s.rad_coef[k][j] = rcoef[6 * k + j];
  }
  s.wall = wall;
  if (wall) {
    s.nu = wp[0];
    s.d_m = wp[1];
    s.tw_min = wp[2];
    s.tw_max = wp[3];
    s.alpha = wp[4];
    s.beta = wp[5];
  }
  s.lam = g_tr.lam;
  s.e2 = g_tr.e2;
  s.lg = g_tr.lg;
  s.ig_type = igt;
  s.n_ig = nig;
  for (int g = 0; g < nig; ++g) {
    s.ig_e[g] = ig[4 * g];
    s.ig_r[g] = ig[4 * g + 1];
    s.ig_t[g] = ig[4 * g + 2];
    s.ig_t0[g] = ig[4 * g + 3];
  }
  std::vector<double> q2(2 * (size_t)n, 0.0);
  s.q_rad = q2.data();
  s.q_tw = q2.data() + n;
  std::vector<unsigned long long> cv(nseg > 0 ? nseg : 1, 0ull);
  if (nseg > 0) {
    s.colmap = colmap.data();
    s.tube_of = tube_of.data();
    s.xm = xm.data();
    s.cvel = cv.data();
  }
  if (launch_energy_sources(s, 0) != cudaSuccess) return 11;
  for (int i = 0; i < n; ++i)
    for (int v = 0; v < ne; ++v) {
      qf_out[(size_t)i * ne + v] = r.qf[0][(size_t)v * ld + colmap[i] + GHOST];
      qc_io[(size_t)i * ne + v] = r.qc[(size_t)v * ld + colmap[i] + GHOST];
    }
  std::memcpy(qrad, q2.data(), 8 * (size_t)n);
  std::memcpy(qtw, q2.data() + n, 8 * (size_t)n);
  if (err) *err = e;
  return 0;
}

// The transport properties (TranDev::tp rows, cells -1..n of each tube)
// of the thread-per-cell kernel (warp == 0) or the warp-per-cell kernel,
// for one tube (packed == 0) or packed tubes; rbound: wall or outlet.
EMU_EXPORT int emu_tran_props(int ntube, const int* ncell, const double* dx, int packed, int rbound, double p_out,
                              const double* qc_aos, int warp, double* props) {
  const int ns = g_ns, ne = ns + 3, prow = TRAN_ROWS_FIXED + 2 * ns;
  std::vector<long long> off(ntube), first(ntube);
  long long cols = 0, ntot = 0;
  for (int t = 0; t < ntube; ++t) {
    off[t] = cols;
    first[t] = ntot;
    cols += ncell[t] + 2 * GHOST;
    ntot += ncell[t];
  }
  Rows r((int)cols, ne);
  for (int t = 0; t < ntube; ++t)
    for (int i = 0; i < ncell[t]; ++i)
      for (int v = 0; v < ne; ++v) r.qc[(size_t)v * cols + off[t] + i + GHOST] = qc_aos[(size_t)(first[t] + i) * ne + v];
  std::vector<int> n(ncell, ncell + ntube), col_tube(cols, 0);
  std::vector<double> dxs(dx, dx + ntube), pout(ntube, p_out);
  std::vector<int4> tiles(1, make_int4(0, 0, 1, 0));
  for (int t = 0; t < ntube; ++t)
    for (long long j = 0; j < ncell[t] + 2 * GHOST; ++j) col_tube[off[t] + j] = t;
  StageArgs a;
  std::memset(&a, 0, sizeof(a));
  unsigned e = 0;
  a.n = packed ? (int)ntot : ncell[0];
  a.ld = (int)cols;
  a.lvir = 2;
  a.ns = ns;
  a.qc = r.qc.data();
  a.qf_in = r.qf[0].data();
  a.dx = dx[0];
  a.rbound = rbound;
  a.p_out = p_out;
  a.strict_newton = 1;
  a.err = &e;
  a.tran = g_tr;
  a.tran.tp = r.tp.data();
  a.tran.flux = r.fl.data();
  if (packed) {
    a.tran.col_tube = col_tube.data();
    a.tubes.tiles = tiles.data();
    a.tubes.n = n.data();
    a.tubes.off = off.data();
    a.tubes.dx = dxs.data();
    a.tubes.p_out = pout.data();
    a.tubes.ntube = ntube;
  }
  const int np = packed ? (int)cols : ncell[0] + 2;
  if (warp)
    emu_launch(k_tran_props_warp, dim3((np + TRAN_WARP_CELLS - 1) / TRAN_WARP_CELLS), dim3(32 * TRAN_WARP_CELLS), 0,
               (cudaStream_t)0, a);
  else
    emu_launch(k_tran_props, dim3((np + TRAN_PROPS_THREADS - 1) / TRAN_PROPS_THREADS), dim3(TRAN_PROPS_THREADS), 0,
               (cudaStream_t)0, a);
  std::memcpy(props, r.tp.data(), (size_t)prow * cols * sizeof(double));
  return e ? 12 : 0;
}

// k_output_rows of one tube with cell centres (i + 1/2) dx
EMU_EXPORT int emu_output_rows(int n, double dx, const double* qf_aos, const double* qc_aos, double* rows) {
  const int ns = g_ns, ne = ns + 3, ld = n + 2 * GHOST;
  Rows r(ld, ne);
  for (int i = 0; i < n; ++i)
    for (int v = 0; v < ne; ++v) {
      r.qf[0][(size_t)v * ld + i + GHOST] = qf_aos[(size_t)i * ne + v];
      r.qc[(size_t)v * ld + i + GHOST] = qc_aos[(size_t)i * ne + v];
    }
  std::vector<double> xm(2 * (size_t)n);
  for (int i = 0; i < n; ++i) {
    xm[i] = (i + 0.5) * dx;
    xm[n + i] = dx;
  }
  OutputArgs a;
  std::memset(&a, 0, sizeof(a));
  a.n = n;
  a.ld = ld;
  a.ns = ns;
  a.qf = r.qf[0].data();
  a.qc = r.qc.data();
  a.xm = xm.data();
  a.out = rows;
  return launch_output_rows(a, 0) == cudaSuccess ? 0 : 11;
}

}  // extern "C"
