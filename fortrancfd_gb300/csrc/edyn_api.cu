// C ABI of the GB300 hot path (see include/edyn_gpu.h).
//
// A context mirrors the state the reference's main_sim keeps between the
// hot-path calls (SRC/main.f90:38-199): the tube's conserved and primitive
// state, now device-resident in structure-of-arrays rows, the stage-0 copy
// of TVDRK3, heat release rates and the device clock of the time loop. The
// host crosses to the device only at these entry points.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "../../include/edyn_gpu.h"
#include "../../include/edyn_surrogate.h"
#include "chem.h"
#include "edyn_dev.cuh"
#include "edyn_kernels.h"
#include "fastmath.cuh"
#include "mechanism.h"
#include "recon.cuh"
#include "transport.h"
#include "h5file.h"

extern "C" int edyn_mech_load_dir(const char* dir, edyn_mech* m, char* err, int errlen);
extern "C" int edyn_mech_write(const edyn_mech* m, const char* path);

namespace {

using namespace edyn;

// The surrogate path of a tube (chem_mode 1): the network the caller
// attached, the gate's tolerances, and the packed work buffers of one source
// step, sized for every cell of the tube.
struct Surr {
  static constexpr int KIN = 64, HID = 256, KOUT = 64;
  bool attached = false;
  bool net = false;            // false: the explicit increment alone (the method without the network)
  const void* wt[4] = {};      // tiled BF16 weights (caller-owned)
  const float* b[4] = {};      // biases (caller-owned)
  const float* norm = nullptr; // mu, isig, omu, osig: 4 x 64 FP32 (caller-owned)
  double rtol = 2.5e-4, atol = 2.5e-10, etol = 1e-6;
  double yfloor = 1e-10, tfloor = 1e-4;
  int nrow = 0, ne = 0;
  unsigned* d_count = nullptr;  // [0] packed rows, [1], [2] rows accepted on the network / explicit candidate
  int* pk_idx = nullptr;
  double *pk_rho = nullptr, *pk_dt = nullptr, *pk_y0 = nullptr, *pk_f0 = nullptr, *pk_y1 = nullptr;
  double *pk_ya = nullptr, *pk_f1 = nullptr, *pk_fa = nullptr;
  void *X = nullptr, *Xt = nullptr, *H[3] = {};
  float* out = nullptr;
  float* zero_out = nullptr;   // [M][64] zeros: the explicit candidate's network output
  float* zero_one = nullptr;   // 64 zeros then 64 ones: its omu and osig
  int* accept = nullptr;
  int* rj_idx = nullptr;
  double *rj_rho = nullptr, *rj_dt = nullptr, *rj_y = nullptr;
  int* d_nrej = nullptr;
  double* wmol = nullptr;      // kg/mol
  double* elem = nullptr;      // [ne][nspe] atoms per molecule
  // counters of the last source step: packed (not inert), accepted on the
  // network's candidate, on the explicit one, fallback cells, right-hand
  // sides of the screen, of the gate, of the fallback integration
  double stats[7] = {};
};

// Several tubes packed side by side in one context's rows (edyn_init_tubes):
// tube t's block of n_t + 2 GHOST columns starts at column off[t]; its cells
// are the packed cells first[t] .. first[t] + n_t - 1.
struct Packed {
  int ntube = 0;
  std::vector<int> n;
  std::vector<long long> off, first;
  std::vector<double> dx, p_out;
  int4* d_tiles = nullptr;
  int ntiles = 0;
  int* d_n = nullptr;
  long long* d_off = nullptr;
  double *d_dx = nullptr, *d_p_out = nullptr, *d_dt = nullptr, *d_time = nullptr;
  int* d_active = nullptr;
  unsigned long long* d_cvel = nullptr;
  int* colmap = nullptr;   // column of each packed cell
  int* tube_of = nullptr;  // tube of each packed cell
  // SMR blocks (edyn_init_blocks): the tubes are the segments of one domain
  bool smr = false;
  double dx_comp = 0.0;    // the dx of calc_dt's dt = cfl dx_comp / max(|u| + a)
  double* d_snap = nullptr;
  double* d_x0 = nullptr;  // the coordinate of each segment's left edge
  std::vector<double> x0;  // the same on the host
};

// A contiguous run of cells in the rows: the whole tube, or one packed tube.
struct Seg {
  long long off, first;
  int n;
};

// Tubes of this many cells and more take the two-pass chemistry by default
// (measured: 20,000 cells of 5 um CH4/air 3.68 -> 2.02 ms per step, 20,000
// of 50 um CH4/O2 4.48 -> 4.56 ms).
constexpr int CHEM_TWO_PASS_CELLS = 10000;

struct Ctx {
  edyn_mech mech;
  ThermoTable tb;
  FluidBC bc;
  int ns = 0, ne = 0, n = 0, lvir = 0, ld = 0;
  int select_time = 1, riemann = 2, flag_acu = 1, flag_muscl = 2, flag_weno = 0;
  int lbound = 0, rbound = 0, do_reaction = 0, strict = 1, chem_mode = 0;
  int acu = ACU_MUSCL, lim = 2, wflag = 3;
  double dx = 0, p_out = 101325.0, t_in = 300.0, rho_u_in = 0.0, rtol = 1e-5, atol = 1e-13;
  cudaStream_t own = nullptr, stream = nullptr;
  double* qf[2] = {nullptr, nullptr};
  int cur = 0;
  double* qc = nullptr;
  double* q0 = nullptr;
  double* acc = nullptr;      // RK4: k1 + 2 k2 + 2 k3 (select_time 2 only)
  double* hrr = nullptr;
  double* hrr_dot = nullptr;  // HRR_dot of the last source step, once evaluated
  double* tchem = nullptr;    // temperature each cell's last integration ended with
  // HRR_dot of the last source step: 0 none (zeros), 1 not yet evaluated (the
  // primitive state is still the one that step left), 2 evaluated into
  // hrr_dot, 3 not yet evaluated, the rows it needs saved in hrr_dot_rows
  int hrr_dot_state = 0;
  double* hrr_dot_rows = nullptr;  // primitive rows the last source step left
  int chem_max_steps = 0;     // integrator step cap per cell (0: the default 4000)
  int precheck = 1;           // single-precision pre-check of the inert-cell test
  int skip_uniform = 1;       // stage: no faces for cells whose stencils hold one state
  // transport (do_tran = 1): the fits, their device tables and the buffers
  // of the per-cell properties and the face fluxes
  int do_tran = 0;
  int spherical = 0;           // is_spherical (the problem file's /problem/ flag)
  std::string chem_dir;        // the mechanism directory (transport fits load from it on demand)
  // energy sources after the chemistry (radiation, wall heat, ignition);
  // src.nrad / wall / ig_type select them
  SourceArgs src{};
  bool src_on = false;
  double clock = 0.0;          // time of the last edyn_step / edyn_advance (the ignition window's clock)
  double* d_tran = nullptr;
  double* d_tp = nullptr;
  double* d_tflux = nullptr;
  int* d_col_tube = nullptr;   // packed tubes with transport: the tube of each column
  TranDev trd{};
  double* staging = nullptr;
  size_t staging_bytes = 0;
  // device clock of the time loop
  double* d_time = nullptr;
  long long* d_nsteps = nullptr;
  long long* d_max_steps = nullptr;  // step budget of the current edyn_advance call
  int* d_active = nullptr;
  double* d_dt = nullptr;
  unsigned long long* d_cvel = nullptr;
  unsigned* d_err = nullptr;
  int* d_cost = nullptr;      // right-hand sides per cell in the last chemistry launch
  unsigned* d_hot = nullptr;  // cells that get a four-warp team in the next one
  double* d_hlast = nullptr;  // step size each cell's integrator proposed last
  // the two-pass source step (screen + listed integration): listed cells,
  // their count, per-cell hot classes and the class histogram
  int* d_list = nullptr;
  unsigned* d_list_count = nullptr;
  unsigned char* d_cls = nullptr;
  unsigned* d_hist = nullptr;
  // runs of identical cells in the two-pass chemistry launch
  unsigned char* d_run_flag = nullptr;
  int* d_heads = nullptr;
  unsigned* d_head_count = nullptr;
  int* d_run_last = nullptr;
  int* d_run_head = nullptr;
  bool listed = false;       // the two-pass form is in use
  cudaGraphExec_t graph = nullptr;
  int graph_steps = 0;
  double graph_cfl = -1, graph_tend = -1;
  int stage_tc = 0;        // cells per stage tile
  ChemState chem;
  // Tables of the species whose elements all occur in the tube (or at the
  // inlet), built when that drops species: the others are zero everywhere
  // and stay zero (no reaction forms a species from absent elements), so
  // the reactions that involve them have zero rates and are left out.
  ChemState chem_sub;
  std::vector<char> sub_keep;
  bool use_sub = false;
  int* d_present = nullptr;  // per species: nonzero somewhere in the tube
  Surr surr;
  Packed pk;
  // output (write_hdf5_b) and restart (read_hdf5_restart)
  double* d_srcq = nullptr;    // [2][n]: Qrad and qTw of the last source step (eos_obj%Qrad, %qTw)
  double* d_out = nullptr;     // [EDYN_OUT_FIXED + ns][n]: the output rows of a snapshot
  double* h_out = nullptr;     // pinned host copy of d_out
  double* d_xm = nullptr;      // [2][n]: cell centres and sizes
  std::vector<double> xm;      // the same on the host
  cudaStream_t out_stream = nullptr;
  cudaEvent_t out_ready = nullptr, out_copied = nullptr;
  bool out_pending = false;    // a snapshot's copy is queued and not yet written
  H5Writer h5;
  std::string err;
};

std::vector<Seg> segs(const Ctx* c) {
  std::vector<Seg> v;
  if (c->pk.ntube == 0) {
    v.push_back({0, 0, c->n});
  } else {
    for (int t = 0; t < c->pk.ntube; ++t) v.push_back({c->pk.off[t], c->pk.first[t], c->pk.n[t]});
  }
  return v;
}

int fail(Ctx* c, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (c) c->err = buf;
  return code;
}

#define CK(call)                                                                                 \
  do {                                                                                           \
    cudaError_t e_ = (call);                                                                     \
    if (e_ != cudaSuccess) return fail(c, EDYN_E_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

// Host evaluation of specific_energy(T, X) (SRC/thermo.f90:356-375) for the
// inlet state, in the reference's molar form.
double host_specific_energy(const edyn_mech& m, double T, const double* x) {
  double ubml = 0.0, wtm = 0.0;
  for (int k = 0; k < m.nspec; ++k) {
    const double* a = m.a[k][T > m.T_mid[k] ? 1 : 0];
    double sum = a[0] + T * (a[1] / 2 + T * (a[2] / 3 + T * (a[3] / 4 + T * a[4] / 5)));
    double h = RU_CGS * T * (sum + a[5] / T);
    ubml += x[k] * (h - RU_CGS * T);
    wtm += x[k] * m.W[k];
  }
  return ubml * 1e-4 / wtm;
}

StageArgs base_args(Ctx* c) {
  StageArgs a;
  std::memset(&a, 0, sizeof(a));
  a.n = c->n;
  a.ld = c->ld;
  a.lvir = c->lvir;
  a.ns = c->ns;
  a.tc = c->stage_tc;
  a.qc = c->qc;
  a.q0 = c->q0;
  a.dx = c->dx;
  a.lbound = c->lbound;
  a.rbound = c->rbound;
  a.p_out = c->p_out;
  a.strict_newton = c->strict;
  a.bc = c->bc;
  a.err = c->d_err;
  a.skip_uniform = c->skip_uniform;
  if (c->do_tran) {
    // the transport flux of a face is not decided by the stencil test of the
    // uniform-region shortcuts (it reads the conserved state): every face
    a.tran = c->trd;
    a.skip_uniform = 0;
  }
  if (c->spherical) {
    // equal face fluxes do not cancel under the face areas
    a.spherical = 1;
    a.skip_uniform = 0;
  }
  if (c->pk.ntube) {
    const Packed& k = c->pk;
    a.tubes = TubeTab{k.d_tiles, k.d_n, k.d_off, k.d_dx, k.d_p_out, k.d_dt, k.d_active, k.d_time, k.ntiles, k.colmap,
                      k.tube_of, k.smr ? k.d_snap : nullptr, k.ntube, k.d_x0};
  }
  return a;
}

static_assert(EDYN_STATUS_NEWTON == EDYN_E_NEWTON && EDYN_STATUS_CHEM == EDYN_E_CHEM &&
                  EDYN_STATUS_STATE == EDYN_E_STATE,
              "device status bits and ABI status classes differ");

// Reads and clears the context's device status word (the stream must be
// synchronised): a call reports the status bits its own kernels set.
int take_status(Ctx* c, const char* what) {
  unsigned e = 0;
  cudaError_t ce = cudaMemcpy(&e, c->d_err, sizeof(e), cudaMemcpyDeviceToHost);
  if (ce != cudaSuccess) return fail(c, EDYN_E_CUDA, "%s: status read: %s", what, cudaGetErrorString(ce));
  if (!e) return EDYN_OK;
  ce = cudaMemset(c->d_err, 0, sizeof(unsigned));
  if (ce != cudaSuccess) return fail(c, EDYN_E_CUDA, "%s: status clear: %s", what, cudaGetErrorString(ce));
  return fail(c, (int)e, "%s: device status 0x%x (%s%s%s)", what, e, (e & EDYN_E_NEWTON) ? "temperature Newton at its cap; " : "",
              (e & EDYN_E_CHEM) ? "chemistry integration failed; " : "",
              (e & EDYN_E_STATE) ? "non-finite, non-positive or clamped state" : "");
}

// Launches the stages of one fluid step. Device-loop mode when dev != 0:
// the stage kernels read step_active/dt from the device and the last
// kernel of the step (this one unless chemistry follows) advances the clock.
int fluid_step(Ctx* c, double dt, bool dev, bool last_is_fluid) {
  StageArgs a = base_args(c);
  a.dt = dt;
  if (dev) {
    a.step_active = c->d_active;
    a.dt_dev = c->d_dt;
  }
  if (c->select_time == 2) {
    // RK4 (SRC/timeintegration.f90:222-356): four stages on the primitive
    // state of the step's start; the last one writes the new primitives
    a.kind = 2;
    a.acc = c->acc;
    a.qf_in = c->qf[c->cur];
    a.qf_out = c->qf[c->cur ^ 1];
    for (int s = 0; s < 4; ++s) {
      a.rk4_stage = s;
      const bool last = s == 3;
      a.cvel_out = (dev && last && last_is_fluid && !c->src_on) ? (c->pk.ntube ? c->pk.d_cvel : c->d_cvel) : nullptr;
      a.time = (dev && last && last_is_fluid) ? c->d_time : nullptr;
      a.nsteps = (dev && last && last_is_fluid) ? c->d_nsteps : nullptr;
      cudaError_t e = launch_stage(a, c->acu, c->lim, c->wflag, c->riemann, c->stream);
      if (e != cudaSuccess) return fail(c, EDYN_E_CUDA, "stage launch: %s", cudaGetErrorString(e));
    }
    c->cur ^= 1;
    return EDYN_OK;
  }
  const int nst = c->select_time == 0 ? 1 : 3;
  for (int s = 0; s < nst; ++s) {
    a.qf_in = c->qf[c->cur];
    a.qf_out = c->qf[c->cur ^ 1];
    if (c->select_time == 0) {
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
    const bool last = (s == nst - 1);
    // with energy sources the source kernel publishes the new state's speed
    a.cvel_out = (dev && last && last_is_fluid && !c->src_on) ? (c->pk.ntube ? c->pk.d_cvel : c->d_cvel) : nullptr;
    a.time = (dev && last && last_is_fluid) ? c->d_time : nullptr;
    a.nsteps = (dev && last && last_is_fluid) ? c->d_nsteps : nullptr;
    cudaError_t e = launch_stage(a, c->acu, c->lim, c->wflag, c->riemann, c->stream);
    if (e != cudaSuccess) return fail(c, EDYN_E_CUDA, "stage launch: %s", cudaGetErrorString(e));
    c->cur ^= 1;
  }
  return EDYN_OK;
}

int surrogate_source_step(Ctx* c, double dt, bool dev);

int chem_source_step(Ctx* c, double dt, bool dev);

// solve_source (SRC/update.f90:100-150): the chemistry, then the energy
// sources. time: the step's time for the ignition window (host calls; the
// device loop reads its clock).
int source_step(Ctx* c, double dt, bool dev, double time = 0.0) {
  int rc = chem_source_step(c, dt, dev);
  if (rc || !c->src_on) return rc;
  SourceArgs s = c->src;
  s.n = c->n;
  s.ld = c->ld;
  s.ns = c->ns;
  s.qf = c->qf[c->cur];
  s.qc = c->qc;
  s.dt = dt;
  s.time = time;
  s.dx = c->dx;
  s.strict_newton = c->strict;
  s.err = c->d_err;
  s.lam = c->trd.lam;
  s.e2 = c->trd.e2;
  s.lg = c->trd.lg;
  s.q_rad = c->d_srcq;
  s.q_tw = c->d_srcq + c->n;
  if (dev) {
    s.dt_dev = c->d_dt;
    s.time_dev = c->d_time;
    s.step_active = c->d_active;
    s.cvel = c->d_cvel;
  }
  if (c->pk.ntube) {
    // SMR segments (one dt for all): columns, centres, per-segment speeds
    const Packed& k = c->pk;
    s.colmap = k.colmap;
    s.tube_of = k.tube_of;
    s.xm = c->d_xm;
    if (dev) {
      s.dt_dev = k.d_dt;
      s.time_dev = k.d_time;
      s.cvel = k.d_cvel;
    }
  }
  cudaError_t e = launch_energy_sources(s, c->stream);
  if (e != cudaSuccess) return fail(c, EDYN_E_CUDA, "energy sources: %s", cudaGetErrorString(e));
  return EDYN_OK;
}

int chem_source_step(Ctx* c, double dt, bool dev) {
  if (!c->do_reaction) return EDYN_OK;
  if (c->chem_mode == 1) return surrogate_source_step(c, dt, dev);
  ChemLaunch L;
  std::memset(&L, 0, sizeof(L));
  L.n = c->n;
  L.ld = c->ld;
  L.qf = c->qf[c->cur];
  L.qc = c->qc;
  L.hrr = c->hrr;
  L.dt = dt;
  L.rtol = c->rtol;
  L.atol = c->atol;
  L.strict_newton = c->strict;
  if (dev) {
    L.step_active = c->d_active;
    L.dt_dev = c->d_dt;
    L.cvel_out = c->src_on ? nullptr : c->d_cvel;  // with sources, their kernel publishes the speed
    L.time = c->d_time;
    L.nsteps = c->d_nsteps;
  }
  L.err = c->d_err;
  L.cost = c->d_cost;
  L.hot = c->d_hot;
  L.hlast = c->d_hlast;
  L.tchem = c->tchem;
  L.max_steps = c->chem_max_steps;
  L.precheck = c->precheck;
  if (c->listed && c->skip_uniform) {
    L.nrow = c->ne;
    L.run_flag = c->d_run_flag;
    L.heads = c->d_heads;
    L.head_count = c->d_head_count;
    L.run_last = c->d_run_last;
    L.run_head = c->d_run_head;
  }
  if (c->pk.ntube) {
    const Packed& k = c->pk;
    L.colmap = k.colmap;
    L.tube_of = k.tube_of;
    L.dt_tube = k.d_dt;
    L.active_tube = k.d_active;
    L.ntube = k.ntube;
    L.cvel_out = nullptr;
    L.time = nullptr;
    if (dev) {
      L.cvel_tube = c->src_on ? nullptr : k.d_cvel;  // with sources, their kernel publishes the speeds
      L.time_tube = k.d_time;
    }
  }
  ChemState& cs = c->use_sub ? c->chem_sub : c->chem;
  cudaError_t e = c->listed ? chem_launch_tube_listed(cs, L, c->d_list, c->d_list_count, c->d_cls, c->d_hist, c->stream)
                            : chem_launch_tube(cs, L, c->stream);
  if (e != cudaSuccess) return fail(c, EDYN_E_CUDA, "chemistry launch: %s", cudaGetErrorString(e));
  return EDYN_OK;
}

// solve_source with the surrogate in front of the implicit integrator
// (chem_mode 1), for the macks call of every tube cell (SRC/source.f90:58):
//  1. the chemistry launch in screen mode: f(y0) and the inert-cell test for
//     every cell; inert cells finish as in the plain path, the others are
//     packed (m rows);
//  2. the network's candidate y0 + dt f0 + correction (tcgen05 GEMMs on the
//     packed rows) and the explicit increment y0 + dt f0;
//  3. the FP64 gate on both (trapezoidal residual with f at the candidate,
//     element conservation), network first;
//  4. the rejected rows compacted and integrated by the implicit integrator;
//  5. every packed row finished (adjust_sum, HRR, qfToQc, QcToqf, speed).
// The host reads the packed and rejected counts to size the launches (two
// synchronisations per step).
int surrogate_source_step(Ctx* c, double dt, bool dev) {
  Surr& z = c->surr;
  if (!z.attached) return fail(c, EDYN_E_ARG, "chem_mode 1 needs a surrogate (edyn_set_surrogate)");
  ChemState& cs = c->use_sub ? c->chem_sub : c->chem;
  cudaStream_t st = c->stream;
  CK(cudaMemsetAsync(z.d_count, 0, 4 * sizeof(unsigned), st));
  ChemLaunch L;
  std::memset(&L, 0, sizeof(L));
  L.n = c->n;
  L.ld = c->ld;
  L.qf = c->qf[c->cur];
  L.qc = c->qc;
  L.hrr = c->hrr;
  L.dt = dt;
  L.rtol = c->rtol;
  L.atol = c->atol;
  L.strict_newton = c->strict;
  if (dev) {
    L.step_active = c->d_active;
    L.dt_dev = c->d_dt;
    L.cvel_out = c->d_cvel;
    L.time = c->d_time;
    L.nsteps = c->d_nsteps;
  } else {
    L.cvel_out = nullptr;
  }
  L.err = c->d_err;
  L.cost = c->d_cost;
  L.hlast = c->d_hlast;
  L.tchem = c->tchem;
  L.max_steps = c->chem_max_steps;
  L.precheck = c->precheck;
  L.screen = 1;
  if (c->skip_uniform) {
    // runs of identical cells: only their heads are screened and packed
    L.nrow = c->ne;
    L.run_flag = c->d_run_flag;
    L.heads = c->d_heads;
    L.head_count = c->d_head_count;
    L.run_last = c->d_run_last;
    L.run_head = c->d_run_head;
  }
  L.pk_count = z.d_count;
  L.pk_idx = z.pk_idx;
  L.pk_rho = z.pk_rho;
  L.pk_dt = z.pk_dt;
  L.pk_y0 = z.pk_y0;
  L.pk_f0 = z.pk_f0;
  cudaError_t e = chem_launch_screen_packed(cs, L, st);
  if (e != cudaSuccess) return fail(c, EDYN_E_CUDA, "chemistry screen launch: %s", cudaGetErrorString(e));
  unsigned cnt[4] = {0, 0, 0, 0};
  CK(cudaMemcpyAsync(cnt, z.d_count, sizeof(cnt), cudaMemcpyDeviceToHost, st));
  ChemCounters k0;
  e = chem_read_counters(cs, &k0, st);  // synchronises the stream
  if (e != cudaSuccess) return fail(c, EDYN_E_CUDA, "counters: %s", cudaGetErrorString(e));
  const int m = (int)cnt[0];
  for (double& v : z.stats) v = 0.0;
  z.stats[0] = m;
  z.stats[4] = (double)k0.rhs;
  if (m == 0) {
    e = chem_follow_packed(cs, L, st);
    if (e != cudaSuccess) return fail(c, EDYN_E_CUDA, "followers: %s", cudaGetErrorString(e));
    return EDYN_OK;
  }
  const int ns = z.nrow - 1;
  const int M = (m + 127) / 128 * 128;
  void* sv = (void*)st;
  const float* mu = z.norm;
  const float* isig = z.norm ? z.norm + 64 : nullptr;
  const float* omu = z.norm ? z.norm + 128 : nullptr;
  const float* osig = z.norm ? z.norm + 192 : nullptr;
  int rc = EDYN_OK;
  if (z.net) {
    rc |= edyn_mlp_features(m, ns, z.pk_rho, z.pk_dt, z.pk_y0, z.wmol, mu, isig, z.X, Surr::KIN, sv);
    rc |= edyn_mlp_tile(z.X, m, Surr::KIN, 128, z.Xt, sv);
    const void* A = z.Xt;
    int K = Surr::KIN;
    for (int l = 0; l < 3; ++l) {
      rc |= edyn_mlp_gemm_tiled(A, z.wt[l], M, Surr::HID, K, EDYN_MLP_EPI_GELU, z.b[l], nullptr, 0, z.H[l],
                                Surr::HID, 1, sv);
      A = z.H[l];
      K = Surr::HID;
    }
    rc |= edyn_mlp_gemm_tiled(A, z.wt[3], M, Surr::KOUT, Surr::HID, EDYN_MLP_EPI_F32, z.b[3], z.out, Surr::KOUT,
                              nullptr, 0, 0, sv);
    rc |= edyn_mlp_decode(m, ns, z.out, Surr::KOUT, omu, osig, z.pk_y0, z.pk_f0, z.pk_dt, z.yfloor, z.tfloor, z.pk_y1,
                          sv);
  }
  // the explicit increment: the decode of a zero network output
  double* expl = z.net ? z.pk_ya : z.pk_y1;
  rc |= edyn_mlp_decode(m, ns, z.zero_out, Surr::KOUT, z.zero_one, z.zero_one + 64, z.pk_y0, z.pk_f0, z.pk_dt,
                        z.yfloor, z.tfloor, expl, sv);
  if (rc) return fail(c, EDYN_E_CUDA | rc, "surrogate network launch failed");
  e = chem_rhs_batch(cs, m, z.pk_rho, z.pk_y1, z.pk_f1, st);
  if (e == cudaSuccess && z.net) e = chem_rhs_batch(cs, m, z.pk_rho, z.pk_ya, z.pk_fa, st);
  if (e != cudaSuccess) return fail(c, EDYN_E_CUDA, "gate right-hand sides: %s", cudaGetErrorString(e));
  rc |= edyn_mlp_gate(m, ns, z.ne, z.pk_y0, z.pk_y1, z.pk_f0, z.pk_f1, z.net ? z.pk_ya : nullptr,
                      z.net ? z.pk_fa : nullptr, z.pk_dt, z.wmol, z.elem, z.rtol, z.atol, z.etol, z.accept,
                      z.d_count + 1, sv);
  rc |= edyn_mlp_compact(m, ns, z.accept, z.pk_rho, z.pk_dt, z.pk_y0, z.rj_idx, z.rj_rho, z.rj_dt, z.rj_y, z.d_nrej,
                         sv);
  if (rc) return fail(c, EDYN_E_CUDA | rc, "surrogate gate launch failed");
  rc = edyn_mlp_status(sv);  // synchronises; reports a GEMM wait that ran out
  if (rc) return fail(c, rc, "surrogate network: a tensor-core kernel's wait ran out");
  int nrej = 0;
  CK(cudaMemcpyAsync(&nrej, z.d_nrej, sizeof(int), cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(cnt, z.d_count, sizeof(cnt), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  z.stats[1] = z.net ? cnt[1] : 0;
  z.stats[2] = z.net ? cnt[2] : cnt[1];
  z.stats[3] = nrej;
  z.stats[5] = z.net ? 2.0 * m : m;
  if (nrej > 0) {
    ChemLaunch B;
    std::memset(&B, 0, sizeof(B));
    B.n = nrej;
    B.rtol = c->rtol;
    B.atol = c->atol;
    B.rho_batch = z.rj_rho;
    B.dt_batch = z.rj_dt;
    B.yiT_batch = z.rj_y;
    B.err = c->d_err;
    B.max_steps = c->chem_max_steps;
    e = chem_launch_batch(cs, B, st);
    if (e != cudaSuccess) return fail(c, EDYN_E_CUDA, "fallback launch: %s", cudaGetErrorString(e));
    rc = edyn_mlp_scatter(nrej, ns, z.rj_idx, z.rj_y, z.pk_y1, sv);
    if (rc) return fail(c, rc, "fallback scatter failed");
    ChemCounters k1;
    e = chem_read_counters(cs, &k1, st);
    if (e != cudaSuccess) return fail(c, EDYN_E_CUDA, "counters: %s", cudaGetErrorString(e));
    z.stats[6] = (double)k1.rhs;
  }
  e = chem_finish_packed(cs, L, m, z.pk_y1, st);
  if (e != cudaSuccess) return fail(c, EDYN_E_CUDA, "packed finish launch: %s", cudaGetErrorString(e));
  e = chem_follow_packed(cs, L, st);
  if (e != cudaSuccess) return fail(c, EDYN_E_CUDA, "followers: %s", cudaGetErrorString(e));
  return EDYN_OK;
}

void drop_graph(Ctx* c);

// The element subset of the mechanism: kept species (renumbered; smap gives
// each one's index in m), and the reactions whose species and named collider
// are all kept, with third-body efficiencies of dropped species removed
// (their concentrations are zero).
void mech_subset(const edyn_mech& m, const std::vector<char>& keep, edyn_mech& o, std::vector<int>& smap) {
  o = m;
  std::vector<int> nid(m.nspec, -1);
  smap.clear();
  int ns = 0;
  for (int k = 0; k < m.nspec; ++k) {
    if (!keep[k]) continue;
    nid[k] = ns;
    smap.push_back(k);
    std::memcpy(o.spec_name[ns], m.spec_name[k], sizeof(o.spec_name[ns]));
    o.W[ns] = m.W[k];
    o.T_lo[ns] = m.T_lo[k];
    o.T_mid[ns] = m.T_mid[k];
    o.T_hi[ns] = m.T_hi[k];
    std::memcpy(o.a[ns], m.a[k], sizeof(o.a[ns]));
    std::memcpy(o.elem_count[ns], m.elem_count[k], sizeof(o.elem_count[ns]));
    ++ns;
  }
  o.nspec = ns;
  int nr = 0;
  for (int i = 0; i < m.nreac; ++i) {
    bool ok = true;
    for (int sl = 0; sl < 6; ++sl)
      if (m.nunk[i][sl] >= 0 && nid[m.nunk[i][sl]] < 0) ok = false;
    if (m.kfal[i] >= 0 && nid[m.kfal[i]] < 0) ok = false;
    if (!ok) continue;
    std::memcpy(o.equation[nr], m.equation[i], sizeof(o.equation[nr]));
    o.rev[nr] = m.rev[i];
    for (int sl = 0; sl < 6; ++sl) {
      o.nu[nr][sl] = m.nu[i][sl];
      o.nunk[nr][sl] = m.nunk[i][sl] >= 0 ? nid[m.nunk[i][sl]] : -1;
    }
    o.A[nr] = m.A[i];
    o.beta[nr] = m.beta[i];
    o.E_R[nr] = m.E_R[i];
    o.tb[nr] = m.tb[i];
    o.kfal[nr] = m.kfal[i] >= 0 ? nid[m.kfal[i]] : -1;
    o.ifop[nr] = m.ifop[i];
    std::memcpy(o.low[nr], m.low[i], sizeof(o.low[nr]));
    std::memcpy(o.troe[nr], m.troe[i], sizeof(o.troe[nr]));
    o.dup[nr] = m.dup[i];
    int ne = 0;
    for (int z = 0; z < m.neff[i]; ++z) {
      if (nid[m.eff_sp[i][z]] < 0) continue;
      o.eff_sp[nr][ne] = nid[m.eff_sp[i][z]];
      o.eff_val[nr][ne] = m.eff_val[i][z];
      ++ne;
    }
    o.neff[nr] = ne;
    ++nr;
  }
  o.nreac = nr;
}

// Picks the chemistry tables for the species present in the tube state
// (present[k]: nonzero somewhere) and at the inlet.
int select_chem_set(Ctx* c, const std::vector<char>& present) {
  const edyn_mech& m = c->mech;
  std::vector<char> el(m.nelem, 0);
  for (int k = 0; k < m.nspec; ++k) {
    const bool here = present[k] || (c->lbound == 1 && c->bc.y_in[k] > 0.0);
    if (!here) continue;
    for (int e = 0; e < m.nelem; ++e)
      if (m.elem_count[k][e] > 0) el[e] = 1;
  }
  std::vector<char> keep(m.nspec, 1);
  int nk = 0;
  for (int k = 0; k < m.nspec; ++k) {
    for (int e = 0; e < m.nelem; ++e)
      if (m.elem_count[k][e] > 0 && !el[e]) keep[k] = 0;
    nk += keep[k];
  }
  const bool want = c->do_reaction && nk < m.nspec && nk > 0;
  if (!want) {
    if (c->use_sub) drop_graph(c);
    c->use_sub = false;
    return EDYN_OK;
  }
  if (keep == c->sub_keep && c->chem_sub.d_tables) {
    if (!c->use_sub) drop_graph(c);
    c->use_sub = true;
    return EDYN_OK;
  }
  std::unique_ptr<edyn_mech> sub(new (std::nothrow) edyn_mech);
  if (!sub) return fail(c, EDYN_E_ARG, "out of host memory for the mechanism subset");
  std::vector<int> smap;
  mech_subset(m, keep, *sub, smap);
  if (sub->nreac < 1) {  // nothing reacts: the full tables do no harm
    if (c->use_sub) drop_graph(c);
    c->use_sub = false;
    return EDYN_OK;
  }
  CK(cudaStreamSynchronize(c->stream));
  drop_graph(c);
  if (c->chem_sub.d_tables) chem_free(c->chem_sub);
  c->chem_sub = ChemState();
  c->sub_keep.clear();
  c->use_sub = false;
  const int rc = chem_init(c->chem_sub, *sub, c->tb, c->stream, smap.data(), m.nspec + 1);
  if (rc) return fail(c, EDYN_E_CUDA, "chemistry tables of the species subset: %s", cudaGetErrorString((cudaError_t)rc));
  c->sub_keep = keep;
  c->use_sub = true;
  return EDYN_OK;
}

// After the state was set from outside: which species occur, then the tables.
int refresh_chem_set(Ctx* c) {
  if (!c->do_reaction) return EDYN_OK;
  // every column between the outermost ghosts (ghost columns hold zeros)
  CK(launch_species_present(c->qc, c->ld, c->ld - 2 * GHOST, c->ns, c->d_present, c->stream));
  std::vector<int> fl(c->ns, 1);
  CK(cudaMemcpyAsync(fl.data(), c->d_present, (size_t)c->ns * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  std::vector<char> present(c->ns);
  for (int k = 0; k < c->ns; ++k) present[k] = fl[k] != 0;
  return select_chem_set(c, present);
}

int ensure_staging(Ctx* c, size_t bytes) {
  if (c->staging_bytes >= bytes) return EDYN_OK;
  if (c->staging) cudaFree(c->staging);
  c->staging = nullptr;
  c->staging_bytes = 0;
  CK(cudaMalloc(&c->staging, bytes));
  c->staging_bytes = bytes;
  return EDYN_OK;
}

void drop_graph(Ctx* c) {
  if (c->graph) cudaGraphExecDestroy(c->graph);
  c->graph = nullptr;
  c->graph_steps = 0;
}

// Evaluates HRR_dot of the last source step into c->hrr_dot while the
// primitive state is still the one that step left.
int eval_hrr_dot(Ctx* c) {
  if (c->hrr_dot_state != 1 && c->hrr_dot_state != 3) return EDYN_OK;
  const double* rows = c->hrr_dot_state == 3 ? c->hrr_dot_rows : c->qf[c->cur];
  cudaError_t e = chem_hrr_dot(c->use_sub ? c->chem_sub : c->chem, c->n, c->ld, rows, c->tchem, c->hrr_dot,
                               c->pk.colmap, c->stream);
  if (e != cudaSuccess) return fail(c, EDYN_E_CUDA, "HRR_dot launch: %s", cudaGetErrorString(e));
  c->hrr_dot_state = 2;
  return EDYN_OK;
}

// Before a fluid step changes the state the last source step left: keep the
// primitive rows HRR_dot needs (the reference's eos_obj%HRR_dot outlives
// the next fluid step), one device-to-device copy of the rows instead of a
// right-hand side per cell; HRR_dot itself is still evaluated only when it
// is downloaded.
int keep_hrr_dot(Ctx* c) {
  if (c->hrr_dot_state != 1) return EDYN_OK;
  const size_t bytes = (size_t)c->ne * c->ld * sizeof(double);
  if (!c->hrr_dot_rows) CK(cudaMalloc(&c->hrr_dot_rows, bytes));
  CK(cudaMemcpyAsync(c->hrr_dot_rows, c->qf[c->cur], bytes, cudaMemcpyDeviceToDevice, c->stream));
  c->hrr_dot_state = 3;
  return EDYN_OK;
}


// Cell centres and sizes of the output's x_m and dx rows: (i + 1/2) dx for
// one tube (the reference accumulates them, SRC/block.f90:264-304, which can
// differ in the last bits; its restart compares them within 1e-7); SMR
// segments follow each other from x = 0.
int cell_geometry(Ctx* c) {
  if (c->pk.ntube && !c->pk.smr)
    return fail(c, EDYN_E_ARG, "output and restart take one tube or one SMR domain per context, not packed tubes");
  const size_t n = (size_t)c->n;
  c->xm.assign(2 * n, 0.0);
  if (!c->pk.ntube) {
    for (size_t i = 0; i < n; ++i) {
      c->xm[i] = ((double)i + 0.5) * c->dx;
      c->xm[n + i] = c->dx;
    }
  } else {
    // SMR segments, each from its left edge (smr_geometry)
    size_t i = 0;
    for (int t = 0; t < c->pk.ntube; ++t) {
      const double d = c->pk.dx[t], x0 = c->pk.x0[t];
      for (int j = 0; j < c->pk.n[t]; ++j, ++i) {
        c->xm[i] = x0 + ((double)j + 0.5) * d;
        c->xm[n + i] = d;
      }
    }
  }
  return EDYN_OK;
}

// SMR: the segments' left edges, x = 0 where the left SMR zone (the leading
// segments whose cells differ from dx_comp) ends (SRC/block.f90:236-237,
// 296-304), and every cell's centre and size on the device (the energy
// sources' positions, the output's x_m and dx); spherical geometry takes
// r = x_m.
int smr_geometry(Ctx* c) {
  Packed& k = c->pk;
  k.x0.assign(k.ntube, 0.0);
  double x = 0.0;
  for (int t = 0; t < k.ntube && k.dx[t] != k.dx_comp; ++t) x -= k.n[t] * k.dx[t];
  for (int t = 0; t < k.ntube; ++t) {
    k.x0[t] = x;
    x += k.n[t] * k.dx[t];
  }
  if (!k.d_x0) CK(cudaMalloc(&k.d_x0, k.ntube * sizeof(double)));
  CK(cudaMemcpy(k.d_x0, k.x0.data(), k.ntube * sizeof(double), cudaMemcpyHostToDevice));
  int rc = cell_geometry(c);
  if (rc) return rc;
  if (!c->d_xm) CK(cudaMalloc(&c->d_xm, c->xm.size() * sizeof(double)));
  CK(cudaMemcpy(c->d_xm, c->xm.data(), c->xm.size() * sizeof(double), cudaMemcpyHostToDevice));
  return EDYN_OK;
}

// set_eos_params + the rows of write_hdf5_b on the device, then their copy
// to pinned host memory on the output stream: the context's stream goes on
// with the next steps while the copy drains.
int output_snapshot(Ctx* c) {
  if (c->out_pending) return fail(c, EDYN_E_ARG, "a snapshot is pending: write it (edyn_output_write) first");
  const size_t n = (size_t)c->n, nrow = (size_t)(EDYN_OUT_FIXED + c->ns);
  if (!c->d_out) {
    int rc = cell_geometry(c);
    if (rc) return rc;
    CK(cudaMalloc(&c->d_out, nrow * n * sizeof(double)));
    CK(cudaMallocHost(&c->h_out, nrow * n * sizeof(double)));
    if (!c->d_xm) CK(cudaMalloc(&c->d_xm, 2 * n * sizeof(double)));
    CK(cudaMemcpy(c->d_xm, c->xm.data(), 2 * n * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaStreamCreateWithFlags(&c->out_stream, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&c->out_ready, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&c->out_copied, cudaEventDisableTiming));
  }
  int rc = eval_hrr_dot(c);
  if (rc) return rc;
  OutputArgs a{};
  a.n = c->n;
  a.ld = c->ld;
  a.ns = c->ns;
  a.qf = c->qf[c->cur];
  a.qc = c->qc;
  a.colmap = c->pk.ntube ? c->pk.colmap : nullptr;
  a.hrr = c->hrr;
  a.hrr_dot = c->hrr_dot_state == 2 ? c->hrr_dot : nullptr;
  a.q_rad = c->d_srcq;
  a.q_tw = c->d_srcq + c->n;
  a.xm = c->d_xm;
  a.wall = c->src.wall;
  a.tw_min = c->src.tw_min;
  a.tw_max = c->src.tw_max;
  a.alpha = c->src.alpha;
  a.beta = c->src.beta;
  a.out = c->d_out;
  // the previous snapshot's copy has left d_out before the rows are rewritten
  CK(cudaStreamWaitEvent(c->stream, c->out_copied, 0));
  CK(launch_output_rows(a, c->stream));
  CK(cudaEventRecord(c->out_ready, c->stream));
  CK(cudaStreamWaitEvent(c->out_stream, c->out_ready, 0));
  CK(cudaMemcpyAsync(c->h_out, c->d_out, nrow * n * sizeof(double), cudaMemcpyDeviceToHost, c->out_stream));
  CK(cudaEventRecord(c->out_copied, c->out_stream));
  c->out_pending = true;
  return EDYN_OK;
}

// waits for the pending snapshot (taking one first when none is queued)
int output_rows_ready(Ctx* c) {
  if (!c->out_pending) {
    int rc = output_snapshot(c);
    if (rc) return rc;
  }
  CK(cudaEventSynchronize(c->out_copied));
  c->out_pending = false;
  return EDYN_OK;
}

// dataset names of write_hdf5_b: the fifteen fields (Fortran's trim keeps
// their leading blanks), then the species names
std::vector<std::string> output_names(const Ctx* c) {
  std::vector<std::string> v = {"rho", "u_x", "  T", "  p", " et", " ek", " ei", "HRR",
                                "HRD", "Qrd", " Tw", "QTw", "x_m", " dx", "idx"};
  for (int k = 0; k < c->ns; ++k) v.push_back(c->mech.spec_name[k]);
  return v;
}

}  // namespace

extern "C" {

const char* edyn_version(void) { return "edyn-gb300 0.1 (sm_103a)"; }

int edyn_mech_compile(const char* chem_dir, const char* out_path, char* err, int errlen) {
  edyn_mech* m = new (std::nothrow) edyn_mech;
  if (!m) return EDYN_E_ARG;
  int rc = edyn_mech_load_dir(chem_dir, m, err, errlen);
  if (rc == 0 && edyn_mech_write(m, out_path) != 0) {
    if (err && errlen > 0) std::snprintf(err, (size_t)errlen, "cannot write %s", out_path);
    rc = 1;
  }
  delete m;
  return rc ? EDYN_E_MECH : EDYN_OK;
}

int edyn_tran_compile(const char* chem_dir, const char* out_path, char* err, int errlen) {
  std::unique_ptr<edyn_mech> m(new (std::nothrow) edyn_mech);
  std::unique_ptr<edyn_tran> t(new (std::nothrow) edyn_tran);
  if (!m || !t) return EDYN_E_ARG;
  if (edyn_mech_load_dir(chem_dir, m.get(), err, errlen) != 0) return EDYN_E_MECH;
  if (edyn_tran_load_dir(chem_dir, t.get(), err, errlen) != 0) return EDYN_E_MECH;
  if (t->kk != m->nspec) {
    if (err && errlen > 0) std::snprintf(err, (size_t)errlen, "transport fits for %d species, mechanism has %d", t->kk, m->nspec);
    return EDYN_E_MECH;
  }
  if (edyn_tran_write(t.get(), m.get(), out_path) != 0) {
    if (err && errlen > 0) std::snprintf(err, (size_t)errlen, "cannot write %s", out_path);
    return EDYN_E_MECH;
  }
  return EDYN_OK;
}

namespace {
// Transport set-up of edyn_init: loads the fits next to the mechanism,
// checks them against it and builds the device tables of TranDev.
int load_tran_tables(Ctx* c) {
  if (c->d_tran) return EDYN_OK;
  const char* chem_dir = c->chem_dir.c_str();
  std::unique_ptr<edyn_tran> t(new (std::nothrow) edyn_tran);
  if (!t) return fail(c, EDYN_E_ARG, "out of host memory");
  char err[512] = {0};
  if (edyn_tran_load_dir(chem_dir, t.get(), err, sizeof(err)) != 0) return fail(c, EDYN_E_MECH, "transport: %s", err);
  const int ns = c->ns;
  if (t->kk != ns) return fail(c, EDYN_E_MECH, "transport fits for %d species, mechanism has %d", t->kk, ns);
  for (int k = 0; k < ns; ++k)
    if (!(std::fabs(t->wt[k] - c->mech.W[k]) <= 1e-6 * c->mech.W[k]))
      return fail(c, EDYN_E_MECH, "transport fits: molecular weight of species %d differs from the mechanism's", k);
  const int npair = ns * (ns - 1) / 2;
  std::vector<double> h;
  auto put = [&](size_t n) {
    size_t o = h.size();
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
  CK(cudaMalloc(&c->d_tran, h.size() * sizeof(double)));
  CK(cudaMemcpy(c->d_tran, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice));
  TranDev& d = c->trd;
  d.eta = c->d_tran + o_eta;
  d.lam = c->d_tran + o_lam;
  d.dif = c->d_tran + o_dif;
  d.wa = c->d_tran + o_wa;
  d.wb = c->d_tran + o_wb;
  d.wc = c->d_tran + o_wc;
  d.W = c->d_tran + o_w;
  d.e2 = c->d_tran + o_e2;
  d.lg = c->d_tran + o_lg;
  d.patmos = t->patmos;
  return EDYN_OK;
}

// do_tran: the fits plus the property and face-flux buffers of the stages
int init_transport(Ctx* c) {
  int rc = load_tran_tables(c);
  if (rc) return rc;
  const size_t ld = (size_t)c->ld;
  const size_t prow = (size_t)(TRAN_ROWS_FIXED + 2 * c->ns);
  CK(cudaMalloc(&c->d_tp, prow * ld * sizeof(double)));
  CK(cudaMalloc(&c->d_tflux, (size_t)c->ne * ld * sizeof(double)));
  CK(cudaMemset(c->d_tp, 0, prow * ld * sizeof(double)));
  CK(cudaMemset(c->d_tflux, 0, (size_t)c->ne * ld * sizeof(double)));
  c->trd.tp = c->d_tp;
  c->trd.flux = c->d_tflux;
  return EDYN_OK;
}
}  // namespace

int edyn_init(const char* chem_dir, int nspe, int nequ, int ncell, int lvir, const int* iflags, int n_iflags,
              const double* rparams, int n_rparams, const double* x_in, void** out) {
  if (!out) return EDYN_E_ARG;
  *out = nullptr;
  Ctx* c = new (std::nothrow) Ctx;
  if (!c) return EDYN_E_ARG;
  char err[512] = {0};
  if (edyn_mech_load_dir(chem_dir, &c->mech, err, sizeof(err)) != 0) {
    int rc = fail(c, EDYN_E_MECH, "mechanism: %s", err);
    *out = c;
    return rc;
  }
  *out = c;
  const edyn_mech& m = c->mech;
  if (nspe != m.nspec || nequ != nspe + 3)
    return fail(c, EDYN_E_ARG, "nspe/nequ (%d/%d) do not match the mechanism (%d species)", nspe, nequ, m.nspec);
  if (m.nspec > EDYN_NS_MAX) return fail(c, EDYN_E_ARG, "too many species (%d > %d)", m.nspec, EDYN_NS_MAX);
  if (!iflags || n_iflags < 8 || !rparams || n_rparams < 1) return fail(c, EDYN_E_ARG, "iflags/rparams too short");
  auto fl = [&](int i, int d) { return i < n_iflags ? iflags[i] : d; };
  auto rp = [&](int i, double d) { return i < n_rparams ? rparams[i] : d; };
  c->select_time = fl(EDYN_IF_SELECT_TIME, 1);
  c->riemann = fl(EDYN_IF_SELECT_RIEMANN, 2);
  c->flag_acu = fl(EDYN_IF_FLAG_ACU, 1);
  c->flag_muscl = fl(EDYN_IF_FLAG_MUSCL, 2);
  c->flag_weno = fl(EDYN_IF_FLAG_WENO, 0);
  c->lbound = fl(EDYN_IF_FLAG_LBOUND, 0);
  c->rbound = fl(EDYN_IF_FLAG_RBOUND, 0);
  c->do_reaction = fl(EDYN_IF_DO_REACTION, 0);
  c->strict = fl(EDYN_IF_STRICT_NEWTON, 1);
  c->chem_mode = fl(EDYN_IF_CHEM_MODE, 0);
  c->do_tran = fl(EDYN_IF_DO_TRAN, 0);
  c->spherical = fl(EDYN_IF_IS_SPHERICAL, 0);
  c->dx = rp(EDYN_RP_DX, 0.0);
  c->p_out = rp(EDYN_RP_P_OUT, 101325.0);
  c->t_in = rp(EDYN_RP_T_IN, 300.0);
  c->rho_u_in = rp(EDYN_RP_RHO_U_IN, 0.0);
  c->rtol = rp(EDYN_RP_RTOL, 1e-5);
  c->atol = rp(EDYN_RP_ATOL, 1e-13);
  if (c->chem_mode != 0 && c->chem_mode != 1)
    return fail(c, EDYN_E_ARG, "chem_mode=%d: 0 (implicit integrator) or 1 (surrogate with fallback)", c->chem_mode);
  if (c->do_tran != 0 && c->do_tran != 1) return fail(c, EDYN_E_ARG, "do_tran=%d must be 0 or 1", c->do_tran);
  if (c->spherical != 0 && c->spherical != 1) return fail(c, EDYN_E_ARG, "is_spherical=%d must be 0 or 1", c->spherical);
  if (c->spherical && (c->select_time == 2 || c->flag_acu == 2))
    return fail(c, EDYN_E_ARG, "spherical geometry takes Euler or TVDRK3 with first order or MUSCL");
  if (c->select_time < 0 || c->select_time > 2)
    return fail(c, EDYN_E_ARG, "select_time=%d not in 0..2 (Euler, TVDRK3, RK4)", c->select_time);
  if (c->riemann < 0 || c->riemann > 2) return fail(c, EDYN_E_ARG, "select_riemann=%d not in 0..2", c->riemann);
  if (c->flag_acu == 0) c->acu = ACU_FIRST;
  else if (c->flag_acu == 1) {
    c->acu = ACU_MUSCL;
    if (c->flag_muscl < 1 || c->flag_muscl > 4) return fail(c, EDYN_E_ARG, "flag_muscl=%d not in 1..4", c->flag_muscl);
    c->lim = c->flag_muscl;
  } else if (c->flag_acu == 2) {
    if (c->flag_weno == 1) c->acu = ACU_WENO3;
    else if (c->flag_weno == 2 || c->flag_weno == 3) {
      c->acu = ACU_WENO5;
      c->wflag = c->flag_weno;
    } else if (c->flag_weno == 4) c->acu = ACU_WENO7;
    else return fail(c, EDYN_E_ARG, "flag_weno=%d not in 1..4", c->flag_weno);
  } else {
    return fail(c, EDYN_E_ARG, "flag_acu=%d not in 0..2", c->flag_acu);
  }
  if (lvir != acu_lvir(c->acu))
    return fail(c, EDYN_E_ARG, "lvir=%d does not match the scheme (needs %d)", lvir, acu_lvir(c->acu));
  if (c->lbound < 0 || c->lbound > 1 || c->rbound < 0 || c->rbound > 1)
    return fail(c, EDYN_E_ARG, "boundary flags must be 0 or 1");
  if (ncell < 16) return fail(c, EDYN_E_ARG, "ncell=%d too small (>= 16)", ncell);
  if (!(c->dx > 0)) return fail(c, EDYN_E_ARG, "dx must be positive");
  c->ns = nspe;
  c->ne = nequ;
  c->n = ncell;
  c->lvir = lvir;
  c->ld = ncell + 2 * GHOST;
  build_thermo_table(m, c->tb);
  std::memset(&c->bc, 0, sizeof(c->bc));
  c->bc.rho_u_in = c->rho_u_in;
  c->bc.t_in = c->t_in;
  if (x_in) {
    double wsum = 0.0;
    for (int k = 0; k < nspe; ++k) wsum += x_in[k] * m.W[k];
    for (int k = 0; k < nspe; ++k) c->bc.y_in[k] = x_in[k] * m.W[k] / wsum;
    c->bc.e_in = host_specific_energy(m, c->t_in, x_in);
  }
  CK(cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking));
  c->stream = c->own;
  const size_t rows = (size_t)nequ * c->ld;
  CK(cudaMalloc(&c->qf[0], rows * sizeof(double)));
  CK(cudaMalloc(&c->qf[1], rows * sizeof(double)));
  CK(cudaMalloc(&c->qc, rows * sizeof(double)));
  CK(cudaMalloc(&c->q0, rows * sizeof(double)));
  if (c->select_time == 2) {
    CK(cudaMalloc(&c->acc, rows * sizeof(double)));
    CK(cudaMemsetAsync(c->acc, 0, rows * sizeof(double), c->stream));
  }
  CK(cudaMalloc(&c->hrr, (size_t)ncell * sizeof(double)));
  CK(cudaMalloc(&c->d_srcq, 2 * (size_t)ncell * sizeof(double)));
  CK(cudaMemsetAsync(c->d_srcq, 0, 2 * (size_t)ncell * sizeof(double), c->stream));
  CK(cudaMalloc(&c->hrr_dot, (size_t)ncell * sizeof(double)));
  CK(cudaMalloc(&c->tchem, (size_t)ncell * sizeof(double)));
  CK(cudaMemsetAsync(c->qf[0], 0, rows * sizeof(double), c->stream));
  CK(cudaMemsetAsync(c->qf[1], 0, rows * sizeof(double), c->stream));
  CK(cudaMemsetAsync(c->qc, 0, rows * sizeof(double), c->stream));
  CK(cudaMemsetAsync(c->q0, 0, rows * sizeof(double), c->stream));
  CK(cudaMemsetAsync(c->hrr, 0, (size_t)ncell * sizeof(double), c->stream));
  CK(cudaMemsetAsync(c->hrr_dot, 0, (size_t)ncell * sizeof(double), c->stream));
  CK(cudaMemsetAsync(c->tchem, 0, (size_t)ncell * sizeof(double), c->stream));
  CK(cudaMalloc(&c->d_time, sizeof(double)));
  CK(cudaMalloc(&c->d_nsteps, sizeof(long long)));
  CK(cudaMalloc(&c->d_max_steps, sizeof(long long)));
  CK(cudaMalloc(&c->d_active, sizeof(int)));
  CK(cudaMalloc(&c->d_dt, sizeof(double)));
  CK(cudaMalloc(&c->d_cvel, sizeof(unsigned long long)));
  CK(cudaMalloc(&c->d_err, sizeof(unsigned)));
  CK(cudaMemsetAsync(c->d_err, 0, sizeof(unsigned), c->stream));
  CK(cudaMalloc(&c->d_cost, (size_t)ncell * sizeof(int)));
  CK(cudaMalloc(&c->d_hot, (HOT_MAX + 1) * sizeof(unsigned)));
  CK(cudaMemsetAsync(c->d_cost, 0, (size_t)ncell * sizeof(int), c->stream));
  CK(cudaMemsetAsync(c->d_hot, 0, (HOT_MAX + 1) * sizeof(unsigned), c->stream));
  CK(cudaMalloc(&c->d_hlast, (size_t)ncell * sizeof(double)));
  CK(cudaMalloc(&c->d_list, (size_t)ncell * sizeof(int)));
  CK(cudaMalloc(&c->d_list_count, sizeof(unsigned)));
  CK(cudaMalloc(&c->d_cls, (size_t)ncell));
  CK(cudaMalloc(&c->d_hist, 64 * sizeof(unsigned)));
  CK(cudaMalloc(&c->d_run_flag, (size_t)ncell));
  CK(cudaMalloc(&c->d_heads, (size_t)ncell * sizeof(int)));
  CK(cudaMalloc(&c->d_head_count, sizeof(unsigned)));
  CK(cudaMalloc(&c->d_run_last, (size_t)((ncell + CHEM_RUN_BLOCK - 1) / CHEM_RUN_BLOCK) * sizeof(int)));
  CK(cudaMalloc(&c->d_run_head, (size_t)ncell * sizeof(int)));
  // From CHEM_TWO_PASS_CELLS on, the two-pass chemistry: the screening pass
  // over the heads of the runs of identical cells, then the integrator over
  // the listed cells; short tubes are bound by their costliest cell, which a
  // second launch would only delay.
  c->listed = ncell >= CHEM_TWO_PASS_CELLS;
  CK(cudaMalloc(&c->d_present, 64 * sizeof(int)));
  CK(cudaMemsetAsync(c->d_hlast, 0, (size_t)ncell * sizeof(double), c->stream));
  int rc = fluid_upload_tables(c->tb, c->stream);
  if (rc == -1) return fail(c, EDYN_E_MECH, "a different mechanism is already loaded in this process");
  if (rc) return fail(c, EDYN_E_CUDA, "constant tables: %s", cudaGetErrorString((cudaError_t)rc));
  rc = chem_init(c->chem, m, c->tb, c->stream);
  if (rc) return fail(c, EDYN_E_CUDA, "chemistry tables: %s", cudaGetErrorString((cudaError_t)rc));
  CK(stage_tiling(c->acu, c->lim, c->wflag, c->riemann, c->ns, c->n, &c->stage_tc, c->spherical));
  c->chem_dir = chem_dir ? chem_dir : ".";
  if (c->do_tran) {
    rc = init_transport(c);
    if (rc) return rc;
  }
  CK(cudaStreamSynchronize(c->stream));
  return EDYN_OK;
}

namespace {
// Stage tiles of packed tubes: each tube split into tiles of tc cells with
// the single-tube rule for its last tile, all tubes' tiles in one table.
int build_tiles(Ctx* c) {
  Packed& k = c->pk;
  std::vector<int4> tl;
  for (int t = 0; t < k.ntube; ++t) {
    const int nb = (k.n[t] + c->stage_tc - 1) / c->stage_tc;
    for (int j = 0; j < nb; ++j) tl.push_back(make_int4(t, j, nb, 0));
  }
  if (k.d_tiles) cudaFree(k.d_tiles);
  k.d_tiles = nullptr;
  CK(cudaMalloc(&k.d_tiles, tl.size() * sizeof(int4)));
  CK(cudaMemcpy(k.d_tiles, tl.data(), tl.size() * sizeof(int4), cudaMemcpyHostToDevice));
  k.ntiles = (int)tl.size();
  return EDYN_OK;
}
}  // namespace

namespace {
// edyn_init_tubes, and edyn_init_blocks (smr): segments of one domain, the
// inflow boundary allowed on the first (x_in), one dt for all.
int init_packed(const char* chem_dir, int nspe, int nequ, int ntube, const int* ncell, int lvir, const int* iflags,
                int n_iflags, const double* rparams, int n_rparams, const double* x_in, bool smr, void** out) {
  if (!out) return EDYN_E_ARG;
  *out = nullptr;
  if (ntube < 1 || !ncell || !rparams || n_rparams < 2 || !iflags || n_iflags < 8) return EDYN_E_ARG;
  long long ntot = 0, cols = 0;
  for (int t = 0; t < ntube; ++t) {
    // SMR segments: down to the reference's blocks (10 cells) -- a segment
    // feeds its neighbour's ghosts from 2 lvir cells; independent tubes >= 16
    if (ncell[t] < (smr ? std::max(8, 2 * lvir) : 16)) return EDYN_E_ARG;
    ntot += ncell[t];
    cols += ncell[t] + 2 * GHOST;
  }
  if (cols > (1ll << 31) - 1) return EDYN_E_ARG;
  if (!smr && n_iflags > EDYN_IF_FLAG_LBOUND && iflags[EDYN_IF_FLAG_LBOUND] != 0) {
    // the inflow boundary needs per-tube inlet data
    int rc = edyn_init(chem_dir, nspe, nequ, 16, lvir, iflags, n_iflags, rparams, n_rparams, nullptr, out);
    if (rc == EDYN_OK) rc = fail((Ctx*)*out, EDYN_E_ARG, "packed tubes take wall or outlet boundaries only");
    return rc ? rc : EDYN_E_ARG;
  }
  if (n_iflags > EDYN_IF_CHEM_MODE && iflags[EDYN_IF_CHEM_MODE] != 0) {
    int rc = edyn_init(chem_dir, nspe, nequ, 16, lvir, iflags, n_iflags, rparams, n_rparams, nullptr, out);
    if (rc == EDYN_OK) rc = fail((Ctx*)*out, EDYN_E_ARG, "packed tubes take the plain chemistry (chem_mode 0)");
    return rc ? rc : EDYN_E_ARG;
  }
  if (!smr && n_iflags > EDYN_IF_IS_SPHERICAL && iflags[EDYN_IF_IS_SPHERICAL] != 0) {
    int rc = edyn_init(chem_dir, nspe, nequ, 16, lvir, iflags, n_iflags, rparams, n_rparams, nullptr, out);
    if (rc == EDYN_OK)
      rc = fail((Ctx*)*out, EDYN_E_ARG, "independent packed tubes are Cartesian (is_spherical 0; SMR domains take it)");
    return rc ? rc : EDYN_E_ARG;
  }
  if (n_iflags > EDYN_IF_DO_TRAN && iflags[EDYN_IF_DO_TRAN] != 0) {
    // The per-column transport kernels reproduce each tube's properties,
    // but two or more tubes stepped with transport lose their right-end
    // cells on the GPU; until that is found, transport takes one tube.
    int rc = edyn_init(chem_dir, nspe, nequ, 16, lvir, iflags, n_iflags, rparams, n_rparams, nullptr, out);
    if (rc == EDYN_OK)
      rc = fail((Ctx*)*out, EDYN_E_ARG, "transport (do_tran 1) takes one tube per context, not packed tubes or SMR");
    return rc ? rc : EDYN_E_ARG;
  }
  // One context whose rows hold every tube's block: its row length is the
  // sum of the blocks, its cell count the sum of the cells.
  int rc = edyn_init(chem_dir, nspe, nequ, (int)(cols - 2 * GHOST), lvir, iflags, n_iflags, rparams, n_rparams,
                     smr ? x_in : nullptr, out);
  if (rc) return rc;
  Ctx* c = (Ctx*)*out;
  Packed& k = c->pk;
  k.ntube = ntube;
  k.smr = smr;
  long long off = 0, first = 0;
  std::vector<int> colmap((size_t)ntot), tube_of((size_t)ntot);
  for (int t = 0; t < ntube; ++t) {
    const double* rp = rparams + (size_t)t * n_rparams;
    k.n.push_back(ncell[t]);
    k.off.push_back(off);
    k.first.push_back(first);
    k.dx.push_back(rp[EDYN_RP_DX]);
    k.p_out.push_back(n_rparams > EDYN_RP_P_OUT ? rp[EDYN_RP_P_OUT] : 101325.0);
    if (!(k.dx.back() > 0)) return fail(c, EDYN_E_ARG, "tube %d: dx must be positive", t);
    for (int i = 0; i < ncell[t]; ++i) {
      colmap[(size_t)(first + i)] = (int)(off + i);
      tube_of[(size_t)(first + i)] = t;
    }
    off += ncell[t] + 2 * GHOST;
    first += ncell[t];
  }
  c->n = (int)ntot;
  const size_t nt = (size_t)ntube;
  CK(cudaMalloc(&k.d_n, nt * sizeof(int)));
  CK(cudaMalloc(&k.d_off, nt * sizeof(long long)));
  CK(cudaMalloc(&k.d_dx, nt * sizeof(double)));
  CK(cudaMalloc(&k.d_p_out, nt * sizeof(double)));
  CK(cudaMalloc(&k.d_dt, nt * sizeof(double)));
  CK(cudaMalloc(&k.d_time, nt * sizeof(double)));
  CK(cudaMalloc(&k.d_active, nt * sizeof(int)));
  CK(cudaMalloc(&k.d_cvel, nt * sizeof(unsigned long long)));
  CK(cudaMalloc(&k.colmap, (size_t)ntot * sizeof(int)));
  CK(cudaMalloc(&k.tube_of, (size_t)ntot * sizeof(int)));
  CK(cudaMemcpy(k.d_n, k.n.data(), nt * sizeof(int), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(k.d_off, k.off.data(), nt * sizeof(long long), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(k.d_dx, k.dx.data(), nt * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(k.d_p_out, k.p_out.data(), nt * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemset(k.d_dt, 0, nt * sizeof(double)));
  CK(cudaMemset(k.d_time, 0, nt * sizeof(double)));
  CK(cudaMemset(k.d_active, 0, nt * sizeof(int)));
  CK(cudaMemcpy(k.colmap, colmap.data(), colmap.size() * sizeof(int), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(k.tube_of, tube_of.data(), tube_of.size() * sizeof(int), cudaMemcpyHostToDevice));
  CK(stage_tiling(c->acu, c->lim, c->wflag, c->riemann, c->ns, c->n, &c->stage_tc, c->spherical));
  c->listed = c->n >= CHEM_TWO_PASS_CELLS;
  if (c->do_tran) {
    // the transport kernels run over every column: each column's tube
    std::vector<int> col_tube((size_t)c->ld, 0);
    for (int t = 0; t < ntube; ++t)
      for (long long j = 0; j < k.n[t] + 2 * GHOST; ++j) col_tube[(size_t)(k.off[t] + j)] = t;
    int* d = nullptr;
    CK(cudaMalloc(&d, col_tube.size() * sizeof(int)));
    CK(cudaMemcpy(d, col_tube.data(), col_tube.size() * sizeof(int), cudaMemcpyHostToDevice));
    c->d_col_tube = d;
    c->trd.col_tube = d;
  }
  if (smr) {
    k.dx_comp = rparams[EDYN_RP_DX];
    const size_t snap = (size_t)(ntube - 1) * 2 * c->ne * 2 * c->lvir;
    if (snap) CK(cudaMalloc(&k.d_snap, snap * sizeof(double)));
  }
  return build_tiles(c);
}
}  // namespace

int edyn_init_tubes(const char* chem_dir, int nspe, int nequ, int ntube, const int* ncell, int lvir,
                    const int* iflags, int n_iflags, const double* rparams, int n_rparams, void** out) {
  return init_packed(chem_dir, nspe, nequ, ntube, ncell, lvir, iflags, n_iflags, rparams, n_rparams, nullptr, false,
                     out);
}

int edyn_init_blocks(const char* chem_dir, int nspe, int nequ, int nseg, const int* ncell, const double* dx, int lvir,
                     const int* iflags, int n_iflags, const double* rparams, int n_rparams, const double* x_in,
                     void** out) {
  if (!out) return EDYN_E_ARG;
  *out = nullptr;
  if (nseg < 1 || !ncell || !dx || !rparams || n_rparams < 1 || !iflags || n_iflags < 8) return EDYN_E_ARG;
  auto refuse = [&](const char* why) {
    int rc = edyn_init(chem_dir, nspe, nequ, 16, lvir, iflags, n_iflags, rparams, n_rparams, nullptr, out);
    if (rc == EDYN_OK) rc = fail((Ctx*)*out, EDYN_E_ARG, "edyn_init_blocks: %s", why);
    return rc ? rc : EDYN_E_ARG;
  };
  if (iflags[EDYN_IF_SELECT_TIME] == 2) return refuse("Euler or TVDRK3 stages only");
  for (int g = 0; g < nseg; ++g) {
    if (!(dx[g] > 0.0)) return refuse("cell sizes must be positive");
    if (g && !(dx[g] == dx[g - 1] || dx[g] == 2.0 * dx[g - 1] || 2.0 * dx[g] == dx[g - 1]))
      return refuse("neighbouring segments' cell sizes must be equal or differ by a factor of two");
  }
  // one rparams row per segment: the context's row with the segment's cell size
  std::vector<double> rp((size_t)nseg * n_rparams);
  for (int g = 0; g < nseg; ++g) {
    for (int j = 0; j < n_rparams; ++j) rp[(size_t)g * n_rparams + j] = rparams[j];
    rp[(size_t)g * n_rparams + EDYN_RP_DX] = dx[g];
  }
  int rc = init_packed(chem_dir, nspe, nequ, nseg, ncell, lvir, iflags, n_iflags, rp.data(), n_rparams, x_in, true,
                       out);
  if (rc == EDYN_OK) {
    ((Ctx*)*out)->pk.dx_comp = rparams[EDYN_RP_DX];
    rc = smr_geometry((Ctx*)*out);
  }
  return rc;
}

int edyn_tube_times(void* ctx, double* time, double* dt) {
  Ctx* c = (Ctx*)ctx;
  if (!c || !c->qc) return EDYN_E_ARG;
  const size_t nt = (size_t)std::max(1, c->pk.ntube);
  if (time) CK(cudaMemcpy(time, c->pk.ntube ? c->pk.d_time : c->d_time, nt * sizeof(double), cudaMemcpyDeviceToHost));
  if (dt) CK(cudaMemcpy(dt, c->pk.ntube ? c->pk.d_dt : c->d_dt, nt * sizeof(double), cudaMemcpyDeviceToHost));
  return EDYN_OK;
}

namespace {
// Cache line key of the stage-tile choice: scheme, species, cells, tubes and
// device, so a choice measured once serves later runs of the same case.
std::string tune_key(Ctx* c) {
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceProp pr;
  std::memset(&pr, 0, sizeof(pr));
  cudaGetDeviceProperties(&pr, dev);
  std::string name(pr.name);
  for (char& ch : name)
    if (ch == ' ') ch = '_';
  char buf[256];
  std::snprintf(buf, sizeof(buf), "stage acu=%d lim=%d weno=%d rm=%d ns=%d n=%d tubes=%d sm=%d %s", c->acu, c->lim,
                c->wflag, c->riemann, c->ns, c->n, c->pk.ntube, pr.multiProcessorCount, name.c_str());
  return buf;
}
}  // namespace

int edyn_autotune(void* ctx, const char* cache_path, int* tile, double* stage_ms) {
  Ctx* c = (Ctx*)ctx;
  if (!c || !c->qc) return EDYN_E_ARG;
  const std::string key = tune_key(c);
  if (cache_path) {
    if (FILE* f = std::fopen(cache_path, "r")) {
      char line[512];
      int best = -1;
      double ms = 0;
      while (std::fgets(line, sizeof(line), f)) {
        const size_t kl = key.size();
        if (std::strncmp(line, key.c_str(), kl) == 0 && line[kl] == ' ') {
          int t = 0;
          double m = 0;
          if (std::sscanf(line + kl, " tile=%d ms=%lf", &t, &m) == 2 && t >= STAGE_MIN_CELLS && t <= STAGE_MAX_CELLS) {
            best = t;
            ms = m;
          }
        }
      }
      std::fclose(f);
      if (best > 0) {
        c->stage_tc = best;
        drop_graph(c);
        if (c->pk.ntube) {
          int rc = build_tiles(c);
          if (rc) return rc;
        }
        if (tile) *tile = best;
        if (stage_ms) *stage_ms = ms;
        return EDYN_OK;
      }
    }
  }
  // Time one fluid stage per candidate tile on the tube's own state with
  // dt = 0: Q - 0 dF = Q, so Qc stays bit for bit as it was; the stage only
  // rewrites the second primitive buffer, which every step writes before
  // it reads it.
  const int tc0 = c->stage_tc;
  // packed tubes time the stage at dt = 0 through their per-tube dt; the
  // tubes' last time steps are put back afterwards
  std::vector<double> dt_saved(c->pk.ntube);
  if (c->pk.ntube)
    CK(cudaMemcpyAsync(dt_saved.data(), c->pk.d_dt, c->pk.ntube * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  int best = tc0;
  float best_ms = 1e30f;
  for (int tc = STAGE_MIN_CELLS; tc <= STAGE_MAX_CELLS; tc += 2) {
    c->stage_tc = tc;
    if (c->pk.ntube) {
      int rc = build_tiles(c);
      if (rc) return rc;
    }
    StageArgs a = base_args(c);
    a.qf_in = c->qf[c->cur];
    a.qf_out = c->qf[c->cur ^ 1];
    a.kind = 0;
    a.save_q0 = 0;
    a.dt = 0.0;
    a.err = nullptr;
    if (c->pk.ntube) {
      // every packed tube at dt = 0: point the per-tube dt at zeros
      CK(cudaMemsetAsync(c->pk.d_dt, 0, c->pk.ntube * sizeof(double), c->stream));
      a.tubes.active = nullptr;
    }
    float ms = 0.f;
    for (int rep = 0; rep < 3; ++rep) {
      CK(cudaEventRecord(e0, c->stream));
      cudaError_t e = launch_stage(a, c->acu, c->lim, c->wflag, c->riemann, c->stream);
      if (e != cudaSuccess) return fail(c, EDYN_E_CUDA, "autotune stage launch: %s", cudaGetErrorString(e));
      CK(cudaEventRecord(e1, c->stream));
      CK(cudaEventSynchronize(e1));
      float m = 0.f;
      CK(cudaEventElapsedTime(&m, e0, e1));
      if (rep > 0) ms = (rep == 1) ? m : std::min(ms, m);  // the first launch warms up
    }
    if (ms < best_ms) {
      best_ms = ms;
      best = tc;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  c->stage_tc = best;
  drop_graph(c);
  if (c->pk.ntube) {
    CK(cudaMemcpyAsync(c->pk.d_dt, dt_saved.data(), c->pk.ntube * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    int rc = build_tiles(c);
    if (rc) return rc;
  }
  if (cache_path) {
    if (FILE* f = std::fopen(cache_path, "a")) {
      std::fprintf(f, "%s tile=%d ms=%.6f\n", key.c_str(), best, (double)best_ms);
      std::fclose(f);
    }
  }
  if (tile) *tile = best;
  if (stage_ms) *stage_ms = best_ms;
  return EDYN_OK;
}

int edyn_set_stage_tile(void* ctx, int cells) {
  Ctx* c = (Ctx*)ctx;
  if (!c || !c->qc) return EDYN_E_ARG;
  if (cells != 0 && (cells < STAGE_MIN_CELLS || cells > STAGE_MAX_CELLS))
    return fail(c, EDYN_E_ARG, "stage tile of %d cells outside [%d, %d] (0: automatic)", cells, STAGE_MIN_CELLS,
                STAGE_MAX_CELLS);
  int tc = cells;
  if (cells == 0) CK(stage_tiling(c->acu, c->lim, c->wflag, c->riemann, c->ns, c->n, &tc, c->spherical));
  c->stage_tc = tc;
  drop_graph(c);
  return c->pk.ntube ? build_tiles(c) : EDYN_OK;
}

int edyn_stage_tile(void* ctx, int* cells, int* threads) {
  Ctx* c = (Ctx*)ctx;
  if (!c || !c->qc) return EDYN_E_ARG;
  if (cells) *cells = c->stage_tc;
  if (threads) *threads = stage_threads(c->stage_tc);
  return EDYN_OK;
}

int edyn_set_stream(void* ctx, void* stream) {
  Ctx* c = (Ctx*)ctx;
  if (!c) return EDYN_E_ARG;
  c->stream = stream ? (cudaStream_t)stream : c->own;
  drop_graph(c);
  return EDYN_OK;
}

int edyn_upload(void* ctx, const double* qf_aos, const double* qc_aos) {
  Ctx* c = (Ctx*)ctx;
  if (!c || !c->qc) return EDYN_E_ARG;
  if (!qc_aos) return fail(c, EDYN_E_ARG, "Qc is required");
  const size_t bytes = (size_t)c->ne * c->n * sizeof(double);
  // Qc and qf each in their half of the staging buffer: the copies back to
  // back, then the transposes
  int rc = ensure_staging(c, 2 * bytes);
  if (rc) return rc;
  double* sc = c->staging;
  double* sf = c->staging + (size_t)c->ne * c->n;
  CK(cudaMemcpyAsync(sc, qc_aos, bytes, cudaMemcpyHostToDevice, c->stream));
  if (qf_aos) CK(cudaMemcpyAsync(sf, qf_aos, bytes, cudaMemcpyHostToDevice, c->stream));
  for (const Seg& g : segs(c)) CK(launch_aos_to_soa(sc + g.first * c->ne, c->ne, g.n, c->qc + g.off, c->ld, c->stream));
  if (qf_aos) {
    for (const Seg& g : segs(c))
      CK(launch_aos_to_soa(sf + g.first * c->ne, c->ne, g.n, c->qf[c->cur] + g.off, c->ld, c->stream));
  } else {
    for (const Seg& g : segs(c)) {
      StageArgs a = base_args(c);
      a.n = g.n;
      a.qc = c->qc + g.off;
      a.qf_in = nullptr;
      a.qf_out = c->qf[c->cur] + g.off;
      a.strict_newton = 1;
      CK(launch_qc_to_qf(a, c->stream));
    }
  }
  for (const Seg& g : segs(c))
    CK(launch_check_state(c->qf[c->cur] + g.off, c->qc + g.off, g.n, c->ns, c->ld, c->d_err, c->stream));
  c->hrr_dot_state = 0;
  int rc2 = refresh_chem_set(c);
  if (rc2) return rc2;
  CK(cudaStreamSynchronize(c->stream));
  return take_status(c, "edyn_upload");
}

int edyn_init_cells(void* ctx, const double* T, const double* p, const double* u, const double* X) {
  Ctx* c = (Ctx*)ctx;
  if (!c || !c->qc || !T || !p || !u || !X) return EDYN_E_ARG;
  const size_t n = (size_t)c->n, ns = (size_t)c->ns;
  const size_t bytes = (3 * n + n * ns) * sizeof(double);
  int rc = ensure_staging(c, std::max(bytes, (size_t)c->ne * n * sizeof(double)));
  if (rc) return rc;
  double* dT = c->staging;
  double* dp = dT + n;
  double* du = dp + n;
  double* dX = du + n;
  CK(cudaMemcpyAsync(dT, T, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(dp, p, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(du, u, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(dX, X, n * ns * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  for (const Seg& g : segs(c)) {
    CK(launch_init_cells(g.n, c->ns, dT + g.first, dp + g.first, du + g.first, dX + g.first * ns, c->ns,
                         c->qf[c->cur] + g.off, c->qc + g.off, c->ld, c->stream));
    CK(launch_check_state(c->qf[c->cur] + g.off, c->qc + g.off, g.n, c->ns, c->ld, c->d_err, c->stream));
  }
  CK(cudaStreamSynchronize(c->stream));
  c->hrr_dot_state = 0;
  int rc2 = refresh_chem_set(c);
  if (rc2) return rc2;
  return take_status(c, "edyn_init_cells");
}

int edyn_calc_dt(void* ctx, double cfl, double* dt) {
  Ctx* c = (Ctx*)ctx;
  if (!c || !c->qc || !dt) return EDYN_E_ARG;
  if (c->pk.ntube)
    return fail(c, EDYN_E_ARG, "packed tubes take their own time steps: step them with edyn_step or edyn_advance");
  CK(cudaMemsetAsync(c->d_cvel, 0, sizeof(unsigned long long), c->stream));
  CK(launch_cvel(c->qf[c->cur], c->n, c->ld, c->d_cvel, c->stream));
  unsigned long long bits = 0;
  CK(cudaMemcpyAsync(&bits, c->d_cvel, sizeof(bits), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  double cv;
  std::memcpy(&cv, &bits, sizeof(cv));
  if (!(cv > 0) || !std::isfinite(cv)) return fail(c, EDYN_E_STATE, "non-finite or zero signal speed");
  *dt = (cfl * c->dx) / cv;
  return EDYN_OK;
}

int edyn_solve_fluid(void* ctx, double dt) {
  Ctx* c = (Ctx*)ctx;
  if (!c || !c->qc) return EDYN_E_ARG;
  if (c->pk.ntube)
    return fail(c, EDYN_E_ARG, "packed tubes take their own time steps: step them with edyn_step or edyn_advance");
  int rc = keep_hrr_dot(c);
  if (rc) return rc;
  rc = fluid_step(c, dt, false, true);
  if (rc) return rc;
  CK(cudaStreamSynchronize(c->stream));
  return take_status(c, "edyn_solve_fluid");
}

int edyn_solve_source(void* ctx, double dt, double time) {
  Ctx* c = (Ctx*)ctx;
  if (!c || !c->qc) return EDYN_E_ARG;
  if (c->pk.ntube)
    return fail(c, EDYN_E_ARG, "packed tubes take their own time steps: step them with edyn_step or edyn_advance");
  int rc = source_step(c, dt, false, time);
  if (rc) return rc;
  if (c->do_reaction) c->hrr_dot_state = 1;
  CK(cudaStreamSynchronize(c->stream));
  return take_status(c, "edyn_solve_source");
}

int edyn_post_step(void* ctx) {
  Ctx* c = (Ctx*)ctx;
  if (!c || !c->qc) return EDYN_E_ARG;
  // Frozen chemistry leaves Qc as the last stage produced it, so the
  // primitive state is already QcToqf(Qc). The chemistry kernel rebuilds qf
  // from the new Qc in its epilogue, so nothing remains to do either way;
  // ghosts are rebuilt from the boundary rule by every consumer.
  return EDYN_OK;
}

int edyn_step(void* ctx, double cfl, double* dt) {
  Ctx* c = (Ctx*)ctx;
  if (!c) return EDYN_E_ARG;
  if (c->pk.ntube) {
    // one step of every tube with its own dt, through the device loop
    double t = 0.0;
    long long n = 0;
    int rc = edyn_advance(ctx, cfl, 1e300, 1, &t, &n);
    if (rc) return rc;
    if (dt) CK(cudaMemcpy(dt, c->pk.d_dt, sizeof(double), cudaMemcpyDeviceToHost));
    return EDYN_OK;
  }
  double d;
  int rc = edyn_calc_dt(ctx, cfl, &d);
  if (rc) return rc;
  // the source step of this call supersedes the last one's HRR_dot
  if (c->do_reaction) c->hrr_dot_state = 0;
  rc = edyn_solve_fluid(ctx, d);
  if (rc) return rc;
  c->clock += d;  // the reference advances time before the step (SRC/main.f90:139)
  rc = edyn_solve_source(ctx, d, c->clock);
  if (rc) return rc;
  rc = edyn_post_step(ctx);
  if (dt) *dt = d;
  return rc;
}

int edyn_advance(void* ctx, double cfl, double tend, long long max_steps, double* time, long long* nsteps) {
  Ctx* c = (Ctx*)ctx;
  if (!c || !c->qc || !time) return EDYN_E_ARG;
  // every step of the loop ends with a source step when chemistry is on, so
  // the HRR_dot of the last one before this call is superseded, not lost
  if (max_steps < 0) return fail(c, EDYN_E_ARG, "max_steps=%lld must be >= 0", max_steps);
  CK(cudaMemcpyAsync(c->d_time, time, sizeof(double), cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemsetAsync(c->d_nsteps, 0, sizeof(long long), c->stream));
  // pageable source: the copy is staged before the call returns, so the
  // stack variable may go out of scope
  const long long budget = max_steps;
  CK(cudaMemcpyAsync(c->d_max_steps, &budget, sizeof(long long), cudaMemcpyHostToDevice, c->stream));
  if (c->pk.ntube) {
    CK(cudaMemsetAsync(c->pk.d_cvel, 0, c->pk.ntube * sizeof(unsigned long long), c->stream));
    CK(launch_cvel(c->qf[c->cur], c->n, c->ld, c->pk.d_cvel, c->stream, c->pk.colmap, c->pk.tube_of));
  } else {
    CK(cudaMemsetAsync(c->d_cvel, 0, sizeof(unsigned long long), c->stream));
    CK(launch_cvel(c->qf[c->cur], c->n, c->ld, c->d_cvel, c->stream));
  }
  if (c->do_reaction && c->chem_mode == 1) {
    // The surrogate path sizes its launches from counts it reads back, so
    // its steps run from the host, one at a time, with the device clock.
    long long done = 0;
    double t = *time;
    while (t < tend && done < max_steps) {
      CK(launch_step_begin(c->d_time, tend, c->d_nsteps, c->d_max_steps, cfl, c->dx, c->d_cvel, c->d_active, c->d_dt,
                           c->stream));
      int rc = fluid_step(c, 0.0, true, false);
      if (!rc) rc = source_step(c, 0.0, true);
      if (rc) return rc;
      long long ns = 0;
      CK(cudaMemcpyAsync(&t, c->d_time, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
      CK(cudaMemcpyAsync(&ns, c->d_nsteps, sizeof(long long), cudaMemcpyDeviceToHost, c->stream));
      CK(cudaStreamSynchronize(c->stream));
      if (ns == done) break;
      done = ns;
    }
    *time = t;
    c->clock = t;
    if (nsteps) *nsteps = done;
    if (done > 0) c->hrr_dot_state = 1;
    return take_status(c, "edyn_advance");
  }
  // Steps per graph: even, so the primitive double buffer returns to the
  // same parity and one captured graph serves every launch.
  const int per_graph = 16;
  if (!c->graph || c->graph_cfl != cfl || c->graph_tend != tend) {
    drop_graph(c);
    const int cur0 = c->cur;
    cudaGraph_t g;
    CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    int rc = 0;
    for (int s = 0; s < per_graph && !rc; ++s) {
      const Packed& k = c->pk;
      cudaError_t e = !k.ntube ? launch_step_begin(c->d_time, tend, c->d_nsteps, c->d_max_steps, cfl, c->dx,
                                                   c->d_cvel, c->d_active, c->d_dt, c->stream)
                      : k.smr ? launch_step_begin_blocks(k.ntube, k.d_time, tend, c->d_nsteps, c->d_max_steps, cfl,
                                                         k.dx_comp, k.d_cvel, k.d_active, k.d_dt, c->d_active,
                                                         c->stream)
                              : launch_step_begin_tubes(k.ntube, k.d_time, tend, c->d_nsteps, c->d_max_steps, cfl,
                                                        k.d_dx, k.d_cvel, k.d_active, k.d_dt, c->d_active, c->stream);
      if (e != cudaSuccess) rc = fail(c, EDYN_E_CUDA, "step_begin: %s", cudaGetErrorString(e));
      if (!rc) rc = fluid_step(c, 0.0, true, !c->do_reaction);
      if (!rc) rc = source_step(c, 0.0, true);
    }
    cudaError_t ec = cudaStreamEndCapture(c->stream, &g);
    if (rc) return rc;
    if (ec != cudaSuccess) return fail(c, EDYN_E_CUDA, "capture: %s", cudaGetErrorString(ec));
    CK(cudaGraphInstantiate(&c->graph, g, 0));
    cudaGraphDestroy(g);
    c->graph_steps = per_graph;
    c->graph_cfl = cfl;
    c->graph_tend = tend;
    if (c->cur != cur0) return fail(c, EDYN_E_ARG, "graph does not preserve the buffer parity");
  }
  long long done = 0;
  double t = *time;
  // packed tubes keep their own clocks on the device; *time reports tube 0's
  double* clock = c->pk.ntube ? c->pk.d_time : c->d_time;
  if (c->pk.ntube) t = -1e300;
  // A graph whose loop test ends the run before its 16th step leaves the new
  // primitive state in the buffer its last active stage wrote; the graph's
  // buffer roles assume all 16 steps, so after an odd number of swaps the
  // state is copied back into the buffer the graph starts from.
  const int swaps_per_step = (c->select_time == 1) ? 3 : 1;
  while (t < tend && done < max_steps) {
    CK(cudaGraphLaunch(c->graph, c->stream));
    long long ns = 0;
    CK(cudaMemcpyAsync(&t, clock, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(&ns, c->d_nsteps, sizeof(long long), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    const long long ran = ns - done;
    if (ran > 0 && ran < per_graph && (ran * swaps_per_step) % 2 == 1)
      CK(cudaMemcpyAsync(c->qf[c->cur], c->qf[c->cur ^ 1], (size_t)c->ne * c->ld * sizeof(double),
                         cudaMemcpyDeviceToDevice, c->stream));
    if (ns == done) break;
    done = ns;
    if (c->pk.ntube) t = -1e300;  // the device's loop test covers every tube
  }
  if (c->pk.ntube) {
    CK(cudaMemcpy(&t, clock, sizeof(double), cudaMemcpyDeviceToHost));
  }
  *time = t;
  c->clock = t;
  if (nsteps) *nsteps = done;
  if (done > 0 && c->do_reaction) c->hrr_dot_state = 1;
  return take_status(c, "edyn_advance");
}

int edyn_download(void* ctx, double* qf_aos, double* qc_aos, double* hrr) {
  Ctx* c = (Ctx*)ctx;
  if (!c || !c->qc) return EDYN_E_ARG;
  const size_t bytes = (size_t)c->ne * c->n * sizeof(double);
  // qf and Qc each in their half of the staging buffer: both transposes,
  // then the copies back to back and one wait
  int rc = ensure_staging(c, 2 * bytes);
  if (rc) return rc;
  double* sf = c->staging;
  double* sc = c->staging + (size_t)c->ne * c->n;
  if (qf_aos)
    for (const Seg& g : segs(c))
      CK(launch_soa_to_aos(c->qf[c->cur] + g.off, c->ne, g.n, c->ld, sf + g.first * c->ne, c->stream));
  if (qc_aos)
    for (const Seg& g : segs(c)) CK(launch_soa_to_aos(c->qc + g.off, c->ne, g.n, c->ld, sc + g.first * c->ne, c->stream));
  if (qf_aos) CK(cudaMemcpyAsync(qf_aos, sf, bytes, cudaMemcpyDeviceToHost, c->stream));
  if (qc_aos) CK(cudaMemcpyAsync(qc_aos, sc, bytes, cudaMemcpyDeviceToHost, c->stream));
  if (hrr) CK(cudaMemcpyAsync(hrr, c->hrr, (size_t)c->n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return EDYN_OK;
}

int edyn_set_surrogate(void* ctx, const void* w0, const void* w1, const void* w2, const void* w3, const float* b0,
                       const float* b1, const float* b2, const float* b3, const float* norm, double rtol, double atol,
                       double etol) {
  Ctx* c = (Ctx*)ctx;
  if (!c || !c->qc) return EDYN_E_ARG;
  const bool net = w0 != nullptr;
  if (net && (!w1 || !w2 || !w3 || !b0 || !b1 || !b2 || !b3 || !norm))
    return fail(c, EDYN_E_ARG, "edyn_set_surrogate: a network needs all four weights, biases and the normalisation");
  for (const void* ptr : {w0, w1, w2, w3})
    if (ptr && (reinterpret_cast<uintptr_t>(ptr) & 15))
      return fail(c, EDYN_E_ARG, "edyn_set_surrogate: tiled weights must be 16-byte aligned");
  if (!(rtol > 0) || !(atol >= 0) || !(etol > 0)) return fail(c, EDYN_E_ARG, "edyn_set_surrogate: bad gate tolerances");
  Surr& z = c->surr;
  const edyn_mech& m = c->mech;
  if (m.nspec + 3 > Surr::KIN) return fail(c, EDYN_E_ARG, "edyn_set_surrogate: %d species do not fit the network's 64 "
                                                         "inputs", m.nspec);
  if (!z.d_count) {
    const size_t n = (size_t)c->n, nrow = (size_t)m.nspec + 1, M = (n + 127) / 128 * 128;
    CK(cudaMalloc(&z.d_count, 4 * sizeof(unsigned)));
    CK(cudaMalloc(&z.pk_idx, n * sizeof(int)));
    CK(cudaMalloc(&z.pk_rho, n * sizeof(double)));
    CK(cudaMalloc(&z.pk_dt, n * sizeof(double)));
    for (double** b : {&z.pk_y0, &z.pk_f0, &z.pk_y1, &z.pk_ya, &z.pk_f1, &z.pk_fa, &z.rj_y})
      CK(cudaMalloc(b, n * nrow * sizeof(double)));
    CK(cudaMalloc(&z.X, M * Surr::KIN * 2));
    CK(cudaMalloc(&z.Xt, M * Surr::KIN * 2));
    for (int l = 0; l < 3; ++l) CK(cudaMalloc(&z.H[l], M * Surr::HID * 2));
    CK(cudaMalloc(&z.out, M * Surr::KOUT * sizeof(float)));
    CK(cudaMalloc(&z.zero_out, M * Surr::KOUT * sizeof(float)));
    CK(cudaMemset(z.zero_out, 0, M * Surr::KOUT * sizeof(float)));
    CK(cudaMalloc(&z.zero_one, 128 * sizeof(float)));
    std::vector<float> zo(128, 0.f);
    for (int j = 64; j < 128; ++j) zo[j] = 1.f;
    CK(cudaMemcpy(z.zero_one, zo.data(), 128 * sizeof(float), cudaMemcpyHostToDevice));
    CK(cudaMalloc(&z.accept, n * sizeof(int)));
    CK(cudaMalloc(&z.rj_idx, n * sizeof(int)));
    CK(cudaMalloc(&z.rj_rho, n * sizeof(double)));
    CK(cudaMalloc(&z.rj_dt, n * sizeof(double)));
    CK(cudaMalloc(&z.d_nrej, sizeof(int)));
    std::vector<double> wm(m.nspec), el((size_t)m.nelem * m.nspec);
    for (int k = 0; k < m.nspec; ++k) {
      wm[k] = m.W[k] * 1e-3;
      for (int e = 0; e < m.nelem; ++e) el[(size_t)e * m.nspec + k] = m.elem_count[k][e];
    }
    CK(cudaMalloc(&z.wmol, wm.size() * sizeof(double)));
    CK(cudaMalloc(&z.elem, el.size() * sizeof(double)));
    CK(cudaMemcpy(z.wmol, wm.data(), wm.size() * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(z.elem, el.data(), el.size() * sizeof(double), cudaMemcpyHostToDevice));
    z.nrow = m.nspec + 1;
    z.ne = m.nelem;
  }
  z.net = net;
  const void* w[4] = {w0, w1, w2, w3};
  const float* b[4] = {b0, b1, b2, b3};
  for (int l = 0; l < 4; ++l) {
    z.wt[l] = w[l];
    z.b[l] = b[l];
  }
  z.norm = norm;
  z.rtol = rtol;
  z.atol = atol;
  z.etol = etol;
  z.attached = true;
  return EDYN_OK;
}

int edyn_surrogate_stats(void* ctx, double* stats) {
  Ctx* c = (Ctx*)ctx;
  if (!c || !c->qc || !stats) return EDYN_E_ARG;
  for (int i = 0; i < 7; ++i) stats[i] = c->surr.stats[i];
  return EDYN_OK;
}

int edyn_output_open(void* ctx, const char* path) {
  Ctx* c = (Ctx*)ctx;
  if (!c || !c->qc || !path) return EDYN_E_ARG;
  int rc = cell_geometry(c);
  if (rc) return rc;
  std::string err;
  if (!c->h5.create(path, err)) return fail(c, EDYN_E_IO, "edyn_output_open: %s", err.c_str());
  return EDYN_OK;
}

int edyn_output_snapshot(void* ctx) {
  Ctx* c = (Ctx*)ctx;
  if (!c || !c->qc) return EDYN_E_ARG;
  return output_snapshot(c);
}

int edyn_output_rows(void* ctx, double* rows) {
  Ctx* c = (Ctx*)ctx;
  if (!c || !c->qc || !rows) return EDYN_E_ARG;
  int rc = output_rows_ready(c);
  if (rc) return rc;
  std::memcpy(rows, c->h_out, (size_t)(EDYN_OUT_FIXED + c->ns) * c->n * sizeof(double));
  return EDYN_OK;
}

int edyn_output_write(void* ctx, int nout, long long nt, double dt, double time_total, double time_restart,
                      double cpu_total, double cpu_restart) {
  Ctx* c = (Ctx*)ctx;
  if (!c || !c->qc) return EDYN_E_ARG;
  if (!c->h5.is_open()) return fail(c, EDYN_E_ARG, "edyn_output_write: no output file is open (edyn_output_open)");
  if (nout < 0 || nout > 999999 || nt < 0 || nt > 2147483647ll)
    return fail(c, EDYN_E_ARG, "edyn_output_write: nout %d or nt %lld out of the file's integer fields", nout, nt);
  int rc = output_rows_ready(c);
  if (rc) return rc;
  const std::string gname = step_group_name(nout, time_total);
  // the attributes write_hdf5_b writes (its loop stops before the eighth,
  // the chemistry directory name)
  const std::vector<H5Attr> attrs = {{"dt", false, dt},
                                     {"time from 0s", false, time_total},
                                     {"time from restart", false, time_restart},
                                     {"cpu time total", false, cpu_total},
                                     {"cpu time restart", false, cpu_restart},
                                     {"number of output", true, (double)nout},
                                     {"number of time step", true, (double)nt}};
  std::string err;
  if (!c->h5.add_group(gname, attrs, output_names(c), c->h_out, c->n, err))
    return fail(c, EDYN_E_IO, "edyn_output_write: %s", err.c_str());
  return EDYN_OK;
}

int edyn_output_close(void* ctx) {
  Ctx* c = (Ctx*)ctx;
  if (!c || !c->qc) return EDYN_E_ARG;
  std::string err;
  if (!c->h5.close(err)) return fail(c, EDYN_E_IO, "edyn_output_close: %s", err.c_str());
  return EDYN_OK;
}

int edyn_restart(void* ctx, const char* path, int* nout, long long* nt, double* time, double* cpu_time) {
  Ctx* c = (Ctx*)ctx;
  if (!c || !c->qc || !path) return EDYN_E_ARG;
  int rc = cell_geometry(c);
  if (rc) return rc;
  H5Reader r;
  std::string err;
  std::vector<H5Object> groups;
  if (!r.open(path, err) || !r.list("", groups, err)) return fail(c, EDYN_E_IO, "edyn_restart: %s", err.c_str());
  if (groups.empty() || !groups.back().group) return fail(c, EDYN_E_IO, "edyn_restart: %s holds no step group", path);
  // the last member in the root group's index order (idx_stepgroup)
  const std::string g = groups.back().name;
  const size_t n = (size_t)c->n, ns = (size_t)c->ns, ne = (size_t)c->ne;
  auto field = [&](const std::string& name, std::vector<double>& v) -> int {
    H5Value x;
    if (!r.read_dataset(g + "/" + name, x, err))
      return fail(c, EDYN_E_IO, "edyn_restart: %s/%s: %s", g.c_str(), name.c_str(), err.c_str());
    if (x.data.size() != n)
      return fail(c, EDYN_E_ARG, "edyn_restart: %s/%s holds %zu cells, the context %zu", g.c_str(), name.c_str(),
                  x.data.size(), n);
    v.swap(x.data);
    return EDYN_OK;
  };
  std::vector<double> rho, u, T, et, xm, idx, dx;
  if ((rc = field("rho", rho)) || (rc = field("u_x", u)) || (rc = field("  T", T)) || (rc = field(" et", et)) ||
      (rc = field("x_m", xm)) || (rc = field("idx", idx)) || (rc = field(" dx", dx)))
    return rc;
  // the reference's consistency checks of the grid (SRC/read_hdf5.f90:327-365)
  for (size_t i = 0; i < n; ++i) {
    if (std::fabs(xm[i] - c->xm[i]) > 1e-7)
      return fail(c, EDYN_E_ARG, "edyn_restart: x_m of cell %zu (%g) does not match the context's (%g)", i + 1, xm[i],
                  c->xm[i]);
    if (idx[i] != (double)(i + 1)) return fail(c, EDYN_E_ARG, "edyn_restart: idx of cell %zu is %g", i + 1, idx[i]);
    if (std::fabs(dx[i] - c->xm[n + i]) > 1e-7)
      return fail(c, EDYN_E_ARG, "edyn_restart: dx of cell %zu (%g) does not match the context's (%g)", i + 1, dx[i],
                  c->xm[n + i]);
  }
  std::vector<double> X(n * ns);
  for (size_t k = 0; k < ns; ++k) {
    std::vector<double> v;
    if ((rc = field(c->mech.spec_name[k], v))) return rc;
    for (size_t i = 0; i < n; ++i) X[i * ns + k] = v[i];
  }
  // Xi2Yi (CKXTY), then set_block_params: qf = (rho, u, T, Y), Qc = (rho,
  // rho u, rho et, rho Y)
  std::vector<double> qf(n * ne), qc(n * ne);
  for (size_t i = 0; i < n; ++i) {
    const double* x = &X[i * ns];
    double sum = 0.0;
    for (size_t k = 0; k < ns; ++k) sum += x[k] * c->mech.W[k];
    double* f = &qf[i * ne];
    double* q = &qc[i * ne];
    f[0] = rho[i];
    f[1] = u[i];
    f[2] = T[i];
    q[0] = rho[i];
    q[1] = rho[i] * u[i];
    q[2] = rho[i] * et[i];
    for (size_t k = 0; k < ns; ++k) {
      const double y = x[k] * c->mech.W[k] / sum;
      f[3 + k] = y;
      q[3 + k] = rho[i] * y;
    }
  }
  H5Value a_time, a_cpu, a_nout, a_nt;
  if (!r.read_attr(g, "time from 0s", a_time, err) || !r.read_attr(g, "cpu time total", a_cpu, err) ||
      !r.read_attr(g, "number of output", a_nout, err) || !r.read_attr(g, "number of time step", a_nt, err) ||
      a_time.data.empty() || a_cpu.data.empty() || a_nout.data.empty() || a_nt.data.empty())
    return fail(c, EDYN_E_IO, "edyn_restart: %s attributes: %s", g.c_str(), err.c_str());
  rc = edyn_upload(ctx, qf.data(), qc.data());
  if (rc) return rc;
  CK(cudaMemsetAsync(c->d_srcq, 0, 2 * n * sizeof(double), c->stream));
  CK(cudaMemsetAsync(c->hrr, 0, n * sizeof(double), c->stream));
  CK(cudaStreamSynchronize(c->stream));
  // read_hdf5_restart's returns: the next output and step numbers
  if (nout) *nout = (int)a_nout.data[0] + 1;
  if (nt) *nt = (long long)a_nt.data[0] + 1;
  if (time) *time = a_time.data[0];
  if (cpu_time) *cpu_time = a_cpu.data[0];
  c->clock = a_time.data[0];
  return EDYN_OK;
}

int edyn_download_source(void* ctx, double* hrr, double* hrr_dot) {
  Ctx* c = (Ctx*)ctx;
  if (!c || !c->qc) return EDYN_E_ARG;
  if (hrr) CK(cudaMemcpyAsync(hrr, c->hrr, (size_t)c->n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  if (hrr_dot) {
    if (c->hrr_dot_state == 0) {
      std::memset(hrr_dot, 0, (size_t)c->n * sizeof(double));
    } else {
      int rc = eval_hrr_dot(c);
      if (rc) return rc;
      CK(cudaMemcpyAsync(hrr_dot, c->hrr_dot, (size_t)c->n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    }
  }
  CK(cudaStreamSynchronize(c->stream));
  return EDYN_OK;
}

int edyn_set_chem_launch(void* ctx, int form) {
  Ctx* c = (Ctx*)ctx;
  if (!c || !c->qc) return EDYN_E_ARG;
  if (form < 0 || form > 2) return fail(c, EDYN_E_ARG, "chemistry launch form %d not in 0..2", form);
  c->listed = form == 2 || (form == 0 && c->n >= CHEM_TWO_PASS_CELLS);
  drop_graph(c);
  return EDYN_OK;
}

int edyn_transport_properties(void* ctx, double* mu, double* kappa, double* dif) {
  Ctx* c = (Ctx*)ctx;
  if (!c || !c->qc) return EDYN_E_ARG;
  if (!c->do_tran) return fail(c, EDYN_E_ARG, "transport properties need a context created with do_tran 1");
  StageArgs a = base_args(c);
  a.qf_in = c->qf[c->cur];
  CK(launch_tran(a, c->stream));
  const size_t ld = (size_t)c->ld, rows = (size_t)(TRAN_ROWS_FIXED + 2 * c->ns);
  std::vector<double> h(rows * ld);
  CK(cudaMemcpyAsync(h.data(), c->d_tp, h.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  for (int i = 0; i < c->n; ++i) {
    // packed tubes: cell i of the numbering (tube after tube) in its tube's block
    size_t col = (size_t)i + GHOST;
    if (c->pk.ntube) {
      int t = 0;
      long long first = i;
      while (first >= c->pk.n[t]) first -= c->pk.n[t++];
      col = (size_t)(c->pk.off[t] + first + GHOST);
    }
    if (mu) mu[i] = h[3 * ld + col];
    if (kappa) kappa[i] = h[4 * ld + col];
    if (dif)
      for (int k = 0; k < c->ns; ++k) dif[(size_t)i * c->ns + k] = h[(TRAN_ROWS_FIXED + c->ns + k) * ld + col];
  }
  return take_status(c, "edyn_transport_properties");
}

namespace {
int sources_allowed(Ctx* c, const char* what) {
  if (c->pk.ntube && !c->pk.smr)
    return fail(c, EDYN_E_ARG, "%s: one tube or one SMR domain per context (independent packed tubes have no energy "
                "sources)", what);
  if (c->chem_mode == 1) return fail(c, EDYN_E_ARG, "%s: not with the surrogate chemistry (chem_mode 1)", what);
  return EDYN_OK;
}
void sources_changed(Ctx* c) {
  c->src_on = c->src.nrad > 0 || c->src.wall || c->src.ig_type;
  drop_graph(c);
}
}  // namespace

int edyn_set_radiation(void* ctx, int nrad, const int* species, const double* coef) {
  Ctx* c = (Ctx*)ctx;
  if (!c || !c->qc) return EDYN_E_ARG;
  if (int rc = sources_allowed(c, "edyn_set_radiation")) return rc;
  if (nrad < 0 || nrad > EDYN_RAD_MAX || (nrad > 0 && (!species || !coef)))
    return fail(c, EDYN_E_ARG, "edyn_set_radiation: %d radiating species (0..%d, with their fits)", nrad, EDYN_RAD_MAX);
  for (int r = 0; r < nrad; ++r)
    if (species[r] < 0 || species[r] >= c->ns)
      return fail(c, EDYN_E_ARG, "edyn_set_radiation: species index %d out of range", species[r]);
  c->src.nrad = nrad;
  for (int r = 0; r < nrad; ++r) {
    c->src.rad_sp[r] = species[r];
    for (int n = 0; n < 6; ++n) c->src.rad_coef[r][n] = coef[6 * r + n];
  }
  sources_changed(c);
  return EDYN_OK;
}

int edyn_set_wall_heat(void* ctx, int on, const double* params) {
  Ctx* c = (Ctx*)ctx;
  if (!c || !c->qc) return EDYN_E_ARG;
  if (int rc = sources_allowed(c, "edyn_set_wall_heat")) return rc;
  if ((on != 0 && on != 1) || (on && !params)) return fail(c, EDYN_E_ARG, "edyn_set_wall_heat: on must be 0 or 1");
  if (on) {
    if (!(params[1] > 0.0)) return fail(c, EDYN_E_ARG, "edyn_set_wall_heat: the diameter must be positive");
    int rc = load_tran_tables(c);  // the conductivity of MCACON
    if (rc) return rc;
    c->src.nu = params[0];
    c->src.d_m = params[1];
    c->src.tw_min = params[2];
    c->src.tw_max = params[3];
    c->src.alpha = params[4];
    c->src.beta = params[5];
  }
  c->src.wall = on;
  sources_changed(c);
  return EDYN_OK;
}

int edyn_set_ignition(void* ctx, int type, int n, const double* energy, const double* radius, const double* duration,
                      const double* start) {
  Ctx* c = (Ctx*)ctx;
  if (!c || !c->qc) return EDYN_E_ARG;
  if (int rc = sources_allowed(c, "edyn_set_ignition")) return rc;
  if (type < 0 || type > 2) return fail(c, EDYN_E_ARG, "edyn_set_ignition: type %d not in 0..2", type);
  if (type && (n < 1 || n > EDYN_IG_MAX || !energy || !radius || !duration || !start))
    return fail(c, EDYN_E_ARG, "edyn_set_ignition: %d sources (1..%d, with their data)", n, EDYN_IG_MAX);
  for (int g = 0; type && g < n; ++g)
    if (!(radius[g] > 0.0)) return fail(c, EDYN_E_ARG, "edyn_set_ignition: radius %d must be positive", g);
  c->src.ig_type = type;
  c->src.n_ig = type ? n : 0;
  for (int g = 0; g < c->src.n_ig; ++g) {
    c->src.ig_e[g] = energy[g];
    c->src.ig_r[g] = radius[g];
    c->src.ig_t[g] = duration[g];
    c->src.ig_t0[g] = start[g];
  }
  sources_changed(c);
  return EDYN_OK;
}

int edyn_set_uniform_skip(void* ctx, int on) {
  Ctx* c = (Ctx*)ctx;
  if (!c || !c->qc) return EDYN_E_ARG;
  if (on != 0 && on != 1) return fail(c, EDYN_E_ARG, "uniform skip=%d must be 0 or 1", on);
  c->skip_uniform = on;
  drop_graph(c);
  return EDYN_OK;
}

int edyn_set_chem_precheck(void* ctx, int on) {
  Ctx* c = (Ctx*)ctx;
  if (!c || !c->qc) return EDYN_E_ARG;
  if (on != 0 && on != 1) return fail(c, EDYN_E_ARG, "precheck=%d must be 0 or 1", on);
  c->precheck = on;
  drop_graph(c);
  return EDYN_OK;
}

int edyn_set_chem_max_steps(void* ctx, int max_steps) {
  Ctx* c = (Ctx*)ctx;
  if (!c || !c->qc) return EDYN_E_ARG;
  if (max_steps < 0) return fail(c, EDYN_E_ARG, "max_steps=%d must be >= 0 (0: the default 4000)", max_steps);
  c->chem_max_steps = max_steps;
  drop_graph(c);
  return EDYN_OK;
}

int edyn_chem_stats(void* ctx, double* stats) {
  Ctx* c = (Ctx*)ctx;
  if (!c || !c->qc || !stats) return EDYN_E_ARG;
  ChemCounters k;
  cudaError_t e = chem_read_counters(c->use_sub ? c->chem_sub : c->chem, &k, c->stream);
  if (e != cudaSuccess) return fail(c, EDYN_E_CUDA, "counters: %s", cudaGetErrorString(e));
  const unsigned long long v[9] = {k.rhs,   k.steps,      k.rejects, k.failed,    k.jac,
                                   k.cells, k.team_cells, k.cells32, k.cells_same};
  for (int i = 0; i < 9; ++i) stats[i] = (double)v[i];
  return EDYN_OK;
}

int edyn_chem_set(void* ctx, int* nspec, int* nreac) {
  Ctx* c = (Ctx*)ctx;
  if (!c || !c->qc) return EDYN_E_ARG;
  const ChemState& s = c->use_sub ? c->chem_sub : c->chem;
  if (nspec) *nspec = s.ns;
  if (nreac) *nreac = s.nr;
  return EDYN_OK;
}

int edyn_chem_cost(void* ctx, int* cost, unsigned* hot) {
  Ctx* c = (Ctx*)ctx;
  if (!c || !c->qc) return EDYN_E_ARG;
  if (cost) CK(cudaMemcpyAsync(cost, c->d_cost, (size_t)c->n * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  if (hot) CK(cudaMemcpyAsync(hot, c->d_hot, (HOT_MAX + 1) * sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return EDYN_OK;
}

namespace {
int check_fn(void* ctx, int n, const double* x, double* max_ulp, bool is_log) {
  Ctx* c = (Ctx*)ctx;
  if (!c || !c->qc || n <= 0 || !x || !max_ulp) return EDYN_E_ARG;
  int rc = ensure_staging(c, (size_t)n * sizeof(double) + 16);
  if (rc) return rc;
  double* xd = c->staging;
  unsigned long long* md = (unsigned long long*)(c->staging + n);
  CK(cudaMemcpyAsync(xd, x, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemsetAsync(md, 0, sizeof(unsigned long long), c->stream));
  if (is_log) CK(chem_check_log(c->chem, n, xd, md, c->stream));
  else CK(chem_check_exp(c->chem, n, xd, md, c->stream));
  unsigned long long bits = 0;
  CK(cudaMemcpyAsync(&bits, md, sizeof(bits), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  std::memcpy(max_ulp, &bits, sizeof(double));
  return EDYN_OK;
}
}  // namespace

int edyn_check_exp(void* ctx, int n, const double* x, double* max_ulp) { return check_fn(ctx, n, x, max_ulp, false); }

int edyn_check_log(void* ctx, int n, const double* x, double* max_ulp) { return check_fn(ctx, n, x, max_ulp, true); }

int edyn_reactors_device(void* ctx, int n, const double* rho_d, const double* dt_d, double* yiT_d, double* stats) {
  Ctx* c = (Ctx*)ctx;
  if (!c || n < 0 || (n > 0 && (!rho_d || !dt_d || !yiT_d))) return EDYN_E_ARG;
  if (n == 0) return EDYN_OK;
  ChemLaunch L;
  std::memset(&L, 0, sizeof(L));
  L.n = n;
  L.rtol = c->rtol;
  L.atol = c->atol;
  L.rho_batch = rho_d;
  L.dt_batch = dt_d;
  L.yiT_batch = yiT_d;
  L.err = c->d_err;
  L.max_steps = c->chem_max_steps;
  cudaError_t e = chem_launch_batch(c->chem, L, c->stream);
  if (e != cudaSuccess) return fail(c, EDYN_E_CUDA, "reactor launch: %s", cudaGetErrorString(e));
  CK(cudaStreamSynchronize(c->stream));
  if (stats) {
    ChemCounters k;
    e = chem_read_counters(c->chem, &k, c->stream);
    if (e != cudaSuccess) return fail(c, EDYN_E_CUDA, "counters: %s", cudaGetErrorString(e));
    stats[0] = (double)k.rhs;
    stats[1] = (double)k.steps;
    stats[2] = (double)k.rejects;
    stats[3] = (double)k.failed;
  }
  return take_status(c, "edyn_reactors");
}

int edyn_chem_rhs_device(void* ctx, int n, const double* rho_d, const double* yiT_d, double* f_d) {
  Ctx* c = (Ctx*)ctx;
  if (!c || n < 0 || (n > 0 && (!rho_d || !yiT_d || !f_d))) return EDYN_E_ARG;
  if (n == 0) return EDYN_OK;
  cudaError_t e = chem_rhs_batch(c->chem, n, rho_d, yiT_d, f_d, c->stream);
  if (e != cudaSuccess) return fail(c, EDYN_E_CUDA, "right-hand side launch: %s", cudaGetErrorString(e));
  return EDYN_OK;
}

int edyn_chem_rhs_tube(void* ctx, int n, const double* rho_d, const double* yiT_d, double* f_d) {
  Ctx* c = (Ctx*)ctx;
  if (!c || !c->qc || n < 0 || (n > 0 && (!rho_d || !yiT_d || !f_d))) return EDYN_E_ARG;
  if (n == 0) return EDYN_OK;
  cudaError_t e = chem_rhs_batch(c->use_sub ? c->chem_sub : c->chem, n, rho_d, yiT_d, f_d, c->stream);
  if (e != cudaSuccess) return fail(c, EDYN_E_CUDA, "right-hand side launch: %s", cudaGetErrorString(e));
  CK(cudaStreamSynchronize(c->stream));
  return EDYN_OK;
}

int edyn_reactors(void* ctx, int n, const double* rho, const double* dt, double* yiT, double* stats) {
  Ctx* c = (Ctx*)ctx;
  if (!c || n < 0) return EDYN_E_ARG;
  if (n == 0) return EDYN_OK;
  const size_t nv = (size_t)c->ns + 1;
  const size_t bytes = ((size_t)n * 2 + (size_t)n * nv) * sizeof(double);
  int rc = ensure_staging(c, bytes);
  if (rc) return rc;
  double* d_rho = c->staging;
  double* d_dt = d_rho + n;
  double* d_y = d_dt + n;
  CK(cudaMemcpyAsync(d_rho, rho, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(d_dt, dt, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(d_y, yiT, (size_t)n * nv * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  rc = edyn_reactors_device(ctx, n, d_rho, d_dt, d_y, stats);
  CK(cudaMemcpyAsync(yiT, d_y, (size_t)n * nv * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return rc;
}

int edyn_last_error(void* ctx, char* buf, int len) {
  Ctx* c = (Ctx*)ctx;
  if (!buf || len <= 0) return EDYN_E_ARG;
  std::snprintf(buf, (size_t)len, "%s", c ? c->err.c_str() : "no context");
  return EDYN_OK;
}

int edyn_finalize(void* ctx) {
  Ctx* c = (Ctx*)ctx;
  if (!c) return EDYN_OK;
  if (c->stream) cudaStreamSynchronize(c->stream);
  drop_graph(c);
  chem_free(c->chem);
  if (c->chem_sub.d_tables) chem_free(c->chem_sub);
  cudaFree(c->d_present);
  {
    Packed& k = c->pk;
    void* bufs[] = {k.d_tiles, k.d_n, k.d_off, k.d_dx, k.d_p_out, k.d_dt, k.d_time, k.d_active, k.d_cvel, k.colmap,
                    k.tube_of, k.d_snap, k.d_x0};
    for (void* b : bufs) cudaFree(b);
  }
  {
    Surr& z = c->surr;
    void* bufs[] = {z.d_count, z.pk_idx, z.pk_rho, z.pk_dt, z.pk_y0, z.pk_f0, z.pk_y1, z.pk_ya, z.pk_f1,
                    z.pk_fa,   z.X,      z.Xt,     z.H[0],  z.H[1],  z.H[2],  z.out,   z.zero_out, z.zero_one,
                    z.accept,  z.rj_idx, z.rj_rho, z.rj_dt, z.rj_y,  z.d_nrej, z.wmol, z.elem};
    for (void* b : bufs) cudaFree(b);
  }
  cudaFree(c->qf[0]);
  cudaFree(c->qf[1]);
  cudaFree(c->qc);
  cudaFree(c->q0);
  cudaFree(c->acc);
  cudaFree(c->hrr);
  cudaFree(c->hrr_dot);
  cudaFree(c->hrr_dot_rows);
  cudaFree(c->tchem);
  cudaFree(c->staging);
  cudaFree(c->d_time);
  cudaFree(c->d_nsteps);
  cudaFree(c->d_max_steps);
  cudaFree(c->d_active);
  cudaFree(c->d_dt);
  cudaFree(c->d_cvel);
  cudaFree(c->d_err);
  cudaFree(c->d_cost);
  cudaFree(c->d_hot);
  cudaFree(c->d_hlast);
  cudaFree(c->d_list);
  cudaFree(c->d_list_count);
  cudaFree(c->d_cls);
  cudaFree(c->d_hist);
  cudaFree(c->d_run_flag);
  cudaFree(c->d_heads);
  cudaFree(c->d_head_count);
  cudaFree(c->d_run_last);
  cudaFree(c->d_run_head);
  cudaFree(c->d_tran);
  cudaFree(c->d_tp);
  cudaFree(c->d_tflux);
  cudaFree(c->d_col_tube);
  cudaFree(c->d_srcq);
  cudaFree(c->d_out);
  cudaFree(c->d_xm);
  if (c->h_out) cudaFreeHost(c->h_out);
  if (c->out_ready) cudaEventDestroy(c->out_ready);
  if (c->out_copied) cudaEventDestroy(c->out_copied);
  if (c->out_stream) cudaStreamDestroy(c->out_stream);
  if (c->own) cudaStreamDestroy(c->own);
  delete c;
  return EDYN_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Fluid step on caller-owned arrays, allocating nothing.
//
// For hosts that own every device array and cannot let the library allocate
// device memory while they run (the state sits in arrays that the host's own
// runtime sized at start-up: a cudaMalloc at step time can fail against that
// runtime's reservation, and a cudaFree synchronises the whole device).
// The step needs scratch beyond its inputs and outputs: the second primitive
// buffer of the stage double buffer and the stage-0 conserved copy of TVDRK3.
// Both live in one statically sized device array, which every GPU that loads
// this library holds until the process exits.
//
// Nothing in the array has to start at zero: a call writes every element it
// reads before reading it (the owned-cell columns of each stage's primitive
// output and of the stage-0 copy; ghost columns are never read, ghost states
// are rebuilt from the boundary rule). All calls share the array and it keeps
// the last call's contents, so calls whose work overlaps on the GPU race on it.
// ---------------------------------------------------------------------------
static __device__ __align__(256) double g_fluid_scratch[EDYN_NOALLOC_SCRATCH_DOUBLES];

namespace {

constexpr int kMaxDevices = 64;

// Device address of g_fluid_scratch on the current device. In host code the
// symbol's name stands for the device array and is not a device address; the
// address is looked up once per device, on the first call made with that
// device current, and cached.
int fluid_scratch(Ctx* c, double** out) {
  int dev = -1;
  CK(cudaGetDevice(&dev));
  int sdev = -1;
  CK(cudaStreamGetDevice(c->stream, &sdev));
  if (sdev != dev)
    return fail(c, EDYN_E_ARG, "edyn_solve_fluid_noalloc: the context's device %d is not the current device %d", sdev,
                dev);
  if (dev < 0 || dev >= kMaxDevices) return fail(c, EDYN_E_ARG, "device ordinal %d out of range", dev);
  static std::mutex mu;
  static double* addr[kMaxDevices] = {};
  std::lock_guard<std::mutex> lock(mu);
  if (!addr[dev]) {
    void* p = nullptr;
    CK(cudaGetSymbolAddress(&p, g_fluid_scratch));
    addr[dev] = static_cast<double*>(p);
  }
  *out = addr[dev];
  return EDYN_OK;
}

}  // namespace

extern "C" int edyn_solve_fluid_noalloc(void* ctx, double* qf_d, double* qc_d, double dt) {
  Ctx* c = (Ctx*)ctx;
  if (!c || !c->qc) return EDYN_E_ARG;
  if (!qf_d || !qc_d)
    return fail(c, EDYN_E_ARG, "edyn_solve_fluid_noalloc: two distinct device arrays (qf, Qc) are required");
  if ((reinterpret_cast<uintptr_t>(qf_d) | reinterpret_cast<uintptr_t>(qc_d)) % alignof(double))
    return fail(c, EDYN_E_ARG, "edyn_solve_fluid_noalloc: qf and Qc must be 8-byte aligned");
  const size_t rows = (size_t)c->ne * c->ld;
  if (c->pk.ntube) return fail(c, EDYN_E_ARG, "edyn_solve_fluid_noalloc: one tube per context");
  if (c->do_tran)
    return fail(c, EDYN_E_ARG, "edyn_solve_fluid_noalloc: transport (do_tran 1) needs the context's property buffers");
  if (c->select_time == 2)
    return fail(c, EDYN_E_ARG, "edyn_solve_fluid_noalloc: RK4 (select_time 2) needs a third scratch array; use "
                               "edyn_solve_fluid");
  // The stage kernel writes qf while it reads and updates Qc in place: the
  // two arrays must not share a byte.
  {
    const uintptr_t f0 = reinterpret_cast<uintptr_t>(qf_d), q0 = reinterpret_cast<uintptr_t>(qc_d);
    const uintptr_t span = rows * sizeof(double);
    if (f0 < q0 + span && q0 < f0 + span)
      return fail(c, EDYN_E_ARG, "edyn_solve_fluid_noalloc: the qf and Qc arrays overlap (each spans %zu bytes)",
                  (size_t)span);
  }
  if (2 * rows > (size_t)EDYN_NOALLOC_SCRATCH_DOUBLES)
    return fail(c, EDYN_E_ARG,
                "edyn_solve_fluid_noalloc: the tube needs 2*nequ*(ncell+8) = %zu doubles of scratch, the static "
                "scratch holds %d (ncell <= %d at nequ = %d)",
                2 * rows, EDYN_NOALLOC_SCRATCH_DOUBLES, EDYN_NOALLOC_SCRATCH_DOUBLES / (2 * c->ne) - 2 * GHOST, c->ne);
  double* scr = nullptr;
  int rc = fluid_scratch(c, &scr);
  if (rc) return rc;

  StageArgs a = base_args(c);
  a.qc = qc_d;
  a.q0 = scr + rows;
  a.dt = dt;
  double* buf[2] = {qf_d, scr};
  int cur = 0;
  const int nst = c->select_time == 0 ? 1 : 3;
  static const double h1[3] = {0.0, 3.0 / 4.0, 1.0 / 3.0};
  static const double h2[3] = {0.0, 1.0 / 4.0, 2.0 / 3.0};
  for (int s = 0; s < nst; ++s) {
    a.qf_in = buf[cur];
    a.qf_out = buf[cur ^ 1];
    a.kind = s == 0 ? 0 : 1;
    a.save_q0 = (s == 0 && nst == 3) ? 1 : 0;
    a.h1 = h1[s];
    a.h2 = h2[s];
    cudaError_t e = launch_stage(a, c->acu, c->lim, c->wflag, c->riemann, c->stream);
    if (e != cudaSuccess) return fail(c, EDYN_E_CUDA, "stage launch: %s", cudaGetErrorString(e));
    cur ^= 1;
  }
  // An odd number of stages leaves the new primitive state in the scratch:
  // copy its owned columns back into the caller's qf.
  const size_t pitch = (size_t)c->ld * sizeof(double);
  CK(cudaMemcpy2DAsync(qf_d + GHOST, pitch, scr + GHOST, pitch, (size_t)c->n * sizeof(double), (size_t)c->ne,
                       cudaMemcpyDeviceToDevice, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return take_status(c, "edyn_solve_fluid_noalloc");
}
