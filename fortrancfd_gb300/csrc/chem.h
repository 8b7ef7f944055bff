// Chemistry (per-cell stiff integrator) launch interface.
#pragma once

#include <cuda_runtime.h>

#include "edyn_dev.cuh"
#include "mechanism.h"

namespace edyn {

// Cells of a tube launch that get a four-warp team, at most.
constexpr int HOT_MAX = 64;

struct ChemCounters {
  unsigned long long rhs, steps, rejects, failed, jac, cells, team_cells;
  unsigned long long cells32;  // inert cells decided by the single-precision pre-check
  unsigned long long cells_same;  // cells given the result of an identical cell (runs)
};

struct ChemState {
  void* d_tables = nullptr;       // packed reaction/species tables (global, staged to smem)
  size_t table_bytes = 0;
  int nr = 0, ns = 0, nf = 0, ntb = 0, nscat = 0, ntbl = 0;
  int nr_pad = 0;
  unsigned* d_next = nullptr;     // work-stealing counter
  ChemCounters* d_count = nullptr;
  int ctas = 0, warps = 0;
  size_t smem = 0;
  int screen_ctas = 0, screen_warps = 0;  // the light screening pass
  size_t screen_smem = 0;
};

struct ChemLaunch {
  int n, ld;
  // tube mode
  double* qf;
  double* qc;
  double* hrr;
  double dt;
  const int* step_active;
  const double* dt_dev;
  unsigned long long* cvel_out;
  double* time;
  long long* nsteps;
  int strict_newton;
  int* cost;        // right-hand sides each cell took in the last launch (n)
  unsigned* hot;    // [0] count, [1..HOT_MAX] cells that get a team next launch
  double* hlast;    // step size each cell's integration proposed at the end of its last window (n)
  // batch mode
  const double* rho_batch;
  const double* dt_batch;
  double* yiT_batch;
  double rtol, atol;
  int max_steps;    // steps (accepted + rejected) per cell before it fails; <= 0: 4000
  double* tchem;    // tube mode: temperature each cell's integration ended with (n), or null
  unsigned* err;
  // screen mode (tube): every cell gets f(y0) and the inert-cell test; the
  // inert ones finish as usual, the others are appended to packed rows (full
  // mechanism layout, nspe + 1 values) for the surrogate path, unfinished
  int screen;
  unsigned* pk_count;   // rows appended (cleared by the caller)
  int* pk_idx;          // cell of each row
  double* pk_rho;       // rho [kg/m^3]
  double* pk_dt;        // dt [s]
  double* pk_y0;        // adjusted [Y, T] before the step
  double* pk_f0;        // f(y0)
  // list mode (tube): k_tube_chem integrates only the cells the screening
  // pass listed (list[0..*list_count)); the pass marks them cost -1
  int* list;
  unsigned* list_count;
  // packed tubes (the cells of several tubes side by side in the rows; null
  // for one tube): column of each cell, its tube, each tube's dt, whether it
  // steps, its signal-speed maximum and clock
  const int* colmap;
  const int* tube_of;
  const double* dt_tube;
  const int* active_tube;
  unsigned long long* cvel_tube;
  double* time_tube;
  int ntube;
  // single-precision pre-check of the inert-cell test (tube mode, single warps)
  int precheck;
  // runs of identical cells (two-pass tube launch; heads null: off): rows
  // of the qf columns compared, per-cell run flags, the heads' list and
  // count, the last head of each block of cells
  int nrow;
  unsigned char* run_flag;
  int* heads;
  unsigned* head_count;
  int* run_last;
  int* run_head;  // the head of a follower that takes its head's integrated result
};
constexpr int CHEM_RUN_BLOCK = 1024;  // cells per block of the run kernels

// smap: tube row of each species of m (3 + smap[k]) when m is a subset of the
// tube's mechanism (NULL: identity); nnorm: components counted in the RMS
// norms (0: ns + 1).
int chem_init(ChemState& s, const edyn_mech& m, const ThermoTable& tb, cudaStream_t st, const int* smap = nullptr,
              int nnorm = 0);
cudaError_t chem_launch_tube(ChemState& s, const ChemLaunch& L, cudaStream_t st);
cudaError_t chem_launch_batch(ChemState& s, const ChemLaunch& L, cudaStream_t st);
// The tube's source step in two passes: a light screening pass over every
// cell (FP64 f(y0), inert cells finished at once, the others listed), then
// the integrator kernel over the listed cells only, then the hot-cell
// selection of the next launch in parallel (cls: n bytes; hist: 33 words).
// The same results as chem_launch_tube up to rounding (a team-listed cell
// that turns out inert is finished by a single warp here, by its team there).
cudaError_t chem_launch_tube_listed(ChemState& s, const ChemLaunch& L, int* list, unsigned* list_count,
                                    unsigned char* cls, unsigned* hist, cudaStream_t st);
// The surrogate path's screen: the light screening pass with packed rows
// (L.pk_*, L.pk_count[0..3] cleared by the caller; [3] counts finished
// CTAs) for the cells that are not inert.
cudaError_t chem_launch_screen_packed(ChemState& s, const ChemLaunch& L, cudaStream_t st);
// FP64 right-hand side d(Y, T)/dt of n reactors (rho SI, yiT rows of ns + 1).
cudaError_t chem_rhs_batch(ChemState& s, int n, const double* rho, const double* yiT, double* f, cudaStream_t st);
cudaError_t chem_read_counters(ChemState& s, ChemCounters* out, cudaStream_t st);
// Finishes the m packed rows of a screened tube launch from their states
// after the step (pk_y1): adjust_sum, HRR, qfToQc, QcToqf, signal speed.
cudaError_t chem_finish_packed(ChemState& s, const ChemLaunch& L, int m, const double* pk_y1, cudaStream_t st);
// The followers of packed heads take their heads' finished columns (runs).
cudaError_t chem_follow_packed(ChemState& s, const ChemLaunch& L, cudaStream_t st);
// HRR_dot [W/m^3] of n tube cells from their primitive rows (qf, SoA with ld)
// and the temperatures their last chemistry step ended with.
cudaError_t chem_hrr_dot(ChemState& s, int n, int ld, const double* qf, const double* tchem, double* out,
                         const int* colmap, cudaStream_t st);
cudaError_t chem_check_exp(ChemState& s, int n, const double* x_d, unsigned long long* maxulp_d, cudaStream_t st);
cudaError_t chem_check_log(ChemState& s, int n, const double* x_d, unsigned long long* maxulp_d, cudaStream_t st);
void chem_free(ChemState& s);

}  // namespace edyn
