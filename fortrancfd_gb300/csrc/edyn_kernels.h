// Host-visible declarations of the device kernels' launch interfaces.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>

namespace edyn {

constexpr int GHOST = 4;          // ghost columns allocated per tube end (max lvir)
constexpr int STAGE_MAX_THREADS = 256; // stage CTA: STAGE_SPLIT threads per cell position, positions = cells + 2
constexpr int STAGE_SPLIT = 4;         // threads per cell position (a power of two, at most 32)
constexpr int STAGE_MIN_CELLS = 8;     // smallest stage tile (the tile rule needs at least lvir cells)
constexpr int STAGE_MAX_CELLS = STAGE_MAX_THREADS / STAGE_SPLIT - 2;
// threads of a stage CTA for a tile of tc cells: STAGE_SPLIT per position, whole warps
constexpr int stage_threads(int tc) { return (STAGE_SPLIT * (tc + 2) + 31) / 32 * 32; }

struct ThermoTable;

// Boundary data of SRC/flow_bound.f90 (inlet) and the outlet pressure.
struct FluidBC {
  double rho_u_in;     // kg/(m^2 s)
  double t_in;         // K
  double e_in;         // specific internal energy at (T_in, X_in), J/kg
  double y_in[64];
};

// Device tables of a context that packs several tubes side by side in the
// same rows (tube t's block of n_t + 2 GHOST columns starts at column
// off[t]): every tile of every tube is one CTA of the same stage launch.
struct TubeTab {
  const int4* tiles;       // per stage CTA: (tube, tile index within the tube, tiles of the tube, 0); null: one tube
  const int* n;            // cells of each tube
  const long long* off;    // column offset of each tube's block
  const double* dx;        // cell size of each tube
  const double* p_out;     // outlet pressure of each tube
  const double* dt;        // time step of each tube in this step
  const int* active;       // each tube steps in this step (its time < tend)
  double* time;            // simulated time of each tube
  int ntiles;              // stage CTAs of all tubes
  const int* colmap;       // column of each cell (its tube's block offset + its index)
  const int* tube_of;      // tube of each cell
  // SMR blocks: the tubes are the segments of one domain, left to right;
  // the ghosts facing another segment come from interpolation_block
  // (SRC/block.f90:475-569) on the segments' end columns, copied here
  // before each stage: per interface j, side 0 (segment j's last 2 lvir
  // cells) and side 1 (segment j+1's first 2 lvir cells), [side][row][cell].
  // Null: independent tubes.
  double* smr_snap;
  int ntube;
  const double* x0;        // SMR: the coordinate of each segment's left edge (cell centres x0 + (i + 1/2) dx); null: 0
};

// Transport of calc_flux_tran (SRC/flux.f90:18-127) when do_tran = 1: the
// device copy of the TRANLIB fits and the two buffers the transport kernels
// write before each stage. flux null: transport off.
struct TranDev {
  const double* eta;  // [ns][4] ln viscosity fits in ln T (TRANLIB's COFETA, cgs)
  const double* lam;  // [ns][4] ln conductivity fits (COFLAM)
  const double* dif;  // [ns (ns - 1) / 2][4] ln D_jk fits at patmos of the pairs j < k, k-major
  const double* wa;   // [ns][ns] Wilke rule, expanded: g_kj = 1 / sqrt(1 + W_k / W_j)
  const double* wb;   //          q_kj g_kj, q_kj = (W_j / W_k)^(1/4)
  const double* wc;   //          q_kj^2 g_kj
  const double* W;    // [ns] molecular weights of the fits (TRANLIB's WT)
  const double* e2;   // table of texp
  const double* lg;   // table of tlog
  double patmos;      // dyn/cm^2
  double* tp;         // cell rows, cells -1..n at column c + GHOST: rho, u, T, mu, kappa, Y_k (ns), D'_k (ns)
  double* flux;       // [ne][ld]: transport flux of face j (cells j-1, j) at column j + GHOST
  const int* col_tube;  // packed tubes: the tube of every column (the columns are each tube's block)
};
constexpr int TRAN_ROWS_FIXED = 5;  // rho, u, T, mu, kappa before the species rows of TranDev::tp

struct StageArgs {
  int n, ld, lvir, ns;
  int tc;                // cells per stage tile (CTA); the CTA has stage_threads(tc) threads
  const double* qf_in;   // primitive rows read by the stencil
  double* qf_out;        // primitive rows written for owned cells
  double* qc;            // conserved rows, updated in place
  double* q0;            // stage-0 conserved rows (TVDRK3)
  int kind;              // 0: Q - c dF (Euler, first TVDRK3 stage); 1: h1 Q0 + h2 (Q - c dF); 2: RK4 stage
  int rk4_stage;         // kind 2: stage 0..3 of RK4 (SRC/timeintegration.f90:222-356)
  double* acc;           // kind 2: k1 + 2 k2 + 2 k3, accumulated over the stages
  int save_q0;           // copy Q into q0 before the update (first TVDRK3 stage)
  double h1, h2;
  double dx, dt;         // dt used when dt_dev is null
  const int* step_active;// device loop: skip the stage when zero
  const double* dt_dev;  // device loop: time step of this step
  double* time;          // last kernel of a step advances time and the step count
  long long* nsteps;
  unsigned long long* cvel_out;  // max signal speed of the new state (bit pattern)
  int lbound, rbound;
  double p_out;
  int strict_newton;     // 1: T Newton starts at 1000 K as the reference
  FluidBC bc;            // inlet data (SRC/flow_bound.f90), passed by value
  unsigned* err;         // status word: EDYN_E_NEWTON / EDYN_E_STATE bits of any cell (may be null)
  TubeTab tubes;         // packed tubes (tubes.tiles null: the single tube above); cvel_out then per tube
  int skip_uniform;      // skip the faces of cells whose stencils hold one state (dF = 0 exactly)
  TranDev tran;          // do_tran: transport fluxes added to the advective ones (tran.flux null: off)
  int spherical;         // is_spherical: spherical geometry, r = (i + 1/2) dx (Euler / TVDRK3, first order / MUSCL)
};

// Energy sources of solve_source after the chemistry (SRC/update.f90:126-147):
// optically thin radiation, micro-flow-reactor wall heat and ignition energy,
// each added to rho E over dt and followed by QcToqf of every cell.
constexpr int EDYN_RAD_MAX = 16;  // radiating species
constexpr int EDYN_IG_MAX = 8;    // ignition sources
struct SourceArgs {
  int n, ld, ns;
  double* qf;               // primitive rows (the current buffer), rewritten
  double* qc;               // conserved rows, energy row updated
  double dt, time;          // host call: the step's dt and time
  const double* dt_dev;     // device loop: the step's dt ...
  const double* time_dev;   // ... and the clock the step already advanced
  const int* step_active;   // device loop: skip when zero
  double dx;                // cell centres at (i + 1/2) dx
  int strict_newton;
  unsigned* err;
  unsigned long long* cvel; // device loop: max signal speed of the new state
  int nrad;                 // radiation: species and Planck-mean fits a0..a5 [1/(m atm)]
  int rad_sp[EDYN_RAD_MAX];
  double rad_coef[EDYN_RAD_MAX][6];
  int wall;                 // wall heat: Nu, diameter [m], Tw(x) = A tanh(alpha (x - beta)) + B
  double nu, d_m, tw_min, tw_max, alpha, beta;
  const double* lam;        // conductivity fits (TranDev::lam), and the texp / tlog tables
  const double* e2;
  const double* lg;
  int ig_type, n_ig;        // ignition: 1 Frendi et al., 2 Zhang et al.; per source E [J], r [m], t, t0 [s]
  double ig_e[EDYN_IG_MAX], ig_r[EDYN_IG_MAX], ig_t[EDYN_IG_MAX], ig_t0[EDYN_IG_MAX];
  double* q_rad;            // per cell: the last radiation loss (eos_obj%Qrad), W/m^3 (may be null)
  double* q_tw;             // per cell: the last wall heat (eos_obj%qTw), W/m^3 (may be null)
  const int* colmap;        // SMR segments: the column of each cell (null: i), ...
  const int* tube_of;       // ... its segment (the signal speed is kept per segment) ...
  const double* xm;         // ... and its centre x_m (null: (i + 1/2) dx)
};

// The output fields of write_hdf5_b (SRC/write_hdf5.f90:140-162) from
// set_eos_params (SRC/block.f90:434-470), one row of n per field:
constexpr int EDYN_OUT_FIXED = 15;  // rho u_x T p et ek ei HRR HRD Qrd Tw QTw x_m dx idx, then X_k
struct OutputArgs {
  int n, ld, ns;
  const double* qf;         // primitive rows (rho, u, T, Y)
  const double* qc;         // conserved rows (the energy row)
  const int* colmap;        // column of cell i (null: i)
  const double* hrr;        // per cell, or null (zeros)
  const double* hrr_dot;
  const double* q_rad;
  const double* q_tw;
  const double* xm;         // [2][n]: cell centre and cell size
  int wall;                 // wall heat on: Tw(x) = A tanh(alpha (x - beta)) + B, else Tw = 0
  double tw_min, tw_max, alpha, beta;
  double* out;              // [EDYN_OUT_FIXED + ns][n]
};

int fluid_upload_tables(const ThermoTable& tb, cudaStream_t s);
size_t stage_smem_bytes(int acu, int ns, int tc);
cudaError_t stage_tiling(int acu, int lim, int wflag, int rm, int ns, int n, int* tc, int sph = 0);
cudaError_t launch_stage(const StageArgs& a, int acu, int lim, int wflag, int rm, cudaStream_t s);
cudaError_t launch_cvel(const double* qf, int n, int ld, unsigned long long* cvel, cudaStream_t s,
                        const int* colmap = nullptr, const int* tube_of = nullptr);
cudaError_t launch_step_begin_tubes(int ntube, const double* time, double tend, const long long* nsteps,
                                    const long long* max_steps, double cfl, const double* dx, unsigned long long* cvel,
                                    int* active, double* dt, int* step_active, cudaStream_t s);
cudaError_t launch_step_begin_blocks(int ntube, const double* time, double tend, const long long* nsteps,
                                     const long long* max_steps, double cfl, double dx_comp, unsigned long long* cvel,
                                     int* active, double* dt, int* step_active, cudaStream_t s);
cudaError_t launch_species_present(const double* qc, int ld, int n, int ns, int* flags, cudaStream_t s);
cudaError_t launch_step_begin(const double* time, double tend, const long long* nsteps, const long long* max_steps,
                              double cfl, double dx, unsigned long long* cvel, int* step_active, double* dt_dev,
                              cudaStream_t s);
cudaError_t launch_aos_to_soa(const double* aos, int ne, int n, double* soa, int ld, cudaStream_t s);
cudaError_t launch_soa_to_aos(const double* soa, int ne, int n, int ld, double* aos, cudaStream_t s);
cudaError_t launch_qc_to_qf(const StageArgs& a, cudaStream_t s);
// Transport properties of cells -1..n and transport fluxes of faces 0..n of
// the stage input (a.tran); launch_stage calls it before the stage kernel.
cudaError_t launch_tran(const StageArgs& a, cudaStream_t s);
cudaError_t launch_energy_sources(const SourceArgs& a, cudaStream_t s);
cudaError_t launch_output_rows(const OutputArgs& a, cudaStream_t s);
cudaError_t launch_check_state(const double* qf, const double* qc, int n, int ns, int ld, unsigned* err,
                               cudaStream_t s);
cudaError_t launch_init_cells(int n, int ns, const double* T, const double* p, const double* u, const double* X,
                              int ldx, double* qf, double* qc, int ld, cudaStream_t s);

}  // namespace edyn
