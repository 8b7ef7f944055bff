/*
 * edyn_gpu.h -- C ABI of the GB300 per-cell hot path of EdynCFD.
 *
 * These entry points replace the reference's Fortran hot-path subroutines
 * (Keisuke043/fortranCFD) for a Fortran host that binds them through
 * ISO_C_BINDING, or for any C/C++/Python caller. Plain pointers and sizes
 * only; every function returns an int status (0 = success, nonzero = a bit
 * set of EDYN_E_* classes); no exception crosses the boundary. Host arrays
 * use the reference's layout: per cell a contiguous vector of nequ doubles,
 * cells consecutive (Fortran qf(nequ, ncell) / Qc(nequ, ncell)), SI units.
 *
 * One context owns one tube (or one batch of reactors) on the current CUDA
 * device, its CUDA stream, its device state and its captured step graphs.
 * A context is used from one host thread at a time.
 */
#ifndef EDYN_GPU_H
#define EDYN_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define EDYN_OK 0
#define EDYN_E_ARG 1        /* invalid argument or unsupported option */
#define EDYN_E_CUDA 2       /* CUDA runtime error */
#define EDYN_E_MECH 4       /* mechanism could not be read */
#define EDYN_E_NEWTON 8     /* a cell's temperature Newton ended at its iteration cap, unconverged */
#define EDYN_E_CHEM 16      /* a cell's chemistry integration failed (step underflow or step cap) */
#define EDYN_E_STATE 32     /* a cell's state is non-finite or non-positive, its T pinned at 20 or
                               6000 K, or an uploaded mass fraction is below -1e-6 */
#define EDYN_E_IO 64        /* an output or restart file could not be written or read */

/* Indices into the iflags array of edyn_init (the solver.inp /params/ and
 * problem-file flags, SRC/params.f90:8-18, 105-142). */
#define EDYN_IF_SELECT_TIME 0     /* 0 Euler, 1 TVDRK3, 2 RK4 (the reference's stale-qf form) */
#define EDYN_IF_SELECT_RIEMANN 1  /* 0 LxF, 1 HLL, 2 HLLC */
#define EDYN_IF_FLAG_ACU 2        /* 0 first order, 1 MUSCL, 2 WENO */
#define EDYN_IF_FLAG_MUSCL 3      /* 1 unlimited, 2 minmod, 3 superbee, 4 MC */
#define EDYN_IF_FLAG_WENO 4       /* 1 WENO3-Z, 2 WENO5-JS, 3 WENO5-Z, 4 WENO7-Z */
#define EDYN_IF_FLAG_LBOUND 5     /* 0 wall, 1 inflow */
#define EDYN_IF_FLAG_RBOUND 6     /* 0 wall, 1 outflow (fixed p_OUT) */
#define EDYN_IF_DO_REACTION 7     /* 0 frozen, 1 per-cell chemistry */
#define EDYN_IF_STRICT_NEWTON 8   /* 1: T Newton starts at 1000 K every call (reference); 0: warm start */
#define EDYN_IF_CHEM_MODE 9       /* 0 plain implicit integrator, 1 surrogate with fallback (edyn_set_surrogate) */
#define EDYN_IF_DO_TRAN 10        /* 0 inviscid, 1 viscous stress, conduction and diffusion (calc_flux_tran) */
#define EDYN_IF_IS_SPHERICAL 11   /* 0 Cartesian, 1 spherical (Euler / TVDRK3; first order or MUSCL) */
#define EDYN_NIFLAGS 12

/* Indices into the rparams array of edyn_init. */
#define EDYN_RP_DX 0        /* cell size dx_comp [m] */
#define EDYN_RP_P_OUT 1     /* outlet pressure [Pa] (bound_flow.txt p_out, converted) */
#define EDYN_RP_T_IN 2      /* inlet temperature [K] */
#define EDYN_RP_RHO_U_IN 3  /* inlet mass flux [kg/m^2/s] */
#define EDYN_RP_RTOL 4      /* chemistry relative tolerance (solver.inp rtol) */
#define EDYN_RP_ATOL 5      /* chemistry absolute tolerance (solver.inp atol) */
#define EDYN_NRPARAMS 6

/* Creates a context for one tube of ncell interior cells.
 * Replaces the set-up the reference does in main_sim before its time loop
 * (SRC/main.f90:30-128: set_thermo, init_solvers' lvir, set_block_params).
 * chem_dir: directory with CHEMKIN chem.inp + therm.dat, or with mech.edyn;
 * with do_tran = 1 also TRANLIB's linking file tran.bin (what set_trans,
 * SRC/trans.f90:20-43, reads) or its text form tran.edyn.
 * nspe/nequ must match the mechanism (nequ = nspe + 3). lvir is checked
 * against the scheme (SRC/params.f90:161-173). x_in: inlet mole fractions
 * (nspe values) or NULL.
 * do_tran = 1 adds calc_flux_tran (SRC/flux.f90:18-127) to every stage:
 * viscous stress, conduction and mixture-averaged diffusion from TRANLIB's
 * MCAVIS / MCACON / MCADIF, with MCAVIS standing in for the MCAVIS_EA that
 * the reference's viscosity_ea calls (SRC/trans.f90:137-151) and its
 * tranlib.f does not define. It is available for one tube per context,
 * not for packed tubes (edyn_init_tubes), SMR domains (edyn_init_blocks) nor
 * edyn_solve_fluid_noalloc, and it turns the uniform-region shortcuts of the
 * stage off.
 * is_spherical = 1 (the problem file's flag, SRC/params.f90:37) solves the
 * spherically symmetric equations with r = (i + 1/2) dx
 * (SRC/flux.f90:272-278, SRC/timeintegration.f90:58-75, 177-198): momentum
 * flux without pressure, face fluxes weighed by (r -+ dx/2)^2 over r^2 dx,
 * and the momentum's Roe-averaged face-pressure gradient applied after the
 * stage combination as the reference writes it. With Euler or TVDRK3 and
 * first order or MUSCL; in one tube or an SMR domain (r = x_m), not in
 * independent packed tubes; no uniform-region shortcuts. */
int edyn_init(const char* chem_dir, int nspe, int nequ, int ncell, int lvir, const int* iflags, int n_iflags,
              const double* rparams, int n_rparams, const double* x_in, void** ctx);

/* Creates a context for ntube independent tubes advanced together, each
 * with its own cell count ncell[t] (>= 16), cell size and outlet pressure
 * (rparams: ntube rows of n_rparams values, the same slots as edyn_init;
 * rtol and atol are taken from the first row) and its own time step
 * dt_t = cfl dx_t / max(|u| + a) over its cells: the reference's one-tube
 * time loop (SRC/main.f90:130-163) run for many tubes in the same kernel
 * launches. The scheme, boundary kinds and chemistry flags are shared;
 * the inflow boundary and the surrogate (chem_mode 1) are not available.
 * The tubes' cells are numbered one tube after another: edyn_upload,
 * edyn_init_cells and edyn_download take and give ncell[0] + ... cells in
 * that order. The context steps through edyn_step (one step of every tube)
 * and edyn_advance (every tube while its own time < tend; *time receives
 * tube 0's); edyn_calc_dt, edyn_solve_fluid and edyn_solve_source refuse
 * it. No counterpart in the reference, which runs one tube per process
 * (its MPI ranks split one tube, SRC/parallel.f90:66-83). */
int edyn_init_tubes(const char* chem_dir, int nspe, int nequ, int ntube, const int* ncell, int lvir,
                    const int* iflags, int n_iflags, const double* rparams, int n_rparams, void** ctx);

/* Creates a context for one domain of SMR blocks (static mesh refinement,
 * SRC/block.f90:91-379): nseg segments, left to right, each a run of
 * ncell[s] (>= max(8, 2 lvir)) cells of size dx[s] (a run of the reference's equal-dx
 * blocks, whose ghost exchange is a copy), neighbouring sizes equal or a
 * factor of two apart. The ghosts facing another segment come from
 * interpolation_block (SRC/block.f90:475-569): the mean of two fine cells on
 * the coarse side, the coarse cell -+ 1/4 of its minmod slope on the fine
 * side; each segment computes its own boundary faces from its own ghosts, as
 * each reference block does. One dt = cfl dx_comp / max(|u| + a) for all,
 * dx_comp = rparams[EDYN_RP_DX] (calc_dt, SRC/update.f90:13-59). rparams is
 * one row as for edyn_init; the first segment may take the inflow boundary
 * (x_in), the last the outflow. Euler or TVDRK3. The cell centres x_m
 * follow the reference's (SRC/block.f90:236-304): x = 0 where the leading
 * segments whose dx differs from dx_comp (the left SMR zone) end; spherical
 * geometry (is_spherical) takes r = x_m, and the energy sources
 * (edyn_set_radiation, _wall_heat, _ignition) their positions from x_m.
 * No transport (do_tran) and no surrogate. Cells are numbered left to
 * right; the context steps through edyn_step / edyn_advance, as packed
 * tubes do. */
int edyn_init_blocks(const char* chem_dir, int nspe, int nequ, int nseg, const int* ncell, const double* dx, int lvir,
                     const int* iflags, int n_iflags, const double* rparams, int n_rparams, const double* x_in,
                     void** ctx);

/* Per-tube simulated times and last time steps (ntube values each, either
 * pointer may be NULL); one value for a single-tube context. */
int edyn_tube_times(void* ctx, double* time, double* dt);

/* Uploads the interior state. qf may be NULL (then qf = QcToqf(Qc)).
 * Mirrors set_block_params filling b_obj%qf / b_obj%Qc (SRC/block.f90:394-431). */
int edyn_upload(void* ctx, const double* qf_aos, const double* qc_aos);

/* Builds the interior state from per-cell T [K], p [Pa], u [m/s] and mole
 * fractions X (ncell x nspe), as initialize_variables does for step
 * profiles (SRC/params.f90:305-580), entirely on the device. */
int edyn_init_cells(void* ctx, const double* T, const double* p, const double* u, const double* X);

/* calc_dt (SRC/update.f90:13): dt = cfl * dx / max(|u| + a). */
int edyn_calc_dt(void* ctx, double cfl, double* dt);

/* solve_fluid (SRC/update.f90:62): one explicit Euler, TVDRK3 or RK4 step.
 * RK4 restates SRC/timeintegration.f90:222-356 as written: its stages update
 * Qc and rebuild the boundary ghosts, but reconstruct from the interior
 * primitive state of the step's start (qf is refreshed only after the last
 * stage), with the reference's stage weights. */
int edyn_solve_fluid(void* ctx, double dt);

/* Size of the static scratch of edyn_solve_fluid_noalloc, in doubles
 * (8 MiB): a tube fits when 2 * nequ * (ncell + 8) <= this value, i.e.
 * ncell <= 9354 with the 53 species of GRI-Mech 3.0 (nequ = 56). */
#define EDYN_NOALLOC_SCRATCH_DOUBLES 1048576

/* One explicit Euler or TVDRK3 fluid step, like edyn_solve_fluid, on arrays
 * that the caller owns, allocating nothing. This entry point has no
 * counterpart in the reference.
 *
 * It is for callers that cannot allocate device memory while they run: a
 * host whose tube state lives in device arrays sized once by its own
 * runtime (OpenACC or CUDA Fortran data regions, a pool allocator that
 * reserves the device up front), where a cudaMalloc at step time can fail
 * against that reservation and a cudaFree synchronises the whole device.
 * The call makes no cudaMalloc, cudaFree or other allocating call; the
 * scratch it needs (the second primitive buffer and the TVDRK3 stage-0
 * copy) is a static device array of EDYN_NOALLOC_SCRATCH_DOUBLES doubles,
 * which every GPU that loads this library holds until the process exits.
 *
 * ctx comes from edyn_init (which allocates, once, at set-up); the call uses
 * its scheme, boundary data, mechanism tables and stream, and neither reads
 * nor writes the context's own state buffers. qf_d and qc_d are two
 * disjoint device arrays (overlapping ones are rejected with EDYN_E_ARG) in
 * the library's device layout: nequ rows of ld = ncell + 8 doubles, row v
 * holding variable v, cell i at column i + 4 (the columns outside the cells
 * are neither read nor written). On entry qf_d holds QcToqf(qc_d); on return
 * qc_d holds the state after the step and qf_d its primitive variables.
 *
 * The entry points that work on the context's own state (edyn_calc_dt,
 * edyn_solve_source, edyn_step, edyn_advance, edyn_download) never see the
 * caller's arrays: on this path the host computes dt from its own state
 * (dt = cfl dx / max(|u| + a), as calc_dt does) and runs its own source
 * step. The call blocks the calling host thread until the step has finished
 * on the context's stream; the status then includes EDYN_E_NEWTON or
 * EDYN_E_STATE when a cell's temperature Newton hit its iteration cap or a
 * cell's state was non-finite, non-positive or clamped.
 *
 * Tubes with 2 * nequ * (ncell + 8) > EDYN_NOALLOC_SCRATCH_DOUBLES are
 * rejected with EDYN_E_ARG and a message naming the limit, and so is RK4
 * (select_time 2), whose stage sum needs a third array. The first call
 * on a device looks up the scratch array's device address with that device
 * current (it must be the context's device); make that first call before
 * any stream capture. All calls share the scratch array, which keeps the
 * last call's contents; nothing in it needs to start at zero, since each call
 * writes every scratch element before reading it. Calls that overlap on the
 * GPU (from two threads, or on two streams) race on it. */
int edyn_solve_fluid_noalloc(void* ctx, double* qf_d, double* qc_d, double dt);

/* solve_source (SRC/update.f90:100): per-cell chemistry over dt, heat
 * release rates, qfToQc (SRC/source.f90:17-84). No-op when frozen. */
int edyn_solve_source(void* ctx, double dt, double time);

/* The boundary + QcToqf block after the source step (SRC/main.f90:149-163). */
int edyn_post_step(void* ctx);

/* One pass of the time loop body: calc_dt, solve_fluid, solve_source,
 * post-step (SRC/main.f90:130-163). Returns the dt used. */
int edyn_step(void* ctx, double cfl, double* dt);

/* Runs the time loop on the device until time >= tend or max_steps steps
 * have run (SRC/main.f90:130: do while (time < tend)), with steps captured
 * in CUDA graphs; *time is read and updated, *nsteps receives the count. */
int edyn_advance(void* ctx, double cfl, double tend, long long max_steps, double* time, long long* nsteps);

/* Copies the interior state back (set_eos_params before output,
 * SRC/block.f90:434). Any pointer may be NULL. hrr receives HRR [W/m^3]
 * of the last source step (SRC/source.f90:70-73), ncell values. */
int edyn_download(void* ctx, double* qf_aos, double* qc_aos, double* hrr);

/* Heat release rates of the last source step, ncell values each (either
 * pointer may be NULL): hrr = HRR (heat_release_rate, SRC/thermo.f90:83-103)
 * and hrr_dot = HRR_dot (heat_release_rate_omegadot, SRC/thermo.f90:105-134),
 * which reaction_macks stores per cell (SRC/source.f90:70-73) for output.
 * HRR_dot is -sum_k W_k h_f,k w_k [W/m^3] with the molar production rates
 * w_k at the state the source step left (rho, Y after adjust_sum, the
 * integration's final T). The library evaluates it when it is first asked
 * for, or before a later fluid step changes that state: in the reference's
 * own order (output right after the source step) it costs nothing on the
 * steps that are not written. Zeros before any source step and when the
 * chemistry is frozen. */
int edyn_download_source(void* ctx, double* hrr, double* hrr_dot);

/* ---- Output and restart files (HDF5) ----
 * The reference's results files: one step group per output below the root
 * group, named nout%06d_time%E11.5 (Fortran edit descriptors), holding one
 * float64 dataset of ncell values per field, in this order (the names are
 * Fortran's trimmed character(32) values, leading blanks kept):
 *   "rho", "u_x", "  T", "  p", " et", " ek", " ei", "HRR", "HRD", "Qrd",
 *   " Tw", "QTw", "x_m", " dx", "idx", then one per species (its name):
 * rho, u, T, p = CKPX(rho, T, X), specific total / kinetic / internal
 * energy (rho E / rho, u^2/2, CKUBML / W), HRR, HRR_dot, the radiation loss,
 * the wall temperature and wall heat of the last source step, the cell
 * centre and size, the 1-based cell index, and the mole fractions X_k.
 * Attributes of the group: "dt", "time from 0s", "time from restart",
 * "cpu time total", "cpu time restart" (float64) and "number of output",
 * "number of time step" (int32), each a one-element array. The files are
 * written without an HDF5 library, in the layout libhdf5 writes with its
 * default settings (superblock version 0, symbol-table groups). One tube or
 * one SMR domain per context (edyn_init_blocks); packed independent tubes
 * are refused. Cell centres are (i - 1/2) dx from the domain's left end. */

/* init_output (SRC/write_hdf5.f90:21-48): creates (truncates) the file
 * path; the next edyn_output_write calls append step groups to it. The
 * reference names it <savedir>/results_nout%06d.h5 after the output number
 * that opens it. */
int edyn_output_open(void* ctx, const char* path);

/* set_eos_params (SRC/block.f90:434-470) on the device, queued on the
 * context's stream, and the rows' copy to pinned host memory on a stream of
 * its own: returns at once, so the time loop can go on while the copy
 * drains. One snapshot may be pending at a time; edyn_output_write (or
 * edyn_output_rows) takes it. */
int edyn_output_snapshot(void* ctx);

/* write_hdf5_b (SRC/write_hdf5.f90:76-347): appends the step group of the
 * pending snapshot (or of a snapshot taken now) to the open file, with the
 * attributes dt, time_total ("time from 0s"), time_restart ("time from
 * restart"), cpu_total, cpu_restart, nout and nt. */
int edyn_output_write(void* ctx, int nout, long long nt, double dt, double time_total, double time_restart,
                      double cpu_total, double cpu_restart);

/* The rows of the pending snapshot (or of one taken now): (15 + nspe) rows
 * of ncell doubles, in the dataset order above. */
int edyn_output_rows(void* ctx, double* rows);

/* fin_output (SRC/write_hdf5.f90:51-73): closes the file. */
int edyn_output_close(void* ctx);

/* read_hdf5_restart (SRC/read_hdf5.f90:13-423) + set_block_params
 * (SRC/block.f90:394-431): reads the last step group (in the root group's
 * name order) of path, checks its x_m, idx and dx against the context's
 * cells (within 1e-7), converts the mole fractions to mass fractions (CKXTY)
 * and sets qf = (rho, u, T, Y) and Qc = (rho, rho u, rho et, rho Y). Returns
 * the next output number and step count (the group's values + 1, as the
 * reference), the simulated time and the CPU time of the group (any
 * pointer may be NULL); the context's clock is set to that time. */
int edyn_restart(void* ctx, const char* path, int* nout, long long* nt, double* time, double* cpu_time);

/* FP64 chemistry right-hand side d(Y_1..Y_nspe, T)/dt of n constant-volume
 * reactors (rows of nspe + 1 values, device pointers; rho in kg/m^3) with
 * the species and reactions the tube's chemistry integrates (edyn_chem_set):
 * when that is a subset, the species outside it must be zero in yiT and get
 * zero rates. The rates are CKWYR's (GRI/cklib.f:9107, called through
 * SRC/thermo.f90); the temperature row is the constant-volume energy
 * balance. Synchronous. No counterpart in the reference beyond those
 * rates. */
int edyn_chem_rhs_tube(void* ctx, int n, const double* rho_d, const double* yiT_d, double* f_d);

/* Form of a tube's chemistry launch: 1 one pass (every cell integrated by
 * the integrator kernel, the costliest on four-warp teams), 2 two passes (a
 * light screening pass evaluates f(y0) and the inert-cell test of every cell
 * at four warps per SM sub-partition and finishes the inert cells; the
 * integrator kernel then takes only the cells it listed), 0 automatic (two
 * passes from 10,000 cells). The forms agree up to rounding: a cell on the
 * four-warp team list that turns out inert is finished by its team in one
 * pass and by a single warp in two, whose sums run in other orders. No
 * counterpart in the reference (a tuning knob of this implementation). */
int edyn_set_chem_launch(void* ctx, int form);

/* Uniform regions (on by default). Fluid stage: a cell whose stencil cells
 * c-r..c+r (r the reconstruction radius) hold one primitive state bit for
 * bit has two faces with identical inputs, so identical fluxes and a flux
 * difference of exactly zero: the stage computes neither the
 * reconstructions nor the fluxes that only such cells need. Chemistry (the
 * two-pass launch): a cell's source step depends on its primitive column
 * and its tube's dt alone, so of a run of cells with columns equal bit for
 * bit only the first is screened; the others receive its finished column,
 * or are integrated one by one when it needs the integrator. Results are
 * bit for bit those of on = 0, which computes every face and every cell as
 * the reference does (SRC/timeintegration.f90:99-219, SRC/source.f90:17-84). */
int edyn_set_uniform_skip(void* ctx, int on);

/* The single-precision pre-check of the integrator's inert-cell test (tube
 * chemistry; on by default). A cell's FP32 right-hand side and gross rates
 * bound its FP64 right-hand side; when the bound already passes the inert
 * test (the whole window's change below 1e-3 of the error tolerance), the
 * cell takes its explicit step with the FP32 right-hand side, which differs
 * from the FP64 one's by under 1e-3 of the tolerance, and no FP64 right-hand
 * side is evaluated. Other cells go through the FP64 test as before. on = 0
 * turns it off (every cell gets the FP64 test). No counterpart in the
 * reference, which integrates every cell with its full solver
 * (SRC/source.f90:58). */
int edyn_set_chem_precheck(void* ctx, int on);

/* Caps the implicit integrator at max_steps steps (accepted + rejected) per
 * cell and call; a cell that reaches the cap fails and the call returns
 * EDYN_E_CHEM. 0 restores the default (4000). No counterpart in the
 * reference, whose missing integrator (SRC/odes.f90) has no documented
 * limit. */
int edyn_set_chem_max_steps(void* ctx, int max_steps);

/* Attaches the chemistry surrogate that a context created with
 * EDYN_IF_CHEM_MODE = 1 puts in front of the implicit integrator in every
 * source step (the macks call of SRC/source.f90:58, for each tube cell).
 * No counterpart in the reference, which integrates every cell.
 *
 * A source step then: evaluates f(y0) and the integrator's inert-cell test
 * for every cell (inert cells take their explicit step as in mode 0); for
 * the others forms the network's candidate y0 + dt f0 + correction (an MLP
 * 64 -> 3 x 256 GELU -> 64 on the tensor cores, BF16 weights, FP32
 * accumulation; see include/edyn_surrogate.h) and the explicit increment
 * y0 + dt f0; accepts per cell the first candidate whose FP64 trapezoidal
 * residual |y1 - y0 - dt (f(y0) + f(y1))/2| stays within atol + rtol
 * max(|y0|, |y1|) in every component (no atol on T) and whose element
 * totals stay within etol; integrates the rest with the implicit
 * integrator. w0..w3: the layers' BF16 weights pre-tiled by edyn_mlp_tile
 * (rows 256, 256, 256, 64; BR = edyn_mlp_tile_rows(rows)); b0..b3 FP32
 * biases; norm: 4 x 64 FP32 (input mean, input 1/std, output mean, output
 * std). All device pointers, owned by the caller, kept alive and unchanged
 * while the context steps. w0 = NULL attaches the method without the
 * network (the explicit increment, gated, then the integrator). The first
 * call allocates the path's work buffers (sized for every cell). */
int edyn_set_surrogate(void* ctx, const void* w0, const void* w1, const void* w2, const void* w3, const float* b0,
                       const float* b1, const float* b2, const float* b3, const float* norm, double rtol, double atol,
                       double etol);

/* Counters of the last surrogate source step, 7 values: cells not inert
 * (handed to the surrogate), accepted on the network's candidate, accepted
 * on the explicit increment, integrated by the fallback, right-hand sides of
 * the screen launch, of the gate, of the fallback integration. No
 * counterpart in the reference. */
int edyn_surrogate_stats(void* ctx, double* stats);

/* Batched reactor call: the macks(dt, nspe+1, yiT, rho) contract of
 * SRC/source.f90:58 for n independent cells in one persistent launch.
 * yiT: n x (nspe+1) [Y_1..Y_nspe, T] in/out; rho [kg/m^3]; dt [s] per cell.
 * Uses the context's mechanism and tolerances. stats (optional, 4 values):
 * total right-hand-side evaluations, steps, rejected steps, failed cells. */
int edyn_reactors(void* ctx, int n, const double* rho, const double* dt, double* yiT, double* stats);

/* Same, on device pointers already resident in GPU memory (no copies). */
int edyn_reactors_device(void* ctx, int n, const double* rho_d, const double* dt_d, double* yiT_d, double* stats);

/* Counters of the last chemistry launch of this context (tube or batch),
 * 9 values: FP64 right-hand-side evaluations, accepted steps, rejected
 * steps, failed cells, Jacobians, cells, cells integrated by a four-warp
 * team, inert cells decided by the single-precision pre-check (no FP64
 * right-hand side; see edyn_set_chem_precheck), cells given the result of
 * an identical neighbour (see edyn_set_uniform_skip).
 * No counterpart in the reference, which reports none (its solver's
 * statistics stay inside macks, SRC/source.f90:58). */
int edyn_chem_stats(void* ctx, double* stats);

/* The species and reactions the tube's chemistry integrates (either may be
 * NULL): the whole mechanism, or, when some elements occur nowhere in the
 * tube state nor at the inlet, the species made of the present elements and
 * the reactions among them (the others have zero concentration and zero
 * rates, so the result is the same). Chosen after every edyn_upload and
 * edyn_init_cells. No counterpart in the reference. */
int edyn_chem_set(void* ctx, int* nspec, int* nreac);

/* Per-cell cost of the last chemistry launch of a tube: cost receives ncell
 * right-hand-side counts; hot (optional, 65 values) the cell list that gets
 * four-warp teams in the next launch ([0] = count). No counterpart in the
 * reference (a load-balance diagnostic of this implementation). */
int edyn_chem_cost(void* ctx, int* cost, unsigned* hot);

/* Self-check of the FP64 exponential used in the chemistry rates against
 * CUDA's exp on n host-supplied arguments in [-700, 700]: *max_ulp receives
 * the largest difference in units in the last place. No counterpart in the
 * reference. */
int edyn_check_exp(void* ctx, int n, const double* x, double* max_ulp);

/* The same self-check for the FP64 natural logarithm of the chemistry rates
 * (positive normal arguments). No counterpart in the reference. */
int edyn_check_log(void* ctx, int n, const double* x, double* max_ulp);

/* Cells per tile of the fluid stage kernel (one CTA per tile: four threads
 * per cell position, cells + 2 positions, rounded up to whole warps). 0 (the
 * default) chooses the tile from the tube length and the kernel's occupancy
 * so that the CTAs fill whole waves of resident slots; 8..62 forces a tile.
 * Results do not depend on the tile. No counterpart in the reference (a
 * tuning knob of this implementation). */
int edyn_set_stage_tile(void* ctx, int cells);

/* Picks the stage tile by measurement: times one fluid stage for each tile
 * of 8..62 cells (every second) on the tube's own state with dt = 0, which
 * leaves the state bit for bit as it was, and keeps the fastest. With a
 * cache_path (a text file, one line per case), a tile measured before for
 * the same scheme, species, cell count, tube count and device is read
 * instead, and a new measurement is appended. tile and stage_ms (either may
 * be NULL) receive the choice and its stage time. Results do not depend on
 * the tile. No counterpart in the reference. */
int edyn_autotune(void* ctx, const char* cache_path, int* tile, double* stage_ms);

/* The stage tile in use: cells per tile and threads per CTA (either may be
 * NULL). No counterpart in the reference. */
int edyn_stage_tile(void* ctx, int* cells, int* threads);

/* Binds the context to a caller-owned CUDA stream (cudaStream_t as void*);
 * NULL returns to the context's own stream. */
int edyn_set_stream(void* ctx, void* stream);

/* Writes the last error message (NUL-terminated, truncated to len). */
int edyn_last_error(void* ctx, char* buf, int len);

/* Releases the context and its device memory. */
int edyn_finalize(void* ctx);

/* Compiles a CHEMKIN mechanism directory into the mech.edyn table format
 * (the role of CKINTERP's chem.bin, GRI/ckinterp.f). */
int edyn_mech_compile(const char* chem_dir, const char* out_path, char* err, int errlen);

/* Energy sources of solve_source after the chemistry (SRC/update.f90:126-147),
 * in the reference's order, each added to rho E over the step and followed
 * by QcToqf of every cell; for one tube or one SMR domain per context (cell
 * positions x_m, edyn_init_blocks), not for independent packed tubes nor
 * with chem_mode 1.
 * Cell i sits at x = (i + 1/2) dx (SMR domains: at its x_m).
 *
 * Optically thin radiation loss (heat_transfer_radiation,
 * SRC/source.f90:88-137; radiation_heat_loss, SRC/radiation.f90:74-121):
 * Q = -4 Kp sigma (T^4 - 300^4), Kp = sum_r kp_r(T) X_r p / (1 atm), with
 * kp_r(T) = coef[6r] + coef[6r+1] T + ... + coef[6r+5] T^5 [1/(m atm)] for
 * species index species[r] (the reference's radiation_file, one line per
 * species). nrad = 0 switches it off. */
int edyn_set_radiation(void* ctx, int nrad, const int* species, const double* coef);

/* Micro-flow-reactor wall heat (heat_transfer_mfr, SRC/source.f90:140-189;
 * SRC/mfr.f90:41-78): Q = -4 lambda Nu (T - Tw(x)) / d^2 with lambda the
 * mixture conductivity (MCACON, from the transport fits next to the
 * mechanism) and Tw(x) = (Tw_max - Tw_min)/2 tanh(alpha (x - beta)) +
 * (Tw_max + Tw_min)/2. params: Nu, d [m], Tw_min [K], Tw_max [K],
 * alpha [1/m], beta [m] (the reference's /mfrwalltemp/ namelist, d in m). */
int edyn_set_wall_heat(void* ctx, int on, const double* params);

/* Ignition energy (energy_source, SRC/source.f90:192-239;
 * SRC/ignitionsource.f90:150-262): type 1 after Frendi et al.
 * (E / (4/3 pi r^3 t) exp(-(pi/4) (x/r)^6)), type 2 after Zhang et al.
 * (E / (pi^1.5 r^3 t) exp(-(x/r)^2)), 0 off; n sources with energy [J],
 * radius [m], duration and start [s], each on while start < time < start +
 * duration (where several are on, the last one's rate applies, as in the
 * reference). time is the step's time: edyn_solve_source's argument, the
 * context's clock in edyn_step (advanced by each step, set by edyn_advance),
 * the device clock in edyn_advance. */
int edyn_set_ignition(void* ctx, int type, int n, const double* energy, const double* radius, const double* duration,
                      const double* start);

/* Writes the transport fits of chem_dir (TRANLIB's linking file tran.bin, as
 * MCINIT reads it, tranlib.f:214-258) in the library's text form tran.edyn,
 * every number to 17 significant digits (it reads back bit for bit). */
int edyn_tran_compile(const char* chem_dir, const char* out_path, char* err, int errlen);

/* Transport properties of the current state of a do_tran context, per
 * interior cell, as calc_flux_tran evaluates them (SRC/flux.f90:51-90, the
 * SRC/trans.f90 wrappers): mu [Pa s] (MCAVIS x 0.1), kappa [W/(m K)]
 * (MCACON x 1e-5) and the diffusivities D'_k = (1 - X_k)/(1 - Y_k) D_k
 * [m^2/s] (MCADIF x 1e-4; 0 where Y_k = 1), dif cell-major (ncell x nspe).
 * Any pointer may be NULL. */
int edyn_transport_properties(void* ctx, double* mu, double* kappa, double* dif);

/* Library version string. */
const char* edyn_version(void);

#ifdef __cplusplus
}
#endif
#endif
