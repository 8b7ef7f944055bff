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
#define EDYN_E_NEWTON 8     /* temperature Newton hit its iteration cap */
#define EDYN_E_CHEM 16      /* a chemistry step was rejected to underflow */
#define EDYN_E_STATE 32     /* non-finite or non-positive state found */

/* Indices into the iflags array of edyn_init (the solver.inp /params/ and
 * problem-file flags, SRC/params.f90:8-18, 105-142). */
#define EDYN_IF_SELECT_TIME 0     /* 0 Euler, 1 TVDRK3, (2 RK4: not supported) */
#define EDYN_IF_SELECT_RIEMANN 1  /* 0 LxF, 1 HLL, 2 HLLC */
#define EDYN_IF_FLAG_ACU 2        /* 0 first order, 1 MUSCL, 2 WENO */
#define EDYN_IF_FLAG_MUSCL 3      /* 1 unlimited, 2 minmod, 3 superbee, 4 MC */
#define EDYN_IF_FLAG_WENO 4       /* 1 WENO3-Z, 2 WENO5-JS, 3 WENO5-Z, 4 WENO7-Z */
#define EDYN_IF_FLAG_LBOUND 5     /* 0 wall, 1 inflow */
#define EDYN_IF_FLAG_RBOUND 6     /* 0 wall, 1 outflow (fixed p_OUT) */
#define EDYN_IF_DO_REACTION 7     /* 0 frozen, 1 per-cell chemistry */
#define EDYN_IF_STRICT_NEWTON 8   /* 1: T Newton starts at 1000 K every call (reference); 0: warm start */
#define EDYN_IF_CHEM_MODE 9       /* 0 plain implicit integrator, 1 surrogate with fallback */
#define EDYN_NIFLAGS 10

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
 * chem_dir: directory with CHEMKIN chem.inp + therm.dat, or with mech.edyn.
 * nspe/nequ must match the mechanism (nequ = nspe + 3). lvir is checked
 * against the scheme (SRC/params.f90:161-173). x_in: inlet mole fractions
 * (nspe values) or NULL. */
int edyn_init(const char* chem_dir, int nspe, int nequ, int ncell, int lvir, const int* iflags, int n_iflags,
              const double* rparams, int n_rparams, const double* x_in, void** ctx);

/* Uploads the interior state. qf may be NULL (then qf = QcToqf(Qc)).
 * Mirrors set_block_params filling b_obj%qf / b_obj%Qc (SRC/block.f90:394-431). */
int edyn_upload(void* ctx, const double* qf_aos, const double* qc_aos);

/* Builds the interior state from per-cell T [K], p [Pa], u [m/s] and mole
 * fractions X (ncell x nspe), as initialize_variables does for step
 * profiles (SRC/params.f90:305-580), entirely on the device. */
int edyn_init_cells(void* ctx, const double* T, const double* p, const double* u, const double* X);

/* calc_dt (SRC/update.f90:13): dt = cfl * dx / max(|u| + a). */
int edyn_calc_dt(void* ctx, double cfl, double* dt);

/* solve_fluid (SRC/update.f90:62): one explicit Euler or TVDRK3 step. */
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
 * nor writes the context's own state buffers. qf_d and qc_d are device
 * arrays in the library's device layout: nequ rows of ld = ncell + 8
 * doubles, row v holding variable v, cell i at column i + 4 (the columns
 * outside the cells are neither read nor written). On entry qf_d holds
 * QcToqf(qc_d); on return qc_d holds the state after the step and qf_d its
 * primitive variables. Returns after the step has finished on the stream.
 *
 * Tubes with 2 * nequ * (ncell + 8) > EDYN_NOALLOC_SCRATCH_DOUBLES are
 * rejected with EDYN_E_ARG and a message naming the limit. The first call
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

/* Batched reactor call: the macks(dt, nspe+1, yiT, rho) contract of
 * SRC/source.f90:58 for n independent cells in one persistent launch.
 * yiT: n x (nspe+1) [Y_1..Y_nspe, T] in/out; rho [kg/m^3]; dt [s] per cell.
 * Uses the context's mechanism and tolerances. stats (optional, 4 values):
 * total right-hand-side evaluations, steps, rejected steps, failed cells. */
int edyn_reactors(void* ctx, int n, const double* rho, const double* dt, double* yiT, double* stats);

/* Same, on device pointers already resident in GPU memory (no copies). */
int edyn_reactors_device(void* ctx, int n, const double* rho_d, const double* dt_d, double* yiT_d, double* stats);

/* Counters of the last chemistry launch of this context (tube or batch),
 * 7 values: right-hand-side evaluations, accepted steps, rejected steps,
 * failed cells, Jacobians, cells, cells integrated by a four-warp team.
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

/* Library version string. */
const char* edyn_version(void);

#ifdef __cplusplus
}
#endif
#endif
