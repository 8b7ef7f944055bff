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
#include "mechanism.h"
#include "recon.cuh"

extern "C" int edyn_mech_load_dir(const char* dir, edyn_mech* m, char* err, int errlen);
extern "C" int edyn_mech_write(const edyn_mech* m, const char* path);

namespace {

using namespace edyn;

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
  double* hrr = nullptr;
  double* staging = nullptr;
  size_t staging_bytes = 0;
  // device clock of the time loop
  double* d_time = nullptr;
  long long* d_nsteps = nullptr;
  int* d_active = nullptr;
  double* d_dt = nullptr;
  unsigned long long* d_cvel = nullptr;
  unsigned* d_err = nullptr;
  int* d_cost = nullptr;      // right-hand sides per cell in the last chemistry launch
  unsigned* d_hot = nullptr;  // cells that get a four-warp team in the next one
  double* d_hlast = nullptr;  // step size each cell's integrator proposed last
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
  std::string err;
};

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
  return a;
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
    a.cvel_out = (dev && last && last_is_fluid) ? c->d_cvel : nullptr;
    a.time = (dev && last && last_is_fluid) ? c->d_time : nullptr;
    a.nsteps = (dev && last && last_is_fluid) ? c->d_nsteps : nullptr;
    cudaError_t e = launch_stage(a, c->acu, c->lim, c->wflag, c->riemann, c->stream);
    if (e != cudaSuccess) return fail(c, EDYN_E_CUDA, "stage launch: %s", cudaGetErrorString(e));
    c->cur ^= 1;
  }
  return EDYN_OK;
}

int source_step(Ctx* c, double dt, bool dev) {
  if (!c->do_reaction) return EDYN_OK;
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
  }
  L.err = c->d_err;
  L.cost = c->d_cost;
  L.hot = c->d_hot;
  L.hlast = c->d_hlast;
  cudaError_t e = chem_launch_tube(c->use_sub ? c->chem_sub : c->chem, L, c->stream);
  if (e != cudaSuccess) return fail(c, EDYN_E_CUDA, "chemistry launch: %s", cudaGetErrorString(e));
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
  CK(launch_species_present(c->qc, c->ld, c->n, c->ns, c->d_present, c->stream));
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
  c->dx = rp(EDYN_RP_DX, 0.0);
  c->p_out = rp(EDYN_RP_P_OUT, 101325.0);
  c->t_in = rp(EDYN_RP_T_IN, 300.0);
  c->rho_u_in = rp(EDYN_RP_RHO_U_IN, 0.0);
  c->rtol = rp(EDYN_RP_RTOL, 1e-5);
  c->atol = rp(EDYN_RP_ATOL, 1e-13);
  if (c->select_time != 0 && c->select_time != 1)
    return fail(c, EDYN_E_ARG, "select_time=%d: only 0 (Euler) and 1 (TVDRK3) are provided", c->select_time);
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
  CK(cudaMalloc(&c->hrr, (size_t)ncell * sizeof(double)));
  CK(cudaMemsetAsync(c->qf[0], 0, rows * sizeof(double), c->stream));
  CK(cudaMemsetAsync(c->qf[1], 0, rows * sizeof(double), c->stream));
  CK(cudaMemsetAsync(c->qc, 0, rows * sizeof(double), c->stream));
  CK(cudaMemsetAsync(c->q0, 0, rows * sizeof(double), c->stream));
  CK(cudaMemsetAsync(c->hrr, 0, (size_t)ncell * sizeof(double), c->stream));
  CK(cudaMalloc(&c->d_time, sizeof(double)));
  CK(cudaMalloc(&c->d_nsteps, sizeof(long long)));
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
  CK(cudaMalloc(&c->d_present, 64 * sizeof(int)));
  CK(cudaMemsetAsync(c->d_hlast, 0, (size_t)ncell * sizeof(double), c->stream));
  int rc = fluid_upload_tables(c->tb, c->stream);
  if (rc == -1) return fail(c, EDYN_E_MECH, "a different mechanism is already loaded in this process");
  if (rc) return fail(c, EDYN_E_CUDA, "constant tables: %s", cudaGetErrorString((cudaError_t)rc));
  rc = chem_init(c->chem, m, c->tb, c->stream);
  if (rc) return fail(c, EDYN_E_CUDA, "chemistry tables: %s", cudaGetErrorString((cudaError_t)rc));
  CK(stage_tiling(c->acu, c->lim, c->wflag, c->riemann, c->ns, c->n, &c->stage_tc));
  CK(cudaStreamSynchronize(c->stream));
  return EDYN_OK;
}

int edyn_set_stage_tile(void* ctx, int cells) {
  Ctx* c = (Ctx*)ctx;
  if (!c || !c->qc) return EDYN_E_ARG;
  if (cells != 0 && (cells < STAGE_MIN_CELLS || cells > STAGE_MAX_CELLS))
    return fail(c, EDYN_E_ARG, "stage tile of %d cells outside [%d, %d] (0: automatic)", cells, STAGE_MIN_CELLS,
                STAGE_MAX_CELLS);
  int tc = cells;
  if (cells == 0) CK(stage_tiling(c->acu, c->lim, c->wflag, c->riemann, c->ns, c->n, &tc));
  c->stage_tc = tc;
  drop_graph(c);
  return EDYN_OK;
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
  int rc = ensure_staging(c, bytes);
  if (rc) return rc;
  CK(cudaMemcpyAsync(c->staging, qc_aos, bytes, cudaMemcpyHostToDevice, c->stream));
  CK(launch_aos_to_soa(c->staging, c->ne, c->n, c->qc, c->ld, c->stream));
  if (qf_aos) {
    CK(cudaMemcpyAsync(c->staging, qf_aos, bytes, cudaMemcpyHostToDevice, c->stream));
    CK(launch_aos_to_soa(c->staging, c->ne, c->n, c->qf[c->cur], c->ld, c->stream));
  } else {
    StageArgs a = base_args(c);
    a.qf_in = nullptr;
    a.qf_out = c->qf[c->cur];
    a.strict_newton = 1;
    CK(launch_qc_to_qf(a, c->stream));
  }
  return refresh_chem_set(c);
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
  CK(launch_init_cells(c->n, c->ns, dT, dp, du, dX, c->ns, c->qf[c->cur], c->qc, c->ld, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return refresh_chem_set(c);
}

int edyn_calc_dt(void* ctx, double cfl, double* dt) {
  Ctx* c = (Ctx*)ctx;
  if (!c || !c->qc || !dt) return EDYN_E_ARG;
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
  int rc = fluid_step(c, dt, false, true);
  if (rc) return rc;
  CK(cudaStreamSynchronize(c->stream));
  return EDYN_OK;
}

int edyn_solve_source(void* ctx, double dt, double time) {
  (void)time;
  Ctx* c = (Ctx*)ctx;
  if (!c || !c->qc) return EDYN_E_ARG;
  int rc = source_step(c, dt, false);
  if (rc) return rc;
  CK(cudaStreamSynchronize(c->stream));
  unsigned e = 0;
  CK(cudaMemcpy(&e, c->d_err, sizeof(e), cudaMemcpyDeviceToHost));
  if (e) return fail(c, (int)e, "chemistry reported status 0x%x", e);
  return EDYN_OK;
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
  double d;
  int rc = edyn_calc_dt(ctx, cfl, &d);
  if (rc) return rc;
  rc = edyn_solve_fluid(ctx, d);
  if (rc) return rc;
  rc = edyn_solve_source(ctx, d, 0.0);
  if (rc) return rc;
  rc = edyn_post_step(ctx);
  if (dt) *dt = d;
  return rc;
}

int edyn_advance(void* ctx, double cfl, double tend, long long max_steps, double* time, long long* nsteps) {
  Ctx* c = (Ctx*)ctx;
  if (!c || !c->qc || !time) return EDYN_E_ARG;
  CK(cudaMemcpyAsync(c->d_time, time, sizeof(double), cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemsetAsync(c->d_nsteps, 0, sizeof(long long), c->stream));
  CK(cudaMemsetAsync(c->d_cvel, 0, sizeof(unsigned long long), c->stream));
  CK(launch_cvel(c->qf[c->cur], c->n, c->ld, c->d_cvel, c->stream));
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
      cudaError_t e = launch_step_begin(c->d_time, tend, cfl, c->dx, c->d_cvel, c->d_active, c->d_dt, c->stream);
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
  while (t < tend && done < max_steps) {
    CK(cudaGraphLaunch(c->graph, c->stream));
    long long ns = 0;
    CK(cudaMemcpyAsync(&t, c->d_time, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(&ns, c->d_nsteps, sizeof(long long), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (ns == done) break;
    done = ns;
  }
  *time = t;
  if (nsteps) *nsteps = done;
  unsigned e = 0;
  CK(cudaMemcpy(&e, c->d_err, sizeof(e), cudaMemcpyDeviceToHost));
  if (e) return fail(c, (int)e, "device status 0x%x", e);
  return EDYN_OK;
}

int edyn_download(void* ctx, double* qf_aos, double* qc_aos, double* hrr) {
  Ctx* c = (Ctx*)ctx;
  if (!c || !c->qc) return EDYN_E_ARG;
  const size_t bytes = (size_t)c->ne * c->n * sizeof(double);
  int rc = ensure_staging(c, bytes);
  if (rc) return rc;
  if (qf_aos) {
    CK(launch_soa_to_aos(c->qf[c->cur], c->ne, c->n, c->ld, c->staging, c->stream));
    CK(cudaMemcpyAsync(qf_aos, c->staging, bytes, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
  }
  if (qc_aos) {
    CK(launch_soa_to_aos(c->qc, c->ne, c->n, c->ld, c->staging, c->stream));
    CK(cudaMemcpyAsync(qc_aos, c->staging, bytes, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
  }
  if (hrr) {
    CK(cudaMemcpyAsync(hrr, c->hrr, (size_t)c->n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
  }
  return EDYN_OK;
}

int edyn_chem_stats(void* ctx, double* stats) {
  Ctx* c = (Ctx*)ctx;
  if (!c || !c->qc || !stats) return EDYN_E_ARG;
  ChemCounters k;
  cudaError_t e = chem_read_counters(c->use_sub ? c->chem_sub : c->chem, &k, c->stream);
  if (e != cudaSuccess) return fail(c, EDYN_E_CUDA, "counters: %s", cudaGetErrorString(e));
  const unsigned long long v[7] = {k.rhs, k.steps, k.rejects, k.failed, k.jac, k.cells, k.team_cells};
  for (int i = 0; i < 7; ++i) stats[i] = (double)v[i];
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
  unsigned st = 0;
  CK(cudaMemcpy(&st, c->d_err, sizeof(st), cudaMemcpyDeviceToHost));
  if (st) {
    CK(cudaMemset(c->d_err, 0, sizeof(unsigned)));
    return fail(c, (int)st, "reactor status 0x%x", st);
  }
  return EDYN_OK;
}

int edyn_chem_rhs_device(void* ctx, int n, const double* rho_d, const double* yiT_d, double* f_d) {
  Ctx* c = (Ctx*)ctx;
  if (!c || n < 0 || (n > 0 && (!rho_d || !yiT_d || !f_d))) return EDYN_E_ARG;
  if (n == 0) return EDYN_OK;
  cudaError_t e = chem_rhs_batch(c->chem, n, rho_d, yiT_d, f_d, c->stream);
  if (e != cudaSuccess) return fail(c, EDYN_E_CUDA, "right-hand side launch: %s", cudaGetErrorString(e));
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
  cudaFree(c->qf[0]);
  cudaFree(c->qf[1]);
  cudaFree(c->qc);
  cudaFree(c->q0);
  cudaFree(c->hrr);
  cudaFree(c->staging);
  cudaFree(c->d_time);
  cudaFree(c->d_nsteps);
  cudaFree(c->d_active);
  cudaFree(c->d_dt);
  cudaFree(c->d_cvel);
  cudaFree(c->d_err);
  cudaFree(c->d_cost);
  cudaFree(c->d_hot);
  cudaFree(c->d_hlast);
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
  if (!qf_d || !qc_d || qf_d == qc_d)
    return fail(c, EDYN_E_ARG, "edyn_solve_fluid_noalloc: two distinct device arrays (qf, Qc) are required");
  if ((reinterpret_cast<uintptr_t>(qf_d) | reinterpret_cast<uintptr_t>(qc_d)) % alignof(double))
    return fail(c, EDYN_E_ARG, "edyn_solve_fluid_noalloc: qf and Qc must be 8-byte aligned");
  const size_t rows = (size_t)c->ne * c->ld;
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
  return EDYN_OK;
}
