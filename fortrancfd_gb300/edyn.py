"""Python host side of the GB300 hot path.

A thin mirror of the reference's hot-path interface over the C ABI of
``include/edyn_gpu.h``: ``Tube`` stands for the reference's per-rank block
state with its calc_dt / solve_fluid / solve_source / post-step calls
(SRC/update.f90:13-150, SRC/main.f90:130-163), ``Reactors`` for the batched
``macks(dt, nspe+1, yiT, rho)`` contract (SRC/source.f90:58). Arrays follow
the reference's layout: per cell a row of ``nequ`` values
(rho, u, T, Y_1..Y_K) or (rho, rho u, rho e, rho Y_k), SI units.

The compiled library is required: importing works without it, but every
call raises ``RuntimeError`` when ``_lib/libedyn_gb300.so`` is missing. There
is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path
from typing import Optional, Sequence

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "_lib" / "libedyn_gb300.so"
GRI30_DIR = PKG / "data" / "gri30"

EDYN_OK = 0
EDYN_E_ARG, EDYN_E_CUDA, EDYN_E_MECH, EDYN_E_NEWTON, EDYN_E_CHEM, EDYN_E_STATE, EDYN_E_IO = 1, 2, 4, 8, 16, 32, 64

# the datasets of a results file's step group before the species' mole
# fractions (write_hdf5_b, SRC/write_hdf5.f90:140-162; Fortran's trim keeps
# the leading blanks)
OUTPUT_FIELDS = ("rho", "u_x", "  T", "  p", " et", " ek", " ei", "HRR", "HRD", "Qrd", " Tw", "QTw", "x_m", " dx",
                 "idx")

# iflags / rparams slots (include/edyn_gpu.h)
IF_SELECT_TIME, IF_SELECT_RIEMANN, IF_FLAG_ACU, IF_FLAG_MUSCL, IF_FLAG_WENO = 0, 1, 2, 3, 4
IF_FLAG_LBOUND, IF_FLAG_RBOUND, IF_DO_REACTION, IF_STRICT_NEWTON, IF_CHEM_MODE = 5, 6, 7, 8, 9
RP_DX, RP_P_OUT, RP_T_IN, RP_RHO_U_IN, RP_RTOL, RP_ATOL = 0, 1, 2, 3, 4, 5

_D = ctypes.POINTER(ctypes.c_double)
_lib = None


class EdynError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"edyn status {code}: {msg}")
        self.code = code


def lib() -> ctypes.CDLL:
    """Loads the in-tree GB300 library; raises if it was not built."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(
            f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`; "
            "the hot path has no CPU fallback")
    L = ctypes.CDLL(str(LIB_PATH))
    vp, ip, dp, i, d, cp = ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), _D, ctypes.c_int, ctypes.c_double, ctypes.c_char_p
    L.edyn_init.argtypes = [cp, i, i, i, i, ip, i, dp, i, dp, ctypes.POINTER(vp)]
    L.edyn_upload.argtypes = [vp, dp, dp]
    L.edyn_init_cells.argtypes = [vp, dp, dp, dp, dp]
    L.edyn_calc_dt.argtypes = [vp, d, dp]
    L.edyn_solve_fluid.argtypes = [vp, d]
    L.edyn_solve_fluid_noalloc.argtypes = [vp, vp, vp, d]
    L.edyn_solve_source.argtypes = [vp, d, d]
    L.edyn_post_step.argtypes = [vp]
    L.edyn_step.argtypes = [vp, d, dp]
    L.edyn_advance.argtypes = [vp, d, d, ctypes.c_longlong, dp, ctypes.POINTER(ctypes.c_longlong)]
    L.edyn_download.argtypes = [vp, dp, dp, dp]
    L.edyn_download_source.argtypes = [vp, dp, dp]
    L.edyn_set_chem_max_steps.argtypes = [vp, i]
    L.edyn_set_chem_launch.argtypes = [vp, i]
    L.edyn_set_chem_precheck.argtypes = [vp, i]
    L.edyn_set_uniform_skip.argtypes = [vp, i]
    L.edyn_init_tubes.argtypes = [cp, i, i, i, ip, i, ip, i, dp, i, ctypes.POINTER(vp)]
    L.edyn_init_blocks.argtypes = [cp, i, i, i, ip, dp, i, ip, i, dp, i, dp, ctypes.POINTER(vp)]
    L.edyn_tube_times.argtypes = [vp, dp, dp]
    L.edyn_autotune.argtypes = [vp, cp, ip, dp]
    L.edyn_chem_rhs_tube.argtypes = [vp, i, vp, vp, vp]
    L.edyn_set_surrogate.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, d, d, d]
    L.edyn_surrogate_stats.argtypes = [vp, dp]
    L.edyn_reactors.argtypes = [vp, i, dp, dp, dp, dp]
    L.edyn_reactors_device.argtypes = [vp, i, vp, vp, vp, dp]
    L.edyn_set_stream.argtypes = [vp, vp]
    L.edyn_chem_stats.argtypes = [vp, dp]
    L.edyn_chem_cost.argtypes = [vp, ip, ctypes.POINTER(ctypes.c_uint)]
    L.edyn_check_exp.argtypes = [vp, i, dp, dp]
    L.edyn_check_log.argtypes = [vp, i, dp, dp]
    L.edyn_set_stage_tile.argtypes = [vp, i]
    L.edyn_chem_set.argtypes = [vp, ip, ip]
    L.edyn_stage_tile.argtypes = [vp, ip, ip]
    L.edyn_last_error.argtypes = [vp, ctypes.c_char_p, i]
    L.edyn_finalize.argtypes = [vp]
    L.edyn_mech_compile.argtypes = [cp, cp, ctypes.c_char_p, i]
    L.edyn_tran_compile.argtypes = [cp, cp, ctypes.c_char_p, i]
    L.edyn_transport_properties.argtypes = [vp, dp, dp, dp]
    L.edyn_set_radiation.argtypes = [vp, i, ip, dp]
    L.edyn_set_wall_heat.argtypes = [vp, i, dp]
    L.edyn_set_ignition.argtypes = [vp, i, i, dp, dp, dp, dp]
    L.edyn_version.restype = ctypes.c_char_p
    ll, llp = ctypes.c_longlong, ctypes.POINTER(ctypes.c_longlong)
    L.edyn_output_open.argtypes = [vp, cp]
    L.edyn_output_snapshot.argtypes = [vp]
    L.edyn_output_rows.argtypes = [vp, dp]
    L.edyn_output_write.argtypes = [vp, i, ll, d, d, d, d, d]
    L.edyn_output_close.argtypes = [vp]
    L.edyn_restart.argtypes = [vp, cp, ip, llp, dp, dp]
    L.edyn_h5_create.argtypes = [cp, ctypes.POINTER(vp)]
    L.edyn_h5_add_group.argtypes = [vp, cp, i, ctypes.POINTER(cp), ip, dp, i, ctypes.POINTER(cp), dp, ll]
    L.edyn_h5_close.argtypes = [vp]
    L.edyn_h5_list.argtypes = [cp, cp, ctypes.c_char_p, ll]
    L.edyn_h5_read.argtypes = [cp, cp, dp, ll, llp]
    L.edyn_h5_attr.argtypes = [cp, cp, cp, dp, ll, llp, ctypes.c_char_p, ll]
    L.edyn_h5_attr_names.argtypes = [cp, cp, ctypes.c_char_p, ll]
    L.edyn_h5_step_name.argtypes = [i, d, ctypes.c_char_p, i]
    L.edyn_h5_error.restype = ctypes.c_char_p
    _lib = L
    return L


def _ptr(a: Optional[np.ndarray]):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_D)


def mech_compile(chem_dir: str, out_path: str) -> None:
    """CHEMKIN directory -> mech.edyn (the CKINTERP step)."""
    buf = ctypes.create_string_buffer(512)
    rc = lib().edyn_mech_compile(str(chem_dir).encode(), str(out_path).encode(), buf, 512)
    if rc:
        raise EdynError(rc, buf.value.decode())


def tran_compile(chem_dir: str, out_path: str) -> None:
    """TRANLIB linking file (chem_dir/tran.bin) -> tran.edyn, the text form
    the library and the package data use."""
    buf = ctypes.create_string_buffer(512)
    rc = lib().edyn_tran_compile(str(chem_dir).encode(), str(out_path).encode(), buf, 512)
    if rc:
        raise EdynError(rc, buf.value.decode())


def species_names(mech_dir: str | os.PathLike = GRI30_DIR) -> list:
    """Species names in mechanism order (from mech.edyn)."""
    txt = (Path(mech_dir) / "mech.edyn").read_text().split()
    i = txt.index("SPECIES")
    n = int(txt[i + 1])
    nel = int(txt[txt.index("ELEMENTS") + 1])
    per = 5 + 14 + nel
    return [txt[i + 2 + k * per] for k in range(n)]


def lvir_for(flag_acu: int, flag_weno: int) -> int:
    """Ghost depth of the scheme (SRC/params.f90:161-173)."""
    if flag_acu == 0:
        return 1
    if flag_acu == 1:
        return 2
    return {1: 2, 2: 3, 3: 3, 4: 4}[flag_weno]


class _Ctx:
    def __init__(self, chem_dir, nspe, ncell, lvir, iflags, rparams, x_in):
        L = lib()
        self._h = ctypes.c_void_p()
        fl = (ctypes.c_int * len(iflags))(*iflags)
        rp = np.ascontiguousarray(rparams, dtype=np.float64)
        xi = None if x_in is None else np.ascontiguousarray(x_in, dtype=np.float64)
        rc = L.edyn_init(str(chem_dir).encode(), nspe, nspe + 3, ncell, lvir, fl, len(iflags), _ptr(rp), len(rp),
                         _ptr(xi), ctypes.byref(self._h))
        self.nspe, self.nequ, self.ncell = nspe, nspe + 3, ncell
        if rc:
            msg = self.last_error()
            self.close()
            raise EdynError(rc, msg)

    def last_error(self) -> str:
        buf = ctypes.create_string_buffer(512)
        lib().edyn_last_error(self._h, buf, 512)
        return buf.value.decode()

    def _check(self, rc: int):
        if rc:
            raise EdynError(rc, self.last_error())

    def set_stream(self, stream_handle: int | None):
        self._check(lib().edyn_set_stream(self._h, ctypes.c_void_p(stream_handle or 0)))

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            lib().edyn_finalize(self._h)
        self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Tube(_Ctx):
    """One 1-D tube on the GPU, driven like the reference's time loop."""

    def __init__(self, ncell: int, dx: float, *, chem_dir=GRI30_DIR, select_time=1, select_riemann=2, flag_acu=1,
                 flag_muscl=2, flag_weno=0, flag_lbound=0, flag_rbound=0, do_reaction=0, strict_newton=1,
                 chem_mode=0, do_tran=0, is_spherical=0, p_out=101325.0, t_in=300.0, rho_u_in=0.0, rtol=1e-5,
                 atol=1e-13,
                 x_in: Optional[Sequence[float]] = None, nspe: Optional[int] = None):
        names = species_names(chem_dir) if (Path(chem_dir) / "mech.edyn").exists() else None
        nspe = nspe if nspe is not None else len(names)
        lv = lvir_for(flag_acu, flag_weno)
        iflags = [select_time, select_riemann, flag_acu, flag_muscl, flag_weno, flag_lbound, flag_rbound,
                  do_reaction, strict_newton, chem_mode, do_tran, is_spherical]
        super().__init__(chem_dir, nspe, ncell, lv, iflags, [dx, p_out, t_in, rho_u_in, rtol, atol], x_in)
        self.names = names if names is not None else [f"S{k + 1}" for k in range(nspe)]
        self.lvir = lv
        self.dx = dx

    def upload(self, qf: Optional[np.ndarray], qc: np.ndarray):
        qc = np.ascontiguousarray(qc, dtype=np.float64)
        qf = None if qf is None else np.ascontiguousarray(qf, dtype=np.float64)
        self._check(lib().edyn_upload(self._h, _ptr(qf), _ptr(qc)))

    def init_cells(self, T, p, u, X):
        T, p, u = (np.ascontiguousarray(a, dtype=np.float64) for a in (T, p, u))
        X = np.ascontiguousarray(X, dtype=np.float64)
        self._check(lib().edyn_init_cells(self._h, _ptr(T), _ptr(p), _ptr(u), _ptr(X)))

    def calc_dt(self, cfl: float) -> float:
        d = ctypes.c_double()
        self._check(lib().edyn_calc_dt(self._h, cfl, ctypes.byref(d)))
        return d.value

    def solve_fluid(self, dt: float):
        self._check(lib().edyn_solve_fluid(self._h, dt))

    def solve_fluid_noalloc(self, qf_ptr: int, qc_ptr: int, dt: float):
        """One fluid step on caller-owned device arrays (nequ rows of
        ncell + 8 doubles, cell i at column i + 4), allocating nothing; the
        scratch is a static device array of the library."""
        self._check(lib().edyn_solve_fluid_noalloc(self._h, ctypes.c_void_p(qf_ptr), ctypes.c_void_p(qc_ptr), dt))

    def solve_source(self, dt: float, time: float = 0.0):
        self._check(lib().edyn_solve_source(self._h, dt, time))

    def post_step(self):
        self._check(lib().edyn_post_step(self._h))

    def step(self, cfl: float) -> float:
        d = ctypes.c_double()
        self._check(lib().edyn_step(self._h, cfl, ctypes.byref(d)))
        return d.value

    def advance(self, cfl: float, tend: float, time: float = 0.0, max_steps: int = 1 << 62):
        t = ctypes.c_double(time)
        n = ctypes.c_longlong(0)
        self._check(lib().edyn_advance(self._h, cfl, tend, max_steps, ctypes.byref(t), ctypes.byref(n)))
        return t.value, n.value

    def chem_stats(self) -> dict:
        """Counters of the last chemistry launch."""
        st = np.zeros(9)
        self._check(lib().edyn_chem_stats(self._h, _ptr(st)))
        keys = ("rhs", "steps", "rejects", "failed", "jac", "cells", "team_cells", "cells32", "cells_same")
        return {k: int(v) for k, v in zip(keys, st)}

    def chem_cost(self):
        """Right-hand sides each cell took in the last chemistry launch, and
        the cells listed for four-warp teams in the next one."""
        cost = np.zeros(self.ncell, dtype=np.int32)
        hot = np.zeros(65, dtype=np.uint32)
        self._check(lib().edyn_chem_cost(self._h, cost.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                         hot.ctypes.data_as(ctypes.POINTER(ctypes.c_uint))))
        return cost, hot[1:1 + int(hot[0])].astype(np.int64)

    def chem_set(self):
        """(species, reactions) the chemistry integrates: the mechanism, or the
        subset of the elements present in the tube."""
        ns, nr = ctypes.c_int(), ctypes.c_int()
        self._check(lib().edyn_chem_set(self._h, ctypes.byref(ns), ctypes.byref(nr)))
        return ns.value, nr.value

    def set_chem_launch(self, form: int = 0) -> None:
        """Chemistry launch form: 0 automatic, 1 one pass, 2 screening pass +
        listed integration (the same results)."""
        self._check(lib().edyn_set_chem_launch(self._h, int(form)))

    def set_chem_precheck(self, on: bool = True) -> None:
        """Single-precision pre-check of the inert-cell test (on by default):
        cells it decides skip the FP64 right-hand side."""
        self._check(lib().edyn_set_chem_precheck(self._h, 1 if on else 0))

    def transport_properties(self):
        """(mu [Pa s], kappa [W/(m K)], D' [m^2/s], ncell x nspe) of the
        current state, as the transport flux evaluates them (do_tran tubes)."""
        mu = np.zeros(self.ncell)
        kap = np.zeros(self.ncell)
        dif = np.zeros((self.ncell, self.nspe))
        self._check(lib().edyn_transport_properties(self._h, _ptr(mu), _ptr(kap), _ptr(dif)))
        return mu, kap, dif

    def set_radiation(self, fits: Optional[dict] = None) -> None:
        """Optically thin radiation loss after the chemistry: {species name:
        (a0, ..., a5)} Planck-mean fits in T [1/(m atm)], as the reference's
        radiation_file; None or {} switches it off."""
        names = species_names()
        fits = fits or {}
        sp = (ctypes.c_int * max(1, len(fits)))(*[names.index(k) for k in fits])
        coef = np.ascontiguousarray([list(v) for v in fits.values()] or [[0.0] * 6], dtype=np.float64)
        self._check(lib().edyn_set_radiation(self._h, len(fits), sp, _ptr(coef)))

    def set_wall_heat(self, nu=None, d=None, tw_min=None, tw_max=None, alpha=None, beta=None) -> None:
        """Micro-flow-reactor wall heat after the chemistry (d [m], alpha
        [1/m], beta [m]); no arguments switch it off."""
        if nu is None:
            self._check(lib().edyn_set_wall_heat(self._h, 0, None))
            return
        p = np.ascontiguousarray([nu, d, tw_min, tw_max, alpha, beta], dtype=np.float64)
        self._check(lib().edyn_set_wall_heat(self._h, 1, _ptr(p)))

    def set_ignition(self, kind: int = 0, sources: Sequence = ()) -> None:
        """Ignition energy after the chemistry: kind 1 (Frendi) or 2 (Zhang),
        sources [(E [J], r [m], duration [s], start [s]), ...]; kind 0 off."""
        a = np.ascontiguousarray(list(sources) or [[0.0] * 4], dtype=np.float64).reshape(-1, 4)
        cols = [np.ascontiguousarray(a[:, j]) for j in range(4)]
        self._check(lib().edyn_set_ignition(self._h, int(kind), len(sources), *[_ptr(c) for c in cols]))

    def set_uniform_skip(self, on: bool = True) -> None:
        """Uniform regions (on by default): the fluid stage computes no faces
        for cells whose stencils hold one state, and the two-pass chemistry
        screens one cell per run of identical cells. The results are bit for
        bit the same."""
        self._check(lib().edyn_set_uniform_skip(self._h, 1 if on else 0))

    def set_stage_tile(self, cells: int = 0) -> None:
        """Cells per fluid stage tile; 0 chooses it from the tube length."""
        self._check(lib().edyn_set_stage_tile(self._h, int(cells)))

    def autotune(self, cache_path=None):
        """Measures the fluid stage tile on this tube (or reads it from the
        cache file) and keeps the fastest; returns (tile, stage ms)."""
        t, ms = ctypes.c_int(), ctypes.c_double()
        cp_ = None if cache_path is None else str(cache_path).encode()
        self._check(lib().edyn_autotune(self._h, cp_, ctypes.byref(t), ctypes.byref(ms)))
        return t.value, ms.value

    def stage_tile(self):
        """(cells per stage tile, threads per stage CTA) in use."""
        cells, threads = ctypes.c_int(), ctypes.c_int()
        self._check(lib().edyn_stage_tile(self._h, ctypes.byref(cells), ctypes.byref(threads)))
        return cells.value, threads.value

    def chem_rhs_device(self, n: int, rho_ptr: int, yiT_ptr: int, f_ptr: int):
        """FP64 right-hand sides of n reactors (device rows of nspe + 1)
        with the species set this tube's chemistry integrates."""
        self._check(lib().edyn_chem_rhs_tube(self._h, n, ctypes.c_void_p(rho_ptr), ctypes.c_void_p(yiT_ptr),
                                             ctypes.c_void_p(f_ptr)))

    def set_surrogate(self, surrogate=None, *, rtol=2.5e-4, atol=2.5e-10, etol=1e-6):
        """Puts a trained surrogate (fortrancfd_gb300.surrogate.Surrogate) in
        front of the implicit integrator of a chem_mode=1 tube; None puts
        the gated explicit increment alone there (the method without the
        network). The tube keeps a reference to the network's device
        arrays."""
        if surrogate is None:
            self._surr_keep = None
            self._check(lib().edyn_set_surrogate(self._h, *([None] * 9), rtol, atol, etol))
            return
        wt, b, norm = surrogate.mlp.device_arrays()
        self._surr_keep = (wt, b, norm)
        ptr = [ctypes.c_void_p(t.data_ptr()) for t in list(wt) + list(b) + [norm]]
        self._check(lib().edyn_set_surrogate(self._h, *ptr, surrogate.rtol, surrogate.atol, surrogate.etol))

    def surrogate_stats(self) -> dict:
        """Counters of the last surrogate source step."""
        st = np.zeros(7)
        self._check(lib().edyn_surrogate_stats(self._h, _ptr(st)))
        keys = ("handed", "accepted_network", "accepted_explicit", "fallback", "screen_rhs", "gate_rhs",
                "fallback_rhs")
        return {k: int(v) for k, v in zip(keys, st)}

    def download_source(self):
        """(HRR, HRR_dot) [W/m^3] of the last source step, one value per cell
        (SRC/source.f90:70-73)."""
        hrr = np.empty(self.ncell)
        hrr_dot = np.empty(self.ncell)
        self._check(lib().edyn_download_source(self._h, _ptr(hrr), _ptr(hrr_dot)))
        return hrr, hrr_dot

    # ---- results files: write_hdf5_b / read_hdf5_restart (SRC/write_hdf5.f90, SRC/read_hdf5.f90)
    def output_names(self) -> list:
        """Dataset names of a step group, in the rows' order."""
        return list(OUTPUT_FIELDS) + list(self.names)

    def output_open(self, path) -> None:
        """init_output: creates (truncates) the results file."""
        self._check(lib().edyn_output_open(self._h, str(path).encode()))

    def output_snapshot(self) -> None:
        """Queues set_eos_params and the rows' device-to-host copy; returns
        at once (one snapshot pending at a time)."""
        self._check(lib().edyn_output_snapshot(self._h))

    def output_rows(self) -> np.ndarray:
        """The output rows ((15 + nspe) x ncell) of the pending snapshot, or
        of one taken now."""
        rows = np.empty((len(OUTPUT_FIELDS) + self.nspe, self.ncell))
        self._check(lib().edyn_output_rows(self._h, _ptr(rows)))
        return rows

    def output_write(self, nout: int, nt: int, dt: float, time_total: float, time_restart: Optional[float] = None,
                     cpu_total: float = 0.0, cpu_restart: float = 0.0) -> None:
        """write_hdf5_b: appends the step group nout%06d_time%E11.5 with the
        pending snapshot's rows (or a snapshot taken now)."""
        tr = time_total if time_restart is None else time_restart
        self._check(lib().edyn_output_write(self._h, int(nout), int(nt), float(dt), float(time_total), float(tr),
                                            float(cpu_total), float(cpu_restart)))

    def output_close(self) -> None:
        """fin_output."""
        self._check(lib().edyn_output_close(self._h))

    def restart(self, path):
        """read_hdf5_restart: the last step group of path becomes the state.
        Returns (nout, nt, time, cpu_time) as the reference's restart sets
        them (the group's output and step numbers + 1)."""
        nout = ctypes.c_int()
        nt = ctypes.c_longlong()
        t = ctypes.c_double()
        cpu = ctypes.c_double()
        self._check(lib().edyn_restart(self._h, str(path).encode(), ctypes.byref(nout), ctypes.byref(nt),
                                       ctypes.byref(t), ctypes.byref(cpu)))
        return nout.value, nt.value, t.value, cpu.value

    def download(self):
        qf = np.empty((self.ncell, self.nequ))
        qc = np.empty((self.ncell, self.nequ))
        hrr = np.empty(self.ncell)
        self._check(lib().edyn_download(self._h, _ptr(qf), _ptr(qc), _ptr(hrr)))
        return qf, qc, hrr


class Tubes(Tube):
    """Several independent tubes advanced together in the same kernel
    launches (edyn_init_tubes): each with its own cell count, cell size,
    outlet pressure and time step; scheme and boundary kinds shared. Cells
    are numbered one tube after another in every array."""

    def __init__(self, ncells: Sequence[int], dxs: Sequence[float], *, p_outs: Optional[Sequence[float]] = None,
                 chem_dir=GRI30_DIR, select_time=1, select_riemann=2, flag_acu=2, flag_muscl=2, flag_weno=3,
                 flag_rbound=1, do_reaction=1, strict_newton=0, rtol=1e-5, atol=1e-13, do_tran=0):
        L = lib()
        names = species_names(chem_dir)
        nspe = len(names)
        lv = lvir_for(flag_acu, flag_weno)
        iflags = [select_time, select_riemann, flag_acu, flag_muscl, flag_weno, 0, flag_rbound, do_reaction,
                  strict_newton, 0, do_tran]
        nt = len(ncells)
        p_outs = [101325.0] * nt if p_outs is None else list(p_outs)
        rp = np.ascontiguousarray([[dxs[t], p_outs[t], 300.0, 0.0, rtol, atol] for t in range(nt)], dtype=np.float64)
        nc = (ctypes.c_int * nt)(*[int(v) for v in ncells])
        fl = (ctypes.c_int * len(iflags))(*iflags)
        self._h = ctypes.c_void_p()
        self.nspe, self.nequ, self.ncell = nspe, nspe + 3, int(sum(ncells))
        self.names = names
        self.ntube, self.ncells = nt, [int(v) for v in ncells]
        self.lvir, self.dx = lv, float(dxs[0])
        rc = L.edyn_init_tubes(str(chem_dir).encode(), nspe, nspe + 3, nt, nc, lv, fl, len(iflags), _ptr(rp), 6,
                               ctypes.byref(self._h))
        if rc:
            msg = self.last_error()
            self.close()
            raise EdynError(rc, msg)

    def times(self):
        """(simulated time, last dt) of every tube."""
        t = np.zeros(self.ntube)
        d = np.zeros(self.ntube)
        self._check(lib().edyn_tube_times(self._h, _ptr(t), _ptr(d)))
        return t, d

    def split(self, a: np.ndarray):
        """Per-tube views of a packed per-cell array."""
        out, i = [], 0
        for n in self.ncells:
            out.append(a[i:i + n])
            i += n
        return out


class Blocks(Tubes):
    """One domain of SMR blocks (edyn_init_blocks): segments of equal-dx
    blocks, left to right, neighbouring cell sizes equal or a factor of two
    apart, ghosts between segments by the reference's interpolation_block,
    one dt = cfl dx_comp / max(|u| + a) for all (dx_comp defaults to the
    first segment's cell size). Cells are numbered left to right; x = 0
    where the leading segments coarser than dx_comp end (the cell centres
    of the energy sources, the spherical radius and the output's x_m)."""

    def __init__(self, ncells: Sequence[int], dxs: Sequence[float], *, dx_comp: Optional[float] = None,
                 chem_dir=GRI30_DIR, select_time=1, select_riemann=2, flag_acu=1, flag_muscl=2, flag_weno=0,
                 flag_lbound=0, flag_rbound=0, do_reaction=0, strict_newton=1, do_tran=0, is_spherical=0,
                 p_out=101325.0, t_in=300.0, rho_u_in=0.0, rtol=1e-5, atol=1e-13,
                 x_in: Optional[Sequence[float]] = None):
        L = lib()
        names = species_names(chem_dir)
        nspe = len(names)
        lv = lvir_for(flag_acu, flag_weno)
        iflags = [select_time, select_riemann, flag_acu, flag_muscl, flag_weno, flag_lbound, flag_rbound, do_reaction,
                  strict_newton, 0, do_tran, is_spherical]
        nt = len(ncells)
        rp = np.ascontiguousarray([dx_comp if dx_comp is not None else dxs[0], p_out, t_in, rho_u_in, rtol, atol],
                                  dtype=np.float64)
        dx = np.ascontiguousarray(dxs, dtype=np.float64)
        nc = (ctypes.c_int * nt)(*[int(v) for v in ncells])
        fl = (ctypes.c_int * len(iflags))(*iflags)
        xi = None if x_in is None else np.ascontiguousarray(x_in, dtype=np.float64)
        self._h = ctypes.c_void_p()
        self.nspe, self.nequ, self.ncell = nspe, nspe + 3, int(sum(ncells))
        self.names = names
        self.ntube, self.ncells = nt, [int(v) for v in ncells]
        self.lvir, self.dx = lv, float(dxs[0])
        rc = L.edyn_init_blocks(str(chem_dir).encode(), nspe, nspe + 3, nt, nc, _ptr(dx), lv, fl, len(iflags),
                                _ptr(rp), 6, _ptr(xi), ctypes.byref(self._h))
        if rc:
            msg = self.last_error()
            self.close()
            raise EdynError(rc, msg)


def _set_chem_max_steps(self, max_steps: int = 0) -> None:
    """Caps the implicit integrator at max_steps steps per cell and call
    (0: the default); a cell at the cap fails with EDYN_E_CHEM."""
    self._check(lib().edyn_set_chem_max_steps(self._h, int(max_steps)))


_Ctx.set_chem_max_steps = _set_chem_max_steps


class Reactors(_Ctx):
    """Batched constant-volume reactors (the macks contract) on the GPU."""

    def __init__(self, *, chem_dir=GRI30_DIR, rtol=1e-5, atol=1e-13, chem_mode=0):
        names = species_names(chem_dir)
        iflags = [1, 2, 1, 2, 0, 0, 0, 1, 1, chem_mode]
        super().__init__(chem_dir, len(names), 16, 2, iflags, [1.0, 101325.0, 300.0, 0.0, rtol, atol], None)

    def integrate(self, rho: np.ndarray, dt: np.ndarray, yiT: np.ndarray, raise_on_fail: bool = True):
        """Advances yiT (n x (nspe+1), [Y, T]) in place; returns the counters."""
        rho = np.ascontiguousarray(rho, dtype=np.float64)
        dt = np.ascontiguousarray(dt, dtype=np.float64)
        assert yiT.dtype == np.float64 and yiT.flags["C_CONTIGUOUS"] and yiT.shape[1] == self.nspe + 1
        st = np.zeros(4)
        rc = lib().edyn_reactors(self._h, yiT.shape[0], _ptr(rho), _ptr(dt), _ptr(yiT), _ptr(st))
        if rc and raise_on_fail:
            raise EdynError(rc, self.last_error())
        return {"rhs": int(st[0]), "steps": int(st[1]), "rejects": int(st[2]), "failed": int(st[3]), "status": rc}

    def check_exp(self, x: np.ndarray) -> float:
        """Largest difference, in ulp of CUDA's exp, of the chemistry's FP64
        exponential on the arguments x (within [-700, 700])."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        out = ctypes.c_double()
        self._check(lib().edyn_check_exp(self._h, len(x), _ptr(x), ctypes.byref(out)))
        return out.value

    def check_log(self, x: np.ndarray) -> float:
        """Largest difference, in ulp of CUDA's log, of the chemistry's FP64
        natural logarithm on the positive arguments x."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        out = ctypes.c_double()
        self._check(lib().edyn_check_log(self._h, len(x), _ptr(x), ctypes.byref(out)))
        return out.value

    def integrate_device(self, n: int, rho_ptr: int, dt_ptr: int, yiT_ptr: int):
        st = np.zeros(4)
        rc = lib().edyn_reactors_device(self._h, n, ctypes.c_void_p(rho_ptr), ctypes.c_void_p(dt_ptr),
                                        ctypes.c_void_p(yiT_ptr), _ptr(st))
        self._check(rc)
        return {"rhs": int(st[0]), "steps": int(st[1]), "rejects": int(st[2]), "failed": int(st[3])}


# ---- HDF5 files without a solver context (include/edyn_h5.h) ----
def output_path(savedir, nout: int) -> str:
    """init_output's file name: ./<savedir>/results_nout%06d.h5."""
    return f"./{savedir}/results_nout{int(nout):06d}.h5"


def step_group_name(nout: int, time: float) -> str:
    """write_hdf5_b's group name: ("nout",i6.6,"_time",e11.5)."""
    buf = ctypes.create_string_buffer(64)
    _h5_check(lib().edyn_h5_step_name(int(nout), float(time), buf, 64))
    return buf.value.decode()


def _h5_check(rc: int):
    if rc:
        raise EdynError(rc, lib().edyn_h5_error().decode())


class H5Writer:
    """A results-format file: step groups of float64 rows with one-element
    float64 (Python float) or int32 (Python int) attributes."""

    def __init__(self, path):
        self._h = ctypes.c_void_p()
        _h5_check(lib().edyn_h5_create(str(path).encode(), ctypes.byref(self._h)))

    def add_group(self, name: str, attrs: dict, rows: dict) -> None:
        an = list(attrs)
        a_names = (ctypes.c_char_p * max(len(an), 1))(*[a.encode() for a in an])
        a_int = (ctypes.c_int * max(len(an), 1))(*[int(isinstance(attrs[a], (int, np.integer))) for a in an])
        a_val = np.array([float(attrs[a]) for a in an] or [0.0])
        rn = list(rows)
        n = len(rows[rn[0]]) if rn else 0
        data = np.ascontiguousarray(np.array([np.asarray(rows[r], dtype=np.float64) for r in rn]).reshape(len(rn), n))
        r_names = (ctypes.c_char_p * max(len(rn), 1))(*[r.encode() for r in rn])
        _h5_check(lib().edyn_h5_add_group(self._h, name.encode(), len(an), a_names, a_int, _ptr(a_val), len(rn),
                                          r_names, _ptr(data) if data.size else None, n))

    def close(self) -> None:
        if self._h.value:
            _h5_check(lib().edyn_h5_close(self._h))
        self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def _h5_text(fn, *args) -> str:
    size = 1 << 16
    while True:
        buf = ctypes.create_string_buffer(size)
        rc = fn(*args, buf, size)
        if rc == EDYN_E_ARG and "too small" in lib().edyn_h5_error().decode() and size < (1 << 28):
            size *= 4
            continue
        _h5_check(rc)
        return buf.value.decode()


def h5_list(path, group: str = "") -> list:
    """Members of a group in its index (name) order; groups end with '/'."""
    return _h5_text(lib().edyn_h5_list, str(path).encode(), group.encode()).splitlines()


def h5_read(path, dataset: str) -> np.ndarray:
    n = ctypes.c_longlong()
    _h5_check(lib().edyn_h5_read(str(path).encode(), dataset.encode(), None, 0, ctypes.byref(n)))
    out = np.empty(n.value)
    _h5_check(lib().edyn_h5_read(str(path).encode(), dataset.encode(), _ptr(out), n.value, ctypes.byref(n)))
    return out


def h5_attr(path, obj: str, name: str):
    """An attribute's values (an array), or its text for string attributes."""
    n = ctypes.c_longlong()
    buf = ctypes.create_string_buffer(1 << 12)
    _h5_check(lib().edyn_h5_attr(str(path).encode(), obj.encode(), name.encode(), None, 0, ctypes.byref(n), buf,
                                 1 << 12))
    if n.value == 0 and buf.value:
        return buf.value.decode()
    out = np.empty(n.value)
    _h5_check(lib().edyn_h5_attr(str(path).encode(), obj.encode(), name.encode(), _ptr(out), n.value,
                                 ctypes.byref(n), None, 0))
    return out


def h5_attr_names(path, obj: str) -> list:
    return _h5_text(lib().edyn_h5_attr_names, str(path).encode(), obj.encode()).splitlines()
