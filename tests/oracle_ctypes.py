"""ctypes binding of the CPU oracle (oracle/_build/libedyn_oracle.so).

Test infrastructure only: the oracle is the checker the GPU library is
compared with, never part of the product path.
"""
from __future__ import annotations

import ctypes
import subprocess
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
ORACLE_SO = ROOT / "oracle" / "_build" / "libedyn_oracle.so"
MECH = ROOT / "fortrancfd_gb300" / "data" / "gri30" / "mech.edyn"
TRAN = ROOT / "fortrancfd_gb300" / "data" / "gri30" / "tran.edyn"
_D = ctypes.POINTER(ctypes.c_double)


def _p(a):
    return None if a is None else np.ascontiguousarray(a).ctypes.data_as(_D)


class Oracle:
    def __init__(self, mech_path: Path = MECH):
        if not ORACLE_SO.exists():
            subprocess.run(["make", "-s", "-C", str(ROOT / "oracle")], check=True)
        L = ctypes.CDLL(str(ORACLE_SO))
        self.L = L
        self.mech = ctypes.create_string_buffer(L.or_mech_sizeof())
        assert L.or_mech_load(str(mech_path).encode(), self.mech) == 0
        vp, d, i = ctypes.c_void_p, ctypes.c_double, ctypes.c_int
        L.or_tube_create.restype = vp
        L.or_tube_create.argtypes = [vp, i, i, ctypes.POINTER(i), _D, _D]
        L.or_tube_destroy.argtypes = [vp]
        L.or_tube_set_interior.argtypes = [vp, _D, _D]
        L.or_tube_get_interior.argtypes = [vp, _D, _D]
        L.or_tube_get_source.argtypes = [vp, _D, _D]
        L.or_output_rows.argtypes = [vp, _D]
        L.or_ckcdyr.argtypes = [vp, d, d, _D, _D, _D]
        L.or_calc_dt.restype = d
        L.or_calc_dt.argtypes = [vp, d]
        L.or_solve_fluid.argtypes = [vp, d]
        L.or_solve_source.argtypes = [vp, d]
        L.or_post_step.argtypes = [vp]
        L.or_step.restype = d
        L.or_step.argtypes = [vp, d]
        L.or_init_cell.argtypes = [vp, d, d, d, _D, _D, _D]
        L.or_reactor.restype = i
        L.or_reactor.argtypes = [vp, d, d, _D, d, d, ctypes.c_void_p]
        L.or_reactor_batch.restype = i
        L.or_reactor_batch.argtypes = [vp, i, _D, _D, _D, d, d, i, ctypes.POINTER(ctypes.c_long)]
        L.or_chem_rhs.argtypes = [vp, d, _D, _D]
        L.or_ckwyr.argtypes = [vp, d, d, _D, _D]
        L.or_ckrop.argtypes = [vp, d, d, _D, _D, _D]
        L.or_cksmh.argtypes = [vp, d, _D]
        L.or_ckhms.argtypes = [vp, d, _D]
        L.or_ckhml.argtypes = [vp, d, _D]
        L.or_ckuml.argtypes = [vp, d, _D]
        L.or_ckcpml.argtypes = [vp, d, _D]
        L.or_ckcvml.argtypes = [vp, d, _D]
        L.or_ckytx.argtypes = [vp, _D, _D]
        L.or_ckxty.argtypes = [vp, _D, _D]
        L.or_temperature_con.restype = d
        L.or_temperature_con.argtypes = [vp, d, _D, ctypes.POINTER(i)]
        L.or_specific_energy.restype = d
        L.or_specific_energy.argtypes = [vp, d, _D]
        L.or_pressure.restype = d
        L.or_pressure.argtypes = [vp, d, d, _D]
        L.or_density.restype = d
        L.or_density.argtypes = [vp, d, d, _D]
        L.or_cv.restype = d
        L.or_cv.argtypes = [vp, d, _D]
        L.or_cp.restype = d
        L.or_cp.argtypes = [vp, d, _D]
        L.or_qc_to_qf.argtypes = [vp, _D, _D]
        L.or_qf_to_qc.argtypes = [vp, _D, _D]
        L.or_muscl3.argtypes = [_D, _D, _D, i]
        L.or_weno5.argtypes = [_D, _D, _D, i]
        L.or_weno3z.argtypes = [_D, _D, _D]
        L.or_weno7z.argtypes = [_D, _D, _D]
        L.or_adjust_sum.argtypes = [i, _D]
        L.or_num_threads.restype = i
        self.tran = ctypes.create_string_buffer(L.or_tran_sizeof())
        assert L.or_tran_load(str(TRAN).encode(), self.tran) == 0
        for fn in ("or_mcsvis", "or_mcscon"):
            getattr(L, fn).argtypes = [vp, d, _D]
        L.or_mcsdif.argtypes = [vp, d, d, _D]
        for fn in ("or_mcavis", "or_mcacon"):
            getattr(L, fn).argtypes = [vp, d, _D, _D]
        L.or_mcadif.argtypes = [vp, d, d, _D, _D]
        for fn in ("or_viscosity", "or_thermal_conductivity"):
            getattr(L, fn).restype = d
            getattr(L, fn).argtypes = [vp, d, _D]
        L.or_diffusivity.argtypes = [vp, d, d, _D, _D]
        L.or_tran_cell.argtypes = [vp, vp, _D, _D, _D, _D, _D, _D, _D, _D]
        L.or_face_flux_tran.argtypes = [vp, vp, _D, _D, d, _D]
        L.or_tube_set_transport.argtypes = [vp, vp]
        L.or_tube_set_sources.argtypes = [vp, vp]
        L.or_tube_set_time.argtypes = [vp, d]
        L.or_sources_sizeof.restype = i
        L.or_tube_set_spherical.argtypes = [vp, i]
        L.or_smr_create.restype = vp
        L.or_smr_create.argtypes = [vp, i, ctypes.POINTER(i), _D, i, ctypes.POINTER(i), _D, _D]
        L.or_smr_destroy.argtypes = [vp]
        L.or_smr_set_interior.argtypes = [vp, _D, _D]
        L.or_smr_get_interior.argtypes = [vp, _D, _D]
        L.or_smr_step.restype = d
        L.or_smr_step.argtypes = [vp, d]
        L.or_smr_segment_all.argtypes = [vp, i, _D]
        L.or_smr_set_transport.argtypes = [vp, vp]
        L.or_smr_set_spherical.argtypes = [vp, ctypes.c_int]
        L.or_smr_set_sources.argtypes = [vp, vp]
        L.or_smr_set_time.argtypes = [vp, d]
        L.or_smr_output_rows.argtypes = [vp, ctypes.c_int, _D]
        self.kk = 53
        self.nequ = self.kk + 3

    # --- per-point helpers
    def vec(self, fn, T):
        out = np.zeros(self.kk)
        getattr(self.L, fn)(self.mech, T, _p(out))
        return out

    def chem_rhs(self, rho_cgs, yiT):
        """d(Y_1..Y_K, T)/dt of a constant-volume adiabatic reactor (the
        function the FP64 reference integrator advances)."""
        out = np.zeros(self.kk + 1)
        self.L.or_chem_rhs(self.mech, rho_cgs, _p(np.ascontiguousarray(yiT, dtype=float)), _p(out))
        return out

    def cdot_ddot(self, rho_cgs, T, Y):
        """CKCDYR: molar creation and destruction rates [mol/cm^3/s]."""
        c = np.zeros(self.kk)
        d = np.zeros(self.kk)
        self.L.or_ckcdyr(self.mech, rho_cgs, T, _p(np.ascontiguousarray(Y, dtype=float)), _p(c), _p(d))
        return c, d

    def wdot(self, rho_cgs, T, Y):
        out = np.zeros(self.kk)
        self.L.or_ckwyr(self.mech, rho_cgs, T, _p(np.ascontiguousarray(Y, dtype=float)), _p(out))
        return out

    def rop(self, rho_cgs, T, Y, nr=325):
        qf = np.zeros(nr)
        qr = np.zeros(nr)
        self.L.or_ckrop(self.mech, rho_cgs, T, _p(np.ascontiguousarray(Y, dtype=float)), _p(qf), _p(qr))
        return qf, qr

    # --- transport (TRANLIB mixture rules, cgs unless noted)
    def pure_viscosity(self, T):
        return self.vec2("or_mcsvis", T)

    def pure_conductivity(self, T):
        return self.vec2("or_mcscon", T)

    def vec2(self, fn, T):
        out = np.zeros(self.kk)
        getattr(self.L, fn)(self.tran, T, _p(out))
        return out

    def binary_diffusion(self, p_cgs, T):
        out = np.zeros((self.kk, self.kk))
        self.L.or_mcsdif(self.tran, p_cgs, T, _p(out))
        return out

    def mix_viscosity(self, T, X):
        out = np.zeros(1)
        self.L.or_mcavis(self.tran, T, _p(np.ascontiguousarray(X, dtype=float)), _p(out))
        return out[0]

    def mix_conductivity(self, T, X):
        out = np.zeros(1)
        self.L.or_mcacon(self.tran, T, _p(np.ascontiguousarray(X, dtype=float)), _p(out))
        return out[0]

    def mix_diffusion(self, p_cgs, T, X):
        out = np.zeros(self.kk)
        self.L.or_mcadif(self.tran, p_cgs, T, _p(np.ascontiguousarray(X, dtype=float)), _p(out))
        return out

    def tran_cell(self, qc):
        """calc_flux_tran's per-cell state from a conserved column:
        (rho, u, T, Y, mu [Pa s], kappa [W/(m K)], D' [m^2/s])."""
        sc = [np.zeros(1) for _ in range(5)]
        y = np.zeros(self.kk)
        dif = np.zeros(self.kk)
        self.L.or_tran_cell(self.mech, self.tran, _p(np.ascontiguousarray(qc, dtype=float)), _p(sc[0]), _p(sc[1]),
                            _p(sc[2]), _p(y), _p(sc[3]), _p(sc[4]), _p(dif))
        return sc[0][0], sc[1][0], sc[2][0], y, sc[3][0], sc[4][0], dif

    def face_flux_tran(self, qcl, qcr, dx):
        g = np.zeros(self.nequ)
        self.L.or_face_flux_tran(self.mech, self.tran, _p(np.ascontiguousarray(qcl, dtype=float)),
                                 _p(np.ascontiguousarray(qcr, dtype=float)), dx, _p(g))
        return g

    def init_cells(self, T, p, u, X):
        n = len(T)
        qf = np.zeros((n, self.nequ))
        qc = np.zeros((n, self.nequ))
        for i in range(n):
            x = np.ascontiguousarray(X[i], dtype=float)
            self.L.or_init_cell(self.mech, float(T[i]), float(p[i]), float(u[i]), _p(x), qf[i].ctypes.data_as(_D),
                                qc[i].ctypes.data_as(_D))
        return qf, qc

    def tube(self, n, lvir, flags, rparams, x_in=None):
        fl = (ctypes.c_int * 8)(*flags[:8])
        rp = np.ascontiguousarray(rparams, dtype=float)
        xi = np.zeros(self.kk) if x_in is None else np.ascontiguousarray(x_in, dtype=float)
        h = self.L.or_tube_create(self.mech, n, lvir, fl, _p(rp), _p(xi))
        return OracleTube(self, h, n, (rp, xi))

    def smr(self, ncells, dxs, lvir, flags, rparams, x_in=None):
        """SMR blocks: segments of ncells[s] cells of size dxs[s], left to
        right, one dt from dx_comp = rparams[0]."""
        nc = (ctypes.c_int * len(ncells))(*ncells)
        dx = np.ascontiguousarray(dxs, dtype=float)
        fl = (ctypes.c_int * 8)(*flags[:8])
        rp = np.ascontiguousarray(rparams, dtype=float)
        xi = np.zeros(self.kk) if x_in is None else np.ascontiguousarray(x_in, dtype=float)
        h = self.L.or_smr_create(self.mech, len(ncells), nc, _p(dx), lvir, fl, _p(rp), _p(xi))
        return OracleSMR(self, h, int(sum(ncells)), (nc, dx, rp, xi))

    def reactor(self, rho_si, dt, yiT, rtol, atol):
        y = np.ascontiguousarray(yiT, dtype=float).copy()
        rc = self.L.or_reactor(self.mech, rho_si, dt, _p(y), rtol, atol, ctypes.c_void_p(
            ctypes.addressof(ctypes.create_string_buffer(64))))
        return y, rc

    def reactor_batch(self, rho, dt, yiT, rtol, atol, nthreads=0):
        y = np.ascontiguousarray(yiT, dtype=float).copy()
        rhs = ctypes.c_long(0)
        fails = self.L.or_reactor_batch(self.mech, len(rho), _p(np.ascontiguousarray(rho, dtype=float)),
                                        _p(np.ascontiguousarray(dt, dtype=float)), _p(y), rtol, atol, nthreads,
                                        ctypes.byref(rhs))
        return y, fails, rhs.value


class Sources(ctypes.Structure):
    """or_sources: the energy sources of solve_source after the chemistry."""
    _fields_ = [("nrad", ctypes.c_int), ("rad_sp", ctypes.c_int * 16), ("rad_coef", (ctypes.c_double * 6) * 16),
                ("wall", ctypes.c_int), ("nu", ctypes.c_double), ("d_m", ctypes.c_double),
                ("tw_min", ctypes.c_double), ("tw_max", ctypes.c_double), ("alpha", ctypes.c_double),
                ("beta", ctypes.c_double), ("tran", ctypes.c_void_p), ("ig_type", ctypes.c_int),
                ("n_ig", ctypes.c_int), ("ig_e", ctypes.c_double * 8), ("ig_r", ctypes.c_double * 8),
                ("ig_t", ctypes.c_double * 8), ("ig_t0", ctypes.c_double * 8)]


class OracleTube:
    def __init__(self, o: Oracle, h, n, keep):
        self.o, self.h, self.n, self._keep = o, h, n, keep

    def set_interior(self, qf, qc):
        self.o.L.or_tube_set_interior(self.h, _p(np.ascontiguousarray(qf)), _p(np.ascontiguousarray(qc)))

    def get(self):
        qf = np.zeros((self.n, self.o.nequ))
        qc = np.zeros((self.n, self.o.nequ))
        self.o.L.or_tube_get_interior(self.h, _p(qf), _p(qc))
        return qf, qc

    def source(self):
        """(HRR, HRR_dot) of the last source step."""
        hrr = np.zeros(self.n)
        hrr_dot = np.zeros(self.n)
        self.o.L.or_tube_get_source(self.h, _p(hrr), _p(hrr_dot))
        return hrr, hrr_dot

    def step(self, cfl):
        return self.o.L.or_step(self.h, cfl)

    def output_rows(self):
        """set_eos_params + write_hdf5_b's rows: (15 + nspe) x n."""
        rows = np.zeros((15 + self.o.nequ - 3, self.n))
        self.o.L.or_output_rows(self.h, _p(rows))
        return rows

    def set_sources(self, radiation=None, wall=None, ignition=None):
        """radiation: [(species index, 6 fit coefficients)]; wall: (Nu, d, Tw_min,
        Tw_max, alpha, beta); ignition: (type, [(E, r, duration, start)])."""
        self._src = make_sources(self.o, radiation, wall, ignition)
        self.o.L.or_tube_set_sources(self.h, ctypes.byref(self._src))

    def set_time(self, time):
        self.o.L.or_tube_set_time(self.h, time)

    def set_spherical(self, on=True):
        """is_spherical = 1: r = (i + 1/2) dx."""
        self.o.L.or_tube_set_spherical(self.h, 1 if on else 0)

    def set_transport(self, on=True):
        """do_tran = 1: calc_flux_tran joins every stage's flux."""
        self.o.L.or_tube_set_transport(self.h, self.o.tran if on else None)

    def calc_dt(self, cfl):
        return self.o.L.or_calc_dt(self.h, cfl)

    def solve_fluid(self, dt):
        self.o.L.or_solve_fluid(self.h, dt)

    def solve_source(self, dt):
        self.o.L.or_solve_source(self.h, dt)

    def post_step(self):
        self.o.L.or_post_step(self.h)

    def __del__(self):
        try:
            self.o.L.or_tube_destroy(self.h)
        except Exception:
            pass


def make_sources(o, radiation=None, wall=None, ignition=None):
    """The oracle's or_sources from radiation [(species, 6 coefficients)],
    wall (Nu, d, Tw_min, Tw_max, alpha, beta) and ignition (type, [(E, r,
    duration, start)])."""
    s = Sources()
    for r, (k, c) in enumerate(radiation or []):
        s.rad_sp[r] = k
        for n in range(6):
            s.rad_coef[r][n] = c[n]
    s.nrad = len(radiation or [])
    if wall is not None:
        s.wall = 1
        s.nu, s.d_m, s.tw_min, s.tw_max, s.alpha, s.beta = wall
        s.tran = ctypes.addressof(o.tran)
    if ignition is not None:
        s.ig_type = ignition[0]
        s.n_ig = len(ignition[1])
        for g, (e, r, d, t0) in enumerate(ignition[1]):
            s.ig_e[g], s.ig_r[g], s.ig_t[g], s.ig_t0[g] = e, r, d, t0
    return s


class OracleSMR:
    def __init__(self, o: Oracle, h, n, keep):
        self.o, self.h, self.n, self._keep = o, h, n, keep

    def set_interior(self, qf, qc):
        self.o.L.or_smr_set_interior(self.h, _p(np.ascontiguousarray(qf)), _p(np.ascontiguousarray(qc)))

    def get(self):
        qf = np.zeros((self.n, self.o.nequ))
        qc = np.zeros((self.n, self.o.nequ))
        self.o.L.or_smr_get_interior(self.h, _p(qf), _p(qc))
        return qf, qc

    def step(self, cfl):
        return self.o.L.or_smr_step(self.h, cfl)

    def set_transport(self, on=True):
        self.o.L.or_smr_set_transport(self.h, self.o.tran if on else None)

    def set_spherical(self, on=True):
        self.o.L.or_smr_set_spherical(self.h, 1 if on else 0)

    def set_sources(self, radiation=None, wall=None, ignition=None):
        self._src = make_sources(self.o, radiation, wall, ignition)
        self.o.L.or_smr_set_sources(self.h, ctypes.byref(self._src))

    def set_time(self, time):
        self.o.L.or_smr_set_time(self.h, time)

    def output_rows(self, ncells):
        """The output rows of the whole domain, segment after segment."""
        parts = []
        for g, n in enumerate(ncells):
            rows = np.zeros((15 + self.o.nequ - 3, n))
            self.o.L.or_smr_output_rows(self.h, g, _p(rows))
            parts.append(rows)
        return np.hstack(parts)

    def segment_all(self, g, n, lvir):
        """Segment g's conserved columns with its ghosts."""
        qc = np.zeros((n + 2 * lvir, self.o.nequ))
        self.o.L.or_smr_segment_all(self.h, g, _p(qc))
        return qc

    def __del__(self):
        try:
            self.o.L.or_smr_destroy(self.h)
        except Exception:
            pass
