"""The allocation-free fluid step (edyn_solve_fluid_noalloc) against the
context-owned one (edyn_solve_fluid), called through the C ABI.

Both start from the same state; the allocation-free step runs on device
arrays that the test owns, with the library's static scratch. After each of
two calls in a row the states must agree within 1e-10 relative to each
variable's magnitude, the bar of the fluid parity tests.
"""
import ctypes

import numpy as np
import pytest

from fortrancfd_gb300 import Tube, configs, edyn

pytestmark = pytest.mark.gpu

TOL = 1e-10
GHOST = 4


def _to_device(torch, aos, ld):
    """(ncell, nequ) host rows -> (nequ, ncell + 8) device rows, cell i at column i + 4."""
    n, ne = aos.shape
    t = torch.zeros((ne, ld), dtype=torch.float64, device="cuda")
    t[:, GHOST:GHOST + n] = torch.from_numpy(np.ascontiguousarray(aos.T)).to("cuda")
    return t


def _to_host(t, n):
    return t[:, GHOST:GHOST + n].T.contiguous().cpu().numpy()


def _rel(a, b):
    scale = np.maximum(np.abs(b).max(axis=0), 1e-300)
    return float((np.abs(a - b) / scale).max())


def _call(tube, qf_d, qc_d, dt):
    return edyn.lib().edyn_solve_fluid_noalloc(tube._h, ctypes.c_void_p(qf_d.data_ptr()),
                                               ctypes.c_void_p(qc_d.data_ptr()), dt)


def _sod_euler():
    case = configs.sod(ncell=316)
    case.flags.update(select_time=0)
    return case


def _detonation():
    case = configs.detonation(ncell=2000)
    case.flags.update(flag_weno=3)
    return case


def _inlet_outlet():
    """Air flowing in at the left (lbound_inlet: 300 K, 60 kg/m^2/s) into a
    pressure step, fixed-pressure outlet at the right: the ghost states that
    read the inlet data and p_out."""
    names = configs.species_names()
    x_air = configs.mole_vector(names, {"O2": 0.21, "N2": 0.79})
    n, dx = 400, 1e-3
    xm = (np.arange(n) + 0.5) * dx
    case = configs.TubeCase("inlet_outlet_air_400", n, dx, np.where(xm < 0.2, 300.0, 350.0),
                            np.where(xm < 0.2, 1.2 * 101325.0, 101325.0), np.where(xm < 0.2, 50.0, 0.0),
                            np.tile(x_air, (n, 1)),
                            dict(select_time=1, select_riemann=2, flag_acu=1, flag_muscl=2, flag_weno=0,
                                 flag_lbound=1, flag_rbound=1, do_reaction=0, p_out=101325.0, t_in=300.0,
                                 rho_u_in=60.0, x_in=x_air), cfl=0.5)
    return case


@pytest.mark.parametrize("make", [configs.sod, _detonation, _sod_euler, _inlet_outlet],
                         ids=["sod_rk3", "detonation_rk3", "sod_euler", "inlet_outlet_rk3"])
def test_noalloc_matches_solve_fluid(make):
    torch = pytest.importorskip("torch")
    case = make()
    flags = {k: v for k, v in case.flags.items() if k != "do_reaction"}
    tube = Tube(case.ncell, case.dx, do_reaction=0, **flags)
    tube.init_cells(case.T, case.p, case.u, case.X)
    qf0, qc0, _ = tube.download()
    ld = case.ncell + 2 * GHOST
    qf_d = _to_device(torch, qf0, ld)
    qc_d = _to_device(torch, qc0, ld)
    torch.cuda.synchronize()
    for _ in range(2):
        dt = tube.calc_dt(case.cfl)
        tube.solve_fluid(dt)
        rc = _call(tube, qf_d, qc_d, dt)
        assert rc == 0, tube.last_error()
        qf_ref, qc_ref, _ = tube.download()
        qf_na, qc_na = _to_host(qf_d, case.ncell), _to_host(qc_d, case.ncell)
        assert np.all(np.isfinite(qf_na)) and np.all(np.isfinite(qc_na))
        assert _rel(qc_na, qc_ref) < TOL
        assert _rel(qf_na, qf_ref) < TOL
    # the step moved the state: the comparison is not between two copies of the input
    assert _rel(qc_na, qc0) > 1e-8
    tube.close()


def test_noalloc_rejects_overlapping_arrays():
    torch = pytest.importorskip("torch")
    case = configs.sod(ncell=256)
    tube = Tube(case.ncell, case.dx)
    ld = case.ncell + 8
    buf = torch.zeros((56 * ld + 1000,), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rc = edyn.lib().edyn_solve_fluid_noalloc(tube._h, ctypes.c_void_p(buf.data_ptr()),
                                             ctypes.c_void_p(buf.data_ptr() + 8 * 1000), 1e-9)
    assert rc == edyn.EDYN_E_ARG
    assert "overlap" in tube.last_error()
    tube.close()


def test_noalloc_rejects_tubes_beyond_the_scratch():
    torch = pytest.importorskip("torch")
    case = configs.sod(ncell=9355)  # 2 * 56 * (9355 + 8) doubles > 2^20
    tube = Tube(case.ncell, case.dx)
    qf_d = torch.zeros((56, case.ncell + 8), dtype=torch.float64, device="cuda")
    qc_d = torch.zeros_like(qf_d)
    torch.cuda.synchronize()
    assert _call(tube, qf_d, qc_d, 1e-9) == edyn.EDYN_E_ARG
    assert "ncell <= 9354" in tube.last_error()
    tube.close()
