"""The fluid kernels' own source on the CPU (test infrastructure, tests/emu):
fortrancfd_gb300/csrc/fluid.cu translated for the host and run through a
CTA emulation (a fiber per thread, __syncthreads, warp shuffles and
__syncwarp honoured, shared memory poisoned with NaN before every CTA),
checked against the oracle on the paths whose device code has not yet run
on a GPU: spherical geometry, transport with every time integrator and in
packed tubes, the energy sources and the output rows. The emulation does
not contract a*b + c into FMAs as nvcc does, so it agrees with the GPU to
rounding, not bit for bit; the bar against the oracle is the GPU tests'
1e-10 (here met at ~1e-14). It checks the kernels' index logic, their
synchronisation and their arithmetic, not the hardware.
"""
import ctypes
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from fortrancfd_gb300 import configs, species_names
from test_sources import RAD_FITS

ROOT = Path(__file__).resolve().parent.parent
CSRC = ROOT / "fortrancfd_gb300" / "csrc"
EMU = Path(__file__).resolve().parent / "emu"
CUDA_INC = Path("/usr/local/cuda/include")
R_SI = 8314.51
_D = ctypes.POINTER(ctypes.c_double)


def _p(a):
    return a.ctypes.data_as(_D)


@pytest.fixture(scope="module")
def emu(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx or not (CUDA_INC / "cuda_runtime_api.h").exists():
        pytest.skip("needs g++ and the CUDA headers")
    import sys
    sys.path.insert(0, str(EMU))
    from host_source import host_source
    d = tmp_path_factory.mktemp("emu")
    (d / "fluid_host.inc").write_text(host_source((CSRC / "fluid.cu").read_text()))
    so = d / "libkernel_host.so"
    cmd = [gxx, "-std=c++17", "-O1", "-ffp-contract=off", "-fPIC", "-shared", "-fvisibility=hidden",
           "-Wl,-Bsymbolic", "-w", f"-I{CUDA_INC}", f"-I{CSRC}",
           f"-I{d}", "-o", str(so), str(EMU / "kernel_host.cpp"), str(CSRC / "mechanism.cpp"),
           str(CSRC / "transport.cpp")]
    subprocess.run(cmd, check=True, capture_output=True)
    L = ctypes.CDLL(str(so))
    assert L.emu_setup(str(ROOT / "fortrancfd_gb300" / "data" / "gri30").encode()) == 0
    return L


def layer(oracle, n, dx, u0=0.0):
    """Burnt gas on the left third, fresh CH4/air beyond, a pressure step
    and a velocity field: every flux term at work."""
    nm = species_names()
    fresh = configs.ch4_air_mixture(nm, 1.0)
    prod = configs.equilibrium_tp(fresh, 2000.0, configs.ATM)
    xm = (np.arange(n) + 0.5) * dx
    w = 0.5 * (1 + np.tanh((0.3 * n * dx - xm) / (4 * dx)))
    X = (1 - w)[:, None] * fresh[None, :] + w[:, None] * prod[None, :]
    return oracle.init_cells(300.0 + 1700.0 * w, configs.ATM * (1 + 0.5 * w), u0 * np.sin(xm / (n * dx) * 5), X)


def oracle_tube(oracle, n, dx, fl, qf, qc):
    st, rm, acu, mus, weno, rb, tran, sph = fl
    lv = 1 if acu == 0 else 2 if acu == 1 else {1: 2, 2: 3, 3: 3, 4: 4}[weno]
    t = oracle.tube(n, lv, [st, rm, acu, mus, weno, 0, rb, 0], [dx, configs.ATM, 300.0, 0.0, 1e-5, 1e-13])
    if tran:
        t.set_transport()
    if sph:
        t.set_spherical()
    t.set_interior(qf, qc)
    return t


def oracle_steps(oracle, t, steps, cfl):
    dts = []
    for _ in range(steps):
        d = oracle.L.or_calc_dt(t.h, cfl)
        oracle.L.or_solve_fluid(t.h, d)
        oracle.L.or_post_step(t.h)
        dts.append(d)
    return np.array(dts)


def emu_fluid(L, ncells, dxs, packed, fl, qf, qc, dts, dx_comp=None):
    nt = len(ncells)
    qc_io = np.ascontiguousarray(qc.copy())
    qf_out = np.zeros_like(qf)
    err = ctypes.c_uint()
    dxc = dxs[0] if dx_comp is None else dx_comp
    rc = L.emu_fluid(nt, (ctypes.c_int * nt)(*ncells), _p(np.ascontiguousarray(dxs, dtype=float)), packed,
                     ctypes.c_double(dxc), (ctypes.c_int * 8)(*fl), ctypes.c_double(configs.ATM),
                     _p(np.ascontiguousarray(qf)), _p(qc_io), _p(qf_out), len(dts) // nt,
                     _p(np.ascontiguousarray(dts, dtype=float)), ctypes.byref(err))
    assert rc == 0, rc
    return qf_out, qc_io, err.value


def close(qf_e, qf_o, tol):
    W = configs.molecular_weights()

    def pres(q):
        return q[:, 0] * R_SI * q[:, 2] * (q[:, 3:] / W).sum(axis=1)

    assert np.all(np.isfinite(qf_e))
    assert np.max(np.abs(pres(qf_e) - pres(qf_o)) / pres(qf_o)) < tol
    assert np.max(np.abs(qf_e[:, 2] - qf_o[:, 2]) / qf_o[:, 2]) < tol
    assert np.max(np.abs(qf_e[:, 0] - qf_o[:, 0]) / qf_o[:, 0]) < tol
    assert np.max(np.abs(qf_e[:, 1] - qf_o[:, 1])) / max(np.abs(qf_o[:, 1]).max(), 1e-300) < tol
    assert np.max(np.abs(qf_e[:, 3:] - qf_o[:, 3:])) / qf_o[:, 3:].max() < tol


# select_time, riemann, flag_acu, flag_muscl, flag_weno, flag_rbound, do_tran, is_spherical
CASES = [
    ((1, 2, 1, 2, 0, 1, 0, 1), 0.0),  # spherical: TVDRK3, HLLC, MUSCL-minmod, outlet
    ((0, 1, 1, 4, 0, 0, 0, 1), 0.0),  # spherical: Euler, HLL, MUSCL-MC, wall
    ((1, 0, 0, 2, 0, 1, 0, 1), 0.0),  # spherical: first order, LxF
    ((1, 2, 1, 2, 0, 1, 1, 0), 5.0),  # transport: planar, TVDRK3
    ((1, 2, 1, 2, 0, 1, 1, 1), 5.0),  # transport: spherical
    ((0, 2, 2, 0, 3, 0, 1, 0), 5.0),  # transport: Euler, WENO5-Z, walls
    ((1, 1, 2, 0, 4, 1, 1, 0), 5.0),  # transport: WENO7-Z, HLL
]


@pytest.mark.parametrize("fl,u0", CASES)
def test_stage_kernels_match_oracle(emu, oracle, fl, u0):
    n, dx = 64, 2e-5
    qf, qc = layer(oracle, n, dx, u0)
    t = oracle_tube(oracle, n, dx, fl, qf, qc)
    dts = oracle_steps(oracle, t, 6, 0.4)
    qf_o, _ = t.get()
    assert np.abs(qf_o[:, 2] - qf[:, 2]).max() > 5.0  # the state moved
    qf_e, _, err = emu_fluid(emu, [n], [dx], 0, fl, qf, qc, dts)
    assert err == 0
    close(qf_e, qf_o, 1e-10)


def test_packed_tubes_with_transport(emu, oracle):
    """Two packed tubes with transport (different cells, sizes and time
    steps) against the same tubes alone: bit for bit; against the oracle
    within 1e-10."""
    fl = (1, 2, 1, 2, 0, 0, 1, 0)
    cases = [(96, 1e-5, 0.0), (128, 2e-5, 8.0)]
    states = [layer(oracle, n, dx, u0) for n, dx, u0 in cases]
    dts = []
    outs = []
    for (n, dx, _), (qf, qc) in zip(cases, states):
        t = oracle_tube(oracle, n, dx, fl, qf, qc)
        dts.append(oracle_steps(oracle, t, 4, 0.5))
        outs.append(t.get()[0])
    dt_packed = np.column_stack(dts).ravel()
    qf_all = np.vstack([s[0] for s in states])
    qc_all = np.vstack([s[1] for s in states])
    qf_p, _, err = emu_fluid(emu, [c[0] for c in cases], [c[1] for c in cases], 1, fl, qf_all, qc_all, dt_packed)
    assert err == 0
    first = 0
    for (n, dx, _), (qf, qc), d, qf_o in zip(cases, states, dts, outs):
        qf_s, _, _ = emu_fluid(emu, [n], [dx], 0, fl, qf, qc, d)
        np.testing.assert_array_equal(qf_p[first:first + n], qf_s)
        close(qf_p[first:first + n], qf_o, 1e-10)
        first += n


def test_energy_sources_match_oracle(emu, oracle):
    nm = species_names()
    n, dx, dt, time = 48, 2e-5, 1e-7, 5e-8
    qf, qc = layer(oracle, n, dx)
    rad = [(nm.index(k), c) for k, c in RAD_FITS.items()]
    wall = (4.0, 2e-3, 373.0, 1300.0, 2e4, 0.5 * n * dx)
    for ig in ((1, [(5e-4, 3e-4, 1e-4, 0.0)]), (2, [(2e-6, 3e-4, 1e-6, 0.0), (1e-6, 1e-4, 1e-6, 1e-8)])):
        t = oracle_tube(oracle, n, dx, (1, 2, 1, 2, 0, 0, 0, 0), qf, qc)
        t.set_sources(radiation=rad, wall=wall, ignition=ig)
        t.set_time(time)
        t.solve_source(dt)
        qf_o, qc_o = t.get()
        rows_o = t.output_rows()
        qc_io = np.ascontiguousarray(qc.copy())
        qf_e = np.zeros_like(qf)
        qrad, qtw = np.zeros(n), np.zeros(n)
        err = ctypes.c_uint()
        igd = np.array([v for s in ig[1] for v in s], dtype=float)
        rc = emu.emu_sources(n, ctypes.c_double(dx), 0, None, None, _p(np.ascontiguousarray(qf)), _p(qc_io), _p(qf_e),
                             ctypes.c_double(dt),
                             ctypes.c_double(time), len(rad), (ctypes.c_int * len(rad))(*[r[0] for r in rad]),
                             _p(np.array([c for _, c in rad], dtype=float).ravel()), 1,
                             _p(np.array(wall, dtype=float)), ig[0], len(ig[1]), _p(igd), _p(qrad), _p(qtw),
                             ctypes.byref(err))
        assert rc == 0 and err.value == 0
        assert np.abs(qf_o[:, 2] - qf[:, 2]).max() > 1.0
        close(qf_e, qf_o, 1e-12)
        np.testing.assert_allclose(qc_io[:, 2], qc_o[:, 2], rtol=1e-13)
        np.testing.assert_allclose(qrad, rows_o[9], rtol=1e-12)
        np.testing.assert_allclose(qtw, rows_o[11], rtol=1e-11, atol=1e-12 * np.abs(rows_o[11]).max())


def test_output_rows_match_oracle(emu, oracle):
    n, dx = 48, 2e-5
    qf, qc = layer(oracle, n, dx, 7.0)
    t = oracle_tube(oracle, n, dx, (1, 2, 1, 2, 0, 0, 0, 0), qf, qc)
    ro = t.output_rows()
    rows = np.zeros_like(ro)
    assert emu.emu_output_rows(n, ctypes.c_double(dx), _p(np.ascontiguousarray(qf)), _p(np.ascontiguousarray(qc)),
                               _p(rows)) == 0
    np.testing.assert_allclose(rows, ro, rtol=1e-14, atol=1e-300)


def smr_state(oracle, ncells, dxs, r0):
    """A pressurised, hot ball of radius r0 in air on SMR segments, with
    qf = QcToqf(Qc) in every cell (a segment's interface ghost is QcToqf of
    an interpolated Qc column)."""
    from oracle_ctypes import _D
    nm = species_names()
    air = configs.mole_vector(nm, {"O2": 0.21, "N2": 0.79})
    xs = np.concatenate([sum(n * d for n, d in zip(ncells[:g], dxs[:g])) + (np.arange(n) + 0.5) * d
                         for g, (n, d) in enumerate(zip(ncells, dxs))])
    inside = xs < r0
    n = len(xs)
    _, qc = oracle.init_cells(np.where(inside, 1500.0, 300.0), np.where(inside, 5 * configs.ATM, configs.ATM),
                              np.zeros(n), np.tile(air, (n, 1)))
    qf = np.zeros_like(qc)
    for i in range(n):
        oracle.L.or_qc_to_qf(oracle.mech, qc[i].ctypes.data_as(_D), qf[i].ctypes.data_as(_D))
    return qf, qc


@pytest.mark.parametrize("fl,short", [((1, 2, 1, 2, 0, 1, 0, 1), 0), ((0, 1, 1, 4, 0, 0, 0, 1), 0),
                                      ((1, 2, 1, 2, 0, 0, 0, 0), 0), ((1, 2, 1, 2, 0, 1, 1, 1), 0),
                                      ((1, 2, 1, 2, 0, 0, 1, 0), 0), ((1, 2, 1, 2, 0, 1, 1, 1), 1),
                                      ((1, 2, 2, 0, 3, 1, 0, 0), 1)])
def test_smr_segments_match_oracle(emu, oracle, fl, short):
    """A hot ball on a fine core with coarser outer segments, spherical (and
    Cartesian), with and without transport: the stage kernels' SMR path
    (interface snapshot, ghosts, r = x_m, the per-column transport kernels)
    against the oracle's SMR blocks."""
    # short: the reference's 10-cell blocks, one segment per level
    ncells, dxs = ([40, 10, 10, 10], [1e-4, 2e-4, 4e-4, 8e-4]) if short else ([40, 24, 16], [1e-4, 2e-4, 4e-4])
    qf, qc = smr_state(oracle, ncells, dxs, 12e-4)
    st, rm, acu, mus, weno, rb, tran, sph = fl
    lv = 2 if acu == 1 else 3
    s = oracle.smr(ncells, dxs, lv, [st, rm, acu, mus, weno, 0, rb, 0], [dxs[0], configs.ATM, 300.0, 0.0, 1e-5, 1e-13])
    if sph:
        s.set_spherical()
    if tran:
        s.set_transport()
    s.set_interior(qf, qc)
    dts = [s.step(0.4) for _ in range(8)]
    qf_o = s.get()[0]
    assert np.abs(qf_o[:, 2] - qf[:, 2]).max() > 5.0
    qf_e, _, err = emu_fluid(emu, ncells, dxs, 2, fl, qf, qc, np.repeat(dts, len(ncells)), dx_comp=dxs[0])
    assert err == 0
    close(qf_e, qf_o, 1e-10)


def test_sources_on_smr_layout_match_one_tube(emu, oracle):
    """The energy-source kernel on three equal-dx SMR segments (columns,
    positions x_m and per-segment speeds of the packed layout) against the
    same cells as one tube."""
    nm = species_names()
    ncells, dx = [30, 30, 30], 2e-5
    n = sum(ncells)
    qf, qc = layer(oracle, n, dx)
    rad = [(nm.index(k), c) for k, c in RAD_FITS.items()]
    rsp = (ctypes.c_int * len(rad))(*[r[0] for r in rad])
    rco = _p(np.array([c for _, c in rad], dtype=float).ravel())
    wall = _p(np.array((4.0, 2e-3, 373.0, 1300.0, 2e4, 0.5 * n * dx), dtype=float))
    igd = _p(np.array([2e-6, 3e-4, 1e-6, 0.0], dtype=float))
    out = []
    for nseg in (0, 3):
        qc_io = np.ascontiguousarray(qc.copy())
        qf_e = np.zeros_like(qf)
        qrad, qtw = np.zeros(n), np.zeros(n)
        err = ctypes.c_uint()
        rc = emu.emu_sources(n, ctypes.c_double(dx), nseg, (ctypes.c_int * 3)(*ncells),
                             _p(np.full(3, dx)), _p(np.ascontiguousarray(qf)), _p(qc_io), _p(qf_e), ctypes.c_double(1e-7),
                             ctypes.c_double(5e-8), len(rad), rsp, rco, 1, wall, 2, 1, igd, _p(qrad), _p(qtw),
                             ctypes.byref(err))
        assert rc == 0 and err.value == 0
        out.append((qf_e, qc_io, qrad, qtw))
    (a, ca, ra, wa), (b, cb, rb, wb) = out
    assert np.abs(a[:, 2] - qf[:, 2]).max() > 1.0
    close(b, a, 1e-12)
    np.testing.assert_allclose(cb[:, 2], ca[:, 2], rtol=1e-13)
    np.testing.assert_allclose(rb, ra, rtol=1e-12)
    np.testing.assert_allclose(wb, wa, rtol=1e-10, atol=1e-12 * np.abs(wa).max())


@pytest.mark.parametrize("packed,rbound", [(0, 0), (0, 1), (1, 0), (1, 1)])
def test_warp_transport_properties_equal_thread_kernel(emu, oracle, packed, rbound):
    """The warp-per-cell property kernel gives the thread-per-cell kernel's
    bits, ghost cells included, in one tube and in packed tubes."""
    cases = [(40, 2e-5, 5.0), (56, 1e-5, 0.0)] if packed else [(70, 2e-5, 5.0)]
    qc = np.vstack([layer(oracle, n, dx, u0)[1] for n, dx, u0 in cases])
    ncells = [c[0] for c in cases]
    cols = sum(n + 8 for n in ncells)
    nrow = 5 + 2 * len(species_names())
    out = []
    for warp in (0, 1):
        props = np.zeros(nrow * cols)
        rc = emu.emu_tran_props(len(cases), (ctypes.c_int * len(cases))(*ncells),
                                _p(np.array([c[1] for c in cases])), packed, rbound, ctypes.c_double(configs.ATM),
                                _p(np.ascontiguousarray(qc)), warp, _p(props))
        assert rc == 0
        out.append(props.reshape(nrow, cols))
    used = np.zeros(cols, bool)
    o = 0
    for n in ncells:
        used[o + 3:o + n + 5] = True  # cells -1..n
        o += n + 8
    assert np.all(np.isfinite(out[0][:, used]))
    np.testing.assert_array_equal(out[1][:, used], out[0][:, used])
