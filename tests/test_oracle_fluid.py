"""Oracle fluid path: reconstruction properties and the Sod tube against the
exact Riemann solution (CPU only). These bound accuracy; parity of the GPU
library with the oracle is checked in test_gpu_fluid.py."""
import ctypes

import numpy as np
import pytest

from fortrancfd_gb300 import configs

P = ctypes.POINTER(ctypes.c_double)


def recon(oracle, fn, s, *flag):
    s = np.ascontiguousarray(s, dtype=float)
    l, r = ctypes.c_double(), ctypes.c_double()
    getattr(oracle.L, fn)(s.ctypes.data_as(P), ctypes.byref(l), ctypes.byref(r), *flag)
    return l.value, r.value


@pytest.mark.parametrize("fn,n,flag", [("or_muscl3", 4, (1,)), ("or_muscl3", 4, (2,)), ("or_muscl3", 4, (3,)),
                                       ("or_muscl3", 4, (4,)), ("or_weno3z", 4, ()), ("or_weno5", 6, (2,)),
                                       ("or_weno5", 6, (3,)), ("or_weno7z", 8, ())])
def test_constant_preserved(oracle, fn, n, flag):
    l, r = recon(oracle, fn, np.full(n, 3.25), *flag)
    assert l == 3.25 and r == 3.25


def test_muscl_linear_exact(oracle):
    for lim in (1, 2):
        l, r = recon(oracle, "or_muscl3", [1.0, 2.0, 3.0, 4.0], lim)
        assert abs(l - 2.5) < 1e-14 and abs(r - 2.5) < 1e-14


def test_minmod_flat_at_extremum(oracle):
    l, r = recon(oracle, "or_muscl3", [1.0, 2.0, 1.0, 0.0], 2)
    assert l == 2.0  # slopes of opposite sign: first order


def test_weno5_smooth_accuracy(oracle):
    # cell averages of sin(x); WENO5 face value at 5th order
    errs = []
    for h in (0.1, 0.05):
        xc = (np.arange(6) - 2.5) * h  # cells i-2..i+3 around face x = 0
        avg = (np.cos(xc - h / 2) - np.cos(xc + h / 2)) / h
        avg = avg + 1.0
        l, _ = recon(oracle, "or_weno5", avg, 3)
        errs.append(abs(l - 1.0))
    assert errs[1] < errs[0] / 16


def exact_sod(x, t, x0, rl, pl, rr, pr, g):
    """Exact ideal-gas Riemann solution (zero initial velocities)."""
    cl, cr = np.sqrt(g * pl / rl), np.sqrt(g * pr / rr)

    def f(p, rk, pk, ck):
        if p > pk:
            a, b = 2 / ((g + 1) * rk), (g - 1) / (g + 1) * pk
            return (p - pk) * np.sqrt(a / (p + b))
        return 2 * ck / (g - 1) * ((p / pk) ** ((g - 1) / (2 * g)) - 1)

    lo, hi = 1e-6 * min(pl, pr), 10 * max(pl, pr)
    for _ in range(200):
        pm = 0.5 * (lo + hi)
        if f(pm, rl, pl, cl) + f(pm, rr, pr, cr) > 0:
            hi = pm
        else:
            lo = pm
    um = 0.5 * (f(pm, rr, pr, cr) - f(pm, rl, pl, cl))
    rml = rl * (pm / pl) ** (1 / g)
    rmr = rr * ((pm / pr + (g - 1) / (g + 1)) / ((g - 1) / (g + 1) * pm / pr + 1))
    sshock = um + (cr * np.sqrt((g + 1) / (2 * g) * pm / pr + (g - 1) / (2 * g)) - um) * 0 + cr * np.sqrt(
        (g + 1) / (2 * g) * pm / pr + (g - 1) / (2 * g))
    cml = cl * (pm / pl) ** ((g - 1) / (2 * g))
    rho = np.empty_like(x)
    for i, xi in enumerate(x):
        s = (xi - x0) / t
        if s < -cl:
            rho[i] = rl
        elif s < um - cml:
            c = 2 / (g + 1) * (cl + (g - 1) / 2 * (0 - s))
            rho[i] = rl * (c / cl) ** (2 / (g - 1))
        elif s < um:
            rho[i] = rml
        elif s < sshock:
            rho[i] = rmr
        else:
            rho[i] = rr
    return rho


def test_sod_against_exact_riemann(oracle):
    case = configs.sod()
    qf0, qc0 = oracle.init_cells(case.T, case.p, case.u, case.X)
    ot = oracle.tube(case.ncell, 2, [1, 2, 1, 2, 0, 0, 0, 0], [case.dx, 101325.0, 300.0, 0.0, 1e-5, 1e-13])
    ot.set_interior(qf0, qc0)
    t = 0.0
    while t < case.tend:
        t += ot.step(case.cfl)
    qf, _ = ot.get()
    xc = (np.arange(case.ncell) + 0.5) * case.dx
    x = np.zeros(53)
    x[:] = case.X[0]
    cp = oracle.L.or_cp(oracle.mech, 320.0, x.ctypes.data_as(P))
    cv = oracle.L.or_cv(oracle.mech, 320.0, x.ctypes.data_as(P))
    g = cp / cv
    rho_ex = exact_sod(xc, t, 0.5, qf0[0, 0], case.p[0], qf0[-1, 0], case.p[-1], g)
    l1 = np.abs(qf[:, 0] - rho_ex).mean() / rho_ex.mean()
    # three discontinuities smeared over a few of 1000 cells with an 8:1
    # density ratio: a few per cent in L1
    assert l1 < 0.05, l1
    assert qf[:, 1].max() > 200.0  # the expansion accelerates the gas


def test_mirror_symmetry(oracle):
    case = configs.sod(ncell=200)
    qf0, qc0 = oracle.init_cells(case.T, case.p, case.u, case.X)
    res = []
    for flip in (False, True):
        a, b = (qf0[::-1].copy(), qc0[::-1].copy()) if flip else (qf0, qc0)
        ot = oracle.tube(case.ncell, 2, [1, 2, 1, 2, 0, 0, 0, 0], [case.dx, 101325.0, 300.0, 0.0, 1e-5, 1e-13])
        ot.set_interior(np.ascontiguousarray(a), np.ascontiguousarray(b))
        for _ in range(40):
            ot.step(0.5)
        qf, _ = ot.get()
        res.append(qf[::-1] if flip else qf)
    assert np.max(np.abs(res[0][:, 2] - res[1][:, 2])) < 1e-9
    assert np.max(np.abs(res[0][:, 1] + res[1][:, 1])) < 1e-9
