"""Pins the oracle's thermodynamics and kinetics (CPU only).

Golden vector: the Cantera TP-equilibrium composition of stoichiometric
CH4/air at 1300 K, 1 atm shipped with the reference
(tests/golden/equil_tp_ch4air_T1300_p1.json). At chemical equilibrium every
reversible reaction's forward and reverse rates of progress must agree; this
checks the NASA-7 Gibbs functions (range selection, coefficient order), the
equilibrium-constant formula of CKRATT and the rate machinery together, with
an R-independent criterion (Q_c / K_c does not depend on the gas constant).
"""
import json
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
EQ = json.loads((ROOT / "tests/golden/equil_tp_ch4air_T1300_p1.json").read_text())
RU = 8.314510e7


def test_equilibrium_detailed_balance(oracle, names):
    X = np.array([EQ["X"][n] for n in names])
    W = np.array([float(l.split()[1]) for l in (ROOT / "fortrancfd_gb300/data/gri30/mech.edyn").read_text().split(
        "SPECIES")[1].strip().split("\n")[1:54]])
    Y = X * W / (X * W).sum()
    T, p = EQ["T"], EQ["p_atm"] * 1.01325e6
    rho = p * (X * W).sum() / (RU * T)
    qf, qr = oracle.rop(rho, T, Y)
    # reactions whose species are all above 1e-14 in mole fraction
    txt = (ROOT / "fortrancfd_gb300/data/gri30/mech.edyn").read_text().split("REACTIONS")[1].strip().split("\n")[1:326]
    checked = 0
    worst = 0.0
    for i, line in enumerate(txt):
        tok = line.split()
        if tok[1] != "1":
            continue
        ks = [int(tok[2 + 2 * q]) for q in range(6)]
        if any(k >= 0 and X[k] < 1e-14 for k in ks):
            continue
        m = max(qf[i], qr[i])
        if m <= 0:
            continue
        worst = max(worst, abs(qf[i] - qr[i]) / m)
        checked += 1
    print('checked', checked, 'worst', worst)
    assert checked >= 40
    assert worst < 1e-10, worst


def test_nasa_continuity_at_tmid(oracle):
    # h, cp and s/R - h/RT of each species are continuous across T_mid
    for T in (1000.0,):
        lo = oracle.vec("or_ckcpml", T)
        hi = oracle.vec("or_ckcpml", T * (1 + 1e-12))
        assert np.max(np.abs(hi - lo) / np.abs(lo)) < 1e-3
        h0, h1 = oracle.vec("or_ckhml", T), oracle.vec("or_ckhml", T * (1 + 1e-12))
        assert np.max(np.abs(h1 - h0) / (np.abs(h0) + RU * T)) < 1e-4


def test_thermo_identities(oracle):
    for T in (300.0, 999.0, 1500.0, 3000.0):
        cp, cv = oracle.vec("or_ckcpml", T), oracle.vec("or_ckcvml", T)
        h, u = oracle.vec("or_ckhml", T), oracle.vec("or_ckuml", T)
        assert np.allclose(cp - cv, RU, rtol=1e-13)
        assert np.allclose(h - u, RU * T, rtol=1e-12)


def test_mole_mass_round_trip(oracle, names):
    rng = np.random.default_rng(0)
    y = rng.random(53)
    y /= y.sum()
    x = np.zeros(53)
    y2 = np.zeros(53)
    import ctypes
    P = ctypes.POINTER(ctypes.c_double)
    oracle.L.or_ckytx(oracle.mech, y.ctypes.data_as(P), x.ctypes.data_as(P))
    oracle.L.or_ckxty(oracle.mech, x.ctypes.data_as(P), y2.ctypes.data_as(P))
    assert np.allclose(y, y2, rtol=1e-14, atol=0)
    assert abs(x.sum() - 1) < 1e-14


def test_production_rates_conserve_mass_and_elements(oracle, names):
    rng = np.random.default_rng(1)
    W = np.array([float(l.split()[1]) for l in (ROOT / "fortrancfd_gb300/data/gri30/mech.edyn").read_text().split(
        "SPECIES")[1].strip().split("\n")[1:54]])
    for T in (900.0, 1500.0, 2500.0):
        y = rng.random(53) ** 4
        y /= y.sum()
        w = oracle.wdot(1e-4, T, y)
        scale = np.abs(W * w).sum()
        assert abs((W * w).sum()) < 1e-12 * scale


def test_temperature_newton_inverts_energy(oracle, names):
    import ctypes
    P = ctypes.POINTER(ctypes.c_double)
    x = np.zeros(53)
    x[names.index("CH4")], x[names.index("O2")], x[names.index("N2")] = 0.095, 0.19, 0.715
    for T in (250.0, 300.0, 999.0, 1001.0, 1700.0, 2900.0):
        e = oracle.L.or_specific_energy(oracle.mech, T, x.ctypes.data_as(P))
        it = ctypes.c_int()
        T2 = oracle.L.or_temperature_con(oracle.mech, e, x.ctypes.data_as(P), ctypes.byref(it))
        assert abs(T2 - T) / T < 1e-10
        assert 1 <= it.value <= 10


def test_adjust_sum_clips_and_normalises(oracle):
    import ctypes
    v = np.array([0.5, -0.1, 0.25, 0.25])
    oracle.L.or_adjust_sum(4, v.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    assert v[1] == 0.0 and abs(v.sum() - 1) < 1e-15 and v[0] == 0.5
