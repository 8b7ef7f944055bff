"""The oracle's energy sources after the chemistry (CPU): optically thin
radiation (SRC/radiation.f90:74-121), micro-flow-reactor wall heat
(SRC/mfr.f90:41-78) and ignition energy (SRC/ignitionsource.f90:150-262),
applied as solve_source applies them (SRC/source.f90:88-239: rho E += dt Q,
then QcToqf). Each is checked against its formula evaluated here from the
oracle's own thermodynamics and conductivity, and for its physical sense.
"""
import numpy as np
import pytest

from fortrancfd_gb300 import configs, species_names

# Planck-mean absorption fits a0..a5 in T [1/(m atm)] of the reference's
# four-species radiation parameter file
# (WORK/Examples/CH4_GRI3.0/SphericalFlame_radiation/rad_params_4sp.txt)
RAD_FITS = {
    "CH4": (1.017015e+1, -7.947312e-3, 4.342446e-7, 1.048611e-9, -2.287861e-13, 0.0),
    "CO": (1.565360e+0, 1.483914e-2, -2.656035e-5, 1.687980e-8, -4.674473e-12, 4.767887e-16),
    "CO2": (3.244420e+1, 7.537513e-2, -1.535140e-4, 9.487940e-8, -2.509259e-11, 2.447995e-15),
    "H2O": (6.869480e+1, -1.523490e-1, 1.417848e-4, -6.620996e-8, 1.524150e-11, -1.373456e-15),
}
SIGMA = 5.6703744191844294e-08
R_SI = 8314.51


def uniform_tube(oracle, n, T, X, dx=1e-4, u=0.0):
    qf, qc = oracle.init_cells(np.asarray(T, float) * np.ones(n), np.full(n, configs.ATM), np.full(n, u),
                               np.tile(X, (n, 1)) if np.ndim(X) == 1 else X)
    t = oracle.tube(n, 2, [1, 2, 1, 2, 0, 0, 0, 0], [dx, configs.ATM, 300.0, 0.0, 1e-5, 1e-13])
    t.set_interior(qf, qc)
    return t, qf, qc


def mole(qf_row, W):
    z = qf_row[3:] / W
    return z / z.sum()


def test_radiation_loss_matches_formula(oracle):
    nm = species_names()
    W = configs.molecular_weights()
    prod = configs.equilibrium_tp(configs.ch4_air_mixture(nm, 1.0), 2000.0, configs.ATM)
    T = np.linspace(1200.0, 2200.0, 8)
    t, qf, qc = uniform_tube(oracle, 8, T, prod)
    t.set_sources(radiation=[(nm.index(k), c) for k, c in RAD_FITS.items()])
    dt = 1e-5
    t.solve_source(dt)
    qf1, qc1 = t.get()
    for i in range(8):
        x = mole(qf[i], W)
        p = qf[i, 0] * R_SI * qf[i, 2] / float(x @ W)
        kp = sum(np.polyval(c[::-1], qf[i, 2]) * x[nm.index(k)] * p / 101325.0 for k, c in RAD_FITS.items())
        q = -4.0 * kp * SIGMA * (qf[i, 2] ** 4 - 300.0 ** 4)
        assert qc1[i, 2] - qc[i, 2] == pytest.approx(dt * q, rel=1e-9)
    assert np.all(qf1[:, 2] < qf[:, 2])
    np.testing.assert_array_equal(qc1[:, 3:], qc[:, 3:])


def test_wall_heat_matches_formula(oracle):
    nm = species_names()
    W = configs.molecular_weights()
    air = configs.mole_vector(nm, {"O2": 0.21, "N2": 0.79})
    n, dx = 16, 1e-3
    t, qf, qc = uniform_tube(oracle, n, 700.0, air, dx=dx)
    wall = (4.0, 2e-3, 373.0, 1300.0, 800.0, 0.5 * n * dx)
    t.set_sources(wall=wall)
    dt = 1e-6
    t.solve_source(dt)
    qf1, qc1 = t.get()
    nu, d, tmin, tmax, alpha, beta = wall
    for i in range(n):
        x = mole(qf[i], W)
        lam = oracle.mix_conductivity(qf[i, 2], x) * 1e-5
        tw = 0.5 * (tmax - tmin) * np.tanh(alpha * ((i + 0.5) * dx - beta)) + 0.5 * (tmax + tmin)
        q = -4.0 * lam * nu * (qf[i, 2] - tw) / d ** 2
        assert qc1[i, 2] - qc[i, 2] == pytest.approx(dt * q, rel=1e-9)
        # the gas moves toward the wall temperature
        assert np.sign(qf1[i, 2] - qf[i, 2]) == np.sign(tw - qf[i, 2])


@pytest.mark.parametrize("kind", [1, 2])
def test_ignition_energy_in_its_window(oracle, kind):
    nm = species_names()
    air = configs.mole_vector(nm, {"O2": 0.21, "N2": 0.79})
    n, dx = 32, 2e-5
    E, r, dur, t0 = 5e-4, 2e-4, 1e-4, 1e-5
    dt = 1e-7
    for time, on in ((5e-5, True), (2e-4, False), (t0, False)):
        t, qf, qc = uniform_tube(oracle, n, 300.0, air, dx=dx)
        t.set_sources(ignition=(kind, [(E, r, dur, t0)]))
        t.set_time(time)
        t.solve_source(dt)
        qf1, qc1 = t.get()
        xm = (np.arange(n) + 0.5) * dx
        pi = 3.14159265359
        if kind == 1:
            rate = E / (4.0 * pi * r ** 3 / 3.0 * dur) * np.exp(-(pi / 4.0) * (xm / r) ** 6)
        else:
            rate = E / (pi ** 1.5 * r ** 3 * dur) * np.exp(-(xm / r) ** 2)
        expect = dt * rate if on else np.zeros(n)
        np.testing.assert_allclose(qc1[:, 2] - qc[:, 2], expect, rtol=1e-9, atol=1e-9 * np.abs(expect).max())
        if on:
            assert qf1[0, 2] > qf[0, 2] + 1.0


def test_several_ignition_sources_last_active_wins(oracle):
    nm = species_names()
    air = configs.mole_vector(nm, {"O2": 0.21, "N2": 0.79})
    n, dx, dt = 16, 2e-5, 1e-7
    a = (5e-4, 2e-4, 1e-4, 0.0)
    b = (1e-4, 1e-4, 1e-4, 0.0)
    out = []
    for srcs in ([a, b], [b], [b, (5e-4, 2e-4, 1e-4, 1.0)]):
        t, qf, qc = uniform_tube(oracle, n, 300.0, air, dx=dx)
        t.set_sources(ignition=(2, srcs))
        t.set_time(5e-5)
        t.solve_source(dt)
        out.append(t.get()[1][:, 2] - qc[:, 2])
    np.testing.assert_array_equal(out[0], out[1])
    np.testing.assert_array_equal(out[2], out[1])
