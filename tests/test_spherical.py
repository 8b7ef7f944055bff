"""Spherical geometry in the oracle (CPU): is_spherical = 1 restated from
SRC/flux.f90:272-278 and SRC/timeintegration.f90:58-75, 177-198. Checked by
exact properties: a uniform gas at rest stays at rest (to rounding); between
the centre (a reflecting wall, zero face area) and a reflecting outer wall,
the volume integrals of mass, species and energy are conserved; a
high-pressure ball expands into the ambient gas with a weaker shock than
the planar problem of the same initial state.
"""
import numpy as np
import pytest

from fortrancfd_gb300 import configs, species_names


def ball(oracle, n, dx, p_in, spherical=True, scheme=(1, 2, 1, 2), T=300.0):
    nm = species_names()
    air = configs.mole_vector(nm, {"O2": 0.21, "N2": 0.79})
    xm = (np.arange(n) + 0.5) * dx
    p = np.where(xm < 0.3 * n * dx, p_in, configs.ATM)
    qf, qc = oracle.init_cells(np.full(n, T), p, np.zeros(n), np.tile(air, (n, 1)))
    st, rm, acu, lim = scheme
    t = oracle.tube(n, 2, [st, rm, acu, lim, 0, 0, 0, 0], [dx, configs.ATM, 300.0, 0.0, 1e-5, 1e-13])
    if spherical:
        t.set_spherical()
    t.set_interior(qf, qc)
    return t, qf, qc


def volumes(n, dx):
    rm = (np.arange(n) + 0.5) * dx
    return rm * rm * dx


def test_uniform_gas_at_rest_stays_at_rest(oracle):
    # to rounding: the HLLC star-state energy rho (E/rho) differs from E in the
    # last bit, a flux that cancels between equal faces in a plane but not
    # under unequal face areas
    t, qf, qc = ball(oracle, 48, 1e-4, configs.ATM)
    for _ in range(10):
        t.step(0.5)
    qf1, qc1 = t.get()
    assert np.abs(qf1[:, 1]).max() < 1e-9
    np.testing.assert_allclose(qc1[:, [0, 2]], qc[:, [0, 2]], rtol=1e-13)
    np.testing.assert_allclose(qf1[:, 2], qf[:, 2], rtol=1e-13)


@pytest.mark.parametrize("scheme", [(1, 2, 1, 2), (0, 1, 1, 2), (1, 0, 0, 2)])
def test_volume_integrals_conserved(oracle, scheme):
    n, dx = 96, 1e-4
    t, qf, qc = ball(oracle, n, dx, 10 * configs.ATM, scheme=scheme)
    for _ in range(40):
        t.step(0.5)
    qf1, qc1 = t.get()
    V = volumes(n, dx)
    for v in [0, 2] + list(range(3, 56)):
        a, b = V @ qc[:, v], V @ qc1[:, v]
        assert abs(b - a) <= 1e-12 * max(abs(a), np.abs(V * qc[:, v]).max()), v
    assert np.abs(qf1[:, 1]).max() > 10.0


def test_spherical_blast_is_weaker_than_planar(oracle):
    n, dx = 128, 1e-4
    ts, _, _ = ball(oracle, n, dx, 10 * configs.ATM)
    tp, _, _ = ball(oracle, n, dx, 10 * configs.ATM, spherical=False)
    for _ in range(60):
        ts.step(0.5)
        tp.step(0.5)
    qs, _ = ts.get()
    qp, _ = tp.get()
    # outside the initial ball the planar shock is stronger
    out = slice(int(0.35 * n), n)
    assert qs[out, 2].max() < qp[out, 2].max()
    assert qs[out, 0].max() < qp[out, 0].max()


@pytest.mark.parametrize("spherical", [True, False])
def test_weak_pulse_decays_as_one_over_r(oracle, spherical):
    """Linear acoustics: an outgoing weak spherical pulse keeps p' r
    constant (its amplitude falls as 1/r), a planar one keeps p'. A 1 %
    isentropic overpressure at r = 1 cm, tracked from 2.2 to 3.4 cm: p' r
    within 10 % in the sphere while p' falls by more than a quarter; p'
    within 10 % in the plane."""
    n, dx = 600, 1e-4
    nm = species_names()
    air = configs.mole_vector(nm, {"O2": 0.21, "N2": 0.79})
    xm = (np.arange(n) + 0.5) * dx
    p = configs.ATM * (1 + 0.01 * np.exp(-((xm - 0.01) / 0.0015) ** 2))
    T = 300.0 * (p / configs.ATM) ** (0.4 / 1.4)
    qf, qc = oracle.init_cells(T, p, np.zeros(n), np.tile(air, (n, 1)))
    t = oracle.tube(n, 2, [1, 2, 1, 2, 0, 0, 0, 0], [dx, configs.ATM, 300.0, 0.0, 1e-5, 1e-13])
    if spherical:
        t.set_spherical()
    t.set_interior(qf, qc)
    W = configs.molecular_weights()
    time, rec = 0.0, []
    for t_probe in (2.5e-5, 5.0e-5):
        while time < t_probe:
            time += t.step(0.5)
        q = t.get()[0]
        pp = q[:, 0] * 8314.51 * q[:, 2] * (q[:, 3:] / W).sum(axis=1) - configs.ATM
        k = int(np.argmax(pp * (xm > 0.012)))
        rec.append((xm[k], pp[k]))
    (r1, p1), (r2, p2) = rec
    assert r2 > r1 + 0.008
    if spherical:
        assert abs(p2 * r2 / (p1 * r1) - 1.0) < 0.1
        assert p2 < 0.75 * p1
    else:
        assert abs(p2 / p1 - 1.0) < 0.1
