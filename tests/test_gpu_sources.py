"""GPU energy sources after the chemistry (radiation, wall heat, ignition)
vs the CPU oracle: the same tube stepped by both, through the host loop
(edyn_step) and the device loop (edyn_advance). Tolerance 1e-10 relative on
p, T, rho (u relative to its peak) for frozen chemistry, as for the fluid
stages; the reacting bar (T 0.1 %, Y 1e-3 of the largest) with chemistry.
"""
import numpy as np
import pytest

from fortrancfd_gb300 import EdynError, Tube, Tubes, configs, species_names
from test_sources import RAD_FITS

pytestmark = pytest.mark.gpu

R_SI = 8314.51


def hot_layer(n, dx):
    nm = species_names()
    fresh = configs.ch4_air_mixture(nm, 1.0)
    prod = configs.equilibrium_tp(fresh, 2000.0, configs.ATM)
    xm = (np.arange(n) + 0.5) * dx
    w = 0.5 * (1 + np.tanh((xm - 0.5 * n * dx) / (4 * dx)))
    X = (1 - w)[:, None] * fresh[None, :] + w[:, None] * prod[None, :]
    return 400.0 + 1600.0 * w, np.full(n, configs.ATM), np.zeros(n), X


def pair(oracle, n, dx, do_reaction, steps, device_loop):
    nm = species_names()
    T, p, u, X = hot_layer(n, dx)
    qf0, qc0 = oracle.init_cells(T, p, u, X)
    rad = [(nm.index(k), c) for k, c in RAD_FITS.items()]
    wall = (4.0, 2e-3, 373.0, 1300.0, 2e4, 0.5 * n * dx)
    # the second source switches on mid-run (dt is ~1e-8 s) and overrides the first
    ig = (2, [(2e-4, 3e-4, 1e-6, 0.0), (1e-4, 1e-4, 1e-6, 1e-7)])
    ot = oracle.tube(n, 2, [1, 2, 1, 2, 0, 0, 0, do_reaction], [dx, configs.ATM, 300.0, 0.0, 1e-5, 1e-13])
    ot.set_interior(qf0, qc0)
    ot.set_sources(radiation=rad, wall=wall, ignition=ig)
    g = Tube(n, dx, flag_acu=1, flag_muscl=2, do_reaction=do_reaction)
    g.upload(qf0, qc0)
    g.set_radiation(RAD_FITS)
    g.set_wall_heat(*wall)
    g.set_ignition(ig[0], ig[1])
    t_o = 0.0
    for _ in range(steps):
        t_o += ot.step(0.5)
    if device_loop:
        t_g, n_g = g.advance(0.5, tend=1e9, max_steps=steps)
        assert n_g == steps
    else:
        t_g = sum(g.step(0.5) for _ in range(steps))
    assert t_g == pytest.approx(t_o, rel=1e-12)
    return ot.get()[0], g.download()[0]


def check(qf_o, qf_g, tol):
    W = configs.molecular_weights()

    def pres(q):
        return q[:, 0] * R_SI * q[:, 2] * (q[:, 3:] / W).sum(axis=1)

    assert np.max(np.abs(pres(qf_g) - pres(qf_o)) / pres(qf_o)) < tol
    assert np.max(np.abs(qf_g[:, 2] - qf_o[:, 2]) / qf_o[:, 2]) < tol
    assert np.max(np.abs(qf_g[:, 0] - qf_o[:, 0]) / qf_o[:, 0]) < tol
    assert np.max(np.abs(qf_g[:, 1] - qf_o[:, 1])) / max(np.abs(qf_o[:, 1]).max(), 1e-300) < tol


@pytest.mark.parametrize("device_loop", [False, True])
def test_sources_frozen_match_oracle(oracle, device_loop):
    qf_o, qf_g = pair(oracle, 96, 2e-5, 0, 24, device_loop)
    check(qf_o, qf_g, 1e-10)
    # the sources acted: the ignition heated the first cells
    assert qf_o[0, 2] > 405.0


def test_sources_with_chemistry_match_oracle(oracle):
    qf_o, qf_g = pair(oracle, 64, 2e-5, 1, 8, True)
    assert np.max(np.abs(qf_g[:, 2] - qf_o[:, 2]) / qf_o[:, 2]) < 1e-3
    assert np.max(np.abs(qf_g[:, 3:] - qf_o[:, 3:])) / qf_o[:, 3:].max() < 1e-3


def test_sources_refused_where_unsupported():
    g = Tubes([64, 64], [1e-5, 1e-5], do_reaction=0)
    with pytest.raises(EdynError):
        g.set_radiation(RAD_FITS)
    t = Tube(64, 1e-5)
    with pytest.raises(EdynError):
        t.set_ignition(3, [(1e-4, 1e-4, 1e-6, 0.0)])
    with pytest.raises(EdynError):
        t.set_wall_heat(4.0, 0.0, 300.0, 400.0, 1.0, 0.0)
    t.set_radiation({})
    t.set_wall_heat()
    t.set_ignition(0)
