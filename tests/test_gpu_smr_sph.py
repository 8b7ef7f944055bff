"""GPU SMR domains with spherical geometry and energy sources vs the CPU
oracle's blocks: r and the sources' positions are each cell's x_m, with
x = 0 where the leading segments coarser than dx_comp end. Tolerance 1e-10
relative on p, T, rho (u relative to its peak), as for the other SMR runs.
"""
import numpy as np
import pytest

from fortrancfd_gb300 import Blocks, configs, species_names
from test_gpu_smr import check
from test_sources import RAD_FITS
from test_smr import RP, sod_state

pytestmark = pytest.mark.gpu


def ball(oracle, ncells, dxs, r0):
    xs = np.concatenate([sum(n * d for n, d in zip(ncells[:g], dxs[:g])) + (np.arange(n) + 0.5) * d
                         for g, (n, d) in enumerate(zip(ncells, dxs))])
    return sod_state(oracle, xs, r0)


@pytest.mark.parametrize("scheme", [(1, 2, 1, 2), (0, 1, 1, 4)])
def test_spherical_ball_on_refined_segments_matches_oracle(oracle, scheme):
    st, rm, acu, mus = scheme
    ncells, dxs = [64, 32, 16], [1e-4, 2e-4, 4e-4]
    qf, qc = ball(oracle, ncells, dxs, 20e-4)
    flags = [st, rm, acu, mus, 0, 0, 1, 0]
    s = oracle.smr(ncells, dxs, 2, flags, [dxs[0]] + RP[1:])
    s.set_spherical()
    s.set_interior(qf, qc)
    b = Blocks(ncells, dxs, select_time=st, select_riemann=rm, flag_acu=acu, flag_muscl=mus, flag_rbound=1,
               is_spherical=1)
    b.upload(qf, qc)
    for _ in range(25):
        assert b.step(0.4) == pytest.approx(s.step(0.4), rel=1e-12)
    qf_o = s.get()[0]
    assert np.abs(qf_o[:, 2] - qf[:, 2]).max() > 5.0
    check(qf_o, b.download()[0])


def test_sources_on_segments_match_oracle(oracle):
    """Radiation, wall heat and a Zhang ignition kernel on a refined domain
    through the device loop."""
    nm = species_names()
    ncells, dxs = [48, 24, 16], [2e-5, 4e-5, 8e-5]
    n = sum(ncells)
    prod = configs.equilibrium_tp(configs.ch4_air_mixture(nm, 1.0), 1800.0, configs.ATM)
    from oracle_ctypes import _D
    _, qc = oracle.init_cells(np.linspace(900.0, 1800.0, n), np.full(n, configs.ATM), np.zeros(n),
                              np.tile(prod, (n, 1)))
    qf = np.zeros_like(qc)
    for i in range(n):
        oracle.L.or_qc_to_qf(oracle.mech, qc[i].ctypes.data_as(_D), qf[i].ctypes.data_as(_D))
    rad = [(nm.index(k), c) for k, c in RAD_FITS.items()]
    wall = (4.0, 2e-3, 373.0, 1300.0, 2e4, 1e-3)
    ig = (2, [(2e-7, 3e-4, 1e-6, 0.0)])
    flags = [1, 2, 1, 2, 0, 0, 0, 0]
    s = oracle.smr(ncells, dxs, 2, flags, [dxs[0]] + RP[1:])
    s.set_interior(qf, qc)
    s.set_sources(radiation=rad, wall=wall, ignition=ig)
    b = Blocks(ncells, dxs)
    b.upload(qf, qc)
    b.set_radiation(RAD_FITS)
    b.set_wall_heat(*wall)
    b.set_ignition(ig[0], ig[1])
    t_o = sum(s.step(0.5) for _ in range(10))
    t_g, n_g = b.advance(0.5, tend=1e9, max_steps=10)
    assert n_g == 10 and t_g == pytest.approx(t_o, rel=1e-12)
    qf_o = s.get()[0]
    assert np.abs(qf_o[:, 2] - qf[:, 2]).max() > 0.1
    check(qf_o, b.download()[0])
    rows = b.output_rows()
    np.testing.assert_allclose(rows[[9, 10, 11]], s.output_rows(ncells)[[9, 10, 11]], rtol=1e-9,
                               atol=1e-9 * np.abs(rows[[9, 11]]).max())


def test_cell_centres_of_a_left_smr_zone():
    """Coarser leading segments put x = 0 where they end."""
    ncells, dxs = [16, 16, 32, 16], [4e-3, 2e-3, 1e-3, 2e-3]
    b = Blocks(ncells, dxs, dx_comp=1e-3)
    n = sum(ncells)
    nm = species_names()
    air = configs.mole_vector(nm, {"O2": 0.21, "N2": 0.79})
    b.init_cells(np.full(n, 300.0), np.full(n, configs.ATM), np.zeros(n), np.tile(air, (n, 1)))
    rows = b.output_rows()
    edges = np.r_[0.0, np.cumsum(np.repeat(dxs, ncells))] - (16 * 4e-3 + 16 * 2e-3)
    np.testing.assert_allclose(rows[12], 0.5 * (edges[:-1] + edges[1:]), rtol=0, atol=1e-15)


def test_ten_cell_segments_match_oracle(oracle):
    """The reference's SMR layout: 10-cell blocks, one per level, beyond a
    fine core (a spherical ball, TVDRK3-HLLC-MUSCL)."""
    ncells, dxs = [60, 10, 10, 10, 10], [1e-4, 2e-4, 4e-4, 8e-4, 1.6e-3]
    qf, qc = ball(oracle, ncells, dxs, 20e-4)
    flags = [1, 2, 1, 2, 0, 0, 1, 0]
    s = oracle.smr(ncells, dxs, 2, flags, [dxs[0]] + RP[1:])
    s.set_spherical()
    s.set_interior(qf, qc)
    b = Blocks(ncells, dxs, flag_rbound=1, is_spherical=1)
    b.upload(qf, qc)
    for _ in range(20):
        assert b.step(0.4) == pytest.approx(s.step(0.4), rel=1e-12)
    check(s.get()[0], b.download()[0])
