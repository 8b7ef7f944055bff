"""GPU SMR blocks (edyn_init_blocks) vs the CPU oracle's blocks: equal-dx
segments reproduce one tube (to rounding); refined segments (fine / coarse /
fine, and the reverse) match the oracle's interpolation_block exchange at
1e-10 relative on p, T, rho (u relative to its peak), under TVDRK3 and Euler,
MUSCL and WENO5-Z, walls and inflow / outflow.
"""
import numpy as np
import pytest

from fortrancfd_gb300 import Blocks, EdynError, Tube, configs, lvir_for, species_names
from test_smr import RP, sod_state

pytestmark = pytest.mark.gpu

R_SI = 8314.51


def check(qf_o, qf_g, tol=1e-10):
    W = configs.molecular_weights()

    def pres(q):
        return q[:, 0] * R_SI * q[:, 2] * (q[:, 3:] / W).sum(axis=1)

    assert np.max(np.abs(pres(qf_g) - pres(qf_o)) / pres(qf_o)) < tol
    assert np.max(np.abs(qf_g[:, 2] - qf_o[:, 2]) / qf_o[:, 2]) < tol
    assert np.max(np.abs(qf_g[:, 0] - qf_o[:, 0]) / qf_o[:, 0]) < tol
    assert np.max(np.abs(qf_g[:, 1] - qf_o[:, 1])) / np.abs(qf_o[:, 1]).max() < tol


def centres(ncells, dxs):
    x, out = 0.0, []
    for n, d in zip(ncells, dxs):
        out.append(x + (np.arange(n) + 0.5) * d)
        x += n * d
    return np.concatenate(out)


def test_equal_segments_reproduce_one_tube(oracle):
    dx = 1e-3
    ncells = [40, 50, 30]
    n = sum(ncells)
    qf, qc = sod_state(oracle, (np.arange(n) + 0.5) * dx, 0.5 * n * dx)
    t = Tube(n, dx, flag_acu=1, flag_muscl=2)
    b = Blocks(ncells, [dx] * 3)
    t.upload(qf, qc)
    b.upload(qf, qc)
    t.advance(0.5, tend=1e9, max_steps=40)
    b.advance(0.5, tend=1e9, max_steps=40)
    # to rounding: a segment's ghost is QcToqf of its neighbour's column on
    # one thread, where the tube reads the neighbour's primitive state, made
    # by the stage's four-lane QcToqf (species sums in another order)
    check(t.download()[0], b.download()[0], tol=1e-11)


@pytest.mark.parametrize("scheme,ncells,dxs", [
    ((1, 2, 1, 2, 0), [100, 40, 60], [1e-3, 2e-3, 1e-3]),
    ((0, 1, 1, 4, 0), [60, 80, 40], [2e-3, 1e-3, 2e-3]),
    ((1, 2, 2, 2, 3), [96, 48, 64], [1e-3, 2e-3, 4e-3]),
])
def test_refined_segments_match_oracle(oracle, scheme, ncells, dxs):
    st, rm, acu, lim, weno = scheme
    lv = lvir_for(acu, weno)
    flags = [st, rm, acu, lim, weno, 0, 0, 0]
    xm = centres(ncells, dxs)
    qf, qc = sod_state(oracle, xm, 0.35 * xm[-1])
    dx_comp = min(dxs)  # the finest level, as the reference's dx_comp
    s = oracle.smr(ncells, dxs, lv, flags, [dx_comp] + RP[1:])
    s.set_interior(qf, qc)
    b = Blocks(ncells, dxs, dx_comp=dx_comp, select_time=st, select_riemann=rm, flag_acu=acu, flag_muscl=lim,
               flag_weno=weno)
    b.upload(qf, qc)
    t_o = sum(s.step(0.5) for _ in range(60))
    t_g, n_g = b.advance(0.5, tend=1e9, max_steps=60)
    assert n_g == 60 and t_g == pytest.approx(t_o, rel=1e-12)
    check(s.get()[0], b.download()[0])


def test_inflow_outflow_blocks_match_oracle(oracle):
    nm = species_names()
    air = configs.mole_vector(nm, {"O2": 0.21, "N2": 0.79})
    ncells, dxs = [64, 32, 32], [5e-4, 1e-3, 2e-3]
    n = sum(ncells)
    xm = centres(ncells, dxs)
    T = 300.0 + 900.0 * np.exp(-((xm - 0.04) / 0.01) ** 2)
    _, qc = oracle.init_cells(T, np.full(n, configs.ATM), np.full(n, 5.0), np.tile(air, (n, 1)))
    from oracle_ctypes import _D

    qf = np.zeros_like(qc)
    for i in range(n):
        oracle.L.or_qc_to_qf(oracle.mech, qc[i].ctypes.data_as(_D), qf[i].ctypes.data_as(_D))
    rho_u_in = 6.0
    rp = [dxs[0], configs.ATM, 300.0, rho_u_in, 1e-5, 1e-13]
    s = oracle.smr(ncells, dxs, 2, [1, 2, 1, 2, 0, 1, 1, 0], rp, x_in=air)
    s.set_interior(qf, qc)
    b = Blocks(ncells, dxs, flag_lbound=1, flag_rbound=1, t_in=300.0, rho_u_in=rho_u_in, x_in=air)
    b.upload(qf, qc)
    for _ in range(50):
        s.step(0.5)
        b.step(0.5)
    check(s.get()[0], b.download()[0])


def test_blocks_refused_where_unsupported():
    with pytest.raises(EdynError):
        Blocks([32, 32], [1e-3, 3e-3])
    with pytest.raises(EdynError):
        Blocks([32, 32], [1e-3, 2e-3], select_time=2)
    with pytest.raises(EdynError):
        Blocks([32, 6], [1e-3, 2e-3])
    with pytest.raises(EdynError, match="transport"):
        Blocks([32, 32], [1e-3, 2e-3], do_tran=1)

