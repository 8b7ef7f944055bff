"""GPU spherical geometry (is_spherical = 1) vs the CPU oracle: a
high-pressure ball expanding into air, centre and outer wall reflecting,
at 1e-10 relative on p, T, rho (u relative to its peak) for the scheme
combinations the spherical stage supports, host loop and device loop.
"""
import numpy as np
import pytest

from fortrancfd_gb300 import EdynError, Tube, Tubes, configs
from test_spherical import ball

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


@pytest.mark.parametrize("select_time,riemann,acu,lim,device_loop",
                         [(1, 2, 1, 2, False), (1, 2, 1, 2, True), (0, 1, 1, 3, False), (1, 0, 0, 2, False),
                          (1, 2, 1, 4, True)])
def test_spherical_ball_matches_oracle(oracle, select_time, riemann, acu, lim, device_loop):
    n, dx, steps = 160, 1e-4, 60
    ot, qf0, qc0 = ball(oracle, n, dx, 10 * configs.ATM, scheme=(select_time, riemann, acu, lim))
    g = Tube(n, dx, select_time=select_time, select_riemann=riemann, flag_acu=acu, flag_muscl=lim,
             is_spherical=1)
    g.upload(qf0, qc0)
    t_o = sum(ot.step(0.5) for _ in range(steps))
    if device_loop:
        t_g, n_g = g.advance(0.5, tend=1e9, max_steps=steps)
        assert n_g == steps
    else:
        t_g = sum(g.step(0.5) for _ in range(steps))
    assert t_g == pytest.approx(t_o, rel=1e-12)
    check(ot.get()[0], g.download()[0])


def test_spherical_refused_where_unsupported():
    for kw in (dict(select_time=2), dict(flag_acu=2, flag_weno=3)):
        with pytest.raises(EdynError):
            Tube(64, 1e-4, is_spherical=1, **kw)
    with pytest.raises(EdynError):
        Tube(64, 1e-4, is_spherical=2)


def test_spherical_flame_kernel_matches_oracle(oracle):
    """The spherical flame configuration shortened (200 cells): spherical
    geometry, transport, chemistry and the ignition energy together, 10
    steps against the oracle at the reacting bar (T 0.1 %, Y 1e-3 of the
    largest mass fraction)."""
    case = configs.spherical_flame(ncell=200)
    fl = case.flags
    qf0, qc0 = oracle.init_cells(case.T, case.p, case.u, case.X)
    ot = oracle.tube(case.ncell, 2, [1, 2, 1, 2, 0, 0, 1, 1], [case.dx, fl["p_out"], 300.0, 0.0, 1e-5, 1e-13])
    ot.set_transport()
    ot.set_spherical()
    ot.set_sources(ignition=fl["ignition"])
    ot.set_interior(qf0, qc0)
    g = Tube(case.ncell, case.dx, flag_acu=1, flag_muscl=2, flag_rbound=1, p_out=fl["p_out"], do_reaction=1,
             do_tran=1, is_spherical=1)
    g.set_ignition(*fl["ignition"])
    g.upload(qf0, qc0)
    for _ in range(10):
        dt_o = ot.step(case.cfl)
        dt_g = g.step(case.cfl)
        assert dt_g == pytest.approx(dt_o, rel=1e-6)
    qf_o, qf_g = ot.get()[0], g.download()[0]
    assert qf_o[0, 2] > 300.5  # the ignition energy heated the centre
    assert np.max(np.abs(qf_g[:, 2] - qf_o[:, 2]) / qf_o[:, 2]) < 1e-3
    assert np.max(np.abs(qf_g[:, 3:] - qf_o[:, 3:])) / qf_o[:, 3:].max() < 1e-3
