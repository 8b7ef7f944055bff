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
