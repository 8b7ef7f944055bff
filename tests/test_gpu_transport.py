"""GPU transport path (do_tran = 1, calc_flux_tran) vs the CPU oracle.

Tolerances: per-cell viscosity, conductivity and diffusivities within 1e-10
relative (the GPU evaluates the same TRANLIB fits with its table-driven
exponential and logarithm and an expanded, rounding-only reordering of
Wilke's sum); tube runs within 1e-10 relative on p, T, rho and u (u relative
to its peak) and 1e-10 of the largest mass fraction on Y, as for the
inviscid stages.
"""
import numpy as np
import pytest

from fortrancfd_gb300 import EdynError, Tube, Tubes, configs, lvir_for, species_names

pytestmark = pytest.mark.gpu

R_SI = 8314.51
TOL = 1e-10


def varied_state(n, seed=3):
    """Cells from cold fresh mixture to hot products, with a velocity field."""
    nm = species_names()
    rng = np.random.default_rng(seed)
    fresh = configs.ch4_air_mixture(nm, 1.0)
    hot = configs.equilibrium_tp(fresh, 2400.0, configs.ATM)
    w = np.clip(np.linspace(-0.2, 1.2, n) + 0.05 * rng.standard_normal(n), 0.0, 1.0)
    X = (1 - w)[:, None] * fresh[None, :] + w[:, None] * hot[None, :]
    T = 300.0 + 2100.0 * w
    u = 20.0 * np.sin(np.linspace(0, 6, n))
    return T, np.full(n, configs.ATM), u, X


def flags_of(case):
    fl = dict(case.flags)
    fl.pop("do_tran", None)
    return fl


def test_transport_properties_match_oracle(oracle):
    n = 300
    T, p, u, X = varied_state(n)
    qf, qc = oracle.init_cells(T, p, u, X)
    g = Tube(n, 1e-5, flag_acu=1, flag_muscl=2, do_tran=1)
    g.upload(qf, qc)
    mu, kap, dif = g.transport_properties()
    for i in range(n):
        _, _, _, _, mu_o, kap_o, dif_o = oracle.tran_cell(qc[i])
        assert abs(mu[i] - mu_o) <= TOL * mu_o, i
        assert abs(kap[i] - kap_o) <= TOL * kap_o, i
        np.testing.assert_allclose(dif[i], dif_o, rtol=TOL, atol=1e-30, err_msg=f"cell {i}")


def test_transport_properties_thread_kernel_match_oracle(oracle):
    """Beyond 40,000 cells the property kernel takes one thread per cell
    (below, one warp per cell, with the same bits): sampled cells of a long
    tube against the oracle."""
    n = 41000
    T, p, u, X = varied_state(n, seed=5)
    qf, qc = oracle.init_cells(T, p, u, X)
    g = Tube(n, 1e-5, flag_acu=1, flag_muscl=2, do_tran=1)
    g.upload(qf, qc)
    mu, kap, dif = g.transport_properties()
    for i in np.linspace(0, n - 1, 60).astype(int):
        _, _, _, _, mu_o, kap_o, dif_o = oracle.tran_cell(qc[i])
        assert abs(mu[i] - mu_o) <= TOL * mu_o, i
        assert abs(kap[i] - kap_o) <= TOL * kap_o, i
        np.testing.assert_allclose(dif[i], dif_o, rtol=TOL, atol=1e-30, err_msg=f"cell {i}")


def run_pair(oracle, case, nsteps, **over):
    fl = {**flags_of(case), **over}
    qf0, qc0 = oracle.init_cells(case.T, case.p, case.u, case.X)
    lv = lvir_for(fl["flag_acu"], fl.get("flag_weno", 0))
    ot = oracle.tube(case.ncell, lv, [fl["select_time"], fl["select_riemann"], fl["flag_acu"], fl["flag_muscl"],
                                      fl.get("flag_weno", 0), fl["flag_lbound"], fl["flag_rbound"],
                                      fl.get("do_reaction", 0)],
                     [case.dx, fl.get("p_out", configs.ATM), fl.get("t_in", 300.0), fl.get("rho_u_in", 0.0), 1e-5,
                      1e-13], x_in=fl.get("x_in"))
    ot.set_transport()
    ot.set_interior(qf0, qc0)
    g = Tube(case.ncell, case.dx, do_tran=1, **fl)
    g.upload(qf0, qc0)
    for _ in range(nsteps):
        dt_o = ot.step(case.cfl)
        dt_g = g.step(case.cfl)
        assert dt_g == pytest.approx(dt_o, rel=1e-12)
    qf_o, _ = ot.get()
    qf_g, _, _ = g.download()
    return qf_o, qf_g


def check(qf_o, qf_g, tol=TOL):
    W = configs.molecular_weights()

    def pres(q):
        return q[:, 0] * R_SI * q[:, 2] * (q[:, 3:] / W).sum(axis=1)

    p_o, p_g = pres(qf_o), pres(qf_g)
    assert np.max(np.abs(p_g - p_o) / p_o) < tol
    assert np.max(np.abs(qf_g[:, 2] - qf_o[:, 2]) / qf_o[:, 2]) < tol
    assert np.max(np.abs(qf_g[:, 0] - qf_o[:, 0]) / qf_o[:, 0]) < tol
    assert np.max(np.abs(qf_g[:, 1] - qf_o[:, 1])) / max(np.abs(qf_o[:, 1]).max(), 1e-300) < tol
    assert np.max(np.abs(qf_g[:, 3:] - qf_o[:, 3:])) / qf_o[:, 3:].max() < tol


def test_planar_flame_nonreacting_matches_oracle(oracle):
    """The planar-flame configuration (inflow / outflow, MUSCL-minmod + HLLC,
    TVDRK3) with transport, 30 steps on 256 cells, chemistry off."""
    case = configs.planar_flame(ncell=256, dx=2e-5, x_c=2.5e-3, width=1e-3, do_reaction=0)
    qf_o, qf_g = run_pair(oracle, case, 30)
    check(qf_o, qf_g)


@pytest.mark.parametrize("select_time,riemann,acu,weno", [(0, 0, 1, 0), (2, 1, 1, 0), (1, 2, 2, 3)])
def test_mixing_layer_schemes_match_oracle(oracle, select_time, riemann, acu, weno):
    """An O2/CH4-rich hot layer in air between walls: Euler, RK4 (the
    reference's stale-qf form) and WENO5-Z TVDRK3 stages with transport."""
    nm = species_names()
    n, dx = 128, 1e-5
    xm = (np.arange(n) + 0.5) * dx
    w = 0.5 * (1 + np.tanh((12 * dx - np.abs(xm - 0.5 * n * dx)) / (3 * dx)))
    air = configs.mole_vector(nm, {"O2": 0.21, "N2": 0.79})
    rich = configs.mole_vector(nm, {"CH4": 0.3, "O2": 0.3, "H2O": 0.1, "N2": 0.3})
    X = (1 - w)[:, None] * air[None, :] + w[:, None] * rich[None, :]
    case = configs.TubeCase("mixing_layer", n, dx, 400.0 + 800.0 * w, np.full(n, configs.ATM), 5.0 * w, X,
                            dict(select_time=select_time, select_riemann=riemann, flag_acu=acu, flag_muscl=2,
                                 flag_weno=weno, flag_lbound=0, flag_rbound=0, do_reaction=0), cfl=0.5)
    qf_o, qf_g = run_pair(oracle, case, 20)
    check(qf_o, qf_g)


def test_planar_flame_reacting_matches_oracle(oracle):
    """Transport and chemistry together on the planar flame's hot side."""
    case = configs.planar_flame(ncell=128, dx=2e-5, x_c=1.2e-3, width=4e-4, do_reaction=1)
    qf_o, qf_g = run_pair(oracle, case, 8)
    # the reacting tubes' parity bar (two integrators at the same
    # tolerances): T within 0.1 %, Y within 1e-3 of the largest mass fraction
    assert np.max(np.abs(qf_g[:, 2] - qf_o[:, 2]) / qf_o[:, 2]) < 1e-3
    assert np.max(np.abs(qf_g[:, 3:] - qf_o[:, 3:])) / qf_o[:, 3:].max() < 1e-3


def test_device_loop_with_transport_matches_host_loop():
    case = configs.planar_flame(ncell=200, dx=2e-5, x_c=2e-3, width=1e-3, do_reaction=0)
    fl = flags_of(case)
    a = Tube(case.ncell, case.dx, do_tran=1, **fl)
    b = Tube(case.ncell, case.dx, do_tran=1, **fl)
    a.init_cells(case.T, case.p, case.u, case.X)
    b.init_cells(case.T, case.p, case.u, case.X)
    for _ in range(20):
        a.step(case.cfl)
    b.advance(case.cfl, tend=1e9, max_steps=20)
    qa, _, _ = a.download()
    qb, _, _ = b.download()
    check(qb, qa, tol=1e-12)


def test_transport_refused_where_unsupported():
    with pytest.raises(EdynError, match="transport"):
        Tubes([64, 64], [1e-5, 1e-5], do_tran=1)
    torch = pytest.importorskip("torch")
    g = Tube(64, 1e-5, do_tran=1)
    qf = torch.zeros((56, 72), dtype=torch.float64, device="cuda")
    qc = torch.zeros((56, 72), dtype=torch.float64, device="cuda")
    with pytest.raises(EdynError, match="transport"):
        g.solve_fluid_noalloc(qf.data_ptr(), qc.data_ptr(), 1e-9)
    with pytest.raises(EdynError):
        Tube(64, 1e-5, do_tran=2)
