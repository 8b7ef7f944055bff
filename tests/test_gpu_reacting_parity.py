"""Reacting-path parity of the GPU library against the CPU oracle.

* The benchmarked 20,000-cell CH4/O2 detonation tube, 100 full steps (fluid +
  chemistry), GPU and oracle at the same integrator tolerances: peak
  temperature within 0.1 % and species within 1e-3 relative (mass fractions
  >= 1e-6; absolute 1e-9 below).
* A 1,000-cell (5 cm) tube of the same detonation to t = 20 us: profiles,
  peak temperature and peak pressure.
* Production rates directly: the FP64 right-hand side d(Y, T)/dt of the GPU
  (edyn_chem_rhs_device, full mechanism; edyn_chem_rhs_tube, the C/H/O
  subset of a CH4/O2 tube) against the oracle's CKWYR-based right-hand side,
  per species within 1e-12 of that species' gross rate (creation plus
  destruction, CKCDYR), so that cancellation near equilibrium does not hide
  or inflate an error; a failure names the species and its largest reaction.
* HRR and HRR_dot (SRC/source.f90:70-73): the library's values against the
  reference formulas (SRC/thermo.f90:83-134) evaluated by the oracle on the
  library's own states within 1e-10 of their gross sums, and against the
  oracle tube's own values within the reacting bars.
* The inflow boundary (lbound_inlet, SRC/boundary.f90:70-103) on a frozen
  tube: p, u, T within 1e-10 relative.
"""
import json
from pathlib import Path

import numpy as np
import pytest

from fortrancfd_gb300 import Reactors, Tube, configs, species_names

pytestmark = pytest.mark.gpu

R_SI = 8314.51
GOLDEN = Path(__file__).resolve().parent / "golden" / "gri30_mech_golden.json"


def species_err(Yg, Yr, floor=1e-6):
    big = np.abs(Yr) >= floor
    rel = np.where(big, np.abs(Yg - Yr) / np.maximum(np.abs(Yr), floor), 0.0)
    ab = np.where(~big, np.abs(Yg - Yr), 0.0)
    return float(rel.max()), float(ab.max())


def pressure(qf, W):
    return qf[:, 0] * R_SI * qf[:, 2] * (qf[:, 3:] / W).sum(axis=1)


def detonation_pair(oracle, case, rtol, atol, strict_newton=1):
    qf0, qc0 = oracle.init_cells(case.T, case.p, case.u, case.X)
    ot = oracle.tube(case.ncell, 3, [1, 2, 2, 2, 3, 0, 1, 1], [case.dx, 101325.0, 300.0, 0.0, rtol, atol])
    ot.set_interior(qf0, qc0)
    g = Tube(case.ncell, case.dx, flag_acu=2, flag_weno=3, flag_rbound=1, do_reaction=1, rtol=rtol, atol=atol,
             strict_newton=strict_newton)
    g.upload(qf0, qc0)
    return ot, g


@pytest.mark.timeout(900)
def test_bench_tube_100_steps_vs_oracle(oracle, names):
    """The 20,000-cell, 50 um CH4/O2 detonation of the benchmark, 100 steps."""
    case = configs.detonation(ncell=20000, length=1.0)
    ot, g = detonation_pair(oracle, case, 1e-6, 1e-14)
    for _ in range(100):
        dt_o = ot.step(case.cfl)
        dt_g = g.step(case.cfl)
        assert dt_g == pytest.approx(dt_o, rel=1e-6)
    qf_o, _ = ot.get()
    qf_g, _, _ = g.download()
    assert abs(qf_g[:, 2].max() - qf_o[:, 2].max()) / qf_o[:, 2].max() < 1e-3
    assert np.max(np.abs(qf_g[:, 2] - qf_o[:, 2]) / qf_o[:, 2]) < 1e-3
    rel_err, abs_err = species_err(qf_g[:, 3:], qf_o[:, 3:])
    assert rel_err < 1e-3, rel_err
    assert abs_err < 1e-9, abs_err
    W = configs.molecular_weights()
    p_o, p_g = pressure(qf_o, W), pressure(qf_g, W)
    assert np.max(np.abs(p_g - p_o) / p_o) < 1e-3
    # the run reacted: the driver's products and the shocked gas are hot
    assert qf_o[:, 2].max() > 2500.0 and (qf_o[:, 2] > 1000.0).sum() > 200


@pytest.mark.timeout(900)
def test_short_tube_to_20us_vs_oracle(oracle, names):
    """A 1,000-cell (5 cm, 50 um) detonation tube run to t = 20 us (about
    2,000 steps, the shock well into the tube): the cells' temperature and
    pressure profiles (L1 within 1 %), peak temperature and pressure
    (0.1 %), and the same steps taken. (The benchmark's 200 us would take
    the oracle tens of minutes: its reaction-front cells need hundreds of
    right-hand sides each, every step.)"""
    case = configs.detonation(ncell=1000, length=0.05)
    ot, g = detonation_pair(oracle, case, 1e-6, 1e-14)
    t_end = 20e-6
    t_o = 0.0
    n_o = 0
    while t_o < t_end:  # the reference's loop test, SRC/main.f90:130
        t_o += ot.step(case.cfl)
        n_o += 1
    t_g, n_g = g.advance(case.cfl, tend=t_end)
    assert n_g == n_o and t_g == pytest.approx(t_o, rel=1e-6)
    qf_o, _ = ot.get()
    qf_g, _, _ = g.download()
    W = configs.molecular_weights()
    p_o, p_g = pressure(qf_o, W), pressure(qf_g, W)
    assert abs(qf_g[:, 2].max() - qf_o[:, 2].max()) / qf_o[:, 2].max() < 1e-3
    assert abs(p_g.max() - p_o.max()) / p_o.max() < 1e-3
    assert np.abs(qf_g[:, 2] - qf_o[:, 2]).sum() / np.abs(qf_o[:, 2]).sum() < 1e-2
    assert np.abs(p_g - p_o).sum() / np.abs(p_o).sum() < 1e-2


def _golden_reactions():
    return json.loads(GOLDEN.read_text())["reactions"]


def _worst_reaction(oracle, rho_cgs, T, Y, species):
    """The reaction with the largest gross rate |q_f| + |q_r| among those in
    which the species takes part (for a failure message)."""
    rx = _golden_reactions()
    qf, qr = oracle.rop(rho_cgs, T, Y)
    best, eq = -1.0, "?"
    for i, r in enumerate(rx):
        if species in r["reac"] or species in r["prod"]:
            v = abs(qf[i]) + abs(qr[i])
            if v > best:
                best, eq = v, r["eq"]
    return eq


def _rhs_check(oracle, names, rho_si, yiT, f_gpu, bar=1e-12):
    W = configs.molecular_weights()
    K = len(names)
    for c in range(len(rho_si)):
        rho_cgs = rho_si[c] * 1e-3
        f_o = oracle.chem_rhs(rho_cgs, yiT[c])
        cd, dd = oracle.cdot_ddot(rho_cgs, yiT[c, K], yiT[c, :K])
        gross = (cd + dd) * W / rho_cgs
        err = np.abs(f_gpu[c, :K] - f_o[:K])
        bad = err > bar * gross + 1e-300
        if bad.any():
            k = int(np.argmax(np.where(gross > 0, err / np.maximum(gross, 1e-300), err)))
            rx = _worst_reaction(oracle, rho_cgs, yiT[c, K], yiT[c, :K], names[k])
            pytest.fail(f"cell {c}: species {names[k]} dY/dt {f_gpu[c, k]:.17e} vs {f_o[k]:.17e} "
                        f"(gross {gross[k]:.3e}, rel {err[k] / max(gross[k], 1e-300):.2e}); "
                        f"largest reaction: {rx}")
        # temperature row: -sum u_k w_k / (rho cv), gross = sum |u_k| (c_k + d_k) / (rho cv)
        uml = oracle.vec("or_ckuml", yiT[c, K])
        cvml = oracle.vec("or_ckcvml", yiT[c, K])
        cv = float((yiT[c, :K] * cvml / W).sum())
        gT = float((np.abs(uml) * (cd + dd)).sum() / (rho_cgs * cv))
        assert abs(f_gpu[c, K] - f_o[K]) <= bar * gT + 1e-300, (c, f_gpu[c, K], f_o[K], gT)


def _hot_tube_states(oracle, ncell=512, steps=6):
    """States of a short CH4/O2 detonation run on the GPU: the costliest cells
    of the last chemistry call and a spread of others."""
    case = configs.detonation(ncell=ncell, length=ncell * 50e-6, driver=64 * 50e-6)
    qf0, qc0 = oracle.init_cells(case.T, case.p, case.u, case.X)
    g = Tube(case.ncell, case.dx, flag_acu=2, flag_weno=3, flag_rbound=1, do_reaction=1, rtol=1e-6, atol=1e-14)
    g.upload(qf0, qc0)
    for _ in range(steps):
        g.step(case.cfl)
    cost, _ = g.chem_cost()
    qf, _, _ = g.download()
    pick = np.unique(np.concatenate([np.argsort(cost)[-48:], np.arange(0, ncell, 37)]))
    rho = np.ascontiguousarray(qf[pick, 0])
    yiT = np.ascontiguousarray(np.concatenate([qf[pick, 3:], qf[pick, 2:3]], axis=1))
    return g, rho, yiT


def test_production_rates_full_mechanism(oracle, names):
    torch = pytest.importorskip("torch")
    from fortrancfd_gb300 import surrogate as S

    rho_a, _, y_a, _ = configs.reactor_batch(96, seed=7)
    g, rho_b, y_b = _hot_tube_states(oracle)
    g.close()
    rho = np.concatenate([rho_a, rho_b])
    yiT = np.ascontiguousarray(np.concatenate([y_a, y_b]))
    r = Reactors()
    R = torch.tensor(rho, device="cuda")
    Y = torch.tensor(yiT, device="cuda")
    F = torch.empty_like(Y)
    S._ck(S._L().edyn_chem_rhs_device(r._h, len(rho), S._p(R), S._p(Y), S._p(F)), "rhs")
    torch.cuda.synchronize()
    _rhs_check(oracle, names, rho, yiT, F.cpu().numpy())


def test_production_rates_species_subset(oracle, names):
    """The CH4/O2 tube integrates the 34 C/H/O species; its right-hand side
    on the tube's states equals the oracle's full-mechanism one (the other
    species are zero and get zero rates)."""
    torch = pytest.importorskip("torch")
    g, rho, yiT = _hot_tube_states(oracle)
    assert g.chem_set()[0] == 34
    R = torch.tensor(rho, device="cuda")
    Y = torch.tensor(yiT, device="cuda")
    F = torch.full_like(Y, np.nan)
    g.chem_rhs_device(len(rho), R.data_ptr(), Y.data_ptr(), F.data_ptr())
    f = F.cpu().numpy()
    K = len(names)
    absent = [k for k in range(K) if yiT[:, k].max() == 0.0 and ("N" in names[k].replace("AR", "") or names[k] == "AR")]
    assert len(absent) == K - 34 and np.all(f[:, absent] == 0.0)
    _rhs_check(oracle, names, rho, yiT, f)


def test_heat_release_rates(oracle, names):
    """HRR and HRR_dot of a reacting tube: the library's values against the
    reference formulas evaluated by the oracle on the library's own states
    (before/after the source step), then against the oracle tube's values."""
    case = configs.detonation(ncell=512, length=512 * 50e-6, driver=64 * 50e-6)
    # warm-started post-step Newton: the downloaded T is the integration's
    # final T to rounding (from 1000 K it would be within the Newton's own
    # stopping test of it)
    ot, g = detonation_pair(oracle, case, 1e-6, 1e-14, strict_newton=0)
    W = configs.molecular_weights()
    hf = oracle.vec("or_ckhms", 298.15)  # erg/g, std_heat_formation
    for _ in range(3):
        ot.step(case.cfl)
        g.step(case.cfl)
    ot.step(case.cfl)
    dt = g.calc_dt(case.cfl)
    g.solve_fluid(dt)
    qf_before, _, _ = g.download()
    g.solve_source(dt)
    g.post_step()
    qf_after, _, _ = g.download()
    hrr, hrr_dot = g.download_source()
    rho_cgs = qf_before[:, 0] * 1e-3
    dY = qf_after[:, 3:] - qf_before[:, 3:]
    terms = rho_cgs[:, None] * hf[None, :] * dY / dt
    hrr_ref = -terms.sum(axis=1) * 1e-1
    gross = np.abs(terms).sum(axis=1) * 1e-1
    assert np.all(np.abs(hrr - hrr_ref) <= 1e-10 * gross + 1e-300)
    dot_ref = np.zeros(case.ncell)
    dot_gross = np.zeros(case.ncell)
    for c in range(case.ncell):
        cd, dd = oracle.cdot_ddot(rho_cgs[c], qf_after[c, 2], qf_after[c, 3:])
        dot_ref[c] = -(W * hf * (cd - dd)).sum() * 1e-1
        dot_gross[c] = (np.abs(W * hf) * (cd + dd)).sum() * 1e-1
    # the library evaluates HRR_dot at the integration's final temperature,
    # the reference's qf(iqtemp)
    assert np.all(np.abs(hrr_dot - dot_ref) <= 1e-10 * dot_gross + 1e-300)
    assert np.abs(hrr_dot).max() > 0 and np.abs(hrr).max() > 0
    # end to end against the oracle tube (independent integrations: the
    # reacting bar, relative to the largest magnitude)
    hrr_o, dot_o = ot.source()
    assert np.abs(hrr - hrr_o).max() <= 1e-3 * np.abs(hrr_o).max()
    assert np.abs(hrr_dot - dot_o).max() <= 1e-3 * np.abs(dot_o).max()
    # a later fluid step does not lose the last source step's HRR_dot
    g.solve_fluid(g.calc_dt(case.cfl))
    _, dot_kept = g.download_source()
    assert np.array_equal(dot_kept, hrr_dot)


def test_inlet_boundary_frozen_parity(oracle, names):
    """lbound_inlet (SRC/boundary.f90:70-103, data from SRC/flow_bound.f90):
    air flowing in at 300 K with 60 kg/m^2/s, a pressure step downstream,
    fixed-pressure outlet; frozen chemistry, MUSCL-minmod + HLLC + TVDRK3.
    p, u, T within 1e-10 relative after 80 steps."""
    W = configs.molecular_weights()
    n = 400
    dx = 1e-3
    x_air = configs.mole_vector(names, {"O2": 0.21, "N2": 0.79})
    xm = (np.arange(n) + 0.5) * dx
    T = np.where(xm < 0.2, 300.0, 350.0)
    p = np.where(xm < 0.2, 1.2 * 101325.0, 101325.0)
    u = np.where(xm < 0.2, 50.0, 0.0)
    X = np.tile(x_air, (n, 1))
    qf0, qc0 = oracle.init_cells(T, p, u, X)
    rho_u_in = 60.0
    ot = oracle.tube(n, 2, [1, 2, 1, 2, 0, 1, 1, 0], [dx, 101325.0, 300.0, rho_u_in, 1e-5, 1e-13], x_in=x_air)
    ot.set_interior(qf0, qc0)
    g = Tube(n, dx, flag_acu=1, flag_muscl=2, flag_lbound=1, flag_rbound=1, p_out=101325.0, t_in=300.0,
             rho_u_in=rho_u_in, x_in=x_air)
    g.upload(qf0, qc0)
    for _ in range(80):
        d_o = ot.step(0.5)
        d_g = g.step(0.5)
        assert d_g == pytest.approx(d_o, rel=1e-12)
    qf_o, _ = ot.get()
    qf_g, _, _ = g.download()
    p_o, p_g = pressure(qf_o, W), pressure(qf_g, W)
    assert float(np.max(np.abs(p_g - p_o) / p_o)) < 1e-10
    assert float(np.max(np.abs(qf_g[:, 2] - qf_o[:, 2]) / qf_o[:, 2])) < 1e-10
    assert float(np.max(np.abs(qf_g[:, 1] - qf_o[:, 1]))) / np.abs(qf_o[:, 1]).max() < 1e-10
    # the inflow is felt: the first cells carry the inlet's mass flux
    assert abs(qf_o[0, 0] * qf_o[0, 1] - rho_u_in) / rho_u_in < 0.2
