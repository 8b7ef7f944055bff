"""GPU chemistry vs the FP64 reference integrator of the oracle.

Bar: species within 1e-3 relative and peak temperature within
0.1% of the FP64 reference for reacting cases. Species below 1e-6 in mass
fraction are compared in absolute terms (1e-9).
"""
import numpy as np
import pytest

from fortrancfd_gb300 import Reactors, Tube, configs

pytestmark = pytest.mark.gpu

REF_RTOL, REF_ATOL = 1e-10, 1e-16


def species_err(Yg, Yr, floor=1e-6):
    big = np.abs(Yr) >= floor
    rel = np.where(big, np.abs(Yg - Yr) / np.maximum(np.abs(Yr), floor), 0.0)
    ab = np.where(~big, np.abs(Yg - Yr), 0.0)
    return float(rel.max()), float(ab.max())


def element_moles(Y, names, W):
    # O, H, C, N, Ar atoms per unit mass
    comp = {"O": [], "H": [], "C": [], "N": []}
    import re
    out = np.zeros((Y.shape[0], 4))
    for k, nm in enumerate(names):
        for e_i, e in enumerate("OHCN"):
            cnt = 0
            for sym, num in re.findall(r"([A-Z][a-z]?)(\d*)", nm.replace("(S)", "")):
                if sym == e:
                    cnt += int(num) if num else 1
            out[:, e_i] += cnt * Y[:, k] / W[k]
    return out


def test_reactor_batch_vs_fp64_reference(oracle, names):
    rho, dt, yiT, _ = configs.reactor_batch(96, seed=3)
    ref, fails, _ = oracle.reactor_batch(rho, dt, yiT, REF_RTOL, REF_ATOL)
    assert fails == 0
    r = Reactors(rtol=1e-6, atol=1e-14)
    y = yiT.copy()
    st = r.integrate(rho, dt, y)
    assert st["failed"] == 0 and st["rhs"] > 0
    K = len(names)
    rel_err, abs_err = species_err(y[:, :K], ref[:, :K])
    assert rel_err < 1e-3, rel_err
    assert abs_err < 1e-9, abs_err
    assert np.max(np.abs(y[:, K] - ref[:, K]) / ref[:, K]) < 1e-3


def test_reactor_conservation(oracle, names):
    rho, dt, yiT, _ = configs.reactor_batch(64, seed=4)
    W = configs.molecular_weights()
    K = len(names)
    r = Reactors(rtol=1e-6, atol=1e-14)
    y = yiT.copy()
    r.integrate(rho, dt, y)
    e0 = element_moles(yiT[:, :K], names, W)
    e1 = element_moles(y[:, :K], names, W)
    assert np.max(np.abs(e1 - e0) / np.maximum(e0, 1e-12)) < 1e-6
    assert np.max(np.abs(y[:, :K].sum(axis=1) - 1.0)) < 1e-8


def test_reactor_matches_oracle_same_tolerance(oracle, names):
    """Same method, same tolerance: only the FP32 Jacobian/LU differ."""
    rho, dt, yiT, _ = configs.reactor_batch(48, seed=5)
    ref, fails, _ = oracle.reactor_batch(rho, dt, yiT, 1e-6, 1e-14)
    y = yiT.copy()
    Reactors(rtol=1e-6, atol=1e-14).integrate(rho, dt, y)
    K = len(names)
    rel_err, _ = species_err(y[:, :K], ref[:, :K])
    assert rel_err < 1e-3


def ignition_delays(integrate, rho, yiT, t_max=1e-3, rise=400.0):
    """Ignition delay of each fresh reactor: the time its temperature first
    exceeds T0 + rise, bracketed by doubling time chunks from 1e-7 s and
    refined by three bisections (to 1/8 of the bracket); reactors that do not
    ignite by t_max get t_max. integrate(rho, dt, y) advances y in place."""
    T0 = yiT[:, -1].copy()
    n = len(rho)
    tau = np.full(n, t_max)
    t = np.zeros(n)
    state = yiT.copy()
    chunk = np.full(n, 1e-7)
    active = np.ones(n, bool)
    while active.any():
        idx = np.nonzero(active)[0]
        out = state[idx].copy()
        integrate(rho[idx], chunk[idx], out)
        ign = out[:, -1] > T0[idx] + rise
        hit, miss = idx[ign], idx[~ign]
        if len(hit):
            lo, hi = np.zeros(len(hit)), chunk[hit].copy()
            for _ in range(3):
                mid = 0.5 * (lo + hi)
                o = state[hit].copy()
                integrate(rho[hit], mid, o)
                up = o[:, -1] > T0[hit] + rise
                hi, lo = np.where(up, mid, hi), np.where(up, lo, mid)
            tau[hit] = t[hit] + hi
            active[hit] = False
        state[miss] = out[~ign]
        t[miss] += chunk[miss]
        chunk[miss] *= 2.0
        active[miss[t[miss] >= t_max]] = False
    return tau


def test_partially_reacted_batch_vs_fp64_reference(oracle, names):
    """The batched-reactor workload: CH4/air reactors with T ~ U[900, 2500] K,
    p log-uniform in [1, 50] atm, phi ~ U[0.5, 2], each advanced a seeded
    fraction U[0, 1] of its own ignition delay (capped at 1 ms: the slowest,
    coolest mixtures are taken in early induction), then one GPU reactor step of
    dt log-uniform in [1e-8, 1e-6] s against the FP64 oracle at tight
    tolerance. The partially reacted states are inputs only: they come from
    the library's reactor batch at rtol 1e-7 (long integrations at the
    oracle's tight tolerance take minutes)."""
    n = 128
    rho, dt, fresh, _ = configs.reactor_batch(n, seed=0)
    pre = Reactors(rtol=1e-7, atol=1e-15)

    def integrate(r, d, y):
        # windows of at most 10 us per call (a call takes at most 4000 steps)
        rem = np.array(d, dtype=float)
        while (rem > 0.0).any():
            idx = np.nonzero(rem > 0.0)[0]
            step = np.minimum(rem[idx], 1e-5)
            sub = np.ascontiguousarray(y[idx])
            st = pre.integrate(np.ascontiguousarray(r[idx]), step, sub)
            assert st["failed"] == 0
            y[idx] = sub
            rem[idx] -= step

    tau = ignition_delays(integrate, rho, fresh)
    frac = np.random.default_rng(100).uniform(0.0, 1.0, n)
    yiT = fresh.copy()
    integrate(rho, frac * tau, yiT)
    ref, fails, _ = oracle.reactor_batch(rho, dt, yiT, REF_RTOL, REF_ATOL)
    assert fails == 0
    r = Reactors(rtol=1e-6, atol=1e-14)
    y = yiT.copy()
    st = r.integrate(rho, dt, y)
    assert st["failed"] == 0
    K = len(names)
    rel_err, abs_err = species_err(y[:, :K], ref[:, :K])
    assert rel_err < 1e-3, rel_err
    assert abs_err < 1e-9, abs_err
    assert np.max(np.abs(y[:, K] - ref[:, K]) / ref[:, K]) < 1e-3
    # the states span fresh to burnt
    assert (yiT[:, K] - fresh[:, K]).max() > 500.0 and np.median(tau) < 1e-3


def test_tube_chemistry_short_run(oracle, names):
    """Reacting detonation tube, a few full steps (fluid + chemistry)."""
    case = configs.detonation(ncell=512, length=512 * 50e-6, driver=64 * 50e-6)
    fl = case.flags
    qf0, qc0 = oracle.init_cells(case.T, case.p, case.u, case.X)
    ot = oracle.tube(case.ncell, 3, [1, 2, 2, 2, 3, 0, 1, 1], [case.dx, 101325.0, 300.0, 0.0, REF_RTOL, REF_ATOL])
    ot.set_interior(qf0, qc0)
    g = Tube(case.ncell, case.dx, flag_acu=2, flag_weno=3, flag_rbound=1, do_reaction=1, rtol=1e-6, atol=1e-14)
    g.upload(qf0, qc0)
    teams = []
    for _ in range(5):
        ot.step(case.cfl)
        g.step(case.cfl)
        teams.append(g.chem_stats()["team_cells"])
    # the costliest cells of each call after the first go to four-warp teams
    assert teams[0] == 0 and min(teams[1:]) > 0, teams
    cost, hot = g.chem_cost()
    assert cost.max() >= 32 and len(hot) > 0
    assert int(np.argmax(cost)) in set(hot.tolist())
    qf_o, _ = ot.get()
    qf_g, _, hrr = g.download()
    K = len(names)
    assert np.max(np.abs(qf_g[:, 2] - qf_o[:, 2]) / qf_o[:, 2]) < 1e-3
    rel_err, abs_err = species_err(qf_g[:, 3:], qf_o[:, 3:])
    assert rel_err < 1e-3, rel_err
    assert abs(qf_g[:, 2].max() - qf_o[:, 2].max()) / qf_o[:, 2].max() < 1e-3
    assert np.all(np.isfinite(hrr))


def test_species_subset_matches_full_tables(oracle, names):
    """CH4/O2 holds no N or Ar: the chemistry integrates the 34 C/H/O species
    and their reactions. Traces of N2 and Ar (mass fraction 1e-300 in the
    driver) bring back the full tables; both give the same tube."""
    case = configs.detonation(ncell=256, length=256 * 50e-6, driver=48 * 50e-6)
    qf0, qc0 = oracle.init_cells(case.T, case.p, case.u, case.X)
    out, sets = [], []
    for trace in (False, True):
        qc = qc0.copy()
        if trace:
            for sp in ("N2", "AR"):
                qc[:8, 3 + names.index(sp)] = qc[:8, 0] * 1e-300
        g = Tube(case.ncell, case.dx, flag_acu=2, flag_weno=3, flag_rbound=1, do_reaction=1, rtol=1e-6, atol=1e-14)
        g.upload(None, qc)
        sets.append(g.chem_set())
        for _ in range(4):
            g.step(case.cfl)
        out.append(g.download()[0])
    K = len(names)
    assert sets[0][0] == 34 and sets[0][1] < sets[1][1] and sets[1] == (K, sets[1][1]), sets
    assert np.max(np.abs(out[0][:, 2] - out[1][:, 2]) / out[1][:, 2]) < 1e-5
    rel_err, abs_err = species_err(out[0][:, 3:], out[1][:, 3:])
    assert rel_err < 1e-3, rel_err
    n_species = [i for i, s in enumerate(names) if "N" in s.replace("AR", "")] + [names.index("AR")]
    assert np.all(out[0][:, 3 + np.array(n_species)] == 0.0)


def test_table_exp_within_one_ulp():
    """The FP64 exponential of the rate evaluation (table-driven, Tang's
    method) against CUDA's exp: at most 1 ulp apart."""
    r = Reactors()
    rng = np.random.default_rng(11)
    x = np.concatenate([rng.uniform(-700.0, 700.0, 1 << 20), rng.uniform(-0.7, 0.7, 1 << 16),
                        rng.uniform(-60.0, 5.0, 1 << 16)])
    assert r.check_exp(x) <= 1.0


def test_table_log_within_two_ulp():
    """The FP64 natural logarithm of the rate evaluation (table-driven)
    against CUDA's log: at most 2 ulp apart, including arguments near 1."""
    r = Reactors()
    rng = np.random.default_rng(12)
    x = np.concatenate([np.exp(rng.uniform(-690.0, 690.0, 1 << 20)), 1.0 + rng.uniform(-0.05, 0.05, 1 << 16),
                        rng.uniform(100.0, 8000.0, 1 << 16)])
    assert r.check_log(x) <= 2.0


def test_chemistry_launch_forms_agree(oracle, names):
    """The one-pass launch and the screening pass + listed integration give
    the same tube up to rounding, stepped from the host and in the device
    loop: an inert cell is finished with the same arithmetic either way and
    listed cells by the same kernel; the one difference is a cell on the
    team list that turns out inert, which the one-pass form finishes on its
    four-warp team and the two-pass form on a single warp (their sums run in
    different orders)."""
    case = configs.detonation(ncell=1024, length=1024 * 50e-6, driver=96 * 50e-6)
    qf0, qc0 = oracle.init_cells(case.T, case.p, case.u, case.X)
    out = []
    for form in (1, 2):
        g = Tube(case.ncell, case.dx, flag_acu=2, flag_weno=3, flag_rbound=1, do_reaction=1, rtol=1e-6, atol=1e-14)
        g.set_chem_launch(form)
        g.upload(qf0, qc0)
        for _ in range(4):
            g.step(case.cfl)
        t, n = g.advance(case.cfl, tend=1e9, max_steps=20)
        out.append(g.download()[0])
    a, b = out
    assert np.max(np.abs(a[:, 2] - b[:, 2]) / b[:, 2]) < 1e-8
    assert np.max(np.abs(a[:, 0] - b[:, 0]) / b[:, 0]) < 1e-8
    rel_err, abs_err = species_err(a[:, 3:], b[:, 3:])
    assert rel_err < 1e-5 and abs_err < 1e-12, (rel_err, abs_err)


def test_single_precision_precheck_agrees_with_fp64_test():
    """The FP32 pre-check of the inert-cell test decides the cold mixture
    ahead of a detonation front without an FP64 right-hand side, in both
    launch forms, and the tube agrees with the same run with every cell
    through the FP64 test: a decided cell's step differs by under 1e-3 of
    its error tolerance (bar: 1e-10 in T and rho, rtol in species)."""
    case = configs.detonation(ncell=1024, length=1024 * 50e-6, driver=96 * 50e-6)
    for form in (1, 2):
        out, stats = [], []
        for pre in (True, False):
            g = Tube(case.ncell, case.dx, flag_acu=2, flag_weno=3, flag_rbound=1, do_reaction=1, rtol=1e-6,
                     atol=1e-14)
            g.set_chem_launch(form)
            g.set_chem_precheck(pre)
            g.set_uniform_skip(False)  # every cell through the screen (no runs of identical cells)
            g.init_cells(case.T, case.p, case.u, case.X)
            for _ in range(6):
                g.step(case.cfl)
            stats.append(g.chem_stats())
            out.append(g.download()[0])
            g.close()
        on, off = stats
        assert off["cells32"] == 0
        assert on["cells32"] > case.ncell // 2, on
        assert on["rhs"] < off["rhs"] - on["cells32"] // 2, (on, off)
        a, b = out
        assert np.max(np.abs(a[:, 2] - b[:, 2]) / b[:, 2]) < 1e-10
        assert np.max(np.abs(a[:, 0] - b[:, 0]) / b[:, 0]) < 1e-10
        rel_err, abs_err = species_err(a[:, 3:], b[:, 3:])
        assert rel_err < 1e-6 and abs_err < 1e-13, (form, rel_err, abs_err)


def test_repeated_runs_are_bit_for_bit():
    """The same reacting tube twice, four-warp teams included (from the
    second launch on), gives the same bits: no step of the chemistry depends
    on the order in which warps or CTAs run."""
    case = configs.detonation(ncell=1024, length=1024 * 50e-6, driver=96 * 50e-6)
    out = []
    for _ in range(2):
        g = Tube(case.ncell, case.dx, flag_acu=2, flag_weno=3, flag_rbound=1, do_reaction=1, rtol=1e-6, atol=1e-14)
        g.init_cells(case.T, case.p, case.u, case.X)
        for _ in range(6):
            g.step(case.cfl)
        teams = g.chem_stats()["team_cells"]
        out.append(g.download()[0])
        g.close()
    assert teams > 0
    assert np.array_equal(out[0], out[1])
