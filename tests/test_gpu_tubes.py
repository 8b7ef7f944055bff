"""Several uneven tubes in one context (edyn_init_tubes): every tube with its
own cell count, cell size, outlet pressure and time step, all advanced in the
same kernel launches (one stage launch over every tube's tiles, one
chemistry launch over every tube's cells).

* Frozen flow: four uneven tubes against four separate oracle tubes, each
  with its own calc_dt: p, u, T within 1e-10 relative, the same per-tube
  simulated times; and bit for bit the same as four single-tube contexts.
* Reacting flow: the same four tubes with chemistry against the oracle:
  species within 1e-3 relative, peak temperature within 0.1 %.
"""
import numpy as np
import pytest

from fortrancfd_gb300 import Tube, Tubes, configs

pytestmark = pytest.mark.gpu

R_SI = 8314.51
FLAGS_O = [1, 2, 2, 2, 3, 0, 1]  # TVDRK3, HLLC, WENO5-Z, wall / outlet


def _cases():
    return configs.uneven_tubes(4, seed=3, cells=(180, 520), length=(0.02, 0.05))


def _pressure(qf, W):
    return qf[:, 0] * R_SI * qf[:, 2] * (qf[:, 3:] / W).sum(axis=1)


def _packed(cases, do_reaction, strict=1, rtol=1e-6, atol=1e-14):
    g = Tubes([c.ncell for c in cases], [c.dx for c in cases], p_outs=[c.flags["p_out"] for c in cases],
              do_reaction=do_reaction, strict_newton=strict, rtol=rtol, atol=atol)
    g.init_cells(np.concatenate([c.T for c in cases]), np.concatenate([c.p for c in cases]),
                 np.concatenate([c.u for c in cases]), np.concatenate([c.X for c in cases]))
    return g


def _oracle_tubes(oracle, cases, do_reaction, rtol=1e-6, atol=1e-14):
    out = []
    for c in cases:
        qf0, qc0 = oracle.init_cells(c.T, c.p, c.u, c.X)
        ot = oracle.tube(c.ncell, 3, FLAGS_O + [do_reaction], [c.dx, c.flags["p_out"], 300.0, 0.0, rtol, atol])
        ot.set_interior(qf0, qc0)
        out.append(ot)
    return out


def test_frozen_uneven_tubes_match_oracle(oracle):
    cases = _cases()
    W = configs.molecular_weights()
    g = _packed(cases, 0)
    ots = _oracle_tubes(oracle, cases, 0)
    nsteps = 30
    t_o = np.zeros(len(cases))
    for _ in range(nsteps):
        for k, ot in enumerate(ots):
            t_o[k] += ot.step(0.4)
        g.step(0.4)
    t_g, _ = g.times()
    assert np.allclose(t_g, t_o, rtol=1e-12, atol=0)
    assert len(set(np.round(t_o / t_o[0], 6))) > 1  # the tubes took different time steps
    qf_g = g.split(g.download()[0])
    for k, ot in enumerate(ots):
        qf_o, _ = ot.get()
        p_o, p_g = _pressure(qf_o, W), _pressure(qf_g[k], W)
        assert float(np.max(np.abs(p_g - p_o) / p_o)) < 1e-10, k
        assert float(np.max(np.abs(qf_g[k][:, 2] - qf_o[:, 2]) / qf_o[:, 2])) < 1e-10, k
        assert float(np.max(np.abs(qf_g[k][:, 1] - qf_o[:, 1]))) / np.abs(qf_o[:, 1]).max() < 1e-10, k


def test_packed_frozen_tubes_equal_single_tube_contexts():
    """The packed launch computes every face and cell with the same
    arithmetic as a one-tube context (tiles do not change results)."""
    cases = _cases()
    g = _packed(cases, 0, strict=0)
    g.advance(0.4, tend=1e9, max_steps=24)
    qf_p = g.split(g.download()[0])
    for k, c in enumerate(cases):
        s = Tube(c.ncell, c.dx, flag_acu=2, flag_weno=3, flag_rbound=1, p_out=c.flags["p_out"], strict_newton=0)
        s.init_cells(c.T, c.p, c.u, c.X)
        s.advance(0.4, tend=1e9, max_steps=24)
        assert np.array_equal(s.download()[0], qf_p[k]), k


def test_reacting_uneven_tubes_match_oracle(oracle, names):
    cases = _cases()
    g = _packed(cases, 1)
    ots = _oracle_tubes(oracle, cases, 1)
    for _ in range(8):
        for ot in ots:
            ot.step(0.4)
        g.step(0.4)
    qf_g = g.split(g.download()[0])
    for k, ot in enumerate(ots):
        qf_o, _ = ot.get()
        assert abs(qf_g[k][:, 2].max() - qf_o[:, 2].max()) / qf_o[:, 2].max() < 1e-3, k
        Yg, Yo = qf_g[k][:, 3:], qf_o[:, 3:]
        big = np.abs(Yo) >= 1e-6
        rel = np.where(big, np.abs(Yg - Yo) / np.maximum(np.abs(Yo), 1e-6), 0.0).max()
        assert rel < 1e-3, (k, rel)
    hrr = g.split(g.download()[2])
    assert all(np.all(np.isfinite(h)) for h in hrr)


def test_packed_reacting_tubes_uniform_skip_is_bit_for_bit():
    """Runs of identical cells never cross a tube boundary: four packed
    reacting tubes through the two-pass chemistry give the same bits with
    the uniform-region shortcuts on and off."""
    cases = _cases()
    out = []
    for on in (True, False):
        g = _packed(cases, 1)
        g.set_chem_launch(2)
        g.set_uniform_skip(on)
        for _ in range(6):
            g.step(0.4)
        qf, qc, hrr = g.download()
        out.append((qf, qc, hrr, g.chem_stats()["cells_same"]))
        g.close()
    assert out[0][3] > 0 and out[1][3] == 0
    for a, b in zip(out[0][:3], out[1][:3]):
        assert np.array_equal(a, b)
