"""The learned surrogate inside the tube's source step (EDYN_IF_CHEM_MODE 1).

A network is trained on the GPU (the library's tcgen05 forward/backward
kernels) on pairs harvested from 5 um CH4/air detonation tubes over a
seeded sweep of equivalence ratio and driver temperature: exactly the cells
that a chem_mode 1 tube hands to its surrogate (those that fail the
integrator's inert-cell test), advanced by the implicit integrator at
rtol 1e-8. It is then attached to a tube of another seed's mixture and
compared with:

* the plain path (chem_mode 0) on the same tube: species within 1e-3
  relative (mass fractions >= 1e-6) and peak temperature within 0.1 %;
* the same path without the network (the gated explicit increment, then the
  integrator): the network must add accepted cells and save right-hand
  sides of the fallback integration, summed over the steps -- a network
  that gains nothing fails here.
"""
import numpy as np
import pytest

from fortrancfd_gb300 import Reactors, Tube

pytestmark = pytest.mark.gpu

STEPS = 30


def species_err(Yg, Yr, floor=1e-6):
    big = np.abs(Yr) >= floor
    return float(np.where(big, np.abs(Yg - Yr) / np.maximum(np.abs(Yr), floor), 0.0).max())


@pytest.fixture(scope="module")
def trained():
    torch = pytest.importorskip("torch")
    from fortrancfd_gb300 import surrogate as S

    cases = S.tube_sweep(4, seed=0)
    rho, dt, y0, y1 = S.harvest_screened(cases, nsteps=80)
    s = S.Surrogate(Reactors(rtol=1e-5, atol=1e-13), S.MLP(seed=0))
    S.train(s, rho, dt, y0, y1, iters=2000, batch=4096, lr=2e-3)
    torch.cuda.synchronize()
    return s


@pytest.fixture(scope="module")
def held_out():
    from fortrancfd_gb300 import surrogate as S

    return S.tube_sweep(1, seed=7)[0]


def _run(case, mode, surr, use_net=True, steps=STEPS, runs=False):
    g = Tube(case.ncell, case.dx, strict_newton=0, rtol=1e-5, atol=1e-13, chem_mode=mode, **case.flags)
    # every cell through the surrogate path unless runs of identical cells
    # are asked for (then only their heads are, with the same results)
    g.set_uniform_skip(runs)
    if mode == 1:
        g.set_surrogate(surr if use_net else None)
    g.init_cells(case.T, case.p, case.u, case.X)
    acc = {"handed": 0, "accepted_network": 0, "accepted_explicit": 0, "fallback": 0, "fallback_rhs": 0}
    for _ in range(steps):
        g.step(case.cfl)
        if mode == 1:
            st = g.surrogate_stats()
            for k in acc:
                acc[k] += st[k]
    qf, _, _ = g.download()
    g.close()
    return qf, acc


def test_tube_surrogate_matches_plain(trained, held_out):
    qf0, _ = _run(held_out, 0, None)
    qf1, acc = _run(held_out, 1, trained)
    assert acc["handed"] > 0
    # every handed cell is accounted for by exactly one of the three ways
    assert acc["accepted_network"] + acc["accepted_explicit"] + acc["fallback"] == acc["handed"]
    assert species_err(qf1[:, 3:], qf0[:, 3:]) < 1e-3
    assert abs(qf1[:, 2].max() - qf0[:, 2].max()) / qf0[:, 2].max() < 1e-3


def test_network_gains_over_the_method_without_it(trained, held_out):
    _, with_net = _run(held_out, 1, trained)
    _, without = _run(held_out, 1, None, use_net=False)
    assert with_net["accepted_network"] > 0, with_net
    assert with_net["fallback"] < without["fallback"], (with_net, without)
    assert with_net["fallback_rhs"] < without["fallback_rhs"], (with_net, without)


def test_runs_of_identical_cells_are_bit_for_bit(trained, held_out):
    """The surrogate path over run heads only (followers take their head's
    finished column) gives the same bits as every cell through it."""
    out = []
    for runs in (True, False):
        g = Tube(held_out.ncell, held_out.dx, strict_newton=0, rtol=1e-5, atol=1e-13, chem_mode=1, **held_out.flags)
        g.set_uniform_skip(runs)
        g.set_surrogate(trained)
        g.init_cells(held_out.T, held_out.p, held_out.u, held_out.X)
        handed = 0
        for _ in range(10):
            g.step(held_out.cfl)
            handed += g.surrogate_stats()["handed"]
        out.append((g.download(), handed))
        g.close()
    (a, ha), (b, hb) = out
    assert 0 < ha < hb, (ha, hb)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
