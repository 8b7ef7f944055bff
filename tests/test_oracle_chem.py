"""Oracle chemistry: the FP64 reference integrator (CPU only).

The reference's own integrator is not shipped, so the FP64 reference is
validated by self-convergence, conservation of mass, elements and internal
energy, and a physical ignition check.
"""
import ctypes

import numpy as np
import pytest

from fortrancfd_gb300 import configs

P = ctypes.POINTER(ctypes.c_double)


def energy(oracle, T, Y):
    W = configs.molecular_weights()
    X = (Y / W) / (Y / W).sum()
    x = np.ascontiguousarray(X)
    return oracle.L.or_specific_energy(oracle.mech, T, x.ctypes.data_as(P))


def test_self_convergence(oracle):
    rho, dt, yiT, _ = configs.reactor_batch(24, seed=7)
    a, fa, _ = oracle.reactor_batch(rho, dt, yiT, 1e-8, 1e-18)
    b, fb, _ = oracle.reactor_batch(rho, dt, yiT, 1e-11, 1e-20)
    assert fa == 0 and fb == 0
    big = np.abs(b[:, :53]) > 1e-8
    assert np.max(np.abs(a[:, :53] - b[:, :53])[big] / np.abs(b[:, :53])[big]) < 1e-5
    assert np.max(np.abs(a[:, 53] - b[:, 53]) / b[:, 53]) < 1e-7


def test_conservation(oracle, names):
    rho, dt, yiT, _ = configs.reactor_batch(24, seed=8)
    y, f, _ = oracle.reactor_batch(rho, dt, yiT, 1e-8, 1e-18)
    assert f == 0
    assert np.max(np.abs(y[:, :53].sum(axis=1) - 1.0)) < 1e-13
    for c in range(24):
        e0 = energy(oracle, yiT[c, 53], yiT[c, :53])
        e1 = energy(oracle, y[c, 53], y[c, :53])
        assert abs(e1 - e0) < 1e-6 * (abs(e0) + 1e6)


def test_ignition(oracle, names):
    W = configs.molecular_weights()
    X = configs.ch4_air_mixture(names, 1.0)
    Y = configs.x_to_y(names, X, W)
    T0, p = 1500.0, 101325.0
    rho = p * (1.0 / (Y / W).sum()) / (8314.51 * T0)
    y = np.concatenate([Y, [T0]])[None, :]
    # called the way the flow solver calls it: 250 windows of 20 us
    for _ in range(250):
        y, f, _ = oracle.reactor_batch(np.array([rho]), np.array([2e-5]), y, 1e-7, 1e-16)
        assert f == 0
    assert y[0, 53] > 2400.0
    assert y[0, names.index("CO2")] > 0.05
