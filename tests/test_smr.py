"""SMR blocks in the oracle (CPU), restated from SRC/block.f90:475-569
(interpolation_block) and the stage tails around it: segments of equal-dx
blocks exchange ghosts by copy, so equal segments must reproduce one tube
bit for bit; at a change of level the ghosts are restricted (mean of two fine
cells) and prolonged (coarse cell +- 1/4 of its minmod slope). A uniform
state stays bit for bit uniform across levels, and a Sod problem on a
fine / coarse / fine grid stays close to the uniform fine grid's.
"""
import numpy as np
import pytest

from fortrancfd_gb300 import configs, species_names
from oracle_ctypes import _D

RP = [1e-3, configs.ATM, 300.0, 0.0, 1e-5, 1e-13]


def sod_state(oracle, xm, xs):
    """The Sod state with qf = QcToqf(Qc) in every cell, so that a block's
    ghost (QcToqf of a copied Qc column) equals its neighbour's qf."""
    nm = species_names()
    x = configs.mole_vector(nm, {"CH4": 0.0950570342, "O2": 0.1901140684, "N2": 0.7148288973})
    left = xm <= xs
    n = len(xm)
    _, qc = oracle.init_cells(np.where(left, 375.0, 300.0), np.where(left, 10 * configs.ATM, configs.ATM),
                              np.zeros(n), np.tile(x, (n, 1)))
    qf = np.zeros_like(qc)
    for i in range(n):
        oracle.L.or_qc_to_qf(oracle.mech, qc[i].ctypes.data_as(_D), qf[i].ctypes.data_as(_D))
    return qf, qc


@pytest.mark.parametrize("flags,lvir", [([1, 2, 1, 2, 0, 0, 0, 0], 2), ([1, 2, 2, 2, 3, 0, 1, 0], 3),
                                        ([0, 1, 1, 4, 0, 0, 0, 0], 2)])
def test_equal_segments_reproduce_one_tube(oracle, flags, lvir):
    n, dx = 120, 1e-3
    xm = (np.arange(n) + 0.5) * dx
    qf, qc = sod_state(oracle, xm, 0.5 * n * dx)
    t = oracle.tube(n, lvir, flags, RP)
    t.set_interior(qf, qc)
    s = oracle.smr([40, 50, 30], [dx, dx, dx], lvir, flags, RP)
    s.set_interior(qf, qc)
    for _ in range(30):
        assert t.step(0.5) == s.step(0.5)
    np.testing.assert_array_equal(s.get()[1], t.get()[1])
    np.testing.assert_array_equal(s.get()[0], t.get()[0])


def test_uniform_state_stays_uniform_across_levels(oracle):
    nm = species_names()
    air = configs.mole_vector(nm, {"O2": 0.21, "N2": 0.79})
    ncells, dxs = [32, 16, 32], [1e-3, 2e-3, 1e-3]
    n = sum(ncells)
    _, qc = oracle.init_cells(np.full(n, 500.0), np.full(n, configs.ATM), np.zeros(n), np.tile(air, (n, 1)))
    qf = np.zeros_like(qc)
    for i in range(n):
        oracle.L.or_qc_to_qf(oracle.mech, qc[i].ctypes.data_as(_D), qf[i].ctypes.data_as(_D))
    s = oracle.smr(ncells, dxs, 2, [1, 2, 1, 2, 0, 0, 0, 0], RP)
    s.set_interior(qf, qc)
    for _ in range(10):
        s.step(0.5)
    np.testing.assert_array_equal(s.get()[1], qc)


def test_refined_sod_close_to_uniform_grid(oracle):
    """Fine (1 mm) / coarse (2 mm) / fine grid against the uniform 1 mm grid:
    the shock and contact cross the coarse block; p and rho within a few
    percent of the jump in L1, and the total mass within 1e-3 (the interface
    fluxes are evaluated once per block, so SMR is not exactly conservative)."""
    dx = 1e-3
    nf = 240
    xm_f = (np.arange(nf) + 0.5) * dx
    flags = [1, 2, 1, 2, 0, 0, 0, 0]
    qf, qc = sod_state(oracle, xm_f, 0.3)
    t = oracle.tube(nf, 2, flags, RP)
    t.set_interior(qf, qc)
    ncells, dxs = [100, 40, 60], [dx, 2 * dx, dx]
    xm_s = np.concatenate([(np.arange(100) + 0.5) * dx, 0.1 + (np.arange(40) + 0.5) * 2 * dx,
                           0.18 + (np.arange(60) + 0.5) * dx])
    qf_s, qc_s = sod_state(oracle, xm_s, 0.3)
    s = oracle.smr(ncells, dxs, 2, flags, RP)
    s.set_interior(qf_s, qc_s)
    for _ in range(120):
        dt = t.step(0.5)
        assert s.step(0.5) == pytest.approx(dt, rel=0.05)
    qf_t, _ = t.get()
    qf_r, qc_r = s.get()
    W = configs.molecular_weights()

    def p(q):
        return q[:, 0] * 8314.51 * q[:, 2] * (q[:, 3:] / W).sum(axis=1)

    ref_p = np.interp(xm_s, xm_f, p(qf_t))
    ref_r = np.interp(xm_s, xm_f, qf_t[:, 0])
    w = np.concatenate([np.full(100, dx), np.full(40, 2 * dx), np.full(60, dx)])
    assert (w * np.abs(p(qf_r) - ref_p)).sum() / w.sum() < 0.03 * 9 * configs.ATM
    assert (w * np.abs(qf_r[:, 0] - ref_r)).sum() / w.sum() < 0.03 * 7 * qf_t[:, 0].min()
    mass0 = (w * qc_s[:, 0]).sum()
    assert abs((w * qc_r[:, 0]).sum() - mass0) < 1e-3 * mass0


def device_ghosts(seg_qc, ncells, dxs, lvir):
    """The GPU's interface ghosts, emulated: the pre-stage snapshot's layout
    ([interface][side][row][cell], 2 lvir cells a side) and the accessors of
    smr_ghost_qc (fortrancfd_gb300/csrc/fluid.cu), for every segment's
    ghosts that face another segment. Returns {(segment, g): column}."""
    S = 2 * lvir
    ne = seg_qc[0].shape[1]
    out = {}
    for t in range(len(ncells)):
        for g in list(range(-lvir, 0)) + list(range(ncells[t], ncells[t] + lvir)):
            left = g < 0
            if (left and t == 0) or (not left and t == len(ncells) - 1):
                continue
            j = t - 1 if left else t
            l = -g if left else g - ncells[t] + 1
            snap = np.zeros((2, ne, S))
            snap[0] = seg_qc[j][ncells[j] - S:ncells[j]].T
            snap[1] = seg_qc[j + 1][0:S].T
            col = np.zeros(ne)
            for v in range(ne):
                sl, sr = snap[0, v], snap[1, v]

                def lx(idx):
                    return sl[S - 1 + idx] if idx <= 0 else (sr[2 * (idx - 1)] + sr[2 * (idx - 1) + 1]) / 2.0

                def rx(idx):
                    return sr[idx] if idx >= 0 else (sl[S - 1 - 2 * (-idx - 1)] + sl[S - 1 - 2 * (-idx - 1) - 1]) / 2.0

                def slope(m, p):
                    return 0.5 * (np.copysign(1.0, m) + np.copysign(1.0, p)) * min(abs(m), abs(p))

                if dxs[j] == dxs[j + 1]:
                    q = lx(-(l - 1)) if left else rx(l - 1)
                elif dxs[j] > dxs[j + 1]:
                    if not left:
                        q = lx(l)
                    else:
                        ic = -((l - 1) // 2)
                        c = lx(ic)
                        d = slope(c - lx(ic - 1), lx(ic + 1) - c)
                        q = c + 0.25 * d if l % 2 == 1 else c - 0.25 * d
                else:
                    if left:
                        q = rx(-l)
                    else:
                        ic = (l - 1) // 2
                        c = rx(ic)
                        d = slope(c - rx(ic - 1), rx(ic + 1) - c)
                        q = c - 0.25 * d if l % 2 == 1 else c + 0.25 * d
                col[v] = q
            out[t, g] = col
    return out


@pytest.mark.parametrize("lvir,dxs", [(1, [1e-3, 2e-3, 1e-3]), (2, [2e-3, 1e-3, 2e-3]), (3, [1e-3, 2e-3, 4e-3]),
                                      (4, [4e-3, 2e-3, 2e-3]), (2, [1e-3, 1e-3, 2e-3])])
def test_interface_ghosts_device_form_matches_oracle(oracle, lvir, dxs):
    """The device's ghost construction (emulated above from its snapshot
    layout and accessors) gives the oracle's interpolation_block ghosts bit
    for bit, for every level relation and ghost depth, on a state with
    non-monotone conserved rows (so that every minmod branch is taken)."""
    ncells = [24, 20, 28]
    n = sum(ncells)
    rng = np.random.default_rng(lvir)
    nm = species_names()
    air = configs.mole_vector(nm, {"O2": 0.21, "N2": 0.79})
    T = 300.0 + 400.0 * rng.random(n)
    _, qc = oracle.init_cells(T, configs.ATM * (1 + 0.5 * rng.random(n)), 50.0 * rng.standard_normal(n),
                              np.tile(air, (n, 1)))
    qf = np.zeros_like(qc)
    for i in range(n):
        oracle.L.or_qc_to_qf(oracle.mech, qc[i].ctypes.data_as(_D), qf[i].ctypes.data_as(_D))
    flags = [1, 2, 1, 2, 0, 0, 0, 0] if lvir <= 2 else [1, 2, 2, 2, 3 if lvir == 3 else 4, 0, 0, 0]
    s = oracle.smr(ncells, dxs, lvir, flags, RP)
    s.set_interior(qf, qc)
    segs = np.split(qc, np.cumsum(ncells)[:-1])
    dev = device_ghosts(segs, ncells, dxs, lvir)
    assert len(dev) == 4 * lvir
    for (t, g), col in dev.items():
        full = s.segment_all(t, ncells[t], lvir)
        np.testing.assert_array_equal(full[g + lvir], col, err_msg=f"segment {t} ghost {g}")


def test_equal_segments_with_transport_reproduce_one_tube(oracle):
    """Transport across block interfaces: with equal cell sizes the blocks'
    ghosts are copies, so the transport flux of every face, recomputed by
    each block from its own ghosts, is the tube's."""
    n, dx = 90, 2e-5
    xm = (np.arange(n) + 0.5) * dx
    nm = species_names()
    w = 0.5 * (1 + np.tanh((xm - 0.5 * n * dx) / (4 * dx)))
    air = configs.mole_vector(nm, {"O2": 0.21, "N2": 0.79})
    rich = configs.mole_vector(nm, {"CH4": 0.3, "O2": 0.3, "H2O": 0.1, "N2": 0.3})
    X = (1 - w)[:, None] * air[None, :] + w[:, None] * rich[None, :]
    _, qc = oracle.init_cells(400.0 + 900.0 * w, np.full(n, configs.ATM), np.zeros(n), X)
    qf = np.zeros_like(qc)
    for i in range(n):
        oracle.L.or_qc_to_qf(oracle.mech, qc[i].ctypes.data_as(_D), qf[i].ctypes.data_as(_D))
    flags = [1, 2, 1, 2, 0, 0, 0, 0]
    rp = [dx] + RP[1:]
    t = oracle.tube(n, 2, flags, rp)
    t.set_transport()
    t.set_interior(qf, qc)
    s = oracle.smr([30, 40, 20], [dx] * 3, 2, flags, rp)
    s.set_transport()
    s.set_interior(qf, qc)
    for _ in range(15):
        assert t.step(0.5) == s.step(0.5)
    np.testing.assert_array_equal(s.get()[1], t.get()[1])


def test_smr_layout_of_the_reference_namelist():
    """configs.smr_segments against the block sizes set_block_size gives
    (SRC/block.f90:176-223): dx_comp 2^(lev_smr - lev) per level, the
    coarsest block outermost, num_smr blocks of ncell_per_block cells each."""
    n, d = configs.smr_segments(1000, 2e-5, 10, lev_smr_n=4, num_smr_n=2)
    assert n == [1000, 20, 20, 20] and d == [2e-5, 4e-5, 8e-5, 1.6e-4]
    n, d = configs.smr_segments(200, 1e-4, 16, lev_smr_0=3, num_smr_0=1, lev_smr_n=2, num_smr_n=1)
    assert n == [16, 16, 200, 16] and d == [4e-4, 2e-4, 1e-4, 2e-4]


def same_state(a, b, tol):
    """rho, T, Y relative; u relative to its peak (it is ~0 at rest)."""
    np.testing.assert_allclose(a[:, [0, 2]], b[:, [0, 2]], rtol=tol)
    np.testing.assert_allclose(a[:, 1], b[:, 1], rtol=0, atol=tol * max(np.abs(b[:, 1]).max(), 1e-300))
    np.testing.assert_allclose(a[:, 3:], b[:, 3:], rtol=0, atol=tol * b[:, 3:].max())


def test_cell_centres_start_where_the_left_smr_zone_ends(oracle):
    """x = 0 at the end of the leading segments coarser than dx_comp
    (SRC/block.f90:236-237, 296-304): the output's x_m row and every
    position-dependent term use these centres."""
    ncells, dxs = [16, 16, 32, 16], [4e-3, 2e-3, 1e-3, 2e-3]
    n = sum(ncells)
    qf, qc = sod_state(oracle, np.arange(n) * 1.0, -1.0)
    s = oracle.smr(ncells, dxs, 2, [1, 2, 1, 2, 0, 0, 0, 0], RP)
    s.set_interior(qf, qc)
    rows = s.output_rows(ncells)
    edges = np.r_[0.0, np.cumsum(np.repeat(dxs, ncells))] - (16 * 4e-3 + 16 * 2e-3)
    np.testing.assert_allclose(rows[12], 0.5 * (edges[:-1] + edges[1:]), rtol=0, atol=1e-15)
    np.testing.assert_array_equal(rows[13], np.repeat(dxs, ncells))


@pytest.mark.parametrize("flags", [[1, 2, 1, 2, 0, 0, 1, 0], [0, 1, 1, 4, 0, 0, 1, 0]])
def test_equal_segments_spherical_reproduce_one_tube(oracle, flags):
    """Spherical geometry on equal-dx segments: r = x_m of each cell, the
    same radii as one tube's (to the rounding of the segment origins)."""
    n, dx = 120, 1e-4
    xm = (np.arange(n) + 0.5) * dx
    qf, qc = sod_state(oracle, xm, 0.3 * n * dx)
    t = oracle.tube(n, 2, flags, [dx] + RP[1:])
    t.set_spherical()
    t.set_interior(qf, qc)
    s = oracle.smr([40, 50, 30], [dx, dx, dx], 2, flags, [dx] + RP[1:])
    s.set_spherical()
    s.set_interior(qf, qc)
    for _ in range(30):
        assert s.step(0.5) == pytest.approx(t.step(0.5), rel=1e-13)
    same_state(s.get()[0], t.get()[0], 1e-11)


def test_refined_spherical_ball_close_to_uniform_grid(oracle):
    """A pressurised ball on a fine core with coarser outer segments (the
    reference's spherical examples refine toward the centre): its shock
    stays close to the uniform fine grid's."""
    dx = 1e-4
    fine = oracle.tube(160, 2, [1, 2, 1, 2, 0, 0, 1, 0], [dx] + RP[1:])
    fine.set_spherical()
    xm = (np.arange(160) + 0.5) * dx
    qf, qc = sod_state(oracle, xm, 20 * dx)
    fine.set_interior(qf, qc)
    ncells, dxs = [64, 24, 12], [dx, 2 * dx, 4 * dx]
    xs = np.r_[(np.arange(64) + 0.5) * dx, 64 * dx + (np.arange(24) + 0.5) * 2 * dx,
               112 * dx + (np.arange(12) + 0.5) * 4 * dx]
    qf2, qc2 = sod_state(oracle, xs, 20 * dx)
    s = oracle.smr(ncells, dxs, 2, [1, 2, 1, 2, 0, 0, 1, 0], [dx] + RP[1:])
    s.set_spherical()
    s.set_interior(qf2, qc2)
    t_f = t_s = 0.0
    while t_f < 2e-5:
        t_f += fine.step(0.4)
    while t_s < t_f:
        t_s += s.step(0.4)
    pf = fine.get()[0][:64, 2]
    ps = s.get()[0][:64, 2]
    assert np.all(np.isfinite(s.get()[0]))
    assert np.max(np.abs(ps - pf)) / pf.max() < 0.05


def test_sources_on_equal_segments_reproduce_one_tube(oracle):
    """Radiation, wall heat and ignition on equal-dx segments: each cell's x_m
    as one tube's, so the same heating (to the rounding of the origins)."""
    from test_sources import RAD_FITS
    nm = species_names()
    n, dx = 90, 2e-5
    prod = configs.equilibrium_tp(configs.ch4_air_mixture(nm, 1.0), 1800.0, configs.ATM)
    _, qc = oracle.init_cells(np.linspace(900.0, 1800.0, n), np.full(n, configs.ATM), np.zeros(n), np.tile(prod, (n, 1)))
    qf = np.zeros_like(qc)
    for i in range(n):
        oracle.L.or_qc_to_qf(oracle.mech, qc[i].ctypes.data_as(_D), qf[i].ctypes.data_as(_D))
    src = dict(radiation=[(nm.index(k), c) for k, c in RAD_FITS.items()],
               wall=(4.0, 2e-3, 373.0, 1300.0, 2e4, 0.5 * n * dx),
               ignition=(2, [(2e-7, 3e-4, 1e-6, 0.0)]))
    flags = [1, 2, 1, 2, 0, 0, 0, 0]
    t = oracle.tube(n, 2, flags, [dx] + RP[1:])
    t.set_interior(qf, qc)
    t.set_sources(**src)
    s = oracle.smr([30, 30, 30], [dx, dx, dx], 2, flags, [dx] + RP[1:])
    s.set_interior(qf, qc)
    s.set_sources(**src)
    for _ in range(8):
        assert s.step(0.5) == pytest.approx(t.step(0.5), rel=1e-13)
    qs, qt = s.get()[0], t.get()[0]
    assert np.abs(qt[:, 2] - qf[:, 2]).max() > 0.1  # the sources acted
    same_state(qs, qt, 1e-11)
    np.testing.assert_allclose(s.output_rows([30, 30, 30])[[9, 10, 11]], t.output_rows()[[9, 10, 11]], rtol=1e-10)
