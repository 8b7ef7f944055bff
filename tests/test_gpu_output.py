"""GPU output and restart (write_hdf5_b / read_hdf5_restart) vs the CPU
oracle: the device's output rows (set_eos_params) against the oracle's on
the same state, within 1e-12 relative (p, ei: the same formulas, another
summation order; the copied rows bit for bit); the results file the GPU
path writes read back by the file-format reader of the tests; a restart
giving back the written state and stepping on as the original tube does;
a snapshot that keeps the state of its own time while the tube steps on.
"""
import numpy as np
import pytest

from fortrancfd_gb300 import OUTPUT_FIELDS, Blocks, EdynError, Tube, Tubes, configs, species_names, step_group_name
from h5_spec import H5Spec
from test_sources import RAD_FITS

pytestmark = pytest.mark.gpu


def layer(n, dx):
    nm = species_names()
    fresh = configs.ch4_air_mixture(nm, 1.0)
    hot = configs.equilibrium_tp(fresh, 2000.0, configs.ATM)
    xm = (np.arange(n) + 0.5) * dx
    w = 0.5 * (1 + np.tanh((xm - 0.5 * n * dx) / (4 * dx)))
    X = (1 - w)[:, None] * fresh[None, :] + w[:, None] * hot[None, :]
    return 400.0 + 1600.0 * w, np.full(n, configs.ATM), 3.0 * np.sin(xm / (n * dx) * 6.0), X


def compare_rows(g, o, n):
    exact = [0, 1, 2, 5, 12, 13, 14]  # rho u T ek x_m dx idx
    for r in exact:
        np.testing.assert_allclose(g[r], o[r], rtol=1e-15, atol=0, err_msg=OUTPUT_FIELDS[r])
    for r in (3, 4, 6):
        np.testing.assert_allclose(g[r], o[r], rtol=1e-12, atol=0, err_msg=OUTPUT_FIELDS[r])
    np.testing.assert_allclose(g[15:], o[15:], rtol=1e-12, atol=1e-300)


def test_output_rows_match_oracle(oracle):
    n, dx = 96, 2e-5
    T, p, u, X = layer(n, dx)
    qf, qc = oracle.init_cells(T, p, u, X)
    ot = oracle.tube(n, 2, [1, 2, 1, 2, 0, 0, 0, 0], [dx, configs.ATM, 300.0, 0.0, 1e-5, 1e-13])
    ot.set_interior(qf, qc)
    g = Tube(n, dx)
    g.upload(qf, qc)
    rows = g.output_rows()
    assert rows.shape == (15 + len(species_names()), n)
    compare_rows(rows, ot.output_rows(), n)
    np.testing.assert_array_equal(rows[7:12], 0.0)


def test_output_source_rows_match_oracle(oracle):
    """Radiation and wall heat through the host loop: Qrd, Tw and QTw of the
    last source step (frozen chemistry, the fluid stages' 1e-10 bar)."""
    nm = species_names()
    n, dx = 64, 2e-5
    T, p, u, X = layer(n, dx)
    qf, qc = oracle.init_cells(T, p, u, X)
    wall = (4.0, 2e-3, 373.0, 1300.0, 2e4, 0.5 * n * dx)
    ot = oracle.tube(n, 2, [1, 2, 1, 2, 0, 0, 0, 0], [dx, configs.ATM, 300.0, 0.0, 1e-5, 1e-13])
    ot.set_interior(qf, qc)
    ot.set_sources(radiation=[(nm.index(k), c) for k, c in RAD_FITS.items()], wall=wall)
    g = Tube(n, dx)
    g.upload(qf, qc)
    g.set_radiation(RAD_FITS)
    g.set_wall_heat(*wall)
    for _ in range(5):
        ot.step(0.5)
        g.step(0.5)
    o, r = ot.output_rows(), g.output_rows()
    for k in (9, 11):
        assert np.all(o[k] != 0.0)
        np.testing.assert_allclose(r[k], o[k], rtol=1e-9, err_msg=OUTPUT_FIELDS[k])
    np.testing.assert_allclose(r[10], o[10], rtol=1e-14)
    np.testing.assert_allclose(r[2], o[2], rtol=1e-10)


def test_results_file_and_restart(tmp_path):
    """Two step groups written on the way; a second tube restarted from the
    file holds the state of the last one and steps on with the original."""
    n, dx = 128, 2e-5
    T, p, u, X = layer(n, dx)
    a = Tube(n, dx, flag_rbound=1)
    a.init_cells(T, p, u, X)
    path = tmp_path / "results_nout000000.h5"
    a.output_open(path)
    t = 0.0
    expect = []
    for nout in range(2):
        for _ in range(6):
            t += a.step(0.5)
        a.output_write(nout, 6 * (nout + 1), 1e-9, t, t, 0.25 * nout, 0.25 * nout)
        expect.append((step_group_name(nout, t), a.output_rows()))
    a.output_close()
    s = H5Spec(path)
    groups = [nm for nm, _ in s.members(s.root)]
    assert groups == [e[0] for e in expect]
    names = a.output_names()
    for gname, rows in expect:
        assert sorted(nm for nm, _ in s.members(s.resolve(gname))) == sorted(names)
        for r, nm in enumerate(names):
            np.testing.assert_array_equal(s.dataset(f"{gname}/{nm}")[1], rows[r])
    at = s.attrs(groups[-1])
    assert at["number of output"] == [1] and at["number of time step"] == [12] and at["time from 0s"] == [t]

    b = Tube(n, dx, flag_rbound=1)
    nout, nt, time, cpu = b.restart(path)
    assert (nout, nt, time, cpu) == (2, 13, t, 0.25)
    qa, ca, _ = a.download()
    qb, cb, _ = b.download()
    np.testing.assert_array_equal(qb[:, :3], qa[:, :3])
    np.testing.assert_allclose(qb[:, 3:], qa[:, 3:], rtol=1e-14, atol=1e-18)
    np.testing.assert_allclose(cb[:, 2], ca[:, 2], rtol=1e-15)
    for _ in range(5):
        da, db = a.step(0.5), b.step(0.5)
        assert db == pytest.approx(da, rel=1e-12)
    qa, _, _ = a.download()
    qb, _, _ = b.download()
    np.testing.assert_allclose(qb[:, :3], qa[:, :3], rtol=1e-12)


def test_snapshot_keeps_its_time(tmp_path):
    """A snapshot queued before more steps writes the state of its own time."""
    n, dx = 96, 2e-5
    T, p, u, X = layer(n, dx)
    a = Tube(n, dx)
    a.init_cells(T, p, u, X)
    for _ in range(3):
        a.step(0.5)
    before = a.output_rows()
    a.output_snapshot()
    with pytest.raises(EdynError, match="pending"):
        a.output_snapshot()
    a.advance(0.5, tend=1e9, max_steps=10)
    path = tmp_path / "r.h5"
    a.output_open(path)
    a.output_write(0, 3, 1e-9, 1e-6)
    a.output_close()
    s = H5Spec(path)
    g = s.members(s.root)[0][0]
    np.testing.assert_array_equal(s.dataset(f"{g}/  T")[1], before[2])
    assert not np.array_equal(a.output_rows()[2], before[2])


def test_smr_domain_output_geometry():
    g = Blocks([32, 16, 32], [2e-5, 4e-5, 2e-5])
    n = 80
    T, p, u, X = layer(n, 2e-5)
    g.init_cells(T, p, u, X)
    rows = g.output_rows()
    dx = np.r_[np.full(32, 2e-5), np.full(16, 4e-5), np.full(32, 2e-5)]
    edges = np.r_[0.0, np.cumsum(dx)]
    np.testing.assert_allclose(rows[12], 0.5 * (edges[:-1] + edges[1:]), rtol=1e-13)
    np.testing.assert_array_equal(rows[13], dx)
    np.testing.assert_array_equal(rows[14], np.arange(1, n + 1))


def test_output_refused_for_packed_tubes(tmp_path):
    g = Tubes([64, 64], [1e-5, 2e-5])
    with pytest.raises(EdynError, match="packed"):
        g.output_open(tmp_path / "x.h5")
    t = Tube(64, 1e-5)
    with pytest.raises(EdynError, match="no output file"):
        t.output_write(0, 0, 1e-9, 0.0)
    w = Tube(32, 1e-5)
    bad = tmp_path / "grid.h5"
    t.output_open(bad)
    t.output_write(0, 0, 1e-9, 0.0)
    t.output_close()
    with pytest.raises(EdynError, match="cells"):
        w.restart(bad)
