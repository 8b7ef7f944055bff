"""Results files (SRC/write_hdf5.f90, SRC/read_hdf5.f90) without an HDF5
library (CPU): the library's writer and reader, and a second reader
written here from the file format (h5_spec), checked against a file that
libhdf5 wrote (the HDF5-based MATLAB 7.3 test file scipy ships, when it is
installed) and against each other on the results layout: the reference's
group and dataset names (leading blanks kept), float64 rows, int32 and
float64 one-element attributes, more members than one symbol-table node
holds, many step groups in one file.
"""
from pathlib import Path

import numpy as np
import pytest

from fortrancfd_gb300 import (OUTPUT_FIELDS, EdynError, H5Writer, configs, h5_attr, h5_attr_names, h5_list, h5_read,
                              species_names, step_group_name)
from h5_spec import H5Spec

R_SI = 8314.51


def libhdf5_file():
    scipy = pytest.importorskip("scipy")
    p = Path(scipy.__file__).parent / "io" / "matlab" / "tests" / "data" / "testhdf5_7.4_GLNX86.mat"
    if not p.exists():
        pytest.skip("scipy's HDF5 test file is not installed")
    return p


def test_readers_read_a_libhdf5_file():
    """A file libhdf5 wrote (a 512-byte user block, a version-2 layout
    message, a string attribute): both readers find the 9 x 1 array
    0, pi/4, ..., 2 pi and its class attribute."""
    p = libhdf5_file()
    expect = np.arange(9) * np.pi / 4
    s = H5Spec(p)
    assert s.base == 512
    assert [n for n, _ in s.members(s.root)] == ["testdouble"]
    dims, vals = s.dataset("testdouble")
    assert dims == [9, 1]
    np.testing.assert_array_equal(vals, expect)
    assert s.attrs("testdouble") == {"MATLAB_class": "double"}
    assert h5_list(p) == ["testdouble"]
    np.testing.assert_array_equal(h5_read(p, "testdouble"), expect)
    assert h5_attr(p, "testdouble", "MATLAB_class") == "double"


def results_rows(n, nspe, seed):
    rng = np.random.default_rng(seed)
    return {name: rng.standard_normal(n) for name in list(OUTPUT_FIELDS) + [f"S{k}" for k in range(nspe)]}


ATTRS = ("dt", "time from 0s", "time from restart", "cpu time total", "cpu time restart", "number of output",
         "number of time step")


def write_results(path, groups):
    with H5Writer(path) as w:
        for name, attrs, rows in groups:
            w.add_group(name, attrs, rows)


def test_results_layout_both_readers(tmp_path):
    """Three step groups of 15 + 53 datasets (nine symbol-table nodes per
    group) with the reference's seven attributes."""
    p = tmp_path / "results_nout000000.h5"
    nm = species_names()
    groups = []
    for k in range(3):
        rows = {name: v for name, v in zip(list(OUTPUT_FIELDS) + nm, results_rows(40, 53, k).values())}
        attrs = dict(zip(ATTRS, [1e-9 * (k + 1), 1e-6 * k, 1e-6 * k, 0.5 * k, 0.5 * k, k, 100 * k]))
        groups.append((step_group_name(k, 1e-6 * k), attrs, rows))
    write_results(p, groups)
    s = H5Spec(p)
    assert s.base == 0 and s.eof == p.stat().st_size
    top = s.members(s.root)  # checks the index invariants too
    assert [n for n, _ in top] == [g[0] for g in groups]
    assert h5_list(p) == [g[0] + "/" for g in groups]
    for name, attrs, rows in groups:
        members = s.members(s.resolve(name))
        assert sorted(n for n, _ in members) == sorted(rows)
        assert h5_list(p, name) == sorted(rows, key=lambda r: r.encode())
        for r, v in rows.items():
            dims, vals = s.dataset(f"{name}/{r}")
            assert dims == [40]
            np.testing.assert_array_equal(vals, v)
            np.testing.assert_array_equal(h5_read(p, f"{name}/{r}"), v)
        a = s.attrs(name)
        assert list(a) == list(ATTRS)  # creation order in the header
        for key in ATTRS:
            assert a[key] == [attrs[key]]
            assert h5_attr(p, name, key)[0] == attrs[key]
        assert isinstance(a["number of output"][0], int) and isinstance(a["dt"][0], float)
        assert h5_attr_names(p, name) == list(ATTRS)


def test_file_is_readable_after_every_group(tmp_path):
    p = tmp_path / "r.h5"
    w = H5Writer(p)
    try:
        for k in range(40):
            w.add_group(step_group_name(k, 2.5e-7 * k), {"number of output": k}, {"rho": np.full(3, float(k))})
            s = H5Spec(p)
            names = [n for n, _ in s.members(s.root)]
            assert len(names) == k + 1 and names == sorted(names)
            assert s.dataset(f"{names[-1]}/rho")[1] == [float(k)] * 3
    finally:
        w.close()
    # the restart's choice: the last group in index order is the last output
    assert h5_list(p)[-1] == step_group_name(39, 2.5e-7 * 39) + "/"


def test_empty_rows_and_empty_file(tmp_path):
    p = tmp_path / "e.h5"
    write_results(p, [])
    assert h5_list(p) == []
    s = H5Spec(p)
    assert s.members(s.root) == []
    q = tmp_path / "z.h5"
    write_results(q, [("g", {}, {"rho": np.zeros(0)})])
    assert h5_read(q, "g/rho").size == 0
    assert H5Spec(q).dataset("g/rho") == ([0], [])


def test_writer_and_reader_errors(tmp_path):
    p = tmp_path / "x.h5"
    with H5Writer(p) as w:
        w.add_group("g", {}, {"a": np.zeros(2)})
        with pytest.raises(EdynError, match="exists"):
            w.add_group("g", {}, {"a": np.zeros(2)})
        with pytest.raises(EdynError, match="members"):
            w.add_group("big", {}, {f"d{k:03d}": np.zeros(1) for k in range(257)})
    with pytest.raises(EdynError, match="no member"):
        h5_read(p, "g/b")
    bad = tmp_path / "not.h5"
    bad.write_bytes(b"plain text, not HDF5" * 10)
    with pytest.raises(EdynError, match="superblock"):
        h5_list(bad)


@pytest.mark.parametrize("t,name", [(0.0, "nout000000_time0.00000E+00"), (1.5e-4, "nout000003_time0.15000E-03"),
                                    (2.0e-3, "nout000003_time0.20000E-02"), (0.123456, "nout000003_time0.12346E+00"),
                                    (12.0, "nout000003_time0.12000E+02"), (9.999996e-5, "nout000003_time0.10000E-03")])
def test_step_group_name_is_fortran_e11_5(t, name):
    nout = 0 if t == 0.0 else 3
    assert step_group_name(nout, t) == name


def test_oracle_output_rows_are_set_eos_params(oracle):
    """The oracle's rows against set_eos_params evaluated here: X from Y,
    p = rho R T / W, ek, et = rho E / rho, and x_m, dx, idx; ei against the
    oracle's own specific_energy; the source rows zero without sources."""
    nm = species_names()
    W = configs.molecular_weights()
    n, dx = 12, 3e-5
    fresh = configs.ch4_air_mixture(nm, 1.0)
    hot = configs.equilibrium_tp(fresh, 2200.0, configs.ATM)
    w = np.linspace(0, 1, n)
    X = (1 - w)[:, None] * fresh[None, :] + w[:, None] * hot[None, :]
    qf, qc = oracle.init_cells(300.0 + 1900.0 * w, np.full(n, configs.ATM), np.linspace(-5, 5, n), X)
    t = oracle.tube(n, 2, [1, 2, 1, 2, 0, 0, 0, 0], [dx, configs.ATM, 300.0, 0.0, 1e-5, 1e-13])
    t.set_interior(qf, qc)
    rows = t.output_rows()
    assert rows.shape == (15 + len(nm), n)
    Y = qf[:, 3:]
    Xo = (Y / W) / (Y / W).sum(axis=1, keepdims=True)
    np.testing.assert_allclose(rows[15:].T, Xo, rtol=1e-14, atol=1e-300)
    np.testing.assert_array_equal(rows[0], qf[:, 0])
    np.testing.assert_array_equal(rows[1], qf[:, 1])
    np.testing.assert_array_equal(rows[2], qf[:, 2])
    np.testing.assert_allclose(rows[3], qf[:, 0] * R_SI * qf[:, 2] / (Xo @ W), rtol=1e-14)
    np.testing.assert_allclose(rows[3], configs.ATM, rtol=1e-12)
    np.testing.assert_allclose(rows[4], qc[:, 2] / qf[:, 0], rtol=1e-15)
    np.testing.assert_array_equal(rows[5], 0.5 * qf[:, 1] ** 2)
    # e_total = e_internal + u^2/2 for the state init_cells built
    np.testing.assert_allclose(rows[4], rows[6] + rows[5], rtol=1e-12)
    np.testing.assert_array_equal(rows[7:12], 0.0)
    np.testing.assert_allclose(rows[12], (np.arange(n) + 0.5) * dx, rtol=1e-15)
    np.testing.assert_array_equal(rows[13], dx)
    np.testing.assert_array_equal(rows[14], np.arange(1, n + 1))


def test_oracle_source_rows_hold_the_last_source_step(oracle):
    """Qrd and QTw are the radiation and wall heat the last source step added
    (rho E grew by dt (Qrad + qTw)); Tw is the wall profile at x_m."""
    from test_sources import RAD_FITS
    nm = species_names()
    prod = configs.equilibrium_tp(configs.ch4_air_mixture(nm, 1.0), 2000.0, configs.ATM)
    n, dx, dt = 10, 1e-3, 1e-6
    qf, qc = oracle.init_cells(np.linspace(900.0, 1900.0, n), np.full(n, configs.ATM), np.zeros(n),
                               np.tile(prod, (n, 1)))
    t = oracle.tube(n, 2, [1, 2, 1, 2, 0, 0, 0, 0], [dx, configs.ATM, 300.0, 0.0, 1e-5, 1e-13])
    t.set_interior(qf, qc)
    wall = (4.0, 2e-3, 373.0, 1300.0, 800.0, 0.5 * n * dx)
    t.set_sources(radiation=[(nm.index(k), c) for k, c in RAD_FITS.items()], wall=wall)
    t.solve_source(dt)
    rows = t.output_rows()
    _, qc1 = t.get()
    assert np.all(rows[9] < 0)
    np.testing.assert_allclose(qc1[:, 2] - qc[:, 2], dt * (rows[9] + rows[11]), rtol=1e-9)
    nu, d, tmin, tmax, alpha, beta = wall
    xm = (np.arange(n) + 0.5) * dx
    np.testing.assert_allclose(rows[10], 0.5 * (tmax - tmin) * np.tanh(alpha * (xm - beta)) + 0.5 * (tmax + tmin),
                               rtol=1e-15)


def restart_state(rows, W):
    """read_hdf5_restart + Xi2Yi + set_block_params on the host (the
    arithmetic edyn_restart performs): qf = (rho, u, T, Y), Qc = (rho,
    rho u, rho et, rho Y)."""
    X = rows[15:].T
    Y = X * W / (X * W).sum(axis=1, keepdims=True)
    rho, u, T, et = rows[0], rows[1], rows[2], rows[4]
    qf = np.column_stack([rho, u, T, Y])
    qc = np.column_stack([rho, rho * u, rho * et, rho[:, None] * Y])
    return qf, qc


def test_results_round_trip_restores_the_state(oracle, tmp_path):
    """Oracle rows through a results file and the restart arithmetic give
    back the state: rho, u, T bit for bit, Y and rho E to rounding."""
    nm = species_names()
    W = configs.molecular_weights()
    n = 16
    fresh = configs.ch4_air_mixture(nm, 0.8)
    hot = configs.equilibrium_tp(fresh, 2100.0, configs.ATM)
    w = np.linspace(0, 1, n)
    X = (1 - w)[:, None] * fresh[None, :] + w[:, None] * hot[None, :]
    qf, qc = oracle.init_cells(300.0 + 1800.0 * w, np.full(n, configs.ATM), np.linspace(0, 30, n), X)
    t = oracle.tube(n, 2, [1, 2, 1, 2, 0, 0, 0, 0], [1e-4, configs.ATM, 300.0, 0.0, 1e-5, 1e-13])
    t.set_interior(qf, qc)
    rows = t.output_rows()
    p = tmp_path / "results_nout000000.h5"
    names = list(OUTPUT_FIELDS) + nm
    write_results(p, [(step_group_name(7, 1e-3), dict(zip(ATTRS, [1e-8, 1e-3, 1e-3, 2.0, 2.0, 7, 1234])),
                       dict(zip(names, rows)))])
    g = h5_list(p)[-1].rstrip("/")
    back = np.array([h5_read(p, f"{g}/{nme}") for nme in names])
    np.testing.assert_array_equal(back, rows)
    qf2, qc2 = restart_state(back, W)
    np.testing.assert_array_equal(qf2[:, :3], qf[:, :3])
    np.testing.assert_allclose(qf2[:, 3:], qf[:, 3:], rtol=1e-14, atol=1e-18)
    np.testing.assert_allclose(qc2[:, 2], qc[:, 2], rtol=1e-15)
    # the restart's returns: the next output and step numbers
    assert h5_attr(p, g, "number of output")[0] + 1 == 8
    assert h5_attr(p, g, "number of time step")[0] + 1 == 1235
