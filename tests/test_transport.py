"""Transport fits and the oracle's TRANLIB restatement (CPU).

The fits in fortrancfd_gb300/data/gri30/tran.edyn are the reference's
TRANLIB linking file (tran.bin) written out by the library. They are pinned
by sources independent of that file's reader:
- re-reading the reference's tran.bin reproduces the committed file (when
  the reference checkout is available);
- every nonpolar species' viscosity fit agrees with Chapman-Enskog theory
  evaluated from the Lennard-Jones parameters of the same file, with the
  collision integrals of Neufeld, Janzen and Aziz (J. Chem. Phys. 57, 1100,
  1972), within 1.5 % from 300 to 3000 K; the binary diffusion fits lie
  within 9 % of the first-approximation formula (up to 8 % above it for the
  pairs of most unequal mass);
- the conductivity fit of every atom is Eucken's 15/4 (R/W) eta of its own
  viscosity fit;
- handbook values of a few gases at 300 K and 1 atm.
The mixture rules are checked in their exact limits (pure gas; a binary
mixture, where the calc_flux_tran diffusivity is the binary coefficient),
and the oracle's face flux and tube stages by exact symmetries and
conservation.
"""
import numpy as np
import pytest

from conftest import ROOT, reference_dir
from fortrancfd_gb300 import configs, species_names

TRAN_TXT = ROOT / "fortrancfd_gb300/data/gri30/tran.edyn"
R_CGS = 8.31451e7


def read_tran():
    lines = TRAN_TXT.read_text().split("\n")
    i = lines.index("SPECIES")
    sp = [ln.split() for ln in lines[i + 1:i + 54]]
    return {
        "names": [s[0] for s in sp],
        "W": np.array([float(s[1]) for s in sp]),
        "eps": np.array([float(s[2]) for s in sp]),
        "sig": np.array([float(s[3]) for s in sp]),
        "dip": np.array([float(s[4]) for s in sp]),
        "nlin": np.array([int(s[7]) for s in sp]),
    }


def omega22(ts):
    return 1.16145 * ts ** -0.14874 + 0.52487 * np.exp(-0.77320 * ts) + 2.16178 * np.exp(-2.43787 * ts)


def omega11(ts):
    return (1.06036 * ts ** -0.15610 + 0.19300 * np.exp(-0.47635 * ts) + 1.03587 * np.exp(-1.52996 * ts)
            + 1.76474 * np.exp(-3.89411 * ts))


def test_committed_fits_reproduce_reference_linking_file(tmp_path):
    ref = reference_dir()
    if ref is None:
        pytest.skip("reference checkout not present")
    from fortrancfd_gb300 import tran_compile

    out = tmp_path / "tran.edyn"
    tran_compile(ref / "WORK/Examples/CH4_GRI3.0/SOD/GRI3.0_CH4", out)
    assert out.read_text() == TRAN_TXT.read_text()


def test_fits_cover_the_mechanism_and_are_symmetric():
    t = read_tran()
    assert t["names"] == species_names()
    np.testing.assert_array_equal(t["W"], configs.molecular_weights())
    lines = TRAN_TXT.read_text().split("\n")
    i = lines.index("COFD")
    cofd = {}
    for ln in lines[i + 1:i + 1 + 53 * 53]:
        v = ln.split()
        cofd[int(v[0]), int(v[1])] = tuple(v[2:])
    assert len(cofd) == 53 * 53
    assert all(cofd[k, j] == cofd[j, k] for k in range(53) for j in range(k))


def test_viscosity_fits_follow_chapman_enskog(oracle):
    t = read_tran()
    nonpolar = t["dip"] == 0
    assert nonpolar.sum() >= 40
    worst = 0.0
    for T in np.geomspace(300.0, 3000.0, 12):
        ce = 2.6693e-5 * np.sqrt(t["W"] * T) / (t["sig"] ** 2 * omega22(T / t["eps"]))
        worst = max(worst, float(np.abs(oracle.pure_viscosity(T) / ce - 1.0)[nonpolar].max()))
    assert worst < 0.015, worst


def test_diffusion_fits_follow_chapman_enskog(oracle):
    t = read_tran()
    W, sig, eps, dip = t["W"], t["sig"], t["eps"], t["dip"]
    worst = 0.0
    for T in (300.0, 1000.0, 2000.0, 3000.0):
        D = oracle.binary_diffusion(1.01325e6, T)
        for j in range(53):
            for k in range(j):
                if dip[j] or dip[k]:
                    continue
                s = 0.5 * (sig[j] + sig[k])
                e = np.sqrt(eps[j] * eps[k])
                ce = 0.0018583 * np.sqrt(T ** 3 * (1 / W[j] + 1 / W[k])) / (s ** 2 * omega11(T / e))
                worst = max(worst, abs(D[j, k] / ce - 1.0))
    assert worst < 0.09, worst


def test_atom_conductivity_is_eucken():
    from oracle_ctypes import Oracle

    o = Oracle()
    t = read_tran()
    atoms = np.nonzero(t["nlin"] == 0)[0]
    assert [t["names"][k] for k in atoms] == ["H", "O", "C", "N", "AR"]
    for T in (300.0, 1200.0, 3000.0):
        vis, con = o.pure_viscosity(T), o.pure_conductivity(T)
        np.testing.assert_allclose(con[atoms], 3.75 * R_CGS / t["W"][atoms] * vis[atoms], rtol=1e-12)


def test_handbook_values_at_300K(oracle):
    nm = species_names()
    vis = oracle.pure_viscosity(300.0) * 0.1       # Pa s
    con = oracle.pure_conductivity(300.0) * 1e-5   # W/(m K)
    D = oracle.binary_diffusion(1.01325e6, 300.0) * 1e-4  # m^2/s
    for s, mu in {"N2": 1.78e-5, "O2": 2.07e-5, "H2": 0.896e-5, "CO2": 1.50e-5, "AR": 2.27e-5,
                  "CH4": 1.12e-5}.items():
        assert vis[nm.index(s)] == pytest.approx(mu, rel=0.03), s
    for s, lam in {"N2": 0.0259, "O2": 0.0263, "H2": 0.183, "AR": 0.0177}.items():
        assert con[nm.index(s)] == pytest.approx(lam, rel=0.05), s
    for (a, b), d in {("O2", "N2"): 2.1e-5, ("H2", "N2"): 7.8e-5}.items():
        assert D[nm.index(a), nm.index(b)] == pytest.approx(d, rel=0.05), (a, b)
    air = configs.mole_vector(nm, {"O2": 0.21, "N2": 0.79})
    assert oracle.mix_viscosity(300.0, air) * 0.1 == pytest.approx(1.85e-5, rel=0.03)


def test_mixture_rules_in_their_exact_limits(oracle):
    nm = species_names()
    for T in (300.0, 1500.0):
        vis, con = oracle.pure_viscosity(T), oracle.pure_conductivity(T)
        for s in ("N2", "H2O", "CH4", "H"):
            x = np.zeros(53)
            x[nm.index(s)] = 1.0
            assert oracle.mix_viscosity(T, x) == pytest.approx(vis[nm.index(s)], rel=1e-14)
            assert oracle.mix_conductivity(T, x) == pytest.approx(con[nm.index(s)], rel=1e-14)
    # binary mixture: (1 - X_1)/(1 - Y_1) D_1 of MCADIF is the binary coefficient
    W = configs.molecular_weights()
    for a, b, xa in (("O2", "N2", 0.3), ("H2", "CH4", 0.6)):
        x = np.zeros(53)
        x[nm.index(a)], x[nm.index(b)] = xa, 1.0 - xa
        y = x * W / (x @ W)
        d = oracle.mix_diffusion(1.01325e6, 1000.0, x)
        D = oracle.binary_diffusion(1.01325e6, 1000.0)
        ia, ib = nm.index(a), nm.index(b)
        assert (1 - x[ia]) / (1 - y[ia]) * d[ia] == pytest.approx(D[ia, ib], rel=1e-12)
        assert (1 - x[ib]) / (1 - y[ib]) * d[ib] == pytest.approx(D[ia, ib], rel=1e-12)


def _cells(oracle, T, u, X, p=101325.0):
    n = len(T)
    return oracle.init_cells(np.asarray(T, float), np.full(n, p), np.asarray(u, float), np.asarray(X, float))


def test_face_flux_symmetries(oracle):
    nm = species_names()
    air = configs.mole_vector(nm, {"O2": 0.21, "N2": 0.79})
    mix = configs.mole_vector(nm, {"CH4": 0.2, "O2": 0.3, "H2O": 0.1, "N2": 0.4})
    _, qc = _cells(oracle, [600.0, 900.0], [3.0, -2.0], [air, mix])
    g = oracle.face_flux_tran(qc[0], qc[1], 1e-4)
    g2 = oracle.face_flux_tran(qc[1], qc[0], 1e-4)
    assert g[0] == 0.0 and np.all(g[1:3] != 0.0)
    np.testing.assert_array_equal(g2[1:], -g[1:])
    # a uniform state carries no transport flux
    assert not oracle.face_flux_tran(qc[0], qc[0], 1e-4).any()
    # pure N2 at rest with a temperature difference: Fourier's law alone
    n2 = configs.mole_vector(nm, {"N2": 1.0})
    _, qc = _cells(oracle, [1000.0, 1010.0], [0.0, 0.0], [n2, n2])
    g = oracle.face_flux_tran(qc[0], qc[1], 1e-4)
    k0 = oracle.tran_cell(qc[0])[5]
    k1 = oracle.tran_cell(qc[1])[5]
    assert g[2] == pytest.approx(-0.5 * (k0 + k1) * 10.0 / 1e-4, rel=1e-9)
    assert g[1] == 0.0 and not g[3:].any()


def test_oracle_tube_diffusion_conserves_and_spreads(oracle):
    """An O2-rich layer in N2 at rest between walls: transport spreads it,
    every species' mass and the total energy stay put."""
    nm = species_names()
    n, dx = 64, 2e-5
    xm = (np.arange(n) + 0.5) * dx
    layer = np.abs(xm - 0.5 * n * dx) < 8 * dx
    X = np.where(layer[:, None], configs.mole_vector(nm, {"O2": 0.6, "N2": 0.4})[None, :],
                 configs.mole_vector(nm, {"O2": 0.1, "N2": 0.9})[None, :])
    qf0, qc0 = _cells(oracle, np.full(n, 800.0), np.zeros(n), X)
    ot = oracle.tube(n, 2, [1, 2, 1, 2, 0, 0, 0, 0], [dx, 101325.0, 300.0, 0.0, 1e-5, 1e-13])
    ot.set_transport()
    ot.set_interior(qf0, qc0)
    for _ in range(10):
        ot.step(0.5)
    qf1, qc1 = ot.get()
    o2 = nm.index("O2")
    np.testing.assert_allclose(qc1[:, 3:].sum(axis=0), qc0[:, 3:].sum(axis=0), rtol=1e-12, atol=1e-15)
    assert qc1[:, 2].sum() == pytest.approx(qc0[:, 2].sum(), rel=1e-12)
    assert qf1[:, 3 + o2].max() < qf0[:, 3 + o2].max()
    # the inviscid run keeps the layer's edge cells as they were to far closer
    ot2 = oracle.tube(n, 2, [1, 2, 1, 2, 0, 0, 0, 0], [dx, 101325.0, 300.0, 0.0, 1e-5, 1e-13])
    ot2.set_interior(qf0, qc0)
    for _ in range(10):
        ot2.step(0.5)
    qf2, _ = ot2.get()
    assert np.abs(qf2[:, 3 + o2] - qf0[:, 3 + o2]).max() < 0.5 * np.abs(qf1[:, 3 + o2] - qf0[:, 3 + o2]).max()


def test_face_flux_device_form_matches_oracle(oracle):
    """k_tran_flux's arithmetic (face averages of the per-cell rows, CKHMS
    from the premixed enthalpy coefficients a1, a2/2, .., a5/5, a6 at the face
    temperature, R_SI h / W) on the oracle's per-cell rows reproduces the
    oracle's face flux to rounding."""
    nm = species_names()
    _, tmid, a, _ = configs._thermo_tables()
    W = configs.molecular_weights()
    mix1 = configs.mole_vector(nm, {"CH4": 0.2, "O2": 0.3, "H2O": 0.1, "N2": 0.4})
    mix2 = configs.equilibrium_tp(configs.ch4_air_mixture(nm, 1.0), 2100.0, configs.ATM)
    _, qc = oracle.init_cells(np.array([700.0, 1900.0]), np.full(2, configs.ATM), np.array([4.0, -3.0]),
                              np.array([mix1, mix2]))
    dx = 2e-5
    L = oracle.tran_cell(qc[0])
    R = oracle.tran_cell(qc[1])
    rho_a, u_a, T_a = 0.5 * (L[0] + R[0]), 0.5 * (L[1] + R[1]), 0.5 * (L[2] + R[2])
    mu_a, k_a = 0.5 * (L[4] + R[4]), 0.5 * (L[5] + R[5])
    tau = -(2.0 / 3.0 * mu_a * (2.0 * ((R[1] - L[1]) / dx)))
    r = (T_a > tmid).astype(int)
    c = a[np.arange(53), r]
    h = ((((c[:, 4] / 5 * T_a + c[:, 3] / 4) * T_a + c[:, 2] / 3) * T_a + c[:, 1] / 2) * T_a + c[:, 0]) * T_a + c[:, 5]
    hs = 8314.51 * h / W
    dif_a = 0.5 * (L[6] + R[6])
    dy = (R[3] - L[3]) / dx
    g = np.zeros(56)
    g[1] = tau
    g[2] = tau * u_a + rho_a * np.sum(-hs * dif_a * dy) - k_a * ((R[2] - L[2]) / dx)
    g[3:] = -(rho_a * dif_a * dy)
    go = oracle.face_flux_tran(qc[0], qc[1], dx)
    scale = np.abs(go).max()
    np.testing.assert_allclose(g, go, rtol=1e-12, atol=1e-12 * scale)


def _fits():
    lines = TRAN_TXT.read_text().split("\n")

    def block(name, n, width):
        i = lines.index(name)
        return np.array([[float(v) for v in ln.split()[width:]] for ln in lines[i + 1:i + 1 + n]])

    ceta, clam = block("COFETA", 53, 1), block("COFLAM", 53, 1)
    cofd = block("COFD", 53 * 53, 2).reshape(53, 53, 4)
    return ceta, clam, cofd


def test_property_kernel_form_matches_oracle(oracle):
    """k_tran_props' arithmetic in NumPy: Wilke's sum expanded into the three
    products with the constant matrices g, q g, q^2 g, and the mixture-
    averaged diffusion from the pair matrix with sum_{j!=k} XX_j W_j taken
    apart from the floored X (the kernel adds a prefix to a suffix). It
    matches the oracle's MCAVIS / MCACON / MCADIF (at the oracle's own T) to
    1e-13 (1e-12 for D') from fresh mixture to products."""
    nm = species_names()
    ceta, clam, cofd = _fits()
    t = read_tran()
    wt = t["W"]
    W = configs.molecular_weights()
    g = 1.0 / np.sqrt(1.0 + wt[:, None] / wt[None, :])
    q = np.sqrt(np.sqrt(wt[None, :] / wt[:, None]))
    wa, wb, wc = g, q * g, q * q * g
    fresh = configs.ch4_air_mixture(nm, 1.0)
    hot = configs.equilibrium_tp(fresh, 2400.0, configs.ATM)
    w = np.linspace(0.0, 1.0, 12)
    X = (1 - w)[:, None] * fresh[None, :] + w[:, None] * hot[None, :]
    _, qc = oracle.init_cells(300.0 + 2100.0 * w, np.full(12, configs.ATM), np.zeros(12), X)
    for c in qc:
        rho, u, T, y, mu_o, kap_o, dif_o = oracle.tran_cell(c)
        sumyow = (y / W).sum()
        x = y / W / sumyow
        p_cgs = 10.0 * 8314.51 * rho * T * sumyow / y.sum()
        L = np.log(T)

        def poly(cf):
            return ((cf[..., 3] * L + cf[..., 2]) * L + cf[..., 1]) * L + cf[..., 0]

        eta, lam = np.exp(poly(ceta)), np.exp(poly(clam))
        kap = 0.5 * ((x * lam).sum() + 1.0 / (x / lam).sum()) * 1e-5
        A, B, C = wa @ x, wb @ (x / np.sqrt(eta)), wc @ (x / eta)
        mu = (x * eta / (A + 2.0 * np.sqrt(eta) * B + eta * C)).sum() * np.sqrt(8.0) * 0.1
        xx = np.maximum(x, 1e-50)
        inv = np.exp(-poly(cofd))
        np.fill_diagonal(inv, 0.0)
        S = inv @ xx
        tot = xx * wt
        sumxw = tot.sum() - tot
        d = sumxw / ((wt * x).sum() * S) * 1013250.0 / p_cgs * 1e-4
        dif = np.where(y == 1.0, 0.0, (1.0 - x) / (1.0 - y) * d)
        assert mu == pytest.approx(mu_o, rel=1e-13)
        assert kap == pytest.approx(kap_o, rel=1e-13)
        np.testing.assert_allclose(dif, dif_o, rtol=1e-12)
