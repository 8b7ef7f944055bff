"""Initial conditions of the benchmark workloads, built the way the
reference's host does (initialize_variables, SRC/params.f90:305-580: step
profiles in T, p, u and mole fractions, the "other species" fill, then
density and energy per cell). Synthetic, seeded; no external data.

Cell centres are (i + 1/2) dx. The reference accumulates them block by
block (SRC/block.f90:256-304); for step profiles whose discontinuity does
not fall on a centre the cell classification is the same.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from .edyn import GRI30_DIR, species_names

ATM = 101325.0


def mole_vector(names, comp: dict, fill: str | None = None) -> np.ndarray:
    x = np.zeros(len(names))
    for k, v in comp.items():
        x[names.index(k)] = v
    if fill is not None:  # "other species" fill (SRC/params.f90:453-459)
        x[names.index(fill)] += 1.0 - x.sum()
    return x


@dataclass
class TubeCase:
    name: str
    ncell: int
    dx: float
    T: np.ndarray
    p: np.ndarray
    u: np.ndarray
    X: np.ndarray
    flags: dict = field(default_factory=dict)
    cfl: float = 0.5
    tend: float = 0.0


def sod(names=None, ncell: int = 1000, length: float = 1.0) -> TubeCase:
    """1-D Sod tube: p_L/p_R = 10, rho_L/rho_R = 8 (T_L = 375 K, T_R = 300 K),
    stoichiometric CH4/air (WORK/Examples/CH4_GRI3.0/SOD/initial.txt:17-24),
    frozen chemistry, MUSCL-minmod + HLLC, TVDRK3, CFL 0.5, walls, 0.6 ms."""
    names = names or species_names(GRI30_DIR)
    dx = length / ncell
    xm = (np.arange(ncell) + 0.5) * dx
    left = xm <= 0.5 * length
    x = mole_vector(names, {"CH4": 0.0950570342, "O2": 0.1901140684, "N2": 0.7148288973}, fill="N2")
    T = np.where(left, 375.0, 300.0)
    p = np.where(left, 10 * ATM, ATM)
    X = np.tile(x, (ncell, 1))
    return TubeCase("sod_ch4air_1000", ncell, dx, T, p, np.zeros(ncell), X,
                    dict(select_time=1, select_riemann=2, flag_acu=1, flag_muscl=2, flag_weno=0,
                         flag_lbound=0, flag_rbound=0, do_reaction=0), cfl=0.5, tend=0.6e-3)


def _thermo_tables(mech_dir=GRI30_DIR):
    txt = (Path(mech_dir) / "mech.edyn").read_text().split()
    ne = int(txt[txt.index("ELEMENTS") + 1])
    enames = [txt[txt.index("ELEMENTS") + 2 + 2 * e] for e in range(ne)]
    i = txt.index("SPECIES")
    n = int(txt[i + 1])
    per = 5 + 14 + ne
    tmid = np.zeros(n)
    a = np.zeros((n, 2, 7))
    comp = np.zeros((n, ne))
    for k in range(n):
        b = i + 2 + k * per
        tmid[k] = float(txt[b + 3])
        a[k] = np.array([float(v) for v in txt[b + 5:b + 19]]).reshape(2, 7)
        comp[k] = [int(v) for v in txt[b + 19:b + 19 + ne]]
    return enames, tmid, a, comp


def gibbs_rt(T, mech_dir=GRI30_DIR):
    """g_k / (R T) of every species from the NASA-7 polynomials."""
    _, tmid, a, _ = _thermo_tables(mech_dir)
    c = a[np.arange(len(tmid)), (T > tmid).astype(int)]
    h = c[:, 0] + c[:, 1] * T / 2 + c[:, 2] * T ** 2 / 3 + c[:, 3] * T ** 3 / 4 + c[:, 4] * T ** 4 / 5 + c[:, 5] / T
    s = c[:, 0] * np.log(T) + c[:, 1] * T + c[:, 2] * T ** 2 / 2 + c[:, 3] * T ** 3 / 3 + c[:, 4] * T ** 4 / 4 + c[:, 6]
    return h - s


def equilibrium_tp(X0: np.ndarray, T: float, p: float, mech_dir=GRI30_DIR, iters: int = 200) -> np.ndarray:
    """Ideal-gas chemical equilibrium at fixed T [K], p [Pa] holding the
    element totals of X0: Gibbs minimisation by the element-potential
    method (n_k = N exp(-g_k/RT - ln(p/p0) + sum_e lambda_e a_ek), Newton on
    lambda and ln N with step damping). Returns mole fractions."""
    _, _, _, comp = _thermo_tables(mech_dir)
    g = gibbs_rt(T, mech_dir) + np.log(p / ATM)
    b = comp.T @ X0
    act = b > 0
    allowed = np.all(comp[:, ~act] == 0, axis=1)
    A = comp[allowed][:, act]
    gk = g[allowed]
    be = b[act]
    ne = A.shape[1]
    # start: one reference species per element (O2, H2, CO, N2, AR) at a
    # mole fraction of 0.1 fixes the element potentials
    enames, _, _, _ = _thermo_tables(mech_dir)
    names = species_names(mech_dir)
    names_ok = [n for n, ok in zip(names, allowed) if ok]
    act_names = [e for e, a_ in zip(enames, act) if a_]
    ref = {"O": "O2", "H": "H2", "C": "CO", "N": "N2", "AR": "AR"}
    rows = [names_ok.index(ref[e]) for e in act_names]
    lam = np.linalg.solve(A[rows], gk[rows] + np.log(0.1))
    lnN = 0.0
    for _ in range(iters):
        mu = np.clip(-gk + lnN + A @ lam, -700, 700)
        n = np.exp(mu)
        N = np.exp(lnN)
        F = np.concatenate([A.T @ n - be, [n.sum() - N]])
        J = np.zeros((ne + 1, ne + 1))
        J[:ne, :ne] = (A * n[:, None]).T @ A
        J[:ne, ne] = A.T @ n
        J[ne, :ne] = A.T @ n
        J[ne, ne] = n.sum() - N
        d = np.linalg.lstsq(J, -F, rcond=None)[0]
        step = 1.0 / max(1.0, np.abs(d).max() / 2.0)
        lam += step * d[:ne]
        lnN += step * d[ne]
        if np.abs(F).max() < 1e-14 * max(1.0, be.max()):
            break
    mu = np.clip(-gk + lnN + A @ lam, -700, 700)
    x = np.zeros(len(g))
    x[allowed] = np.exp(mu)
    return x / x.sum()


def detonation(names=None, ncell: int = 20000, length: float = 1.0, driver: float = 0.01, T_drv: float = 3000.0,
               p_drv: float = 30 * ATM, phi: float = 1.0, p0: float = ATM, T0: float = 300.0,
               oxidizer: str = "O2", weno: int = 3) -> TubeCase:
    """CH4 detonation tube: fresh stoichiometric CH4/O2 at 1 atm, 300 K; a
    driver at x <= 1 cm holding the TP-equilibrium products of the fresh
    mixture at 3000 K, 30 atm; reflecting left wall, fixed-pressure outlet at
    1 atm on the right; WENO5 + HLLC, TVDRK3, CFL 0.4."""
    names = names or species_names(GRI30_DIR)
    dx = length / ncell
    xm = (np.arange(ncell) + 0.5) * dx
    drv = xm <= driver
    if oxidizer == "O2":
        fresh = mole_vector(names, {"CH4": phi / (phi + 2.0), "O2": 2.0 / (phi + 2.0)})
    else:  # air: O2 + 3.76 N2
        n = phi + 2.0 * 4.76
        fresh = mole_vector(names, {"CH4": phi / n, "O2": 2.0 / n, "N2": 2.0 * 3.76 / n})
    # equilibrium products of the fresh mixture at the driver's T and p
    burnt = equilibrium_tp(fresh, T_drv, p_drv)
    T = np.where(drv, T_drv, T0)
    p = np.where(drv, p_drv, p0)
    X = np.where(drv[:, None], burnt[None, :], fresh[None, :])
    return TubeCase(f"ch4_{oxidizer.lower()}_detonation_{ncell}", ncell, dx, T, p, np.zeros(ncell), X,
                    dict(select_time=1, select_riemann=2, flag_acu=2, flag_muscl=2, flag_weno=weno,
                         flag_lbound=0, flag_rbound=1, do_reaction=1, p_out=p0), cfl=0.4, tend=200e-6)


def planar_flame(names=None, ncell: int = 1000, dx: float = 2.0e-5, T_lo: float = 300.0, T_hi: float = 2400.0,
                 x_c: float = 1.4e-2, width: float = 2.0e-3, u_in: float = 1.0, do_reaction: int = 1) -> TubeCase:
    """Planar CH4/air flame with transport, the reference's planar-flame
    example (WORK/Examples/CH4_GRI3.0/PlanarFlame_Xe: pla_flame.inp,
    initial.txt, bound_flow.txt) with N2 in place of its Xe diluent, which
    GRI-Mech 3.0 lacks, and one uniform grid in place of its SMR blocks:
    stoichiometric CH4/O2/N2 (0.0951/0.1901/0.7148) at 1 atm, temperature
    T_lo + (T_hi - T_lo)(erf((x - x_c)/width) + 1)/2 (SRC/params.f90:374-377),
    constant mass flux rho u = rho_in u_in, inflow at 300 K, 1 m/s on the
    left, outflow at 1 atm on the right; MUSCL-minmod + HLLC, TVDRK3, CFL
    0.5, transport and chemistry on."""
    from math import erf

    names = names or species_names(GRI30_DIR)
    xm = (np.arange(ncell) + 0.5) * dx
    fresh = mole_vector(names, {"CH4": 0.0950570342, "O2": 0.1901140684, "N2": 0.7148288973})
    T = T_lo + 0.5 * (T_hi - T_lo) * (np.array([erf((x - x_c) / width) for x in xm]) + 1.0)
    p = np.full(ncell, ATM)
    X = np.tile(fresh, (ncell, 1))
    W = molecular_weights()
    wm = float(fresh @ W)
    rho = p * wm / (8314.51 * T)
    rho_in = ATM * wm / (8314.51 * T_lo)
    u = rho_in * u_in / rho
    return TubeCase(f"ch4_air_planar_flame_{ncell}", ncell, dx, T, p, u, X,
                    dict(select_time=1, select_riemann=2, flag_acu=1, flag_muscl=2, flag_weno=0,
                         flag_lbound=1, flag_rbound=1, do_reaction=do_reaction, do_tran=1, p_out=ATM, t_in=T_lo,
                         rho_u_in=rho_in * u_in, x_in=fresh), cfl=0.5, tend=0.2)


def spherical_flame(names=None, ncell: int = 2000, dx: float = 2.0e-5, do_reaction: int = 1) -> TubeCase:
    """Spherical CH4/air flame kernel, the reference's spherical-flame
    example (WORK/Examples/CH4_GRI3.0/SphericalFlame: sph_flame.inp,
    initial.txt, igsource.inp) on one uniform grid in place of its SMR
    blocks: stoichiometric CH4/O2/N2 at 300 K, 1 atm, at rest; spherical
    geometry with the centre a wall and an outflow at 1 atm at r = ncell dx;
    an ignition energy after Frendi et al. of 0.5 mJ within 500 um for the
    first 100 us; MUSCL-minmod + HLLC, TVDRK3, CFL 0.2, transport and
    chemistry on. flags['ignition'] holds (kind, [(E, r, duration, start)])."""
    names = names or species_names(GRI30_DIR)
    fresh = mole_vector(names, {"CH4": 0.0950570342, "O2": 0.1901140684, "N2": 0.7148288973})
    return TubeCase(f"ch4_air_spherical_flame_{ncell}", ncell, dx, np.full(ncell, 300.0), np.full(ncell, ATM),
                    np.zeros(ncell), np.tile(fresh, (ncell, 1)),
                    dict(select_time=1, select_riemann=2, flag_acu=1, flag_muscl=2, flag_weno=0, flag_lbound=0,
                         flag_rbound=1, do_reaction=do_reaction, do_tran=1, is_spherical=1, p_out=ATM,
                         ignition=(1, [(0.5e-3, 500e-6, 100e-6, 0.0)])), cfl=0.2, tend=2.0e-2)


def smr_segments(nx_comp: int, dx_comp: float, ncell_per_block: int, lev_smr_0: int = 0, num_smr_0: int = 0,
                 lev_smr_n: int = 0, num_smr_n: int = 0):
    """Segments (cells, cell size) of the reference's SMR layout
    (set_block_size, SRC/block.f90:91-379): the computational blocks at
    dx_comp, then on each side, from the inside out, levels 2..lev_smr of
    num_smr blocks each with the cell size doubling per level. Equal-size
    blocks merge into one segment. For edyn_init_blocks / Blocks."""
    left = [(num_smr_0 * ncell_per_block, dx_comp * 2 ** (lev - 1)) for lev in range(lev_smr_0, 1, -1)]
    right = [(num_smr_n * ncell_per_block, dx_comp * 2 ** (lev - 1)) for lev in range(2, lev_smr_n + 1)]
    segs = [s for s in left + [(nx_comp, dx_comp)] + right if s[0] > 0]
    return [n for n, _ in segs], [d for _, d in segs]


def ch4_air_mixture(names, phi: float) -> np.ndarray:
    n = phi + 2.0 * 4.76
    return mole_vector(names, {"CH4": phi / n, "O2": 2.0 / n, "N2": 2.0 * 3.76 / n})


def x_to_y(names, X: np.ndarray, W: np.ndarray) -> np.ndarray:
    Y = X * W
    return Y / Y.sum(axis=-1, keepdims=True)


def molecular_weights(mech_dir=GRI30_DIR) -> np.ndarray:
    txt = (mech_dir / "mech.edyn").read_text().split()
    i = txt.index("SPECIES")
    n = int(txt[i + 1])
    nel = int(txt[txt.index("ELEMENTS") + 1])
    per = 5 + 14 + nel
    return np.array([float(txt[i + 2 + k * per + 1]) for k in range(n)])


def reactor_batch(n: int, seed: int = 0, names=None):
    """Fresh CH4/air reactors: T ~ U[900, 2500] K, p log-uniform in
    [1, 50] atm, phi ~ U[0.5, 2.0], dt log-uniform in [1e-8, 1e-6] s.
    Returns (rho [kg/m^3], dt [s], yiT (n x (K+1)), phi)."""
    names = names or species_names(GRI30_DIR)
    W = molecular_weights()
    rng = np.random.default_rng(seed)
    T = rng.uniform(900.0, 2500.0, n)
    p = ATM * np.exp(rng.uniform(np.log(1.0), np.log(50.0), n))
    phi = rng.uniform(0.5, 2.0, n)
    dt = np.exp(rng.uniform(np.log(1e-8), np.log(1e-6), n))
    X = np.stack([ch4_air_mixture(names, f) for f in phi])
    Y = x_to_y(names, X, W)
    wbar = 1.0 / (Y / W).sum(axis=1)
    rho = p * wbar / (8314.51 * T)
    yiT = np.concatenate([Y, T[:, None]], axis=1)
    return rho, dt, np.ascontiguousarray(yiT), phi


def uneven_tubes(ntube: int, seed: int = 0, cells=(2000, 50000), length=(0.1, 1.0), names=None):
    """The uneven batch: ntube independent CH4/air detonation tubes with cell
    counts ~ U[cells], tube lengths ~ U[length] m, equivalence ratio
    phi ~ U[0.7, 1.4], initial pressure ~ U[0.5, 5] atm and driver
    temperature ~ U[2500, 3500] K (seeded); 1 cm driver at 30 atm holding
    the fresh mixture's TP-equilibrium products; wall left, fixed-pressure
    outlet (at the tube's initial pressure) right; WENO5-Z + HLLC + SSP-RK3,
    CFL 0.4. Returns the tubes' TubeCase list (p_out in each case's flags)."""
    names = names or species_names(GRI30_DIR)
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(ntube):
        n = int(rng.integers(cells[0], cells[1] + 1))
        L = float(rng.uniform(*length))
        phi = float(rng.uniform(0.7, 1.4))
        p0 = ATM * float(rng.uniform(0.5, 5.0))
        tdrv = float(rng.uniform(2500.0, 3500.0))
        case = detonation(names, ncell=n, length=L, phi=phi, T_drv=tdrv, p0=p0, oxidizer="air")
        case.flags["p_out"] = p0
        out.append(case)
    return out
