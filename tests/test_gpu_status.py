"""Failure paths reported through the status words of the C ABI.

The reference stops on bad input (`stop`) or continues silently (the capped
temperature Newton, SRC/thermo.f90:244-255); the library returns EDYN_E_*
bits instead. Every failure here is made on the host (a broken state, a bad
argument, a second mechanism, a step cap of one, a zero wait limit); no
kernel faults, traps or hangs, and the context keeps working afterwards.
"""
import numpy as np
import pytest

from fortrancfd_gb300 import EdynError, Reactors, Tube, configs, edyn

pytestmark = pytest.mark.gpu


def _sod_tube(oracle, ncell=128):
    case = configs.sod(ncell=ncell)
    qf0, qc0 = oracle.init_cells(case.T, case.p, case.u, case.X)
    return case, Tube(case.ncell, case.dx), qf0, qc0


def _status(excinfo):
    return excinfo.value.code


def test_nan_state_upload(oracle):
    case, g, qf0, qc0 = _sod_tube(oracle)
    qc = qc0.copy()
    qc[17, 2] = np.nan
    with pytest.raises(EdynError) as ei:
        g.upload(None, qc)
    assert _status(ei) & edyn.EDYN_E_STATE
    # the context still works: a sound state uploads and steps
    g.upload(qf0, qc0)
    g.step(case.cfl)


def test_negative_mass_fraction_upload(oracle, names):
    case, g, qf0, qc0 = _sod_tube(oracle)
    qf = qf0.copy()
    k = 3 + names.index("O2")
    qf[5, k] = -0.01
    with pytest.raises(EdynError) as ei:
        g.upload(qf, qc0)
    assert _status(ei) & edyn.EDYN_E_STATE
    assert "clamped state" in g.last_error() or "non-finite" in g.last_error()


def test_too_cold_state_upload(oracle):
    case, g, qf0, qc0 = _sod_tube(oracle)
    qf = qf0.copy()
    qf[40, 2] = 10.0
    with pytest.raises(EdynError) as ei:
        g.upload(qf, qc0)
    assert _status(ei) & edyn.EDYN_E_STATE


def test_state_broken_mid_run_is_reported_by_the_step(oracle):
    """A cell whose energy is far below any temperature the tables hold
    drives its Newton to the 20 K clamp during the fluid stage: the step
    reports EDYN_E_STATE (the reference would clamp and continue)."""
    case, g, qf0, qc0 = _sod_tube(oracle)
    qc = qc0.copy()
    qc[60, 2] = -1e9  # rho e hugely negative: no temperature matches it
    # the uploaded conserved row is finite and positive where checked at
    # upload (rho e may be negative for a cold gas), so upload passes qf
    g.upload(qf0, qc)
    with pytest.raises(EdynError) as ei:
        g.step(case.cfl)
    assert _status(ei) & edyn.EDYN_E_STATE


def test_unknown_time_integrator_rejected():
    case = configs.sod(ncell=64)
    with pytest.raises(EdynError) as ei:
        Tube(case.ncell, case.dx, select_time=3)
    assert _status(ei) == edyn.EDYN_E_ARG
    assert "select_time=3" in str(ei.value)


def test_surrogate_mode_needs_a_surrogate(oracle):
    """chem_mode 1 without an attached surrogate: the source step refuses
    (EDYN_E_ARG) instead of silently running the plain integrator."""
    case = configs.detonation(ncell=256, length=256 * 50e-6, driver=48 * 50e-6)
    g = Tube(case.ncell, case.dx, flag_acu=2, flag_weno=3, flag_rbound=1, do_reaction=1, chem_mode=1)
    g.init_cells(case.T, case.p, case.u, case.X)
    with pytest.raises(EdynError) as ei:
        g.step(case.cfl)
    assert _status(ei) == edyn.EDYN_E_ARG and "edyn_set_surrogate" in str(ei.value)
    with pytest.raises(EdynError):
        Tube(case.ncell, case.dx, chem_mode=2)


def test_second_mechanism_rejected(tmp_path):
    """The thermo tables live in constant memory, one set per process: a
    context with a different mechanism is refused with EDYN_E_MECH."""
    Tube(64, 1e-3)  # the GRI-Mech 3.0 tables are loaded
    src = (edyn.GRI30_DIR / "mech.edyn").read_text().split("\n")
    # perturb one NASA-7 coefficient of the first species
    out, done = [], False
    for line in src:
        if not done and line.startswith("H2 "):
            parts = line.split()
            parts[5] = repr(float(parts[5]) * 1.001)
            line = " ".join(parts)
            done = True
        out.append(line)
    assert done
    d = tmp_path / "other"
    d.mkdir()
    (d / "mech.edyn").write_text("\n".join(out))
    with pytest.raises(EdynError) as ei:
        Tube(64, 1e-3, chem_dir=d)
    assert _status(ei) == edyn.EDYN_E_MECH


def test_integrator_step_cap_reports_chem_failure():
    """A step cap of one step per cell makes every cell that needs an
    implicit step fail: the batch call returns EDYN_E_CHEM with the failed
    cells counted; the cap lifted, the same batch integrates."""
    rho, dt, yiT, _ = configs.reactor_batch(64, seed=9)
    r = Reactors(rtol=1e-6, atol=1e-14)
    r.set_chem_max_steps(1)
    y = yiT.copy()
    st = r.integrate(rho, dt, y, raise_on_fail=False)
    assert st["status"] & edyn.EDYN_E_CHEM and st["failed"] > 0
    r.set_chem_max_steps(0)
    y = yiT.copy()
    st = r.integrate(rho, dt, y)
    assert st["status"] == 0 and st["failed"] == 0


def test_tube_step_cap_reports_chem_failure(oracle):
    case = configs.detonation(ncell=256, length=256 * 50e-6, driver=48 * 50e-6)
    qf0, qc0 = oracle.init_cells(case.T, case.p, case.u, case.X)
    g = Tube(case.ncell, case.dx, flag_acu=2, flag_weno=3, flag_rbound=1, do_reaction=1, rtol=1e-6, atol=1e-14)
    g.upload(qf0, qc0)
    g.set_chem_max_steps(1)
    with pytest.raises(EdynError) as ei:
        g.step(case.cfl)
    assert _status(ei) & edyn.EDYN_E_CHEM
    assert "chemistry integration failed" in g.last_error()


def test_surrogate_gemm_wait_runs_out_and_recovers():
    """The tensor-core GEMM's gating waits given a zero limit: the kernels
    give up, drain the copies and products they issued, free their TMEM and
    set the status that edyn_mlp_status reports as EDYN_E_SURR. With the
    limit restored the same products come out right."""
    torch = pytest.importorskip("torch")
    from fortrancfd_gb300 import surrogate as S

    g = torch.Generator(device="cuda").manual_seed(3)
    A = torch.randn(256, 256, device="cuda", generator=g).to(torch.bfloat16)
    B = torch.randn(128, 256, device="cuda", generator=g).to(torch.bfloat16)
    At, Bt = S.tile(A, 128), S.tile(B, S.tile_rows(128))
    C = torch.zeros(256, 128, device="cuda")
    ref = A.float() @ B.float().T
    try:
        S.set_wait_limit(0)
        S.gemm_tiled(At, Bt, 256, 128, 256, S.EPI_F32, C32=C)
        with pytest.raises(EdynError) as ei:
            S.status()
        assert ei.value.code == 64  # EDYN_E_SURR
        C2 = torch.zeros(256, 128, device="cuda")
        S.gemm(A, B, 256, 128, 256, S.EPI_F32, C32=C2)
        with pytest.raises(EdynError):
            S.status()
    finally:
        S.set_wait_limit(2_000_000_000)
    S.gemm_tiled(At, Bt, 256, 128, 256, S.EPI_F32, C32=C)
    S.gemm(A, B, 256, 128, 256, S.EPI_F32, C32=C2)
    S.status()
    for out in (C, C2):
        assert float(((out - ref).abs().max() / ref.abs().max()).item()) < 1e-4
