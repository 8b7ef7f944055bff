"""Chemistry surrogate on the GPU: the tensor-core GEMM against torch FP32
matmuls, the MLP's gradients against the float64 CPU oracle
(oracle/mlp_ref.py), and the trained, gated surrogate against the FP64
reference integrator.

Tolerances: GEMM products 1e-4 relative to the largest |C| (FP32
accumulation in a different order); fused GELU / GELU' epilogues 1e-2
relative (BF16 output rounding); MLP loss 2e-3 and weight/bias gradients
4e-2 relative Frobenius error against the oracle, which sees the same BF16
weights and inputs but keeps every activation in float64 (the GPU rounds
activations and back-propagated signals to BF16); gated surrogate +
fallback: species within 1e-3 relative (species >= 1e-6) and T within
1e-3 relative of the FP64 reference.
"""
import sys
from pathlib import Path

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

sys.path.insert(0, str(Path(__file__).resolve().parents[1] / "oracle"))


def _bf(x):
    return x.to(torch.bfloat16)


@pytest.mark.parametrize("M,N,K", [(128, 64, 64), (300, 256, 192), (257, 128, 256), (1000, 320, 64), (64, 256, 4096)])
def test_gemm_matches_torch(M, N, K):
    from fortrancfd_gb300 import surrogate as S

    g = torch.Generator(device="cuda").manual_seed(M + N + K)
    A = _bf(torch.randn(M, K, device="cuda", generator=g))
    B = _bf(torch.randn(N, K, device="cuda", generator=g))
    bias = torch.randn(N, device="cuda", generator=g)
    C = torch.full((M, N), float("nan"), device="cuda")
    S.gemm(A, B, M, N, K, S.EPI_F32, bias=bias, C32=C)
    S.status()
    ref = A.float() @ B.float().T + bias
    err = ((C - ref).abs().max() / ref.abs().max()).item()
    assert err < 1e-4, err


@pytest.mark.parametrize("M,N,K", [(128, 64, 64), (256, 256, 192), (384, 128, 256), (1024, 320, 64), (128, 256, 4096)])
def test_bulk_copy_gemm_matches_torch(M, N, K):
    from fortrancfd_gb300 import surrogate as S

    g = torch.Generator(device="cuda").manual_seed(M + 2 * N + K)
    A = _bf(torch.randn(M, K, device="cuda", generator=g))
    B = _bf(torch.randn(N, K, device="cuda", generator=g))
    bias = torch.randn(N, device="cuda", generator=g)
    C = torch.full((M, N), float("nan"), device="cuda")
    S.gemm_tiled(S.tile(A, 128), S.tile(B, S.tile_rows(N)), M, N, K, S.EPI_F32, bias=bias, C32=C)
    S.status()
    ref = A.float() @ B.float().T + bias
    err = ((C - ref).abs().max() / ref.abs().max()).item()
    assert err < 1e-4, err


def test_bulk_copy_forward_equals_thread_copy_forward():
    """The inference path (tiled operands, bulk copies, tiled GELU output)
    issues the same products in the same order as the training path: the
    outputs agree bit for bit."""
    from fortrancfd_gb300 import surrogate as S

    m = S.MLP(seed=3)
    g = torch.Generator(device="cuda").manual_seed(7)
    X = torch.zeros(640, S.KIN, device="cuda")
    X[:, : S.NIN] = torch.randn(640, S.NIN, device="cuda", generator=g)
    X16 = _bf(X)
    a = m.forward(X16).clone()
    b = m.forward_tiled(X16).clone()
    S.status()
    assert torch.equal(a, b), (a - b).abs().max().item()


def test_gemm_epilogues():
    from fortrancfd_gb300 import surrogate as S

    g = torch.Generator(device="cuda").manual_seed(5)
    M, N, K = 256, 256, 128
    A = _bf(torch.randn(M, K, device="cuda", generator=g) * 0.2)
    B = _bf(torch.randn(N, K, device="cuda", generator=g) * 0.2)
    bias = torch.randn(N, device="cuda", generator=g) * 0.1
    Z = torch.empty(M, N, device="cuda")
    H = torch.empty(M, N, dtype=torch.bfloat16, device="cuda")
    S.gemm(A, B, M, N, K, S.EPI_GELU, bias=bias, C32=Z, C16=H)
    z = A.float() @ B.float().T + bias
    h = torch.nn.functional.gelu(z)
    assert ((Z - z).abs().max() / z.abs().max()).item() < 1e-4
    assert ((H.float() - h).abs().max() / h.abs().max()).item() < 1e-2
    D16 = torch.empty(M, N, dtype=torch.bfloat16, device="cuda")
    D32 = torch.empty(M, N, device="cuda")
    S.gemm(A, B, M, N, K, S.EPI_DGELU, C32=D32, C16=D16, Z=z.contiguous())
    S.status()
    zz = z.double()
    dg = 0.5 * (1 + torch.erf(zz / 2 ** 0.5)) + zz * torch.exp(-0.5 * zz * zz) / (2 * np.pi) ** 0.5
    d = (A.double() @ B.double().T) * dg
    assert ((D32.double() - d).abs().max() / d.abs().max()).item() < 1e-4
    assert ((D16.double() - d).abs().max() / d.abs().max()).item() < 1e-2


def test_gradients_match_oracle():
    import mlp_ref

    from fortrancfd_gb300 import surrogate as S

    m = S.MLP(seed=1)
    M = 512
    g = torch.Generator(device="cuda").manual_seed(2)
    X = torch.zeros(M, S.KIN, device="cuda")
    X[:, : S.NIN] = torch.randn(M, S.NIN, device="cuda", generator=g)
    X16 = _bf(X)
    T = torch.zeros(M, S.KOUT, device="cuda")
    T[:, : S.NOUT] = torch.randn(M, S.NOUT, device="cuda", generator=g)
    # a few Adam steps first, so the biases and the last layer are not at
    # their initial values
    for _ in range(3):
        m.forward(X16, train=True)
        m.loss_grad(T)
        m.backward(M)
        m.adam(1e-3)
    m.forward(X16, train=True)
    loss = m.loss_grad(T).item()
    m.backward(M)
    S.status()
    Ws = [w.float().double().cpu().numpy() for w in m.W16]
    bs = [b.double().cpu().numpy() for b in m.b]
    lo, gW, gb = mlp_ref.loss_and_grads(Ws, bs, X16.double().cpu().numpy(), T.double().cpu().numpy(), S.NOUT)
    assert abs(loss - lo) / lo < 2e-3, (loss, lo)
    for l in range(len(Ws)):
        a, b = m.gW[l].double().cpu().numpy(), gW[l]
        e = np.linalg.norm(a - b) / np.linalg.norm(b)
        assert e < 4e-2, ("W", l, e)
        a, b = m.gb[l].double().cpu().numpy(), gb[l]
        e = np.linalg.norm(a - b) / np.linalg.norm(b)
        assert e < 4e-2, ("b", l, e)


def species_err(Yg, Yr, floor=1e-6):
    big = np.abs(Yr) >= floor
    rel = np.where(big, np.abs(Yg - Yr) / np.maximum(np.abs(Yr), floor), 0.0)
    return float(rel.max())


@pytest.fixture(scope="module")
def trained():
    from fortrancfd_gb300 import Reactors, configs
    from fortrancfd_gb300 import surrogate as S

    case = configs.detonation(ncell=2000, length=0.1)
    rho, dt, y0, y1 = S.harvest_tube(case, nsteps=1200, every=20)
    plain = Reactors(rtol=1e-6, atol=1e-14)
    s = S.Surrogate(plain, S.MLP(seed=0))
    hist = S.train(s, rho, dt, y0, y1, iters=3000, batch=4096, lr=2e-3, log_every=500)
    held = configs.detonation(ncell=2000, length=0.1, phi=1.2, T_drv=3300.0)
    hrho, hdt, hy0, hy1 = S.harvest_tube(held, nsteps=600, every=50)
    return s, hist, (hrho, hdt, hy0, hy1)


def test_training_lowers_loss(trained):
    _, hist, _ = trained
    assert hist[-1][1] < 0.5 * hist[0][1], hist


def test_gated_surrogate_matches_reference(trained):
    """Held-out states of another tube run (phi 1.2, 3300 K driver): the
    surrogate-with-fallback result is within the species/T bars of the FP64
    reference; the network's candidate is the one accepted for most cells;
    and adding the network loses no accepted cell against the same gate on
    the explicit increment alone (the method without the network). The
    fallback rates of both are printed."""
    s, _, (rho, dt, y0, ref) = trained
    d = lambda a: torch.tensor(a, device="cuda")  # noqa: E731
    y = d(y0)
    st = s.apply(d(rho), d(dt), y)
    out = y.cpu().numpy()
    assert species_err(out[:, :-1], ref[:, :-1]) < 1e-3
    assert np.max(np.abs(out[:, -1] - ref[:, -1]) / ref[:, -1]) < 1e-3
    y = d(y0)
    st0 = s.apply(d(rho), d(dt), y, zero_net=True)
    out0 = y.cpu().numpy()
    assert species_err(out0[:, :-1], ref[:, :-1]) < 1e-3
    print(f"fallback rate: network {st['fallback_rate']:.4f} ({st['accepted_network']} cells took the network's "
          f"candidate), explicit increment only {st0['fallback_rate']:.4f}")
    assert st["accepted_network"] > 0.5 * st["cells"]
    assert st["accepted"] >= st0["accepted"], (st, st0)


def test_decode_gate_compact_scatter_match_numpy():
    """The cell-path kernels against NumPy restatements on a synthetic
    batch: decode (y1 = y0 + dt f0 + c (|dt f0| + floor), Y clipped at 0)
    within 1e-14 of the size of its terms; the gate's accept flags exactly, with every
    synthetic residual at least 4x inside or outside its bound and one
    element's moles kept or broken by 100x its tolerance; compaction and
    scatter exactly."""
    from fortrancfd_gb300 import Reactors
    from fortrancfd_gb300 import surrogate as S
    from fortrancfd_gb300.surrogate import NS, _L, _p, _stream

    rng = np.random.default_rng(11)
    n, nv = 300, NS + 1
    s = S.Surrogate(Reactors(rtol=1e-6, atol=1e-14), S.MLP(seed=0))
    y0 = np.abs(rng.normal(0, 0.05, (n, nv)))
    y0[:, -1] = rng.uniform(300, 3000, n)
    f0 = rng.normal(0, 1e3, (n, nv))
    dt = 10 ** rng.uniform(-9, -7, n)
    out = rng.normal(0, 1, (n, S.KOUT)).astype(np.float32)
    omu = rng.normal(0, 0.1, S.KOUT).astype(np.float32)
    osig = rng.uniform(0.5, 2, S.KOUT).astype(np.float32)
    d = lambda a: torch.tensor(np.ascontiguousarray(a), device="cuda")  # noqa: E731
    # every device array is held by a name for the whole call: a temporary
    # would go back to the allocator (and to the next argument) at once
    with s:
        out_d, omu_d, osig_d, y0_d, f0_d, dt_d = d(out), d(omu), d(osig), d(y0), d(f0), d(dt)
        y1d = torch.empty(n, nv, dtype=torch.float64, device="cuda")
        S._ck(_L().edyn_mlp_decode(n, NS, _p(out_d), S.KOUT, _p(omu_d), _p(osig_d), _p(y0_d), _p(f0_d), _p(dt_d),
                                   S.YFLOOR, S.TFLOOR, _p(y1d), _stream()), "decode")
        y1 = y1d.cpu().numpy()
    e = dt[:, None] * f0
    cols = np.r_[np.arange(1, NS + 1), 0]  # component k (Y_0..Y_52, T) -> output column
    c = out[:, cols].astype(np.float64) * osig[cols].astype(np.float64) + omu[cols].astype(np.float64)
    floor = np.r_[np.full(NS, S.YFLOOR), S.TFLOOR]
    ref = y0 + e + c * (np.abs(e) + floor)
    ref[:, :NS] = np.maximum(ref[:, :NS], 0.0)
    # rounding (and FMA contraction) is relative to the terms, not the sum
    scale = np.abs(y0) + np.abs(e) + np.abs(c) * (np.abs(e) + floor)
    assert np.all(np.abs(y1 - ref) <= 1e-14 * scale)

    # gate: residual r = y1 - y0 - dt (f0 + f1) / 2 set to +-0.25x or +-4x
    # its bound per component; candidate a: first 100 cells inside, the rest
    # with one component outside; candidate b (second): cells 100..199 inside
    yb0 = np.abs(rng.normal(0.02, 0.01, (n, nv)))
    yb0[:, -1] = rng.uniform(800, 2500, n)
    E = s.elem.cpu().numpy()
    W = s.W_kg

    def candidate(scale_in, bad_cells, bad_col):
        y = yb0 * (1 + rng.uniform(-1e-7, 1e-7, yb0.shape))  # tiny change: elements held to ~1e-7
        f0g = rng.normal(0, 1e2, (n, nv))
        bound = np.r_[np.full(NS, s.atol), 0.0][None, :] + s.rtol * np.maximum(np.abs(yb0), np.abs(y))
        r = scale_in * bound * rng.choice([-1.0, 1.0], (n, nv))
        r[bad_cells, bad_col] = 4.0 * bound[bad_cells, bad_col]
        f1g = 2.0 * (y - yb0 - r) / dt[:, None] - f0g  # so that y - y0 - dt (f0 + f1)/2 = r
        return y, f0g, f1g

    ya, f0a, f1a = candidate(0.25, np.arange(100, n), 5)
    yb, _, _ = candidate(0.25, np.r_[np.arange(100), np.arange(200, n)], 7)
    # the second candidate's f1, for its own residual with the shared f0
    rb_bound = np.r_[np.full(NS, s.atol), 0.0][None, :] + s.rtol * np.maximum(np.abs(yb0), np.abs(yb))
    rb = 0.25 * rb_bound
    rb[np.r_[np.arange(100), np.arange(200, n)], 7] = 4.0 * rb_bound[np.r_[np.arange(100), np.arange(200, n)], 7]
    fbb = 2.0 * (yb - yb0 - rb) / dt[:, None] - f0a
    # cell 150: its second candidate breaks an element balance by far more than etol
    k_c = int(np.argmax(E[0]))  # a species that holds element 0
    yb[150, k_c] *= 1 + 100 * s.etol * (E[0] / W * yb0[150, :NS]).sum() / (E[0, k_c] / W[k_c] * yb0[150, k_c])
    fbb[150] = 2.0 * (yb[150] - yb0[150] - 0.25 * rb_bound[150]) / dt[150] - f0a[150]
    with s:
        y1g = d(ya)
        yb0_d, f0a_d, f1a_d, yb_d, fbb_d, dt_d = d(yb0), d(f0a), d(f1a), d(yb), d(fbb), d(dt)
        acc = torch.empty(n, dtype=torch.int32, device="cuda")
        cnt = torch.zeros(2, dtype=torch.int32, device="cuda")
        S._ck(_L().edyn_mlp_gate(n, NS, s.ne, _p(yb0_d), _p(y1g), _p(f0a_d), _p(f1a_d), _p(yb_d), _p(fbb_d),
                                 _p(dt_d), _p(s.wmol), _p(s.elem), s.rtol, s.atol, s.etol, _p(acc), _p(cnt),
                                 _stream()), "gate")
        a = acc.cpu().numpy()
        y1_out = y1g.cpu().numpy()
    want = np.zeros(n, dtype=np.int32)
    want[:100] = 1
    want[100:200] = 2
    want[150] = 0
    assert np.array_equal(a, want), np.nonzero(a != want)
    assert np.array_equal(cnt.cpu().numpy(), [100, 99])
    assert np.array_equal(y1_out[100:150], yb[100:150]) and np.array_equal(y1_out[:100], ya[:100])

    # compaction of the rejected cells, in cell order, and the scatter back
    rho = rng.uniform(0.1, 10, n)
    with s:
        idx = torch.empty(n, dtype=torch.int32, device="cuda")
        rp = torch.empty(n, dtype=torch.float64, device="cuda")
        dp = torch.empty(n, dtype=torch.float64, device="cuda")
        yp = torch.empty(n, nv, dtype=torch.float64, device="cuda")
        nr = torch.zeros(1, dtype=torch.int32, device="cuda")
        a_d, rho_d, dt_d, yb0_d = d(a), d(rho), d(dt), d(yb0)
        S._ck(_L().edyn_mlp_compact(n, NS, _p(a_d), _p(rho_d), _p(dt_d), _p(yb0_d), _p(idx), _p(rp), _p(dp),
                                    _p(yp), _p(nr), _stream()), "compact")
        m = int(nr.item())
        rej = np.nonzero(a == 0)[0]
        assert m == len(rej)
        assert np.array_equal(idx[:m].cpu().numpy(), rej)
        assert np.array_equal(rp[:m].cpu().numpy(), rho[rej]) and np.array_equal(dp[:m].cpu().numpy(), dt[rej])
        assert np.array_equal(yp[:m].cpu().numpy(), yb0[rej])
        tgt = torch.zeros(n, nv, dtype=torch.float64, device="cuda")
        S._ck(_L().edyn_mlp_scatter(m, NS, _p(idx), _p(yp), _p(tgt), _stream()), "scatter")
        t_np = tgt.cpu().numpy()
    assert np.array_equal(t_np[rej], yb0[rej]) and not t_np[a != 0].any()
