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
