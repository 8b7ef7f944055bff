"""The MLP oracle (oracle/mlp_ref.py) against central finite differences of
its own loss: every weight and bias gradient within 1e-6 relative (float64,
step 1e-6) on a small network."""
import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parents[1] / "oracle"))
import mlp_ref  # noqa: E402


def _net(rng, dims):
    Ws = [rng.normal(0, (2.0 / dims[i]) ** 0.5, (dims[i + 1], dims[i])) for i in range(len(dims) - 1)]
    bs = [rng.normal(0, 0.1, dims[i + 1]) for i in range(len(dims) - 1)]
    return Ws, bs


def test_gradients_match_finite_differences():
    rng = np.random.default_rng(3)
    dims = [6, 9, 8, 5]
    Ws, bs = _net(rng, dims)
    X = rng.normal(size=(7, 6))
    T = rng.normal(size=(7, 5))
    n_real = 4
    _, gW, gb = mlp_ref.loss_and_grads(Ws, bs, X, T, n_real)
    h = 1e-6
    for l in range(len(Ws)):
        for arr, g in ((Ws[l], gW[l]), (bs[l], gb[l])):
            fd = np.zeros_like(arr)
            it = np.nditer(arr, flags=["multi_index"])
            for _ in it:
                i = it.multi_index
                old = arr[i]
                arr[i] = old + h
                lp = mlp_ref.loss_and_grads(Ws, bs, X, T, n_real)[0]
                arr[i] = old - h
                lm = mlp_ref.loss_and_grads(Ws, bs, X, T, n_real)[0]
                arr[i] = old
                fd[i] = (lp - lm) / (2 * h)
            err = np.abs(fd - g).max() / max(np.abs(g).max(), 1e-12)
            assert err < 1e-6, (l, err)


def test_padded_output_columns_get_no_gradient():
    rng = np.random.default_rng(4)
    Ws, bs = _net(rng, [4, 8, 6])
    X = rng.normal(size=(5, 4))
    T = rng.normal(size=(5, 6))
    _, gW, gb = mlp_ref.loss_and_grads(Ws, bs, X, T, 3)
    assert np.all(gW[-1][3:] == 0) and np.all(gb[-1][3:] == 0)
