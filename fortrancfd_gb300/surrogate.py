"""Chemistry surrogate with per-cell gating and fallback to the implicit
integrator.

The reference integrates every cell's chemistry with its implicit solver
(``reaction_macks`` -> ``macks(dt, nspe+1, yiT, rho)``,
SRC/source.f90:17-84). This module adds a learned path for the same call:

* an MLP (64 padded inputs -> 3 x 256 GELU -> 64 padded outputs; BF16
  weights, FP32 accumulation) whose dense layers are the tcgen05 GEMM of
  ``csrc/mlp.cu`` with fused bias/GELU epilogues, trained on the GPU by the
  same kernels (forward, backward with the GELU derivative fused into the
  data-gradient GEMM, Adam on FP32 master weights);
* inputs x = (T, log p, Box-Cox(Y_k, 0.1), log dt), standardised;
* output: per component (Y_k, T) the correction of the explicit increment
  dt f(y0) in units of its own size, so
  y1 = y0 + dt f0 + c (|dt f0| + floor);
* a gate per cell in FP64: the trapezoidal residual
  y1 - y0 - dt (f(y0) + f(y1)) / 2 within rtol max(|y0|, |y1|, floor), and
  every element's moles within etol; cells that fail go to the implicit
  integrator (``edyn_reactors_device``), and the fallback rate is reported.

Everything on the cell path runs in the library's kernels; torch supplies
device memory, streams and (training only) the batch sampling.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np
import torch

from . import configs
from .edyn import GRI30_DIR, EdynError, Reactors, lib

NS = 53
NIN = NS + 3           # T, log p, 53 Box-Cox Y, log dt
KIN = 64               # padded input width
NOUT = NS + 1          # T, 53 Y
KOUT = 64              # padded output width
HID = 256
DEPTH = 3
YFLOOR = 1e-10         # floor of the species correction unit
TFLOOR = 1e-4          # floor of the temperature correction unit [K]
CLIP = 8.0             # training targets are clipped to [-CLIP, CLIP] units

EPI_F32, EPI_GELU, EPI_DGELU = 0, 1, 2

_bound = False


def _L():
    global _bound
    L = lib()
    if not _bound:
        vp, i, d, f, l = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_float, ctypes.c_long
        L.edyn_mlp_gemm.argtypes = [vp, i, vp, i, i, i, i, i, vp, vp, i, vp, i, vp, i, vp]
        L.edyn_mlp_status.argtypes = [vp]
        L.edyn_mlp_transpose.argtypes = [vp, i, i, vp, vp]
        L.edyn_mlp_colsum.argtypes = [vp, i, i, vp, vp]
        L.edyn_mlp_mse.argtypes = [vp, vp, i, i, i, vp, vp, vp, vp]
        L.edyn_mlp_adam.argtypes = [vp, vp, vp, vp, l, f, f, f, f, i, vp, vp]
        L.edyn_mlp_features.argtypes = [i, i, vp, vp, vp, vp, vp, vp, vp, i, vp]
        L.edyn_mlp_decode.argtypes = [i, i, vp, i, vp, vp, vp, vp, vp, d, d, vp, vp]
        L.edyn_mlp_gate.argtypes = [i, i, i, vp, vp, vp, vp, vp, vp, vp, vp, vp, d, d, d, vp, vp, vp]
        L.edyn_mlp_compact.argtypes = [i, i, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp]
        L.edyn_mlp_scatter.argtypes = [i, i, vp, vp, vp, vp]
        L.edyn_chem_rhs_device.argtypes = [vp, i, vp, vp, vp]
        L.edyn_mlp_gemm_tiled.argtypes = [vp, vp, i, i, i, i, vp, vp, i, vp, i, i, vp]
        L.edyn_mlp_tile.argtypes = [vp, i, i, i, vp, vp]
        L.edyn_mlp_tile_rows.argtypes = [i]
        L.edyn_mlp_set_wait_limit.argtypes = [ctypes.c_ulonglong]
        _bound = True
    return L


def _p(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def _ck(rc: int, what: str):
    if rc:
        raise EdynError(rc, what)


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def gemm(A, B, M, N, K, epi, bias=None, C32=None, C16=None, Z=None):
    """C = A B^T on the tensor cores (A [M][K], B [N][K] BF16) with the fused
    epilogue ``epi`` (see include/edyn_surrogate.h)."""
    _ck(_L().edyn_mlp_gemm(_p(A), A.stride(0), _p(B), B.stride(0), M, N, K, epi, _p(bias), _p(C32),
                           C32.stride(0) if C32 is not None else 0, _p(C16), C16.stride(0) if C16 is not None else 0,
                           _p(Z), Z.stride(0) if Z is not None else 0, _stream()), "mlp gemm")


def gemm_tiled(At, Bt, M, N, K, epi, bias=None, C32=None, C16=None, c16_tiled=False):
    """The bulk-copy GEMM on pre-tiled operands (see tile())."""
    _ck(_L().edyn_mlp_gemm_tiled(_p(At), _p(Bt), M, N, K, epi, _p(bias), _p(C32),
                                 C32.stride(0) if C32 is not None else 0, _p(C16),
                                 C16.shape[-1] if C16 is not None else 0, int(c16_tiled), _stream()), "mlp gemm tiled")


def tile_rows(N):
    return _L().edyn_mlp_tile_rows(N)


def tile(x, br, out=None):
    """Row-major [R][K] BF16 -> the tiled operand layout with br-row blocks
    (rows padded with zeros to a multiple of br); returned flat."""
    R, K = x.shape
    Rp = (R + br - 1) // br * br
    out = torch.empty(Rp * K, dtype=x.dtype, device=x.device) if out is None else out
    _ck(_L().edyn_mlp_tile(_p(x), R, K, br, _p(out), _stream()), "mlp tile")
    return out


def transpose(x, out=None):
    r, c = x.shape
    out = torch.empty((c, r), dtype=x.dtype, device=x.device) if out is None else out
    _ck(_L().edyn_mlp_transpose(_p(x), r, c, _p(out), _stream()), "mlp transpose")
    return out


def status():
    _ck(_L().edyn_mlp_status(_stream()), "mlp kernel wait ran out")


def set_wait_limit(ns: int) -> None:
    """Limit of the GEMM kernels' gating waits (default 2 s; 0: give up at
    once, which exercises the failure path)."""
    _ck(_L().edyn_mlp_set_wait_limit(int(ns)), "mlp wait limit")


def element_matrix(mech_dir=GRI30_DIR):
    _, _, _, comp = configs._thermo_tables(mech_dir)
    return np.ascontiguousarray(comp.T)  # [ne][ns]


def raw_features(rho, dt, yiT, W_kg):
    """The network inputs before standardisation, in FP64 (host; used for the
    normalisation statistics): T, log p, Box-Cox(Y, 0.1), log dt."""
    T = yiT[:, -1]
    p = rho * 8.31446261815324 * T * (yiT[:, :-1] / W_kg).sum(axis=1)
    bc = (np.maximum(yiT[:, :-1], 1e-30) ** 0.1 - 1.0) * 10.0
    return np.concatenate([T[:, None], np.log(p)[:, None], bc, np.log(dt)[:, None]], axis=1)


@dataclass
class MLP:
    """Parameters, optimiser state and work buffers of the surrogate MLP."""

    seed: int = 0
    device: str = "cuda"
    W: list = field(default_factory=list)      # FP32 master weights [N][K]
    b: list = field(default_factory=list)
    W16: list = field(default_factory=list)    # BF16 copies [N][K]
    W16T: list = field(default_factory=list)   # BF16 transposes [K][N] (backward)
    step_count: int = 0

    def __post_init__(self):
        dims = [KIN] + [HID] * DEPTH + [KOUT]
        g = torch.Generator().manual_seed(self.seed)
        dev = self.device
        for l in range(DEPTH + 1):
            n, k = dims[l + 1], dims[l]
            fan = NIN if l == 0 else k
            w = torch.randn(n, k, generator=g) * (2.0 / fan) ** 0.5
            if l == 0:
                w[:, NIN:] = 0
            if l == DEPTH:
                w *= 0.1
                w[NOUT:, :] = 0
            self.W.append(w.to(dev).contiguous())
            self.b.append(torch.zeros(n, device=dev))
        self.W16 = [w.to(torch.bfloat16).contiguous() for w in self.W]
        self.W16T = [w.t().contiguous().to(torch.bfloat16) for w in self.W]
        self.mW = [torch.zeros_like(w) for w in self.W]
        self.vW = [torch.zeros_like(w) for w in self.W]
        self.mb = [torch.zeros_like(b) for b in self.b]
        self.vb = [torch.zeros_like(b) for b in self.b]
        self.gW = [torch.zeros_like(w) for w in self.W]
        self.gb = [torch.zeros_like(b) for b in self.b]
        self.mu = torch.zeros(KIN, device=dev)
        self.isig = torch.zeros(KIN, device=dev)
        self.isig[:NIN] = 1.0
        self.omu = torch.zeros(KOUT, device=dev)
        self.osig = torch.ones(KOUT, device=dev)
        self._buf = {}

    # -- buffers ---------------------------------------------------------
    def _bufs(self, M):
        if M not in self._buf:
            d, bf = self.device, torch.bfloat16
            self._buf[M] = dict(
                H=[None] + [torch.empty(M, HID, dtype=bf, device=d) for _ in range(DEPTH)],
                Z=[torch.empty(M, HID, device=d) for _ in range(DEPTH)],
                Y=torch.empty(M, KOUT, device=d),
                dY32=torch.empty(M, KOUT, device=d),
                dY16=torch.empty(M, KOUT, dtype=bf, device=d),
                dZ32=[torch.empty(M, HID, device=d) for _ in range(DEPTH)],
                dZ16=[torch.empty(M, HID, dtype=bf, device=d) for _ in range(DEPTH)],
                GT={n: torch.empty(n, M, dtype=bf, device=d) for n in (KOUT, HID)},
                HT={n: torch.empty(n, M, dtype=bf, device=d) for n in (KIN, HID)},
                loss=torch.zeros(1, dtype=torch.float64, device=d),
            )
        return self._buf[M]

    # -- passes ----------------------------------------------------------
    def forward(self, X16, train=False):
        """Network output (FP32 [M][KOUT]) for BF16 inputs X16 [M][KIN]."""
        M = X16.shape[0]
        B = self._bufs(M)
        B["H"][0] = X16
        for l in range(DEPTH):
            gemm(B["H"][l], self.W16[l], M, HID, B["H"][l].shape[1], EPI_GELU, bias=self.b[l],
                 C32=B["Z"][l] if train else None, C16=B["H"][l + 1])
        gemm(B["H"][DEPTH], self.W16[DEPTH], M, KOUT, HID, EPI_F32, bias=self.b[DEPTH], C32=B["Y"])
        return B["Y"]

    def forward_tiled(self, X16):
        """forward() for inference through the bulk-copy GEMM: the inputs and
        weights are tiled once, each layer writes its activations tiled for
        the next. X16 rows: a multiple of 128."""
        M = X16.shape[0]
        if getattr(self, "_tiled_at", None) != self.step_count:
            self.Wt = [tile(w, tile_rows(w.shape[0])) for w in self.W16]
            self._tiled_at = self.step_count
        key = ("tiled", M)
        if key not in self._buf:
            d, bf = self.device, torch.bfloat16
            self._buf[key] = dict(X=torch.empty(M * KIN, dtype=bf, device=d),
                                  H=[torch.empty(M * HID, dtype=bf, device=d) for _ in range(DEPTH)],
                                  Y=torch.empty(M, KOUT, device=d))
        B = self._buf[key]
        tile(X16, 128, B["X"])
        A, K = B["X"], KIN
        for l in range(DEPTH):
            gemm_tiled(A, self.Wt[l], M, HID, K, EPI_GELU, bias=self.b[l], C16=B["H"][l], c16_tiled=True)
            A, K = B["H"][l], HID
        gemm_tiled(A, self.Wt[DEPTH], M, KOUT, HID, EPI_F32, bias=self.b[DEPTH], C32=B["Y"])
        return B["Y"]

    def device_arrays(self):
        """(tiled BF16 weights, FP32 biases, normalisation 4 x 64) of the
        current parameters, for a tube's surrogate path."""
        if getattr(self, "_tiled_at", None) != self.step_count:
            self.Wt = [tile(w, tile_rows(w.shape[0])) for w in self.W16]
            self._tiled_at = self.step_count
        norm = torch.cat([self.mu, self.isig, self.omu, self.osig]).contiguous()
        return self.Wt, self.b, norm

    def loss_grad(self, target):
        """Mean-square error of the last forward output against target (FP32
        [M][KOUT], zeros in the padded columns) and its gradient; returns the
        loss as a device scalar."""
        M = target.shape[0]
        B = self._bufs(M)
        B["loss"].zero_()
        _ck(_L().edyn_mlp_mse(_p(B["Y"]), _p(target), M, KOUT, NOUT, _p(B["dY32"]), _p(B["dY16"]), _p(B["loss"]),
                              _stream()), "mlp mse")
        return B["loss"]

    def backward(self, M):
        """Gradients gW, gb of the loss whose output gradient loss_grad left
        in the buffers of batch size M (a multiple of 64)."""
        B = self._bufs(M)
        G16, G32 = B["dY16"], B["dY32"]
        for l in range(DEPTH, -1, -1):
            n, k = self.W[l].shape
            GT = transpose(G16, B["GT"][n])
            HT = transpose(B["H"][l], B["HT"][k])
            gemm(GT, HT, n, k, M, EPI_F32, C32=self.gW[l])
            _ck(_L().edyn_mlp_colsum(_p(G32), M, n, _p(self.gb[l]), _stream()), "mlp colsum")
            if l > 0:
                gemm(G16, self.W16T[l], M, k, n, EPI_DGELU, C32=B["dZ32"][l - 1], C16=B["dZ16"][l - 1],
                     Z=B["Z"][l - 1])
                G16, G32 = B["dZ16"][l - 1], B["dZ32"][l - 1]

    def adam(self, lr, b1=0.9, b2=0.999, eps=1e-8):
        self.step_count += 1
        L, s = _L(), _stream()
        for l in range(DEPTH + 1):
            _ck(L.edyn_mlp_adam(_p(self.W[l]), _p(self.gW[l]), _p(self.mW[l]), _p(self.vW[l]), self.W[l].numel(), lr,
                                b1, b2, eps, self.step_count, _p(self.W16[l]), s), "mlp adam")
            _ck(L.edyn_mlp_adam(_p(self.b[l]), _p(self.gb[l]), _p(self.mb[l]), _p(self.vb[l]), self.b[l].numel(), lr,
                                b1, b2, eps, self.step_count, None, s), "mlp adam")
            if l > 0:
                transpose(self.W16[l], self.W16T[l])


class Surrogate:
    """The trained network plus the gate, applied to batches of reactors
    (the macks contract: rho [kg/m^3], dt [s], yiT rows (Y_1..Y_ns, T))."""

    def __init__(self, reactors: Reactors, mlp: MLP | None = None, *, rtol=2.5e-4, yfloor_gate=1e-6, etol=1e-6):
        self.r = reactors
        self.mlp = mlp or MLP()
        dev = self.mlp.device
        W = configs.molecular_weights()
        self.W_kg = W * 1e-3
        self.wmol = torch.tensor(self.W_kg, dtype=torch.float64, device=dev)
        E = element_matrix()
        self.ne = E.shape[0]
        self.elem = torch.tensor(E, dtype=torch.float64, device=dev)
        self.rtol, self.atol, self.etol = rtol, rtol * yfloor_gate, etol
        self.stats = {}
        # one stream for the network's kernels and the context's chemistry
        # kernels (a NULL stream would send the latter to the context's own
        # stream, unordered with the former)
        self.stream = torch.cuda.Stream(device=dev)
        self.r.set_stream(self.stream.cuda_stream)

    def __enter__(self):
        self.stream.wait_stream(torch.cuda.current_stream())
        self._ctx = torch.cuda.stream(self.stream)
        self._ctx.__enter__()
        return self

    def __exit__(self, *exc):
        self._ctx.__exit__(*exc)
        self.stream.synchronize()
        return False

    # -- pieces of the cell path -----------------------------------------
    def rhs(self, rho, yiT, out=None):
        out = torch.empty_like(yiT) if out is None else out
        _ck(_L().edyn_chem_rhs_device(self.r._h, yiT.shape[0], _p(rho), _p(yiT), _p(out)), "chemistry rhs")
        return out

    def features(self, rho, dt, yiT):
        n = yiT.shape[0]
        M = (n + 127) // 128 * 128
        X = torch.zeros(M, KIN, dtype=torch.bfloat16, device=yiT.device)
        _ck(_L().edyn_mlp_features(n, NS, _p(rho), _p(dt), _p(yiT), _p(self.wmol), _p(self.mlp.mu), _p(self.mlp.isig),
                                   _p(X), KIN, _stream()), "mlp features")
        return X

    def candidate(self, rho, dt, yiT, f0, zero_net=False):
        """y1 from the network (or, with zero_net, the explicit increment
        alone: the method without the network)."""
        n = yiT.shape[0]
        y1 = torch.empty_like(yiT)
        if zero_net:
            out = torch.zeros(n, KOUT, device=yiT.device)
            omu, osig = torch.zeros_like(self.mlp.omu), torch.ones_like(self.mlp.osig)
        else:
            out = self.mlp.forward_tiled(self.features(rho, dt, yiT))
            omu, osig = self.mlp.omu, self.mlp.osig
        _ck(_L().edyn_mlp_decode(n, NS, _p(out), KOUT, _p(omu), _p(osig), _p(yiT), _p(f0), _p(dt), YFLOOR, TFLOOR,
                                 _p(y1), _stream()), "mlp decode")
        return y1

    def gate(self, rho, dt, y0, y1, f0, ya=None):
        """Accept flags of the candidate y1 (and, where it fails, of the
        second candidate ya, copied into y1 where it passes)."""
        n = y0.shape[0]
        f1 = self.rhs(rho, y1)
        fa = self.rhs(rho, ya) if ya is not None else None
        acc = torch.empty(n, dtype=torch.int32, device=y0.device)
        cnt = torch.zeros(2, dtype=torch.int32, device=y0.device)
        _ck(_L().edyn_mlp_gate(n, NS, self.ne, _p(y0), _p(y1), _p(f0), _p(f1), _p(ya), _p(fa), _p(dt), _p(self.wmol),
                               _p(self.elem), self.rtol, self.atol, self.etol, _p(acc), _p(cnt), _stream()),
            "mlp gate")
        return acc, cnt

    def apply(self, rho, dt, yiT, zero_net=False):
        """Advances the device batch yiT (float64 [n][ns+1]) over dt in place:
        the surrogate where the gate accepts it, the implicit integrator for
        the rest. Returns the counters (accepted cells, fallback rate, the
        integrator's right-hand sides)."""
        if yiT.shape[0] == 0:
            self.stats = {"cells": 0, "accepted": 0, "accepted_network": 0, "fallback_rate": 0.0, "integrator_rhs": 0,
                          "integrator_steps": 0}
            return self.stats
        with self:
            return self._apply(rho, dt, yiT, zero_net)

    def _apply(self, rho, dt, yiT, zero_net):
        n = yiT.shape[0]
        f0 = self.rhs(rho, yiT)
        if zero_net:
            y1 = self.candidate(rho, dt, yiT, f0, True)
            acc, cnt = self.gate(rho, dt, yiT, y1, f0)
        else:
            # the network's candidate, and the explicit increment where the
            # network's fails
            y1 = self.candidate(rho, dt, yiT, f0)
            acc, cnt = self.gate(rho, dt, yiT, y1, f0, self.candidate(rho, dt, yiT, f0, True))
        dev = yiT.device
        idx = torch.empty(n, dtype=torch.int32, device=dev)
        rho_p = torch.empty(n, dtype=torch.float64, device=dev)
        dt_p = torch.empty(n, dtype=torch.float64, device=dev)
        y_p = torch.empty_like(yiT)
        nrej = torch.zeros(1, dtype=torch.int32, device=dev)
        _ck(_L().edyn_mlp_compact(n, NS, _p(acc), _p(rho), _p(dt), _p(yiT), _p(idx), _p(rho_p), _p(dt_p), _p(y_p),
                                  _p(nrej), _stream()), "mlp compact")
        status()
        m = int(nrej.item())
        st = {"rhs": 0, "steps": 0}
        if m:
            st = self.r.integrate_device(m, rho_p.data_ptr(), dt_p.data_ptr(), y_p.data_ptr())
            _ck(_L().edyn_mlp_scatter(m, NS, _p(idx), _p(y_p), _p(y1), _stream()), "mlp scatter")
        yiT.copy_(y1)
        c = cnt.cpu().numpy()
        self.stats = {"cells": n, "accepted": n - m, "accepted_network": int(c[0]) if not zero_net else 0,
                      "fallback_rate": m / n, "integrator_rhs": st["rhs"], "integrator_steps": st["steps"]}
        return self.stats


# -- training data and training --------------------------------------------

def harvest_tube(case, nsteps=2000, every=20, rtol=1e-8, atol=1e-16, tube_rtol=1e-6, tube_atol=1e-14):
    """(rho, dt, y0, y1) pairs from a reacting tube run: every `every` steps
    the interior states and the step's dt, advanced over dt by the implicit
    integrator at (rtol, atol). Host numpy arrays."""
    from .edyn import Tube

    g = Tube(case.ncell, case.dx, rtol=tube_rtol, atol=tube_atol, **case.flags)
    g.init_cells(case.T, case.p, case.u, case.X)
    ref = Reactors(rtol=rtol, atol=atol)
    R, D, Y0 = [], [], []
    for s in range(nsteps):
        dt = g.step(case.cfl)
        if s % every == every - 1:
            qf, _, _ = g.download()
            R.append(qf[:, 0].copy())
            D.append(np.full(case.ncell, dt))
            Y0.append(np.concatenate([qf[:, 3:], qf[:, 2:3]], axis=1))
    g.close()
    rho, dt, y0 = np.concatenate(R), np.concatenate(D), np.ascontiguousarray(np.concatenate(Y0))
    y1 = y0.copy()
    ref.integrate(rho, dt, y1)
    ref.close()
    return rho, dt, y0, y1


def tube_sweep(n_cases, seed, *, ncell=4000, dx=5e-6, oxidizer="air"):
    """Detonation tubes of the surrogate's training sweep: 5 um cells,
    equivalence ratio phi ~ U[0.7, 1.4] and driver temperature ~ U[2500,
    3500] K (seeded), the 1 cm driver and the rest as the benchmark tube."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_cases):
        phi, tdrv = rng.uniform(0.7, 1.4), rng.uniform(2500.0, 3500.0)
        out.append(configs.detonation(ncell=ncell, length=ncell * dx, phi=phi, T_drv=tdrv, oxidizer=oxidizer))
    return out


def harvest_screened(cases, nsteps=100, every=1, rtol=1e-8, atol=1e-16, tube_rtol=1e-5, tube_atol=1e-13,
                     device="cuda"):
    """(rho, dt, y0, y1) pairs of the cells a chem_mode=1 tube hands to its
    surrogate: every `every` steps of each case, the state the source step
    sees (after the fluid step; Y adjust_summed) of the cells that fail the
    integrator's inert-cell test (||dt f(y0)||_w > 1e-3 with the tube's
    tolerances), advanced over the step's dt by the implicit integrator at
    (rtol, atol). Host arrays (float64)."""
    from .edyn import Tube

    R, D, Y0 = [], [], []
    for case in cases:
        g = Tube(case.ncell, case.dx, rtol=tube_rtol, atol=tube_atol, strict_newton=0, **case.flags)
        g.init_cells(case.T, case.p, case.u, case.X)
        for st in range(nsteps):
            dt = g.calc_dt(case.cfl)
            g.solve_fluid(dt)
            if st % every == every - 1:
                qf, _, _ = g.download()
                y = np.concatenate([np.maximum(qf[:, 3:], 0.0), qf[:, 2:3]], axis=1)
                y[:, :-1] /= y[:, :-1].sum(axis=1, keepdims=True)
                rho = torch.tensor(qf[:, 0], device=device)
                yd = torch.tensor(np.ascontiguousarray(y), device=device)
                f0 = torch.empty_like(yd)
                g.chem_rhs_device(len(rho), rho.data_ptr(), yd.data_ptr(), f0.data_ptr())
                w = tube_atol + tube_rtol * yd.abs()
                nrm = torch.sqrt(((dt * f0 / w) ** 2).mean(dim=1))
                keep = nrm > 1e-3
                R.append(rho[keep])
                D.append(torch.full((int(keep.sum()),), dt, dtype=torch.float64, device=device))
                Y0.append(yd[keep])
            g.solve_source(dt)
        g.close()
    rho, dt, y0 = torch.cat(R), torch.cat(D), torch.cat(Y0).contiguous()
    y1 = y0.clone()
    ref = Reactors(rtol=rtol, atol=atol)
    # windows of 2^16 reactors per call
    for a in range(0, len(rho), 1 << 16):
        b = min(len(rho), a + (1 << 16))
        blk = y1[a:b].contiguous()
        ref.integrate_device(b - a, rho[a:b].contiguous().data_ptr(), dt[a:b].contiguous().data_ptr(),
                             blk.data_ptr())
        y1[a:b] = blk
    ref.close()
    torch.cuda.synchronize()
    return rho.cpu().numpy(), dt.cpu().numpy(), y0.cpu().numpy(), y1.cpu().numpy()


def train(s: Surrogate, rho, dt, y0, y1, *, iters=3000, batch=4096, lr=1e-3, seed=0, log_every=0):
    """Fits s.mlp to the pairs (host numpy arrays) on the GPU with the
    library's kernels. Returns the loss history [(iter, loss)]."""
    with s:
        return _train(s, rho, dt, y0, y1, iters, batch, lr, seed, log_every)


def _train(s, rho, dt, y0, y1, iters, batch, lr, seed, log_every):
    dev = s.mlp.device
    m = s.mlp
    f0 = s.rhs(torch.tensor(rho, device=dev), torch.tensor(y0, device=dev)).cpu().numpy()
    # The gate tries the network first and the explicit increment second, so
    # the network is needed only where the explicit increment misses the
    # gate's bar against the reference: train on those cells, plus a tenth
    # of the others so that the inputs stay broad.
    e = dt[:, None] * f0
    atol = np.r_[np.full(NS, s.atol), 0.0][None, :]
    miss = np.abs(y0 + e - y1) / (atol + s.rtol * np.maximum(np.abs(y0), np.abs(y1)))
    keep = (miss.max(axis=1) > 0.5) | (np.random.default_rng(seed).random(len(rho)) < 0.1)
    rho, dt, y0, y1, f0, e = rho[keep], dt[keep], y0[keep], y1[keep], f0[keep], e[keep]
    raw = raw_features(rho, dt, y0, s.W_kg)
    mu = raw.mean(axis=0)
    sig = raw.std(axis=0) + 1e-6
    m.mu.zero_()
    m.isig.zero_()
    m.mu[:NIN] = torch.tensor(mu, dtype=torch.float32)
    m.isig[:NIN] = torch.tensor(1.0 / sig, dtype=torch.float32)
    rho_d = torch.tensor(rho, device=dev)
    dt_d = torch.tensor(dt, device=dev)
    y0_d = torch.tensor(y0, device=dev)
    unit = np.abs(e) + np.where(np.arange(NS + 1) == NS, TFLOOR, YFLOOR)[None, :]
    c = np.clip((y1 - y0 - e) / unit, -CLIP, CLIP)
    cols = np.concatenate([c[:, NS:], c[:, :NS]], axis=1)  # output column 0 = T, k + 1 = Y_k
    omu = cols.mean(axis=0)
    osig = cols.std(axis=0) + 1e-3
    m.omu.zero_()
    m.osig.fill_(1.0)
    m.omu[:NOUT] = torch.tensor(omu, dtype=torch.float32)
    m.osig[:NOUT] = torch.tensor(osig, dtype=torch.float32)
    tgt = torch.zeros(len(rho), KOUT, device=dev)
    tgt[:, :NOUT] = torch.tensor((cols - omu) / osig, dtype=torch.float32)
    X = s.features(rho_d, dt_d, y0_d)[: len(rho)]
    n = len(rho)
    gen = torch.Generator(device=dev).manual_seed(seed)
    hist = []
    for it in range(iters):
        lr_t = lr * 0.5 * (1 + np.cos(np.pi * it / iters))
        sel = torch.randint(0, n, (batch,), device=dev, generator=gen)
        xb = X.index_select(0, sel)
        tb = tgt.index_select(0, sel)
        m.forward(xb, train=True)
        loss = m.loss_grad(tb)
        m.backward(batch)
        m.adam(lr_t)
        if log_every and (it % log_every == 0 or it == iters - 1):
            hist.append((it, float(loss.item())))
    status()
    return hist


def _main():
    """Times the MLP's forward pass (four tensor-core GEMMs with fused
    epilogues; the bulk-copy path on tiled operands and the thread-copy path
    on row-major ones) on a batch of random standardised inputs (rows a
    multiple of 128); prints one JSON line with the dense BF16 rates."""
    import argparse
    import json

    ap = argparse.ArgumentParser(description=_main.__doc__)
    ap.add_argument("--rows", type=int, default=1 << 20)
    ap.add_argument("--reps", type=int, default=10)
    ap.add_argument("--path", choices=["both", "tiled", "copy"], default="both")
    a = ap.parse_args()
    m = MLP(seed=0)
    X = torch.randn(a.rows, KIN, device="cuda").to(torch.bfloat16)
    flops = 2.0 * a.rows * (KIN * HID + (DEPTH - 1) * HID * HID + HID * KOUT)
    res = {"rows": a.rows, "flops_per_row": flops / a.rows}
    paths = {"tiled": m.forward_tiled, "copy": m.forward}
    for name in (["tiled", "copy"] if a.path == "both" else [a.path]):
        fn = paths[name]
        for _ in range(3):
            fn(X)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(a.reps):
            fn(X)
        e1.record()
        e1.synchronize()
        status()
        ms = e0.elapsed_time(e1) / a.reps
        res[name] = {"forward_ms": ms, "tflops": flops / ms / 1e9}
    print(json.dumps(res))


if __name__ == "__main__":
    _main()
