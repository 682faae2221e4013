"""Learned warm start for MINRES: a small 3-D convolutional network maps a
geometry to the interface-force field the solve starts from.

No counterpart in the reference: its ``MinresSolver::solve`` takes an
``initial_guess`` (src/solver/MinresSolver.hpp:23, used at
src/solver/MinresSolver.cpp:68-70) that its driver never fills.

* Input per voxel: solid indicator and support indicator (channels 0 and 1 of
  16; the tensor cores take input channels in blocks of 16).
* Output per voxel: the three force components for a unit pressure gradient
  along x (channels 0..2 of 16).  Other load directions rotate the geometry
  so that the load lies along x, predict, and rotate the field back: the
  discrete operator is invariant under axis permutations.
* Layers: 3x3x3 convolutions with dilations 1, 2, 4, 8, 1 (receptive field 33
  voxels), ReLU between them, all on the GPU through the ``fp_nn_*`` kernels
  of libfftperm (BF16 tensor cores, FP32 accumulation, Adam on FP32 masters).
* Training pairs come from the plain FP64 solver itself: geometry ->
  converged interface forces for the unit x gradient.
* Loss: relative squared error of the predicted forces on the support after
  per-component mean removal (the operator's null space).
* At solve time the guess is scaled by the factor that minimises the initial
  residual (one operator apply) and kept only if it lowers that residual
  below the zero start's; otherwise MINRES starts from zero, and MINRES
  always judges the final error.

PyTorch provides device memory and the stream handle only; every operation
of the network is a kernel of libfftperm.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _capi
from . import geometry as G

CH = 16  # channel block of the tensor-core kernels


@dataclass
class Layer:
    cin: int
    cout: int
    dil: int
    relu: bool


DEFAULT_LAYERS = [Layer(CH, 32, 1, True), Layer(32, 32, 2, True), Layer(32, 32, 4, True),
                  Layer(32, 32, 8, True), Layer(32, CH, 1, False)]


def _torch():
    import torch

    if not torch.cuda.is_available():
        raise RuntimeError("the learned warm start needs a CUDA device")
    return torch


def _ptr(t) -> C.c_void_p:
    return C.c_void_p(t.data_ptr())


def _ok(rc: int, what: str):
    if rc != _capi.FP_OK:
        raise _capi.FpError(rc, what)


class WarmStartNet:
    """The network, its FP32 master weights, Adam state and BF16 copies."""

    def __init__(self, layers=None, seed: int = 0):
        torch = _torch()
        self.lib = _capi.load()
        self.layers = list(layers or DEFAULT_LAYERS)
        self.stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        rng = np.random.default_rng(seed)
        self.params = []
        for ly in self.layers:
            fan_in = 27 * ly.cin
            w = rng.standard_normal((27, ly.cout, ly.cin)) * np.sqrt(2.0 / fan_in)
            if not ly.relu:
                w *= 0.1
            w32 = torch.tensor(w.ravel(), dtype=torch.float32, device="cuda")
            b32 = torch.zeros(ly.cout, dtype=torch.float32, device="cuda")
            p = dict(w=w32, b=b32, mw=torch.zeros_like(w32), vw=torch.zeros_like(w32),
                     mb=torch.zeros_like(b32), vb=torch.zeros_like(b32),
                     wf=torch.empty(27 * ly.cout * ly.cin, dtype=torch.bfloat16, device="cuda"),
                     wt=torch.empty(27 * ly.cout * ly.cin, dtype=torch.bfloat16, device="cuda"),
                     gw=torch.zeros_like(w32), gb=torch.zeros_like(b32))
            self.params.append(p)
        self.step_count = 0
        self._refresh_bf16()

    # -- weights -----------------------------------------------------------
    def _refresh_bf16(self):
        """BF16 copies from the masters: an Adam step with zero gradient and lr 0."""
        for ly, p in zip(self.layers, self.params):
            zeros = p["gw"].zero_()
            _ok(self.lib.fp_nn_adam(_ptr(p["w"]), _ptr(p["mw"]), _ptr(p["vw"]), _ptr(zeros),
                                    p["w"].numel(), 0.0, 0.9, 0.999, 1e-8, 1.0, 1.0, ly.cout, ly.cin,
                                    _ptr(p["wf"]), _ptr(p["wt"]), self.stream), "adam")

    def state(self) -> dict:
        out = {}
        for i, p in enumerate(self.params):
            out["w%d" % i] = p["w"].cpu().numpy()
            out["b%d" % i] = p["b"].cpu().numpy()
        return out

    def load_state(self, st: dict):
        torch = _torch()
        for i, p in enumerate(self.params):
            p["w"].copy_(torch.tensor(np.asarray(st["w%d" % i]), dtype=torch.float32))
            p["b"].copy_(torch.tensor(np.asarray(st["b%d" % i]), dtype=torch.float32))
        self._refresh_bf16()

    # -- forward / backward -------------------------------------------------
    def forward(self, feat, shape, keep: bool = False):
        """feat: BF16 [samples*n, 16].  Returns the FP32 output [samples*n, 16]
        and, with keep, the BF16 layer inputs for the backward pass."""
        torch = _torch()
        nz, ny, nx = shape
        total = feat.shape[0]
        x = feat
        acts = [x]
        out = None
        for li, (ly, p) in enumerate(zip(self.layers, self.params)):
            last = li == len(self.layers) - 1
            if last:
                out = torch.empty((total, ly.cout), dtype=torch.float32, device="cuda")
                _ok(self.lib.fp_nn_conv(nx, ny, nz, total, ly.dil, 1, _ptr(x), ly.cin, _ptr(p["wf"]),
                                        _ptr(p["b"]), ly.cout, 0, _ptr(out), None, self.stream), "conv")
            else:
                y = torch.empty((total, ly.cout), dtype=torch.bfloat16, device="cuda")
                _ok(self.lib.fp_nn_conv(nx, ny, nz, total, ly.dil, 1, _ptr(x), ly.cin, _ptr(p["wf"]),
                                        _ptr(p["b"]), ly.cout, int(ly.relu), None, _ptr(y),
                                        self.stream), "conv")
                x = y
                if keep:
                    acts.append(x)
        return out, (acts if keep else None)

    def backward(self, dout, acts, shape):
        """dout: FP32 [total, cout_last] gradient of the loss; fills gw, gb."""
        torch = _torch()
        nz, ny, nx = shape
        total = dout.shape[0]
        dy = torch.empty((total, self.layers[-1].cout), dtype=torch.bfloat16, device="cuda")
        _ok(self.lib.fp_nn_relu_back(_ptr(dout), None, total, self.layers[-1].cout,
                                     self.layers[-1].cout, _ptr(dy), self.stream), "relu_back")
        chunk = 4096
        nchunks = (total + chunk - 1) // chunk
        for li in range(len(self.layers) - 1, -1, -1):
            ly, p = self.layers[li], self.params[li]
            x = acts[li]
            co16 = (ly.cout + 15) // 16 * 16
            partial = torch.empty(nchunks * 27 * co16 * ly.cin, dtype=torch.float32, device="cuda")
            _ok(self.lib.fp_nn_wgrad(nx, ny, nz, total, ly.dil, _ptr(dy), ly.cout, _ptr(x), ly.cin,
                                     chunk, _ptr(partial), _ptr(p["gw"]), self.stream), "wgrad")
            _ok(self.lib.fp_nn_bias_grad(_ptr(dy), total, ly.cout, _ptr(p["gb"]), self.stream), "bgrad")
            if li == 0:
                break
            dx = torch.empty((total, ly.cin), dtype=torch.float32, device="cuda")
            _ok(self.lib.fp_nn_conv(nx, ny, nz, total, ly.dil, -1, _ptr(dy), ly.cout, _ptr(p["wt"]),
                                    None, ly.cin, 0, _ptr(dx), None, self.stream), "dgrad")
            prev = self.layers[li - 1]
            dy = torch.empty((total, ly.cin), dtype=torch.bfloat16, device="cuda")
            _ok(self.lib.fp_nn_relu_back(_ptr(dx), _ptr(x) if prev.relu else None, total, ly.cin,
                                         ly.cin, _ptr(dy), self.stream), "relu_back")

    def adam_step(self, lr: float, b1: float = 0.9, b2: float = 0.999, eps: float = 1e-8):
        self.step_count += 1
        c1 = 1.0 - b1 ** self.step_count
        c2 = 1.0 - b2 ** self.step_count
        for ly, p in zip(self.layers, self.params):
            _ok(self.lib.fp_nn_adam(_ptr(p["w"]), _ptr(p["mw"]), _ptr(p["vw"]), _ptr(p["gw"]),
                                    p["w"].numel(), lr, b1, b2, eps, c1, c2, ly.cout, ly.cin,
                                    _ptr(p["wf"]), _ptr(p["wt"]), self.stream), "adam")
            _ok(self.lib.fp_nn_adam(_ptr(p["b"]), _ptr(p["mb"]), _ptr(p["vb"]), _ptr(p["gb"]),
                                    p["b"].numel(), lr, b1, b2, eps, c1, c2, 0, 0, None, None,
                                    self.stream), "adam")


# ---------------------------------------------------------------------------
# data
# ---------------------------------------------------------------------------

def features(mask: np.ndarray, support: np.ndarray):
    """BF16 [n, 16] device tensor: channel 0 solid, channel 1 support."""
    torch = _torch()
    n = mask.size
    f = np.zeros((n, CH), dtype=np.float32)
    f[:, 0] = (np.asarray(mask).ravel() == 0)
    f[support, 1] = 1.0
    return torch.tensor(f, device="cuda").to(torch.bfloat16)


@dataclass
class Sample:
    mask: np.ndarray
    support: np.ndarray      # ascending flat indices
    target: np.ndarray       # [n, 3] forces on the support (mean-free), zero elsewhere
    tnorm: float


def solve_sample(mask: np.ndarray, tol: float = 1e-8, maxit: int = 20000) -> Sample:
    """Training pair from the plain FP64 solver: unit gradient along x."""
    from .permeability import PermeabilityProblem

    with PermeabilityProblem(mask.shape, precision="fp64") as p:
        p.set_geometry(mask)
        sup = p.support()
        _, st, x = p.solve_load_case((1.0, 0.0, 0.0), tol, maxit, want_solution=True)
    t = np.zeros((mask.size, 3), dtype=np.float32)
    t[sup] = x.reshape(-1, 3)
    return Sample(mask=mask, support=sup, target=t, tnorm=float(np.sum(x.astype(np.float64) ** 2)))


def make_training_set(count: int, n: int = 32, seed: int = 10000) -> list:
    """Half overlapping spheres (radius 2-5), half Gaussian fields (correlation
    length 3-6), porosity in [0.3, 0.8]."""
    out = []
    for i in range(count):
        rng = np.random.default_rng(seed + i)
        phi = float(rng.uniform(0.3, 0.8))
        if i % 2 == 0:
            m = G.spheres(n, float(rng.uniform(2.0, 5.0)), phi, seed=seed + i)
        else:
            m = G.gaussian_field(n, float(rng.uniform(3.0, 6.0)), phi, seed=seed + i)
        out.append(solve_sample(m))
    return out


def _batch_tensors(samples):
    torch = _torch()
    feat = torch.cat([features(s.mask, s.support) for s in samples])
    tgt = torch.tensor(np.concatenate([s.target for s in samples]), device="cuda")
    sup = np.zeros(sum(s.mask.size for s in samples), dtype=np.uint8)
    off = 0
    for s in samples:
        sup[off + s.support] = 1
        off += s.mask.size
    supd = torch.tensor(sup, device="cuda")
    tn = torch.tensor([s.tnorm for s in samples], dtype=torch.float32, device="cuda")
    return feat, tgt, supd, tn


def loss_and_grad(net: WarmStartNet, out, tgt, supd, tn, n: int, samples: int):
    torch = _torch()
    dout = torch.empty_like(out)
    stats = torch.empty(4 * samples, dtype=torch.float32, device="cuda")
    loss = torch.empty(samples, dtype=torch.float32, device="cuda")
    _ok(net.lib.fp_nn_loss(_ptr(out), out.shape[1], _ptr(tgt), _ptr(supd), n, samples, _ptr(tn),
                           _ptr(stats), _ptr(dout), _ptr(loss), net.stream), "loss")
    return loss, dout


def train(net: WarmStartNet, data: list, epochs: int = 40, batch: int = 4, lr: float = 2e-3,
          seed: int = 0) -> list:
    """Adam over mini-batches of equal-shape samples; returns the mean loss per epoch."""
    shape = data[0].mask.shape
    n = data[0].mask.size
    rng = np.random.default_rng(seed)
    hist = []
    for ep in range(epochs):
        order = rng.permutation(len(data))
        tot = 0.0
        for b0 in range(0, len(order), batch):
            idx = order[b0:b0 + batch]
            feat, tgt, supd, tn = _batch_tensors([data[i] for i in idx])
            out, acts = net.forward(feat, shape, keep=True)
            loss, dout = loss_and_grad(net, out, tgt, supd, tn, n, len(idx))
            net.backward(dout, acts, shape)
            step_lr = lr * (0.5 * (1 + np.cos(np.pi * ep / max(1, epochs))))
            net.adam_step(step_lr)
            tot += float(loss.sum().item())
        hist.append(tot / len(data))
    return hist


def evaluate(net: WarmStartNet, data: list) -> float:
    """Mean relative squared error of the prediction on the support."""
    shape = data[0].mask.shape
    n = data[0].mask.size
    tot = 0.0
    for s in data:
        feat, tgt, supd, tn = _batch_tensors([s])
        out, _ = net.forward(feat, shape)
        loss, _ = loss_and_grad(net, out, tgt, supd, tn, n, 1)
        tot += float(loss.sum().item())
    return tot / len(data)


# ---------------------------------------------------------------------------
# inference as the MINRES initial guess
# ---------------------------------------------------------------------------

_PERM = {0: (0, 1, 2), 1: (0, 2, 1), 2: (2, 1, 0)}  # array axes (z, y, x) swapped so the load is along x


def predict_guess(net: WarmStartNet, mask: np.ndarray, support: np.ndarray, direction: int) -> np.ndarray:
    """Compact initial guess [3 * nb] (the solver's [3*local + comp] layout)
    for a unit pressure gradient along `direction`."""
    perm = _PERM[direction]
    m = np.ascontiguousarray(np.transpose(mask, perm))
    sup_mask = np.zeros(mask.size, dtype=bool)
    sup_mask[support] = True
    sup_r = np.flatnonzero(np.transpose(sup_mask.reshape(mask.shape), perm))
    out, _ = net.forward(features(m, sup_r), m.shape)
    f = out[:, :3].float().cpu().numpy().reshape(m.shape + (3,))
    # back to the original frame: axes, then components (x is the last array axis)
    f = np.transpose(f, perm + (3,))
    comp = {0: (0, 1, 2), 1: (1, 0, 2), 2: (2, 1, 0)}[direction]
    f = f[..., list(comp)].reshape(-1, 3)
    g = f[support].astype(np.float64)
    g -= g.mean(axis=0)
    return g.ravel()


def solve_load_case_warm(problem, net: WarmStartNet, direction: int, tol: float, maxit: int):
    """fp_solve_load_case from the network's guess, scaled by the factor that
    minimises the initial residual |b - s A x0| (one operator apply); from
    zero when that does not lower the residual below |b|.  Returns
    (avg velocity, stats, used_guess, initial relative residual)."""
    grad = np.zeros(3)
    grad[direction] = 1.0
    sup = problem.support()
    x0 = predict_guess(net, problem.mask, sup, direction)
    b = problem.build_rhs(grad)
    ax = problem.operator_apply(x0)
    den = float(ax @ ax)
    scale = float(b @ ax) / den if den > 0 else 0.0
    x0 *= scale
    rel0 = float(np.linalg.norm(b - scale * ax) / np.linalg.norm(b))
    use = scale > 0 and rel0 < 1.0
    avg, st, _ = problem.solve_load_case(grad, tol, maxit, x0=x0 if use else None)
    return avg, st, use, rel0
