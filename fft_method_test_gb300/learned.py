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


# ---------------------------------------------------------------------------
# the 4-level U-Net (16 -> 128 channels)
# ---------------------------------------------------------------------------

# (name, cin, cout, level, relu): encoder convolutions with ReLU and 2x average
# pooling between levels, a second convolution at the coarsest level, decoder
# convolutions (no activation) whose outputs are up-sampled 2x, added to the
# encoder output of the finer level and passed through ReLU, and the head.
UNET = [("enc0", CH, 16, 0, True), ("enc1", 16, 32, 1, True), ("enc2", 32, 64, 2, True),
        ("enc3", 64, 128, 3, True), ("bott", 128, 128, 3, True), ("dec3", 128, 64, 3, False),
        ("dec2", 64, 32, 2, False), ("dec1", 32, 16, 1, False), ("head", 16, CH, 0, False)]

# channel pairs (cout rounded to 16, cin) the tensor-core weight gradient covers
_WGRAD_TC = {(16, 16), (16, 32), (32, 16), (32, 32), (64, 32), (32, 64), (64, 64)}


class UNetWarmStart:
    """The warm-start network of four resolution levels (16 -> 128 channels).

    Every convolution runs on the tcgen05 tensor-core kernel (fp_nn_conv_tc:
    forward and data gradient); weight gradients use the mma.sync kernel where
    it covers the channel counts and the CUDA-core kernel otherwise; pooling,
    up-sampling and the skip additions are their own kernels.  Grids must be
    divisible by 8 along each axis."""

    def __init__(self, seed: int = 0):
        torch = _torch()
        self.lib = _capi.load()
        self.stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        rng = np.random.default_rng(seed)
        self.params = {}
        for name, cin, cout, _, relu in UNET:
            fan_in = 27 * cin
            w = rng.standard_normal((27, cout, cin)) * np.sqrt(2.0 / fan_in)
            if name == "head":
                w *= 0.1
            w32 = torch.tensor(w.ravel(), dtype=torch.float32, device="cuda")
            b32 = torch.zeros(cout, dtype=torch.float32, device="cuda")
            self.params[name] = dict(
                w=w32, b=b32, mw=torch.zeros_like(w32), vw=torch.zeros_like(w32),
                mb=torch.zeros_like(b32), vb=torch.zeros_like(b32),
                wf=torch.empty(27 * cout * cin, dtype=torch.bfloat16, device="cuda"),
                wt=torch.empty(27 * cout * cin, dtype=torch.bfloat16, device="cuda"),
                gw=torch.zeros_like(w32), gb=torch.zeros_like(b32), cin=cin, cout=cout)
        self.step_count = 0
        self._refresh_bf16()

    def _refresh_bf16(self):
        for p in self.params.values():
            zeros = p["gw"].zero_()
            _ok(self.lib.fp_nn_adam(_ptr(p["w"]), _ptr(p["mw"]), _ptr(p["vw"]), _ptr(zeros),
                                    p["w"].numel(), 0.0, 0.9, 0.999, 1e-8, 1.0, 1.0, p["cout"],
                                    p["cin"], _ptr(p["wf"]), _ptr(p["wt"]), self.stream), "adam")

    def state(self) -> dict:
        out = {}
        for k, p in self.params.items():
            out[k + "_w"] = p["w"].cpu().numpy()
            out[k + "_b"] = p["b"].cpu().numpy()
        return out

    def load_state(self, st: dict):
        torch = _torch()
        for k, p in self.params.items():
            p["w"].copy_(torch.tensor(np.asarray(st[k + "_w"]), dtype=torch.float32))
            p["b"].copy_(torch.tensor(np.asarray(st[k + "_b"]), dtype=torch.float32))
        self._refresh_bf16()

    # -- building blocks ----------------------------------------------------
    def _conv(self, name, x, shape, total, out32=False, relu=None, sign=1):
        torch = _torch()
        p = self.params[name]
        nz, ny, nx = shape
        cin, cout = (p["cin"], p["cout"]) if sign > 0 else (p["cout"], p["cin"])
        w = p["wf"] if sign > 0 else p["wt"]
        relu_on = (UNET_RELU[name] if relu is None else relu) and sign > 0
        if out32:
            y = torch.empty((total, cout), dtype=torch.float32, device="cuda")
            o32, o16 = _ptr(y), None
        else:
            y = torch.empty((total, cout), dtype=torch.bfloat16, device="cuda")
            o32, o16 = None, _ptr(y)
        bias = _ptr(p["b"]) if sign > 0 else None
        _ok(self.lib.fp_nn_conv_tc(nx, ny, nz, total, 1, sign, _ptr(x), cin, _ptr(w), bias, cout,
                                   int(relu_on), o32, o16, self.stream), "conv_tc " + name)
        return y

    def _pool(self, x, shape, samples, c):
        torch = _torch()
        nz, ny, nx = shape
        y = torch.empty((x.shape[0] // 8, c), dtype=torch.bfloat16, device="cuda")
        _ok(self.lib.fp_nn_pool2(nx, ny, nz, samples, c, _ptr(x), _ptr(y), self.stream), "pool2")
        return y

    def _up_add(self, coarse, skip, shape, samples, c):
        torch = _torch()
        nz, ny, nx = shape
        y = torch.empty_like(skip)
        _ok(self.lib.fp_nn_up2_add(nx, ny, nz, samples, c, _ptr(coarse), _ptr(skip), 1, _ptr(y),
                                   self.stream), "up2_add")
        return y

    # -- forward / backward -------------------------------------------------
    def forward(self, feat, shape, samples: int, keep: bool = False):
        """feat: BF16 [samples*n, 16].  Returns the FP32 output [samples*n, 16]
        and, with keep, the saved activations for the backward pass."""
        s = [tuple(d >> l for d in shape) for l in range(4)]
        t = [int(np.prod(s[l])) * samples for l in range(4)]
        a = {"feat": feat}
        a["e0"] = self._conv("enc0", feat, s[0], t[0])
        a["p0"] = self._pool(a["e0"], s[0], samples, 16)
        a["e1"] = self._conv("enc1", a["p0"], s[1], t[1])
        a["p1"] = self._pool(a["e1"], s[1], samples, 32)
        a["e2"] = self._conv("enc2", a["p1"], s[2], t[2])
        a["p2"] = self._pool(a["e2"], s[2], samples, 64)
        a["e3"] = self._conv("enc3", a["p2"], s[3], t[3])
        a["b3"] = self._conv("bott", a["e3"], s[3], t[3])
        c3 = self._conv("dec3", a["b3"], s[3], t[3])
        a["u2"] = self._up_add(c3, a["e2"], s[2], samples, 64)
        c2 = self._conv("dec2", a["u2"], s[2], t[2])
        a["u1"] = self._up_add(c2, a["e1"], s[1], samples, 32)
        c1 = self._conv("dec1", a["u1"], s[1], t[1])
        a["u0"] = self._up_add(c1, a["e0"], s[0], samples, 16)
        out = self._conv("head", a["u0"], s[0], t[0], out32=True)
        return out, (dict(acts=a, s=s, t=t, samples=samples) if keep else None)

    def _to_bf16(self, d, post=None):
        """BF16 copy of an FP32 gradient, masked where post <= 0 (ReLU)."""
        torch = _torch()
        total, c = d.shape
        y = torch.empty((total, c), dtype=torch.bfloat16, device="cuda")
        _ok(self.lib.fp_nn_relu_back(_ptr(d), _ptr(post) if post is not None else None, total, c, c,
                                     _ptr(y), self.stream), "relu_back")
        return y

    def _grads(self, name, dy, x, shape, total):
        """Weight and bias gradients of one convolution from its BF16 output
        gradient dy and its BF16 input x."""
        torch = _torch()
        p = self.params[name]
        nz, ny, nx = shape
        cin, cout = p["cin"], p["cout"]
        chunk = 4096
        nchunks = (total + chunk - 1) // chunk
        if (cout, cin) in _WGRAD_TC:
            partial = torch.empty(nchunks * 27 * cout * cin, dtype=torch.float32, device="cuda")
            _ok(self.lib.fp_nn_wgrad(nx, ny, nz, total, 1, _ptr(dy), cout, _ptr(x), cin, chunk,
                                     _ptr(partial), _ptr(p["gw"]), self.stream), "wgrad " + name)
        else:
            chunk = 1024
            nchunks = (total + chunk - 1) // chunk
            partial = torch.empty(nchunks * 27 * cout * cin, dtype=torch.float32, device="cuda")
            _ok(self.lib.fp_nn_wgrad_cc(nx, ny, nz, total, 1, _ptr(dy), cout, _ptr(x), cin, chunk,
                                        _ptr(partial), _ptr(p["gw"]), self.stream), "wgrad_cc " + name)
        _ok(self.lib.fp_nn_bias_grad(_ptr(dy), total, cout, _ptr(p["gb"]), self.stream), "bgrad")

    def _up_back(self, d, post, shape, samples, c):
        torch = _torch()
        nz, ny, nx = shape
        dskip = torch.empty_like(d)
        dcoarse = torch.empty((d.shape[0] // 8, c), dtype=torch.float32, device="cuda")
        _ok(self.lib.fp_nn_up2_add_back(nx, ny, nz, samples, c, _ptr(d), _ptr(post), _ptr(dskip),
                                        _ptr(dcoarse), self.stream), "up2_add_back")
        return dskip, dcoarse

    def _pool_back(self, dcoarse, dfine, shape, samples, c):
        nz, ny, nx = shape
        _ok(self.lib.fp_nn_pool2_back(nx, ny, nz, samples, c, _ptr(dcoarse), _ptr(dfine),
                                      self.stream), "pool2_back")

    def backward(self, dout, saved):
        """dout: FP32 [total, 16] gradient of the loss; fills gw, gb."""
        a, s, t, B = saved["acts"], saved["s"], saved["t"], saved["samples"]
        dy = self._to_bf16(dout)
        self._grads("head", dy, a["u0"], s[0], t[0])
        d_u0 = self._conv("head", dy, s[0], t[0], out32=True, sign=-1)
        d_e0, d_c1 = self._up_back(d_u0, a["u0"], s[0], B, 16)
        dy = self._to_bf16(d_c1)
        self._grads("dec1", dy, a["u1"], s[1], t[1])
        d_u1 = self._conv("dec1", dy, s[1], t[1], out32=True, sign=-1)
        d_e1, d_c2 = self._up_back(d_u1, a["u1"], s[1], B, 32)
        dy = self._to_bf16(d_c2)
        self._grads("dec2", dy, a["u2"], s[2], t[2])
        d_u2 = self._conv("dec2", dy, s[2], t[2], out32=True, sign=-1)
        d_e2, d_c3 = self._up_back(d_u2, a["u2"], s[2], B, 64)
        dy = self._to_bf16(d_c3)
        self._grads("dec3", dy, a["b3"], s[3], t[3])
        d_b3 = self._conv("dec3", dy, s[3], t[3], out32=True, sign=-1)
        dy = self._to_bf16(d_b3, a["b3"])
        self._grads("bott", dy, a["e3"], s[3], t[3])
        d_e3 = self._conv("bott", dy, s[3], t[3], out32=True, sign=-1)
        dy = self._to_bf16(d_e3, a["e3"])
        self._grads("enc3", dy, a["p2"], s[3], t[3])
        d_p2 = self._conv("enc3", dy, s[3], t[3], out32=True, sign=-1)
        self._pool_back(d_p2, d_e2, s[2], B, 64)
        dy = self._to_bf16(d_e2, a["e2"])
        self._grads("enc2", dy, a["p1"], s[2], t[2])
        d_p1 = self._conv("enc2", dy, s[2], t[2], out32=True, sign=-1)
        self._pool_back(d_p1, d_e1, s[1], B, 32)
        dy = self._to_bf16(d_e1, a["e1"])
        self._grads("enc1", dy, a["p0"], s[1], t[1])
        d_p0 = self._conv("enc1", dy, s[1], t[1], out32=True, sign=-1)
        self._pool_back(d_p0, d_e0, s[0], B, 16)
        dy = self._to_bf16(d_e0, a["e0"])
        self._grads("enc0", dy, a["feat"], s[0], t[0])

    def adam_step(self, lr: float, b1: float = 0.9, b2: float = 0.999, eps: float = 1e-8):
        self.step_count += 1
        c1 = 1.0 - b1 ** self.step_count
        c2 = 1.0 - b2 ** self.step_count
        for p in self.params.values():
            _ok(self.lib.fp_nn_adam(_ptr(p["w"]), _ptr(p["mw"]), _ptr(p["vw"]), _ptr(p["gw"]),
                                    p["w"].numel(), lr, b1, b2, eps, c1, c2, p["cout"], p["cin"],
                                    _ptr(p["wf"]), _ptr(p["wt"]), self.stream), "adam")
            _ok(self.lib.fp_nn_adam(_ptr(p["b"]), _ptr(p["mb"]), _ptr(p["vb"]), _ptr(p["gb"]),
                                    p["b"].numel(), lr, b1, b2, eps, c1, c2, 0, 0, None, None,
                                    self.stream), "adam")


UNET_RELU = {name: relu for name, _, _, _, relu in UNET}


# ---------------------------------------------------------------------------
# U-Net data, training and use
# ---------------------------------------------------------------------------

@dataclass
class Pair:
    """A training pair kept on the device: fluid mask (u8 [n]), support
    indicator (u8 [n]), target forces (FP32 [n, 3], zero off the support,
    mean-free on it) and the target's squared norm."""
    mask: object
    sup: object
    target: object
    tnorm: float


def features_gpu(mask_u8, sup_u8):
    """BF16 [n, 16] input: channel 0 solid, channel 1 support."""
    torch = _torch()
    f = torch.zeros((mask_u8.numel(), CH), dtype=torch.bfloat16, device="cuda")
    f[:, 0] = (mask_u8 == 0).to(torch.bfloat16)
    f[:, 1] = sup_u8.to(torch.bfloat16)
    return f


def c5_geometry(n: int, seed: int) -> np.ndarray:
    """A training geometry: even seeds overlapping spheres of radius
    uniform in [3, 10], odd seeds Gaussian random fields of correlation length
    uniform in [4, 8]; porosity uniform in [0.3, 0.8]."""
    rng = np.random.default_rng(seed)
    phi = float(rng.uniform(0.3, 0.8))
    if seed % 2 == 0:
        return G.spheres(n, 3.0, phi, seed=seed, radius_max=10.0)
    return G.gaussian_field(n, float(rng.uniform(4.0, 8.0)), phi, seed=seed)


def make_pairs(count: int, n: int = 64, seed: int = 10000, tol: float = 1e-6,
               precision: str = "mixed") -> list:
    """Training pairs from the solver itself: geometry -> converged interface
    forces for a unit pressure gradient along x."""
    from .permeability import PermeabilityProblem

    torch = _torch()
    out = []
    with PermeabilityProblem((n, n, n), precision=precision) as p:
        for i in range(count):
            m = c5_geometry(n, seed + i)
            p.set_geometry(m)
            sup = p.support()
            _, st, x = p.solve_load_case((1.0, 0.0, 0.0), tol, 20000, want_solution=True)
            t = np.zeros((m.size, 3), dtype=np.float32)
            t[sup] = x.reshape(-1, 3)
            s = np.zeros(m.size, dtype=np.uint8)
            s[sup] = 1
            out.append(Pair(mask=torch.tensor(m.ravel(), device="cuda"),
                            sup=torch.tensor(s, device="cuda"),
                            target=torch.tensor(t, device="cuda"),
                            tnorm=float(np.sum(x.astype(np.float64) ** 2))))
    return out


def _pair_batch(pairs):
    torch = _torch()
    feat = torch.cat([features_gpu(q.mask, q.sup) for q in pairs])
    tgt = torch.cat([q.target for q in pairs])
    sup = torch.cat([q.sup for q in pairs])
    tn = torch.tensor([q.tnorm for q in pairs], dtype=torch.float32, device="cuda")
    return feat, tgt, sup, tn


def train_unet(net: UNetWarmStart, pairs: list, n: int, epochs: int = 8, batch: int = 4,
               lr: float = 1e-3, seed: int = 0) -> list:
    """Adam over mini-batches with a cosine learning-rate schedule; returns the
    mean loss (relative squared error on the support) per epoch."""
    rng = np.random.default_rng(seed)
    shape = (n, n, n)
    hist = []
    for ep in range(epochs):
        order = rng.permutation(len(pairs))
        tot = 0.0
        for b0 in range(0, len(order), batch):
            idx = order[b0:b0 + batch]
            feat, tgt, sup, tn = _pair_batch([pairs[i] for i in idx])
            out, saved = net.forward(feat, shape, len(idx), keep=True)
            loss, dout = loss_and_grad(net, out, tgt, sup, tn, n ** 3, len(idx))
            net.backward(dout, saved)
            net.adam_step(lr * 0.5 * (1 + np.cos(np.pi * ep / max(1, epochs))))
            tot += float(loss.sum().item())
        hist.append(tot / len(pairs))
    return hist


def evaluate_unet(net: UNetWarmStart, pairs: list, n: int) -> float:
    tot = 0.0
    for q in pairs:
        feat, tgt, sup, tn = _pair_batch([q])
        out, _ = net.forward(feat, (n, n, n), 1)
        loss, _ = loss_and_grad(net, out, tgt, sup, tn, n ** 3, 1)
        tot += float(loss.sum().item())
    return tot / len(pairs)


def predict_guess_unet(net: UNetWarmStart, mask: np.ndarray, support: np.ndarray,
                       direction: int) -> np.ndarray:
    """Compact initial guess [3 * nb] for a unit pressure gradient along
    `direction`: the geometry is transposed so that the load lies along x,
    the network predicts, and the field is transposed back (the discrete
    operator is invariant under axis permutations)."""
    torch = _torch()
    perm = _PERM[direction]
    m = np.ascontiguousarray(np.transpose(mask, perm))
    sup_mask = np.zeros(mask.size, dtype=np.uint8)
    sup_mask[support] = 1
    sup_r = np.ascontiguousarray(np.transpose(sup_mask.reshape(mask.shape), perm))
    feat = features_gpu(torch.tensor(m.ravel(), device="cuda"), torch.tensor(sup_r.ravel(), device="cuda"))
    out, _ = net.forward(feat, m.shape, 1)
    del feat
    # the support voxels' outputs, gathered on the device: voxel (z, y, x) of
    # the cell sits at the permuted coordinates in the transposed frame
    coords = np.unravel_index(support, mask.shape)
    idx_r = np.ravel_multi_index(tuple(coords[a] for a in perm), m.shape)
    f = out[torch.tensor(idx_r, device="cuda")][:, :3].double().cpu().numpy()
    del out
    # components back to (x, y, z): x of the transposed frame is the load axis
    comp = {0: (0, 1, 2), 1: (1, 0, 2), 2: (2, 1, 0)}[direction]
    g = f[:, list(comp)]
    g -= g.mean(axis=0)
    return g.ravel()
