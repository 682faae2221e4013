"""The learned warm start: its tensor-core kernels against the CPU
restatement (oracle/nn_ref.py), a gradient check of the whole network, and
what the trained network gains as the MINRES initial guess.  No reference
counterpart (the reference's MinresSolver::solve takes an initial guess that
nothing fills)."""
import numpy as np
import pytest

from conftest import rel_err
from fft_method_test_gb300 import geometry as G

pytestmark = pytest.mark.gpu


def _t(a, dtype):
    import torch

    return torch.tensor(np.ascontiguousarray(a), dtype=dtype, device="cuda")


def _conv_case(seed, shape=(6, 8, 10), batch=2, cin=16, cout=32, dil=2):
    import nn_ref as R

    rng = np.random.default_rng(seed)
    x = R.bf16(rng.standard_normal((batch,) + shape + (cin,)))
    w = R.bf16(rng.standard_normal((27, cout, cin)) * 0.1)
    b = rng.standard_normal(cout).astype(np.float32).astype(np.float64)
    return x, w, b


def test_conv_forward_matches_cpu(gpu_lib):
    import ctypes as C

    import nn_ref as R
    import torch

    x, w, b = _conv_case(1)
    B, nz, ny, nx, cin = x.shape
    cout = w.shape[1]
    total = B * nz * ny * nx
    xd, wd = _t(x.reshape(total, cin), torch.bfloat16), _t(w.ravel(), torch.bfloat16)
    bd = _t(b, torch.float32)
    out = torch.empty((total, cout), dtype=torch.float32, device="cuda")
    out16 = torch.empty((total, cout), dtype=torch.bfloat16, device="cuda")
    rc = gpu_lib.fp_nn_conv(nx, ny, nz, total, 2, 1, C.c_void_p(xd.data_ptr()), cin,
                            C.c_void_p(wd.data_ptr()), C.c_void_p(bd.data_ptr()), cout, 1,
                            C.c_void_p(out.data_ptr()), C.c_void_p(out16.data_ptr()), None)
    assert rc == 0
    torch.cuda.synchronize()
    ref = R.conv(x, w, 2, bias=b, relu=True).reshape(total, cout)
    assert rel_err(out.cpu().numpy(), ref) < 1e-5
    assert rel_err(out16.float().cpu().numpy(), R.bf16(ref)) < 1e-2


def test_conv_data_and_weight_gradients_match_cpu(gpu_lib):
    import ctypes as C

    import nn_ref as R
    import torch

    x, w, _ = _conv_case(2, cout=16)
    B, nz, ny, nx, cin = x.shape
    cout = w.shape[1]
    total = B * nz * ny * nx
    rng = np.random.default_rng(3)
    dy = R.bf16(rng.standard_normal((B, nz, ny, nx, cout)))
    wt = np.ascontiguousarray(np.transpose(w, (0, 2, 1)))  # [tap][cin][cout]
    dyd = _t(dy.reshape(total, cout), torch.bfloat16)
    wtd = _t(wt.ravel(), torch.bfloat16)
    dx = torch.empty((total, cin), dtype=torch.float32, device="cuda")
    assert gpu_lib.fp_nn_conv(nx, ny, nz, total, 2, -1, C.c_void_p(dyd.data_ptr()), cout,
                              C.c_void_p(wtd.data_ptr()), None, cin, 0, C.c_void_p(dx.data_ptr()),
                              None, None) == 0
    xd = _t(x.reshape(total, cin), torch.bfloat16)
    chunk = 64
    nch = (total + chunk - 1) // chunk
    partial = torch.empty(nch * 27 * 16 * cin, dtype=torch.float32, device="cuda")
    dw = torch.empty(27 * cout * cin, dtype=torch.float32, device="cuda")
    assert gpu_lib.fp_nn_wgrad(nx, ny, nz, total, 2, C.c_void_p(dyd.data_ptr()), cout,
                               C.c_void_p(xd.data_ptr()), cin, chunk, C.c_void_p(partial.data_ptr()),
                               C.c_void_p(dw.data_ptr()), None) == 0
    db = torch.empty(cout, dtype=torch.float32, device="cuda")
    assert gpu_lib.fp_nn_bias_grad(C.c_void_p(dyd.data_ptr()), total, cout,
                                   C.c_void_p(db.data_ptr()), None) == 0
    torch.cuda.synchronize()
    assert rel_err(dx.cpu().numpy(), R.conv_data_grad(dy, w, 2).reshape(total, cin)) < 1e-5
    assert rel_err(dw.cpu().numpy(), R.conv_weight_grad(dy, x, 2).ravel()) < 1e-5
    assert rel_err(db.cpu().numpy(), dy.reshape(total, cout).sum(axis=0)) < 1e-5
    # the data gradient is the adjoint of the forward convolution
    y = R.conv(x, w, 2)
    assert abs(np.sum(y * dy) - np.sum(x * R.conv_data_grad(dy, w, 2))) < 1e-9 * np.abs(y * dy).sum()


def test_network_gradient_matches_cpu(gpu_lib):
    """Whole-network gradient (three layers, ReLU, dilations, loss on the
    support) against the CPU restatement with the same BF16 rounding."""
    import nn_ref as R
    import torch

    from fft_method_test_gb300 import learned as L

    shape = (8, 8, 8)
    layers = [L.Layer(16, 16, 1, True), L.Layer(16, 16, 2, True), L.Layer(16, 16, 1, False)]
    net = L.WarmStartNet(layers, seed=4)
    rng = np.random.default_rng(5)
    masks = [G.spheres(8, 1.5, 0.6, seed=s) for s in (1, 2)]
    sups = []
    for m in masks:
        solid = m == 0
        nb = np.zeros_like(solid)
        for ax in range(3):
            for sh in (1, -1):
                nb |= np.roll(m == 1, sh, ax)
        sups.append(np.flatnonzero(solid & nb))
    feat = torch.cat([L.features(m, s) for m, s in zip(masks, sups)])
    tgt = np.zeros((2, 512, 3))
    supb = np.zeros((2, 512), dtype=bool)
    for b, s in enumerate(sups):
        t = rng.standard_normal((len(s), 3))
        tgt[b, s] = t - t.mean(axis=0)
        supb[b, s] = True
    tn = np.array([np.sum(tgt[b] ** 2) for b in range(2)])
    out, acts = net.forward(feat, shape, keep=True)
    loss, dout = L.loss_and_grad(net, out, _t(tgt.reshape(-1, 3), torch.float32),
                                 _t(supb.ravel().astype(np.uint8), torch.uint8),
                                 _t(tn, torch.float32), 512, 2)
    net.backward(dout, acts, shape)
    torch.cuda.synchronize()
    # CPU: the same network with BF16 rounding at the kernels' points
    ws = [R.bf16(p["w"].cpu().numpy().reshape(27, ly.cout, ly.cin)) for ly, p in zip(layers, net.params)]
    bs = [p["b"].cpu().numpy().astype(np.float64) for p in net.params]
    x0 = feat.float().cpu().numpy().reshape((2,) + shape + (16,))
    xs = [x0]
    h = x0
    for i, ly in enumerate(layers[:-1]):
        h = R.bf16(R.conv(h, ws[i], ly.dil, bias=bs[i], relu=True))
        xs.append(h)
    y = R.conv(h, ws[-1], layers[-1].dil, bias=bs[-1])
    lref, dref = R.loss_grad(y.reshape(2, 512, 16), tgt, supb)
    assert rel_err(loss.cpu().numpy(), lref) < 1e-4
    dy = R.bf16(dref.reshape((2,) + shape + (16,)))
    for i in range(len(layers) - 1, -1, -1):
        gw = R.conv_weight_grad(dy, xs[i], layers[i].dil)
        assert rel_err(net.params[i]["gw"].cpu().numpy(), gw.ravel()) < 1e-3, i
        assert rel_err(net.params[i]["gb"].cpu().numpy(), dy.reshape(-1, 16).sum(axis=0)) < 1e-3, i
        if i == 0:
            break
        dx = R.conv_data_grad(dy, ws[i], layers[i].dil)
        dy = R.bf16(dx * (xs[i] > 0))


def test_training_lowers_the_loss(gpu_lib):
    from fft_method_test_gb300 import learned as L

    data = L.make_training_set(8, n=16, seed=300)
    net = L.WarmStartNet(seed=1)
    before = L.evaluate(net, data)
    hist = L.train(net, data, epochs=15, batch=4, lr=2e-3)
    after = L.evaluate(net, data)
    assert after < 0.7 * before, (before, after, hist)


def test_trained_network_lowers_the_initial_residual(gpu_lib):
    """What training buys: on held-out cells the trained network's (scaled)
    guess starts MINRES at a lower residual than an untrained network's, and
    the solve from it reaches the same velocity."""
    from fft_method_test_gb300 import learned as L
    from fft_method_test_gb300.permeability import PermeabilityProblem

    data = L.make_training_set(48, n=24, seed=400)
    trained = L.WarmStartNet(seed=2)
    L.train(trained, data, epochs=30, batch=8, lr=2e-3)
    untrained = L.WarmStartNet(seed=2)
    rel_t, rel_u = [], []
    for seed in (501, 502, 503):
        m = G.gaussian_field(24, 4.0, 0.5, seed=seed)
        with PermeabilityProblem(m.shape, precision="fp64") as p:
            p.set_geometry(m)
            a0, s0, _ = p.solve_load_case((1.0, 0.0, 0.0), 1e-9, 5000)
            a1, s1, used, r1 = L.solve_load_case_warm(p, trained, 0, 1e-9, 5000)
            _, _, _, r2 = L.solve_load_case_warm(p, untrained, 0, 1e-9, 5000)
        assert s1["converged"] and rel_err(a1, a0) < 1e-7
        rel_t.append(r1)
        rel_u.append(r2)
    assert np.mean(rel_t) < np.mean(rel_u) - 0.05, (rel_t, rel_u)
    assert max(rel_t) < 1.0


# ---------------------------------------------------------------------------
# the tcgen05 convolution and the U-Net
# ---------------------------------------------------------------------------

def _conv_ref_torch(x, w, shape, dil, sign, bias, relu):
    """Periodic 3x3x3 convolution in float64 (torch): y[v][o] = sum_tap
    sum_i x[v + sign*dil*off(tap)][i] w[tap][o][i]."""
    import torch

    nz, ny, nx = shape
    cin, cout = x.shape[1], w.shape[1]
    S = x.shape[0] // (nx * ny * nz)
    x5 = x.reshape(S, nz, ny, nx, cin).double()
    out = torch.zeros(S, nz, ny, nx, cout, dtype=torch.float64)
    s = sign * dil
    for tap in range(27):
        dz, dy, dx = tap // 9 - 1, (tap // 3) % 3 - 1, tap % 3 - 1
        out += torch.roll(x5, shifts=(-s * dz, -s * dy, -s * dx), dims=(1, 2, 3)) @ w[tap].double().T
    out = out.reshape(-1, cout)
    if bias is not None:
        out += bias.double()
    return torch.clamp(out, min=0) if relu else out


@pytest.mark.parametrize("cin,cout", [(16, 16), (16, 32), (32, 64), (64, 128), (128, 128), (128, 64),
                                      (32, 16)])
@pytest.mark.parametrize("shape,samples,dil,sign", [((8, 8, 8), 2, 1, 1), ((7, 5, 6), 1, 2, -1)])
def test_conv_tcgen05_matches_reference(gpu_lib, cin, cout, shape, samples, dil, sign):
    """fp_nn_conv_tc (tcgen05.mma, TMEM accumulator) against a float64 torch
    convolution of the same BF16 inputs: FP32 output to 1e-5, BF16 output to
    BF16 rounding; the error flag of the bounded waits stays clear."""
    import ctypes as C

    import torch

    torch.manual_seed(cin * 7 + cout)
    n = int(np.prod(shape))
    x = torch.randn(samples * n, cin, device="cuda").to(torch.bfloat16)
    w = (torch.randn(27, cout, cin, device="cuda") * 0.1).to(torch.bfloat16)
    b = torch.randn(cout, device="cuda")
    o32 = torch.full((samples * n, cout), float("nan"), device="cuda")
    o16 = torch.empty((samples * n, cout), dtype=torch.bfloat16, device="cuda")
    rc = gpu_lib.fp_nn_conv_tc(shape[2], shape[1], shape[0], samples * n, dil, sign,
                               C.c_void_p(x.data_ptr()), cin, C.c_void_p(w.data_ptr()),
                               C.c_void_p(b.data_ptr()), cout, 1, C.c_void_p(o32.data_ptr()),
                               C.c_void_p(o16.data_ptr()), None)
    assert rc == 0
    torch.cuda.synchronize()
    flag = C.c_int(1)
    assert gpu_lib.fp_nn_tc_error(C.byref(flag), 1) == 0 and flag.value == 0
    want = _conv_ref_torch(x.float().cpu(), w.float().cpu(), shape, dil, sign, b.cpu(), True)
    scale = float(want.abs().max())
    assert float((o32.double().cpu() - want).abs().max()) < 1e-5 * scale
    assert float((o16.double().cpu() - want).abs().max()) < 1e-2 * scale


def _unet_ref_loss(params, feat, shape, tgt, sup, tn):
    """The U-Net in float32 torch (autograd), with the BF16 roundings of the
    GPU path at the same places; returns the summed relative squared error of
    the mean-free prediction on the support (the fp_nn_loss definition)."""
    import torch
    import torch.nn.functional as F

    def r16(t):
        return t.to(torch.bfloat16).float()

    class GradToBf16(torch.autograd.Function):
        """Identity whose backward rounds the gradient to BF16, as the GPU
        path does with the gradient of every convolution output."""

        @staticmethod
        def forward(ctx, t):
            return t.view_as(t)

        @staticmethod
        def backward(ctx, g):
            return g.to(torch.bfloat16).float()

    def conv(name, x, s, relu):
        w, b = params[name]
        nz, ny, nx = s
        cout, cin = w.shape[1], w.shape[2]
        S = x.shape[0] // (nz * ny * nx)
        x5 = x.reshape(S, nz, ny, nx, cin).permute(0, 4, 1, 2, 3)
        x5 = F.pad(x5, (1, 1, 1, 1, 1, 1), mode="circular")
        k = w.reshape(3, 3, 3, cout, cin).permute(3, 4, 0, 1, 2)
        y = F.conv3d(x5, k) + b.view(1, -1, 1, 1, 1)
        y = GradToBf16.apply(y.permute(0, 2, 3, 4, 1).reshape(-1, cout))
        return torch.relu(y) if relu else y

    def pool(x, s, c):
        nz, ny, nx = s
        S = x.shape[0] // (nz * ny * nx)
        x5 = x.reshape(S, nz, ny, nx, c).permute(0, 4, 1, 2, 3)
        return F.avg_pool3d(x5, 2).permute(0, 2, 3, 4, 1).reshape(-1, c)

    def up_add(cz, skip, s, c):
        nz, ny, nx = s
        S = skip.shape[0] // (nz * ny * nx)
        c5 = cz.reshape(S, nz // 2, ny // 2, nx // 2, c)
        c5 = c5.repeat_interleave(2, 1).repeat_interleave(2, 2).repeat_interleave(2, 3)
        return torch.relu(c5.reshape(-1, c) + skip)

    s = [tuple(d >> l for d in shape) for l in range(4)]
    e0 = r16(conv("enc0", feat, s[0], True))
    p0 = r16(pool(e0, s[0], 16))
    e1 = r16(conv("enc1", p0, s[1], True))
    p1 = r16(pool(e1, s[1], 32))
    e2 = r16(conv("enc2", p1, s[2], True))
    p2 = r16(pool(e2, s[2], 64))
    e3 = r16(conv("enc3", p2, s[3], True))
    b3 = r16(conv("bott", e3, s[3], True))
    c3 = r16(conv("dec3", b3, s[3], False))
    u2 = r16(up_add(c3, e2, s[2], 64))
    c2 = r16(conv("dec2", u2, s[2], False))
    u1 = r16(up_add(c2, e1, s[1], 32))
    c1 = r16(conv("dec1", u1, s[1], False))
    u0 = r16(up_add(c1, e0, s[0], 16))
    out = conv("head", u0, s[0], False)
    n = int(np.prod(shape))
    S = out.shape[0] // n
    loss = 0.0
    for k in range(S):
        o = out[k * n:(k + 1) * n, :3]
        m = sup[k * n:(k + 1) * n].bool()
        om = o[m] - o[m].mean(dim=0)
        loss = loss + ((om - tgt[k * n:(k + 1) * n][m]) ** 2).sum() / tn[k]
    return loss


def test_unet_gradients_match_torch_autograd(gpu_lib):
    """The U-Net's forward and backward passes (tcgen05 convolutions and data
    gradients, weight gradients, pooling, up-sampling with skips) against
    torch autograd of the same network in FP32 with the GPU path's BF16
    roundings of activations and of the convolution output gradients: loss to
    1e-2 and every weight gradient to 8e-2 in the relative 2-norm."""
    import torch

    from fft_method_test_gb300 import learned as L

    shape, samples = (16, 16, 16), 2
    n = int(np.prod(shape))
    net = L.UNetWarmStart(seed=3)
    rng = np.random.default_rng(4)
    masks = [G.spheres(16, 3.0, 0.6, seed=40 + k) for k in range(samples)]
    sup = torch.zeros(samples * n, dtype=torch.uint8, device="cuda")
    tgt = torch.zeros(samples * n, 3, device="cuda")
    for k, m in enumerate(masks):
        solid = np.flatnonzero(m.ravel() == 0)
        sup[k * n + torch.tensor(solid, device="cuda")] = 1
        t = rng.standard_normal((len(solid), 3)).astype(np.float32)
        t -= t.mean(axis=0)
        tgt[k * n + torch.tensor(solid, device="cuda")] = torch.tensor(t, device="cuda")
    tn = torch.stack([(tgt[k * n:(k + 1) * n] ** 2).sum() for k in range(samples)]).float()
    mask_t = torch.tensor(np.concatenate([m.ravel() for m in masks]), device="cuda")
    feat = L.features_gpu(mask_t, sup)
    out, saved = net.forward(feat, shape, samples, keep=True)
    loss, dout = L.loss_and_grad(net, out, tgt, sup, tn, n, samples)
    net.backward(dout, saved)
    torch.cuda.synchronize()
    params = {}
    for name, p in net.params.items():
        w = p["wf"].float().reshape(27, p["cout"], p["cin"]).clone().requires_grad_(True)
        b = p["b"].clone().requires_grad_(True)
        params[name] = (w, b)
    ref = _unet_ref_loss(params, feat.float(), shape, tgt, sup, tn)
    ref.backward()
    assert abs(float(loss.sum()) - float(ref.detach())) < 1e-2 * abs(float(ref.detach()))
    for name, p in net.params.items():
        gw = params[name][0].grad.reshape(-1)
        err = float(torch.linalg.norm(p["gw"] - gw) / torch.linalg.norm(gw))
        assert err < 8e-2, (name, err)
