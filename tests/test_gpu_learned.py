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
