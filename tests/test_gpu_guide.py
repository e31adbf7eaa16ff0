"""The path-guiding network on the tensor cores (tcgen05) against a plain
PyTorch fp32 reference of the same computation: fp16-rounded weights and
inputs, fp32 accumulation, bias, ReLU, activations rounded to fp16 between
layers."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LAYERS = [(7, 64), (64, 64), (64, 64), (64, 64), (64, 40)]  # (in, out)
TOL = 2e-3  # relative to the output scale: fp16 activations (2^-11) and fp32 sums in another order


def unpack(p):
    out, o = [], 0
    for kin, kout in LAYERS:
        W = p[o:o + kin * kout].reshape(kout, kin)
        o += kin * kout
        b = p[o:o + kout]
        o += kout
        out.append((W, b))
    assert o == len(p)
    return out


def torch_forward(p, x):
    import torch
    h = torch.tensor(x, dtype=torch.float32).half().float()
    layers = unpack(p)
    for i, (W, b) in enumerate(layers):
        Wt = torch.tensor(W).half().float()
        h = h @ Wt.T + torch.tensor(b)
        if i < len(layers) - 1:
            h = torch.relu(h).half().float()
    return h.numpy()


@pytest.mark.parametrize("n", [1, 1000, 70001])
def test_forward_matches_torch_fp32(gpu, n):
    import torch
    gpu.guide_init(seed=3)
    p = gpu.guide_params()
    assert p.shape == (15592,) and np.abs(p).max() <= 1.0
    rng = np.random.default_rng(n)
    x = rng.uniform(-1, 1, (n, 7)).astype(np.float32)
    dx = torch.tensor(x, device="cuda:0")
    dout = torch.full((n, 40), float("nan"), device="cuda:0")
    torch.cuda.synchronize()
    gpu.guide_forward_dev(dx.data_ptr(), n, dout.data_ptr())
    got = dout.cpu().numpy()
    want = torch_forward(p, x)
    scale = np.abs(want).max()
    err = np.abs(got - want).max()
    print(f"n={n}: max |gpu - torch| = {err:.3e}, output scale {scale:.3e}")
    assert np.isfinite(got).all()
    assert err <= TOL * scale


def test_forward_structured_weights(gpu):
    """Weights that make each layer's layout mistakes visible: every output
    depends on a distinct input column."""
    import torch
    rng = np.random.default_rng(7)
    p = rng.normal(0, 0.3, 15592).astype(np.float32)
    gpu.guide_set_params(p)
    assert np.array_equal(gpu.guide_params(), p)
    n = 256
    x = rng.normal(0, 1, (n, 7)).astype(np.float32)
    dx = torch.tensor(x, device="cuda:0")
    dout = torch.zeros((n, 40), device="cuda:0")
    torch.cuda.synchronize()
    gpu.guide_forward_dev(dx.data_ptr(), n, dout.data_ptr())
    want = torch_forward(p, x)
    got = dout.cpu().numpy()
    assert np.abs(got - want).max() <= TOL * np.abs(want).max()


def torch_params(p, requires_grad=False):
    import torch
    out = []
    for W, b in unpack(p):
        Wt = torch.tensor(W).half().float().requires_grad_(requires_grad)
        bt = torch.tensor(b).requires_grad_(requires_grad)
        out.append((Wt, bt))
    return out


def torch_net(layers, x):
    import torch
    h = x.half().float()
    for i, (W, b) in enumerate(layers):
        h = h @ W.T + b
        if i < len(layers) - 1:
            h = torch.relu(h).half().float()
    return h


def flat_grads(layers):
    import torch
    return torch.cat([t.grad.reshape(-1) for W, b in layers for t in (W, b)]).numpy()


@pytest.mark.parametrize("n", [5, 300, 20000])
def test_backward_matches_torch_autograd(gpu, n):
    import torch
    rng = np.random.default_rng(11 + n)
    p = rng.normal(0, 0.25, 15592).astype(np.float32)
    gpu.guide_set_params(p)
    x = rng.normal(0, 1, (n, 7)).astype(np.float32)
    dout = rng.normal(0, 1, (n, 40)).astype(np.float32)
    dx, dd = torch.tensor(x, device="cuda:0"), torch.tensor(dout, device="cuda:0")
    dg = torch.full((15592,), float("nan"), device="cuda:0")
    torch.cuda.synchronize()
    gpu.guide_backward_dev(dx.data_ptr(), dd.data_ptr(), n, dg.data_ptr())
    got = dg.cpu().numpy()
    layers = torch_params(p, True)
    (torch_net(layers, torch.tensor(x)) * torch.tensor(dout)).sum().backward()
    want = flat_grads(layers)
    o = 0
    for i, (kin, kout) in enumerate(LAYERS):
        for name, size in (("W", kin * kout), ("b", kout)):
            g, w = got[o:o + size], want[o:o + size]
            err = np.abs(g - w).max() / max(np.abs(w).max(), 1e-12)
            print(f"n={n} layer {i} {name}: max rel err {err:.2e}")
            assert err < 2e-2, (i, name, err)  # dZ rounded to fp16 on the tensor-core path
            o += size


def mixture_nll(out, d, w):
    """-sum w log p / sum w for the vMF mixture parametrisation of the network."""
    import math

    import torch
    z = out.reshape(-1, 8, 5)
    logpi = torch.log_softmax(z[..., 0], -1)
    from tracer_gb300.native import GpuContext
    s = z[..., 1].clamp(*GpuContext.GUIDE_LOG_KAPPA)
    kappa = torch.exp(s)
    m = z[..., 2:5]
    mu = m / (m.norm(dim=-1, keepdim=True) + 1e-6)
    c = (mu * d[:, None, :]).sum(-1)
    lognorm = torch.log(kappa) - math.log(2 * math.pi) - torch.log1p(-torch.exp(-2 * kappa))
    logp = torch.logsumexp(logpi + lognorm + kappa * (c - 1), -1)
    return -(w * logp).sum() / w.sum()


def test_loss_gradient_matches_torch_autograd(gpu):
    import torch
    rng = np.random.default_rng(5)
    n = 3000
    gpu.guide_init(seed=9)
    p = gpu.guide_params()
    x = rng.normal(0, 1, (n, 7)).astype(np.float32)
    d = rng.normal(0, 1, (n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    w = rng.exponential(1.0, n).astype(np.float32)
    w[:50] = 0.0
    dx, ddir, dw = (torch.tensor(a, device="cuda:0") for a in (x, d, w))
    ddout = torch.zeros((n, 40), device="cuda:0")
    torch.cuda.synchronize()
    loss = gpu.guide_loss_dev(dx.data_ptr(), ddir.data_ptr(), dw.data_ptr(), n, ddout.data_ptr())
    out = torch_net(torch_params(p), torch.tensor(x)).detach().requires_grad_(True)
    ref = mixture_nll(out, torch.tensor(d), torch.tensor(w))
    ref.backward()
    print(f"loss gpu {loss:.6f} torch {ref.item():.6f}")
    assert abs(loss - ref.item()) <= 1e-3 * abs(ref.item())
    g, want = ddout.cpu().numpy(), out.grad.numpy()
    assert np.abs(g - want).max() <= 1e-2 * np.abs(want).max()


def test_training_learns_a_direction_field(gpu):
    """Directions drawn around a mean that depends on the input: Adam steps on
    the tensor-core network must lower the mixture NLL well below the uniform
    sphere's log(4 pi)."""
    import math

    import torch
    rng = np.random.default_rng(2)
    gpu.guide_init(seed=1)
    n = 8192
    losses = []
    for step in range(300):
        x = rng.uniform(-1, 1, (n, 7)).astype(np.float32)
        mean = np.stack([np.cos(2 * x[:, 0]), np.sin(2 * x[:, 0]), x[:, 1]], 1)
        d = mean / np.linalg.norm(mean, axis=1, keepdims=True) + rng.normal(0, 0.15, (n, 3))
        d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
        w = np.ones(n, np.float32)
        dx, ddir, dw = (torch.tensor(a, device="cuda:0") for a in (x, d, w))
        torch.cuda.synchronize()
        losses.append(gpu.guide_train_step_dev(dx.data_ptr(), ddir.data_ptr(), dw.data_ptr(), n, 3e-3))
    print("loss", [round(v, 3) for v in losses[::30]], "uniform", round(math.log(4 * math.pi), 3))
    assert all(np.isfinite(losses))
    assert np.mean(losses[-20:]) < math.log(4 * math.pi) - 1.0


def _batch(rng, n, zero_weights=0):
    x = rng.normal(0, 1, (n, 7)).astype(np.float32)
    d = rng.normal(0, 1, (n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    w = rng.exponential(1.0, n).astype(np.float32)
    w[:zero_weights] = 0.0
    return x, d, w


def _torch_grad(p, x, d, w):
    import torch
    layers = torch_params(p, True)
    loss = mixture_nll(torch_net(layers, torch.tensor(x)), torch.tensor(d), torch.tensor(w))
    loss.backward()
    return loss.item(), flat_grads(layers)


def _step(gpu, x, d, w, lr):
    import torch
    dx, ddir, dw = (torch.tensor(a, device="cuda:0") for a in (x, d, w))
    torch.cuda.synchronize()
    return gpu.guide_train_step_dev(dx.data_ptr(), ddir.data_ptr(), dw.data_ptr(), len(x), lr)


@pytest.mark.parametrize("n", [77, 3000, 65536])
def test_fused_training_step_against_torch(gpu, n):
    """One Adam step through the fused kernels (forward, loss and backward in
    one tcgen05 launch, Adam and the weight images in a second): the loss is
    torch's, and Adam's first step moves every parameter by lr against the
    sign of torch's fp32 gradient (m / sqrt(v) = g / |g| after one step)."""
    rng = np.random.default_rng(n)
    gpu.guide_init(seed=4)
    p = gpu.guide_params()
    x, d, w = _batch(rng, n, zero_weights=min(20, n // 4))
    want_loss, g = _torch_grad(p, x, d, w)
    lr = 1e-4
    loss = _step(gpu, x, d, w, lr)
    delta = gpu.guide_params().astype(np.float64) - p
    print(f"n={n} loss gpu {loss:.6f} torch {want_loss:.6f}")
    assert abs(loss - want_loss) <= 1e-3 * abs(want_loss)
    o = 0
    for i, (kin, kout) in enumerate(LAYERS):
        for name, size in (("W", kin * kout), ("b", kout)):
            gg, dd = g[o:o + size], delta[o:o + size]
            big = np.abs(gg) > 2e-2 * np.abs(gg).max()
            agree = (np.sign(dd[big]) == -np.sign(gg[big])).mean()
            print(f"  layer {i} {name}: {big.sum()} significant gradients, sign agreement {agree:.4f}")
            assert agree >= 0.99, (i, name, agree)
            assert np.abs(np.abs(dd[big]) - lr).max() <= 0.05 * lr
            o += size
    # the packed images follow the parameters: a forward pass matches torch on the new parameters
    import torch
    p1 = gpu.guide_params()
    xs = x[:256]
    dxs = torch.tensor(xs, device="cuda:0")
    out = torch.zeros((len(xs), 40), device="cuda:0")
    torch.cuda.synchronize()
    gpu.guide_forward_dev(dxs.data_ptr(), len(xs), out.data_ptr())
    want = torch_forward(p1, xs)
    assert np.abs(out.cpu().numpy() - want).max() <= TOL * np.abs(want).max()


def test_fused_training_step_gradient_magnitudes(gpu):
    """Two Adam steps on two batches: the second update is
    -lr (0.09 g_a + 0.1 g_b) / 0.19 / sqrt((0.000999 g_a^2 + 0.001 g_b^2) / 0.001999),
    which depends on the ratio of the two batches' gradients per parameter,
    so it checks gradient magnitudes, not only signs (lr small enough that
    the first step does not move the second gradient)."""
    rng = np.random.default_rng(21)
    gpu.guide_init(seed=6)
    p = gpu.guide_params()
    xa, da, wa = _batch(rng, 4000)
    xb, db, wb = _batch(rng, 2500)
    _, ga = _torch_grad(p, xa, da, wa)
    _, gb = _torch_grad(p, xb, db, wb)
    lr = 1e-6
    _step(gpu, xa, da, wa, lr)
    p1 = gpu.guide_params().astype(np.float64)
    _step(gpu, xb, db, wb, lr)
    delta = gpu.guide_params().astype(np.float64) - p1
    ga, gb = ga.astype(np.float64), gb.astype(np.float64)
    want = -lr * ((0.09 * ga + 0.1 * gb) / 0.19) / np.sqrt((0.000999 * ga ** 2 + 0.001 * gb ** 2) / 0.001999)
    sig = np.maximum(np.abs(ga), np.abs(gb)) > 5e-2 * np.maximum(np.abs(ga).max(), np.abs(gb).max())
    err = np.abs(delta - want)[sig] / lr
    print(f"{sig.sum()} parameters; |update - expected| / lr: median {np.median(err):.4f}, "
          f"99th percentile {np.percentile(err, 99):.4f}")
    # fp32 parameters near 0.1-1 resolve an update of 1e-6 to ~1e-7 / 1e-6
    assert np.percentile(err, 95) <= 0.1


def test_fused_training_step_is_deterministic(gpu):
    """The gradient partials of the CTAs are summed in a fixed order: the same
    step from the same state gives bit-identical parameters."""
    rng = np.random.default_rng(3)
    x, d, w = _batch(rng, 20000)
    outs = []
    for _ in range(2):
        gpu.guide_init(seed=8)
        for _ in range(3):
            _step(gpu, x, d, w, 1e-3)
        outs.append(gpu.guide_params())
    assert np.array_equal(outs[0].view(np.uint32), outs[1].view(np.uint32))
