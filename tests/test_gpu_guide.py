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
