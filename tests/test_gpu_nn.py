"""Learned initial guess: the network's own GPU kernels against the CPU
oracle (oracle/nn_oracle.py).

  - one 3x3 convolution (tcgen05 implicit GEMM with TMA-loaded NHWC BF16
    activations) equals the oracle's BF16-rounded result to one BF16 ulp;
  - the whole network's loss and parameter gradient (forward, backward
    through every layer, pooling, upsampling, concatenation and the head)
    agree with the oracle: loss within 1e-3 relative, gradient within 3e-2
    relative L2 error and cosine similarity above 0.999 (the residual
    difference is BF16 rounding of activations that the GPU sums in FP32 and
    the oracle in float64);
  - Adam steps on a fixed batch lower the loss.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import nn_oracle as nno

pytestmark = pytest.mark.gpu


def smooth_fields(rng, nb, H, W):
    y, x = np.mgrid[0:H, 0:W]
    out = np.zeros((nb, H, W))
    for k in range(4):
        a, b = rng.integers(1, 4, 2)
        ph = rng.uniform(0, 2 * np.pi, (nb, 1, 1))
        out += rng.normal(size=(nb, 1, 1)) * np.sin(np.pi * a * y / H + ph) * np.cos(np.pi * b * x / W)
    return out


def make_batch(seed, nb, H, W):
    rng = np.random.default_rng(seed)
    raw = np.zeros((nb, 3, H, W), np.float32)
    raw[:, 0] = 2.0 * smooth_fields(rng, nb, H, W)
    raw[:, 1] = 1e4 * smooth_fields(rng, nb, H, W)
    raw[:, 2] = 50.0 * smooth_fields(rng, nb, H, W)
    sf_new = (raw[:, 2] + 0.5 * smooth_fields(rng, nb, H, W)).astype(np.float32)
    return raw, sf_new


@pytest.mark.parametrize("nb,H,W,cin,cout", [(2, 8, 64, 16, 32), (1, 16, 256, 32, 64), (1, 8, 128, 96, 128),
                                             (2, 4, 32, 256, 256), (1, 16, 128, 192, 64)])
def test_conv3x3_matches_oracle(gpu_lib, nb, H, W, cin, cout):
    from tracer_code_gb300.learned import conv3x3
    rng = np.random.default_rng(cin * 7 + cout)
    x = nno.bf16(rng.normal(size=(nb, H, W, cin)).astype(np.float32))
    w = (rng.normal(size=(cout, 9, cin)) / np.sqrt(9 * cin)).astype(np.float32)
    b = rng.normal(size=cout).astype(np.float32) * 0.1
    xd = torch.from_numpy(x).to(torch.bfloat16).cuda()
    wd = torch.from_numpy(w).cuda()
    bd = torch.from_numpy(b).cuda()
    yd = torch.zeros((nb, H, W, cout), dtype=torch.bfloat16, device="cuda")
    conv3x3(xd.data_ptr(), nb, H, W, cin, wd.data_ptr(), bd.data_ptr(), cout, True, yd.data_ptr())
    torch.cuda.synchronize()
    got = yd.float().cpu().numpy()
    ref = nno.conv3x3(x, w.astype(np.float64), b.astype(np.float64), relu=True)
    # one BF16 ulp (2^-8 relative) plus the FP32-vs-float64 summation difference
    tol = np.abs(ref) * 2.0 ** -7 + 1e-5
    assert np.all(np.abs(got - ref) <= tol), float(np.abs(got - ref).max())


def test_network_gradient_matches_oracle(gpu_lib):
    from tracer_code_gb300.learned import Net
    nb, H, W = 2, 64, 128
    raw, sf_new = make_batch(5, nb, H, W)
    net = Net(nb, H, W, seed=11)
    params = net.get_params()
    rd = torch.from_numpy(raw).cuda()
    sd = torch.from_numpy(sf_new).cuda()
    loss = net.loss_backward(rd.data_ptr(), sd.data_ptr(), nb)
    g = net.get_grads().astype(np.float64)
    lo, go, _ = nno.loss_and_grads(params, raw, sf_new)
    assert abs(loss - lo) <= 1e-3 * lo, (loss, lo)
    rel = np.linalg.norm(g - go) / np.linalg.norm(go)
    cos = float(g @ go / (np.linalg.norm(g) * np.linalg.norm(go)))
    assert rel <= 3e-2 and cos >= 0.999, (rel, cos)
    # every layer receives a gradient of the right size (per-layer check)
    lay, head, _ = nno.param_layout()
    for l, (w, b, cout, cin) in enumerate(lay):
        gl, ol = g[w:b + cout], go[w:b + cout]
        assert np.linalg.norm(gl - ol) <= 0.1 * np.linalg.norm(ol) + 1e-12, l
    net.close()


def test_adam_lowers_the_loss(gpu_lib):
    from tracer_code_gb300.learned import Net
    nb, H, W = 4, 64, 128
    raw, sf_new = make_batch(9, nb, H, W)
    net = Net(nb, H, W, seed=3)
    rd = torch.from_numpy(raw).cuda()
    sd = torch.from_numpy(sf_new).cuda()
    losses = []
    for _ in range(30):
        losses.append(net.loss_backward(rd.data_ptr(), sd.data_ptr(), nb))
        net.adam(1e-3)
    assert losses[-1] < 0.5 * losses[0], losses[::5]
    net.close()
