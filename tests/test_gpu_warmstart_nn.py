"""tcgen05 BF16 network kernels (forward, data and weight gradients) against
the CPU restatement oracle/nn_oracle.py, which mirrors the BF16 rounding
points; tolerances are relative L2: output 3e-3 (8e-3 with 4 levels), full
gradient 1e-2 (BF16 products, FP32 sums in another order).  Batched calls against single-image
calls, and the feature kernel against its numpy restatement."""
import numpy as np
import pytest

from oracle import nn_oracle
from quantumvortices_gb300.warmstart import WarmStartNet

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _data(h, seed=0):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(seed)
    inp = rng.standard_normal((3, h, h)).astype(np.float32)
    tgt = (0.3 * rng.standard_normal((2, h, h))).astype(np.float32)
    return inp, tgt, torch.from_numpy(inp).cuda(), torch.from_numpy(tgt).cuda()


@pytest.mark.parametrize("h,base,levels", [(32, 16, 2), (64, 16, 3), (64, 32, 4)])
def test_forward_matches_oracle(h, base, levels):
    torch = pytest.importorskip("torch")
    net = WarmStartNet(h, h, base, levels, seed=3)
    inp, tgt, di, dt = _data(h)
    out = torch.empty((2, h, h), dtype=torch.float32, device="cuda")
    net.forward(di, out)
    ref, _ = nn_oracle.forward(net.get_params().astype(np.float64), inp.astype(np.float64), base, levels)
    # FP32 sums in another order flip BF16 roundings of stored activations;
    # each level adds a few (measured on GB300: 6.0e-3 with 4 levels)
    assert rel(out.cpu().numpy(), ref) < (3e-3 if levels <= 3 else 8e-3)
    net.close()


@pytest.mark.parametrize("h,base,levels", [(32, 16, 2), (64, 16, 3)])
def test_gradient_matches_oracle(h, base, levels):
    net = WarmStartNet(h, h, base, levels, seed=5)
    inp, tgt, di, dt = _data(h, seed=1)
    loss, g = net.loss_grad(di, dt)
    rloss, rg = nn_oracle.loss_grad(net.get_params().astype(np.float64), inp.astype(np.float64),
                                    tgt.astype(np.float64), base, levels)
    assert abs(loss - rloss) <= 3e-3 * rloss
    assert rel(g, rg) < 1e-2
    # per layer
    o = 0
    for ci, co, _ in nn_oracle.layers(base, levels):
        n = co * 9 * ci
        assert rel(g[o:o + n], rg[o:o + n]) < 5e-2, (ci, co)
        o += n + co
    net.close()


def test_training_reduces_loss():
    """Adam on a learnable map (half of the first two input channels)."""
    torch = pytest.importorskip("torch")
    net = WarmStartNet(64, 64, 16, 3, seed=7)
    inp, _, di, _ = _data(64, seed=2)
    dt = (0.5 * di[:2]).contiguous()
    torch.cuda.synchronize()  # the network reads it on its own stream
    l0 = net.train_step(di, dt, 2e-3, want_loss=True)
    for _ in range(150):
        last = net.train_step(di, dt, 2e-3, want_loss=True)
    assert last < 0.3 * l0, (l0, last)
    net.close()


@pytest.mark.parametrize("h,base,levels", [(128, 16, 2), (128, 32, 2)])
def test_row_block_conv_matches_oracle(h, base, levels):
    """Widths that are multiples of 128 take the row-block convolution for the
    narrow layers: forward and gradient against the oracle as above."""
    torch = pytest.importorskip("torch")
    net = WarmStartNet(h, h, base, levels, seed=11)
    inp, tgt, di, dt = _data(h, seed=3)
    out = torch.empty((2, h, h), dtype=torch.float32, device="cuda")
    net.forward(di, out)
    prm = net.get_params().astype(np.float64)
    ref, _ = nn_oracle.forward(prm, inp.astype(np.float64), base, levels)
    assert rel(out.cpu().numpy(), ref) < 3e-3
    loss, g = net.loss_grad(di, dt)
    rloss, rg = nn_oracle.loss_grad(prm, inp.astype(np.float64), tgt.astype(np.float64), base, levels)
    assert abs(loss - rloss) <= 3e-3 * rloss
    assert rel(g, rg) < 1e-2
    net.close()


def test_row_block_conv_matches_generic_kernel_at_512():
    """512^2, 4 levels (row blocks of 4 and 2 rows, 16/32/64 channels): the
    row-block kernel against the generic implicit-GEMM kernel (same BF16
    products, FP32 sums in another order): output and gradient within 1e-3."""
    import os
    torch = pytest.importorskip("torch")
    h = 512
    inp, tgt, di, dt = _data(h, seed=4)
    res = []
    for flag in ("0", "1"):
        os.environ["VK_CONV_ROWS"] = flag
        try:
            net = WarmStartNet(h, h, 32, 4, seed=2)
        finally:
            os.environ.pop("VK_CONV_ROWS", None)
        out = torch.empty((2, h, h), dtype=torch.float32, device="cuda")
        net.forward(di, out)
        loss, g = net.loss_grad(di, dt)
        res.append((out.cpu().numpy(), loss, g))
        net.close()
    (o0, l0, g0), (o1, l1, g1) = res
    assert rel(o1, o0) < 1e-3 and abs(l1 - l0) <= 1e-3 * l0 and rel(g1, g0) < 1e-3


@pytest.mark.parametrize("h,base,levels", [(64, 16, 3), (128, 32, 2)])
def test_batched_calls_match_single_image_calls(h, base, levels):
    """A batch of 3 images: each image's output equals its single-image
    forward, and the batch gradient is the mean of the single-image
    gradients (the batch loss is the mean over the images)."""
    torch = pytest.importorskip("torch")
    net = WarmStartNet(h, h, base, levels, seed=13, batch=3)
    data = [_data(h, seed=20 + i) for i in range(3)]
    xb = torch.stack([d[2] for d in data]).contiguous()
    yb = torch.stack([d[3] for d in data]).contiguous()
    torch.cuda.synchronize()  # the network reads them on its own stream
    out = torch.empty((3, 2, h, h), dtype=torch.float32, device="cuda")
    net.forward(xb, out)
    lb, gb = net.loss_grad(xb, yb)
    net.set_batch(1)
    one = torch.empty((2, h, h), dtype=torch.float32, device="cuda")
    gs, ls = [], []
    for i, d in enumerate(data):
        net.forward(d[2], one)
        assert rel(out[i].cpu().numpy(), one.cpu().numpy()) < 1e-5
        l1, g1 = net.loss_grad(d[2], d[3])
        ls.append(l1)
        gs.append(g1)
    assert abs(lb - np.mean(ls)) <= 1e-5 * lb
    # the batch's output gradient carries 1/3 where a single image's carries
    # 1, so its BF16 roundings differ (measured 1.4e-4)
    assert rel(gb, np.mean(gs, axis=0)) < 1e-3
    net.close()


def test_feature_kernel_matches_numpy():
    torch = pytest.importorskip("torch")
    h = 128
    net = WarmStartNet(h, h, 16, 2, seed=1)
    rng = np.random.default_rng(6)
    psi = rng.standard_normal((h, h)) + 1j * rng.standard_normal((h, h))
    pos = rng.uniform(0, 2 * np.pi, (10, 2))
    width = 2 * np.sqrt(2) * 2 * np.pi / h
    out = torch.empty((3, h, h), dtype=torch.float32, device="cuda")
    net.features(psi, pos, width, out)
    ref = nn_oracle.features(h, h, pos, psi, width)
    assert rel(out.cpu().numpy(), ref) < 1e-6
    net.close()


@pytest.mark.parametrize("h,base,levels,narrow", [(128, 32, 3, False), (64, 32, 4, False), (128, 16, 3, True)])
def test_tma_conv_matches_cp_async_conv(h, base, levels, narrow):
    """Layers whose input has 64k channels run on the TMA-fed kernel
    (VK_CONV_TMA=1: periodic padding, TMA tiles in the 128-byte swizzle
    layout, 3- or 4-stage mbarrier ring), and with VK_CONV_TMA_NARROW=1 the 16- and
    32-channel layers too (32- and 64-byte swizzle); the K order is that of
    the cp.async kernels, so forward outputs and gradients agree to FP32
    rounding (a batch of 2)."""
    import os
    torch = pytest.importorskip("torch")
    if narrow:
        os.environ["VK_CONV_TMA_NARROW"] = "1"
    data = [_data(h, seed=30 + i) for i in range(2)]
    xb = torch.stack([d[2] for d in data]).contiguous()
    yb = torch.stack([d[3] for d in data]).contiguous()
    torch.cuda.synchronize()
    res = []
    for flag in ("0", "1"):
        os.environ["VK_CONV_TMA"] = flag
        try:
            net = WarmStartNet(h, h, base, levels, seed=9, batch=2)
        finally:
            os.environ.pop("VK_CONV_TMA", None)
        out = torch.empty((2, 2, h, h), dtype=torch.float32, device="cuda")
        net.forward(xb, out)
        loss, g = net.loss_grad(xb, yb)
        res.append((out.cpu().numpy(), loss, g))
        net.close()
    os.environ.pop("VK_CONV_TMA_NARROW", None)
    (o0, l0, g0), (o1, l1, g1) = res
    assert rel(o1, o0) < 1e-5 and abs(l1 - l0) <= 1e-5 * l0 and rel(g1, g0) < 1e-4


def test_training_graph_matches_plain_launches():
    """From the second step of a batch size the training step replays one
    CUDA graph (inputs copied into fixed buffers, Adam's lr and bias
    corrections read from device memory); VK_NN_GRAPH=0 launches the same
    kernels one by one.  The weight-gradient sums use float atomics, so two
    runs agree to FP32 rounding, not bit for bit: parameters after six Adam
    steps within 1e-5 (relative L2), losses within 1e-4."""
    import os
    torch = pytest.importorskip("torch")
    data = [_data(64, seed=50 + i) for i in range(2)]
    xb = torch.stack([d[2] for d in data]).contiguous()
    yb = torch.stack([d[3] for d in data]).contiguous()
    torch.cuda.synchronize()
    res = []
    for flag in ("0", "1"):
        os.environ["VK_NN_GRAPH"] = flag
        try:
            net = WarmStartNet(64, 64, 16, 3, seed=11, batch=2)
        finally:
            os.environ.pop("VK_NN_GRAPH", None)
        p0 = net.get_params()
        losses = [net.train_step(xb, yb, 1e-3, want_loss=True) for _ in range(6)]
        res.append((p0, net.get_params(), losses))
        net.close()
    (a0, a, la), (b0, b, lb) = res
    assert np.array_equal(a0, b0) and not np.array_equal(a, a0)
    assert rel(b, a) < 1e-5
    assert all(abs(x - y) <= 1e-4 * abs(x) for x, y in zip(la, lb))
