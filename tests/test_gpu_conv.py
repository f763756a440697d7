"""The tensor-core convolutions of the learned pressure guess against a CPU
FP64 convolution.

Every kernel of the network -- forward (with bias, skip addend and ReLU),
backward-data (with the skip addend and the ReLU mask of the layer below),
weight gradient and bias gradient -- runs through the C-ABI on the GPU and
is compared with torch's float64 conv3d (and its autograd) on the CPU, on
the same BF16-rounded inputs and weights.  Tolerances: the outputs of the
forward and backward-data kernels are BF16 (relative rounding 2^-9), so
they must agree to 4e-3 relative L2 and 1 % of the largest value; the
weight and bias gradients are FP32 sums of exact BF16 products and must
agree to 1e-4.

The whole network's gradient (hydro_net_gradient, 11 layers, pooling,
upsampling, skip connections) is compared with torch autograd in float64
on the same samples and weights; its activations are BF16 on the GPU, so
each layer's gradient must agree to 5 % relative L2 (cosine >= 0.995).
"""
import ctypes

import numpy as np
import pytest

from hydro_gb300 import capi

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
F = torch.nn.functional

PAIRS = [(16, 16), (16, 32), (32, 16), (32, 32), (32, 64), (64, 32), (64, 64)]
GRID = (12, 20, 6, 2)  # nx, ny, nz, nb: not multiples of the 8 x 16 x 4 tile


def _bf(t):
    """Round to BF16 and back (the values the kernels see)."""
    return t.to(torch.bfloat16).to(torch.float64)


def _ncdhw(x):  # [nb, nz, ny, nx, c] -> [nb, c, nz, ny, nx]
    return x.permute(0, 4, 1, 2, 3)


def _cl(x):  # [nb, c, nz, ny, nx] -> [nb, nz, ny, nx, c]
    return x.permute(0, 2, 3, 4, 1)


def _rel(a, b):
    return float((a - b).norm() / b.norm())


def _close_bf16(got, ref):
    assert _rel(got, ref) <= 4e-3, _rel(got, ref)
    assert float((got - ref).abs().max()) <= 1e-2 * float(ref.abs().max())


@pytest.fixture(scope="module")
def lib(built):
    return capi.load()


@pytest.mark.parametrize("cin,cout", PAIRS)
def test_conv_forward(lib, cin, cout):
    nx, ny, nz, nb = GRID
    g = torch.Generator().manual_seed(cin * 100 + cout)
    x = _bf(torch.randn(nb, nz, ny, nx, cin, generator=g, dtype=torch.float64))
    w = torch.randn(cout, cin, 3, 3, 3, generator=g, dtype=torch.float64) / np.sqrt(27 * cin)
    b = torch.randn(cout, generator=g, dtype=torch.float64) * 0.1
    add = _bf(torch.randn(nb, nz, ny, nx, cout, generator=g, dtype=torch.float64) * 0.5)
    ref = F.relu(_cl(F.conv3d(_ncdhw(x), _bf(w), b.float().double(), padding=1)) + add)
    dx = x.to(torch.bfloat16).contiguous().cuda()
    dw = w.float().contiguous().cuda()
    db = b.float().contiguous().cuda()
    dadd = add.to(torch.bfloat16).contiguous().cuda()
    dy = torch.empty(nb, nz, ny, nx, cout, dtype=torch.bfloat16, device="cuda")
    torch.cuda.synchronize()
    st = lib.hydro_conv3d_forward(nx, ny, nz, nb, cin, cout, dx.data_ptr(), dw.data_ptr(),
                                  db.data_ptr(), dadd.data_ptr(), 1, dy.data_ptr(), None)
    assert st == capi.OK
    _close_bf16(dy.cpu().double(), ref)


@pytest.mark.parametrize("cin,cout", PAIRS)
def test_conv_backward_data(lib, cin, cout):
    nx, ny, nz, nb = GRID
    g = torch.Generator().manual_seed(7 + cin * 100 + cout)
    w = torch.randn(cout, cin, 3, 3, 3, generator=g, dtype=torch.float64) / np.sqrt(27 * cout)
    gy = _bf(torch.randn(nb, nz, ny, nx, cout, generator=g, dtype=torch.float64))
    add = _bf(torch.randn(nb, nz, ny, nx, cin, generator=g, dtype=torch.float64) * 0.5)
    mask = _bf(torch.randn(nb, nz, ny, nx, cin, generator=g, dtype=torch.float64))
    x = torch.zeros(nb, cin, nz, ny, nx, dtype=torch.float64, requires_grad=True)
    F.conv3d(x, _bf(w), padding=1).backward(_ncdhw(gy))
    ref = (_cl(x.grad) + add) * (mask > 0)
    dgy = gy.to(torch.bfloat16).contiguous().cuda()
    dw = w.float().contiguous().cuda()
    dadd = add.to(torch.bfloat16).contiguous().cuda()
    dmask = mask.to(torch.bfloat16).contiguous().cuda()
    dgx = torch.empty(nb, nz, ny, nx, cin, dtype=torch.bfloat16, device="cuda")
    torch.cuda.synchronize()
    st = lib.hydro_conv3d_backward_data(nx, ny, nz, nb, cin, cout, dgy.data_ptr(), dw.data_ptr(),
                                        dadd.data_ptr(), dmask.data_ptr(), dgx.data_ptr(), None)
    assert st == capi.OK
    _close_bf16(dgx.cpu().double(), ref)


@pytest.mark.parametrize("cin,cout", PAIRS)
def test_conv_backward_weight(lib, cin, cout):
    nx, ny, nz, nb = GRID
    g = torch.Generator().manual_seed(11 + cin * 100 + cout)
    x = _bf(torch.randn(nb, nz, ny, nx, cin, generator=g, dtype=torch.float64))
    gy = _bf(torch.randn(nb, nz, ny, nx, cout, generator=g, dtype=torch.float64))
    w = torch.zeros(cout, cin, 3, 3, 3, dtype=torch.float64, requires_grad=True)
    F.conv3d(_ncdhw(x), w, padding=1).backward(_ncdhw(gy))
    ref_w = w.grad.reshape(cout, cin, 27)
    ref_b = gy.sum(dim=(0, 1, 2, 3))
    dx = x.to(torch.bfloat16).contiguous().cuda()
    dgy = gy.to(torch.bfloat16).contiguous().cuda()
    dw = torch.full((cout, cin, 27), float("nan"), dtype=torch.float32, device="cuda")
    db = torch.full((cout,), float("nan"), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    st = lib.hydro_conv3d_backward_weight(nx, ny, nz, nb, cin, cout, dx.data_ptr(),
                                          dgy.data_ptr(), dw.data_ptr(), db.data_ptr(), None)
    assert st == capi.OK
    assert _rel(dw.cpu().double(), ref_w) <= 1e-4, _rel(dw.cpu().double(), ref_w)
    assert _rel(db.cpu().double(), ref_b) <= 1e-4


# ------------------------------------------------------------ network ----
def _torch_net(params, shapes, x0):
    """The network of include/hydro_net.h in float64 (weights BF16-rounded
    as the kernels use them); x0: [nb, 16, nz, ny, nx]."""
    off = 0
    W, B = [], []
    for cin, cout in shapes:
        nw = cout * cin * 27
        W.append(_bf(params[off:off + nw].reshape(cout, cin, 3, 3, 3)).requires_grad_(True))
        off += nw
        B.append(params[off:off + cout].clone().requires_grad_(True))
        off += cout

    def c(x, i, relu=True, add=None):
        y = F.conv3d(x, W[i], B[i], padding=1)
        if add is not None:
            y = y + add
        return F.relu(y) if relu else y

    e1a = c(x0, 0)
    e1b = c(e1a, 1)
    e2a = c(F.avg_pool3d(e1b, 2), 2)
    e2b = c(e2a, 3)
    e3a = c(F.avg_pool3d(e2b, 2), 4)
    e3b = c(e3a, 5)
    d2a = c(F.interpolate(e3b, scale_factor=2, mode="nearest"), 6, add=e2b)
    d2b = c(d2a, 7)
    d1a = c(F.interpolate(d2b, scale_factor=2, mode="nearest"), 8, add=e1b)
    d1b = c(d1a, 9)
    out = c(d1b, 10, relu=False)
    return out, W, B


def test_network_gradient_vs_torch(built):
    from hydro_gb300.net import Net
    n, nb = (16, 16, 12), 2
    net = Net(n, batch=nb, seed=3)
    nc = n[0] * n[1] * n[2]
    rng = np.random.default_rng(5)
    samples, host = [], []
    for b in range(nb):
        f = rng.normal(size=nc)
        rho = rng.uniform(1.0, 10.0, size=nc)
        p = rng.normal(size=nc)
        df, drho, dp = (torch.from_numpy(a).cuda() for a in (f, rho, p))
        s = torch.empty(net.sample_bytes, dtype=torch.uint8, device="cuda")
        net.pack(df.data_ptr(), drho.data_ptr(), dp.data_ptr(), 0.1, s.data_ptr())
        samples.append(s)
        host.append((f, rho, p))
    torch.cuda.synchronize()
    loss, grad = net.gradient(samples)
    params = torch.from_numpy(net.get_params().astype(np.float64))
    # the samples as the kernels see them (BF16 after normalisation)
    x0 = torch.zeros(nb, 16, n[2], n[1], n[0], dtype=torch.float64)
    tgt = torch.zeros(nb, n[2], n[1], n[0], dtype=torch.float64)
    for b, (f, rho, p) in enumerate(host):
        fn = (f - f.mean()) / f.std()
        pn = (p - p.mean()) / p.std()
        x0[b, 0] = _bf(torch.from_numpy(fn)).reshape(n[2], n[1], n[0])
        x0[b, 1] = _bf(torch.from_numpy(rho * 0.1)).reshape(n[2], n[1], n[0])
        tgt[b] = _bf(torch.from_numpy(pn)).reshape(n[2], n[1], n[0])
    out, W, B = _torch_net(params, net.layer_shapes(), x0)
    ref_loss = 0.5 * ((out[:, 0] - tgt) ** 2).mean()
    ref_loss.backward()
    assert abs(loss - float(ref_loss)) <= 0.02 * float(ref_loss), (loss, float(ref_loss))
    off = 0
    for i, (cin, cout) in enumerate(net.layer_shapes()):
        nw = cout * cin * 27
        gw = torch.from_numpy(grad[off:off + nw].astype(np.float64))
        rw = W[i].grad.reshape(-1)
        off += nw
        gb = torch.from_numpy(grad[off:off + cout].astype(np.float64))
        rb = B[i].grad
        off += cout
        if i == 0:  # padded input channels 2..15 carry zero inputs
            gw = gw.reshape(cout, cin, 27)[:, :2].reshape(-1)
            rw = rw.reshape(cout, cin, 27)[:, :2].reshape(-1)
        if i == 10:  # padded output channels 1..15 carry no loss
            gw = gw.reshape(cout, cin, 27)[:1].reshape(-1)
            rw = rw.reshape(cout, cin, 27)[:1].reshape(-1)
            gb, rb = gb[:1], rb[:1]
        cos = float(gw @ rw / (gw.norm() * rw.norm()))
        assert _rel(gw, rw) <= 0.05 and cos >= 0.995, (i, _rel(gw, rw), cos)
        assert _rel(gb, rb) <= 0.05 or float((gb - rb).abs().max()) <= 1e-6, (i, _rel(gb, rb))
    net.close()
