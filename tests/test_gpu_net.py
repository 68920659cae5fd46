"""The learned initial guess on the GPU. The BF16 tensor-core 3x3x3
convolution (pgb_conv3d_bf16, tcgen05) against a plain PyTorch FP32
convolution of the same BF16-rounded inputs and weights: outputs agree to
BF16 rounding and the padding stays zero; the adjoint weight image gives
the transposed convolution. The whole network's loss and gradients against
a PyTorch FP32 replica on the CPU, and training lowering the loss."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _lib():
    from pamr_amrd_gb300.learned import conv_lib
    return conv_lib()


def _geom(W, H, D):
    import ctypes as C
    vt, mg = C.c_long(), C.c_long()
    _lib().pgb_conv3d_geometry(W, H, D, C.byref(vt), C.byref(mg))
    return vt.value, mg.value


def _index(W, H, D, margin):
    z, y, x = torch.meshgrid(torch.arange(D), torch.arange(H), torch.arange(W), indexing="ij")
    return (margin + (x + 1) + (W + 2) * ((y + 1) + (H + 2) * (z + 1))).reshape(-1).cuda()


def to_layout(X, vtot, margin):
    """X: (D, H, W, C) -> act[C/8][vtot][8] BF16, zero elsewhere"""
    D, H, W, Cn = X.shape
    act = torch.zeros(Cn // 8, vtot, 8, dtype=torch.bfloat16, device="cuda")
    P = _index(W, H, D, margin)
    Xb = X.reshape(-1, Cn).to(torch.bfloat16)
    for cb in range(Cn // 8):
        act[cb, P, :] = Xb[:, 8 * cb:8 * cb + 8]
    return act, P


def from_layout(act, P, shape):
    D, H, W, Cn = shape
    out = torch.empty(D * H * W, Cn, device="cuda")
    for cb in range(Cn // 8):
        out[:, 8 * cb:8 * cb + 8] = act[cb, P, :].float()
    return out.reshape(D, H, W, Cn)


@pytest.mark.parametrize("cin,cout", [(16, 16), (16, 32), (32, 16), (32, 32), (32, 64), (64, 64), (64, 16)])
@pytest.mark.parametrize("vol", [(16, 12, 10), (128, 6, 5), (4, 4, 4), (2, 2, 2), (40, 24, 37)])
@pytest.mark.parametrize("adjoint", [0, 1])
def test_conv3d_matches_torch(cin, cout, vol, adjoint):
    L = _lib()
    W, H, D = vol
    g = torch.Generator(device="cpu").manual_seed(cin * 1000 + cout + W + adjoint)
    w = (torch.randn(27, cin, cout, generator=g) / np.sqrt(27 * cin)).cuda()
    wb = w.to(torch.bfloat16).float()
    ci_, co_ = (cout, cin) if adjoint else (cin, cout)
    X = torch.randn(D, H, W, ci_, generator=g).cuda()
    bias = (0.1 * torch.randn(co_, generator=g)).cuda()
    vtot, margin = _geom(W, H, D)
    act, P = to_layout(X, vtot, margin)
    # buffers start zeroed; the planes the output tiles cover are filled with
    # junk to see the kernel write every voxel there (interior and padding)
    plane = (W + 2) * (H + 2)
    lo, hi = margin + plane, margin + (D + 1) * plane
    out = torch.zeros(co_ // 8, vtot, 8, dtype=torch.bfloat16, device="cuda")
    out[:, lo:hi, :] = 7.0
    img = torch.zeros(27 * cin * cout, dtype=torch.bfloat16, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    assert L.pgb_conv3d_pack_weights(w.data_ptr(), img.data_ptr(), cin, cout, adjoint, None) == 0
    rc = L.pgb_conv3d_bf16(act.data_ptr(), out.data_ptr(), img.data_ptr(), bias.data_ptr(), W, H, D,
                           ci_, co_, 1, err.data_ptr(), None)
    torch.cuda.synchronize()
    assert rc == 0 and int(err.item()) == 0
    # reference: cross-correlation with w_t[co, ci, dz, dy, dx] = w[tap][ci][co]
    wt = wb.reshape(3, 3, 3, cin, cout).permute(4, 3, 0, 1, 2).contiguous()
    xin = X.to(torch.bfloat16).float().permute(3, 0, 1, 2).unsqueeze(0)
    if adjoint:
        ref = torch.nn.functional.conv_transpose3d(xin, wt, padding=1)
    else:
        ref = torch.nn.functional.conv3d(xin, wt, padding=1)
    ref = torch.nn.functional.leaky_relu(ref[0] + bias.view(-1, 1, 1, 1), 0.125).permute(1, 2, 3, 0)
    got = from_layout(out, P, (D, H, W, co_))
    tol = 1e-2 * ref.abs() + 2e-3 * ref.abs().max()
    assert torch.all((got - ref).abs() <= tol), float((got - ref).abs().max())
    mask = torch.ones(vtot, dtype=torch.bool, device="cuda")
    mask[P] = False
    assert torch.all(out[:, mask, :] == 0)
    assert lo <= int(P.min()) and int(P.max()) < hi


# ------------------------------------------------------------- the network --
def _torch_net(net, flat, x):
    """plain FP32 PyTorch replica of the network (same parameters), on the
    CPU: the oracle of the GPU forward and backward kernels"""
    F = torch.nn.functional
    P = {k: (torch.tensor(w).requires_grad_(True), torch.tensor(b).requires_grad_(True))
         for k, (w, b) in net.split(flat.copy()).items()}

    def conv(name, a, relu=True):
        w, b = P[name]
        wt = w.reshape(3, 3, 3, w.shape[1], w.shape[2]).permute(4, 3, 0, 1, 2)
        y = F.conv3d(a, wt, b, padding=1)
        return F.leaky_relu(y, 0.125) if relu else y

    up = lambda a: F.interpolate(a, scale_factor=2, mode="nearest")  # noqa: E731
    e1 = [conv("tc0", conv("in", x))]
    for v in range(1, net.NLEV):
        e1.append(conv(f"tc{2 * v}", conv(f"tc{2 * v - 1}", F.avg_pool3d(e1[v - 1], 2))))
    d = e1[-1]
    for v in range(net.NLEV - 2, -1, -1):
        d = conv(f"tc{net.dec_layer(v)}", up(d) + e1[v])
    return conv("out", d, relu=False), P


def _smooth_field(n, rng, amp=1.0):
    x = np.linspace(-1, 1, n)
    Z, Y, X = np.meshgrid(x, x, x, indexing="ij")
    f = np.zeros((n, n, n))
    for _ in range(4):
        c = rng.uniform(-0.5, 0.5, 3)
        w = rng.uniform(0.2, 0.5)
        f += amp * rng.uniform(0.2, 1.0) * np.exp(-((X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2) / w ** 2)
    return f


def test_net_gradients_match_torch_fp32():
    from pamr_amrd_gb300.learned import Net
    n = 65
    rng = np.random.default_rng(7)
    net = Net(n, seed=3)
    net.set_scales(2.0, 0.5)
    rho = _smooth_field(n, rng)
    ut = (0.3 * _smooth_field(n, rng)).astype(np.float32)
    d_rho = torch.from_numpy(rho.reshape(-1)).cuda()
    d_ut = torch.from_numpy(ut.reshape(-1)).cuda()
    loss = net.loss_grad(d_rho.data_ptr(), d_ut.data_ptr())
    grads = net.split(net.params(1))
    flat = net.params(0)
    pb = flat.copy()   # the tensor-core layers use BF16 weights
    o = 0
    for name, ci, co in Net.LAYERS:
        k = 27 * ci * co
        if name.startswith("tc"):
            pb[o:o + k] = torch.tensor(pb[o:o + k]).to(torch.bfloat16).float().numpy()
        o += k + co
    x = torch.tensor(2.0 * rho[:n - 1, :n - 1, :n - 1], dtype=torch.float32)[None, None]
    y, P = _torch_net(net, pb, x)
    tgt = torch.tensor(ut[:n - 1, :n - 1, :n - 1] / 0.5)[None, None]
    d = (y - tgt)[..., 1:, 1:, 1:]
    ref_loss = (d * d).mean()
    ref_loss.backward()
    assert abs(loss - ref_loss.item()) <= 0.03 * ref_loss.item(), (loss, ref_loss.item())
    for name, _, _ in Net.LAYERS:
        for k, ours in enumerate(grads[name]):
            ref = P[name][k].grad.detach().cpu().numpy().reshape(-1)
            ours = ours.reshape(-1)
            cos = float(np.dot(ours, ref) / (np.linalg.norm(ours) * np.linalg.norm(ref) + 1e-30))
            assert cos > 0.97, (name, k, cos)
    net.close()


def test_net_training_reduces_the_loss():
    from pamr_amrd_gb300.learned import Net
    n = 65
    rng = np.random.default_rng(8)
    net = Net(n, seed=5)
    rho = _smooth_field(n, rng)
    ut = (0.5 * _smooth_field(n, rng)).astype(np.float32)
    d_rho = torch.from_numpy(rho.reshape(-1)).cuda()
    d_ut = torch.from_numpy(ut.reshape(-1)).cuda()
    losses = [net.train_step(d_rho.data_ptr(), d_ut.data_ptr(), 1e-3) for _ in range(60)]
    assert losses[-1] < 0.2 * losses[0], (losses[0], losses[-1])
    u = torch.zeros(n ** 3, dtype=torch.float64, device="cuda")
    net.predict(d_rho.data_ptr(), u.data_ptr())
    torch.cuda.synchronize()
    uu = u.cpu().numpy().reshape(n, n, n)
    assert np.all(uu[0] == 0) and np.all(uu[:, :, -1] == 0) and np.isfinite(uu).all()
    net.close()


def test_bias_free_net_is_homogeneous():
    """with the biases held at zero the guess scales with the source: a
    power-of-two factor commutes with every rounding, so exactly"""
    from pamr_amrd_gb300.learned import Net
    n = 65
    rng = np.random.default_rng(9)
    net = Net(n, seed=6)
    net.set_bias_free(True)
    rho = _smooth_field(n, rng)
    ut = (0.5 * _smooth_field(n, rng)).astype(np.float32)
    d_rho = torch.from_numpy(rho.reshape(-1)).cuda()
    d_ut = torch.from_numpy(ut.reshape(-1)).cuda()
    for _ in range(5):
        net.train_step(d_rho.data_ptr(), d_ut.data_ptr(), 1e-3)
    p = net.split(net.params(0))
    assert all(not np.any(b) for _, b in p.values())
    u1 = torch.zeros(n ** 3, dtype=torch.float64, device="cuda")
    u4 = torch.zeros_like(u1)
    d_rho4 = 4.0 * d_rho
    net.predict(d_rho.data_ptr(), u1.data_ptr())
    net.predict(d_rho4.data_ptr(), u4.data_ptr())
    torch.cuda.synchronize()
    assert float(u1.abs().max()) > 0
    assert torch.equal(u4, 4.0 * u1)
    net.close()


def test_rescale_restores_the_amplitude():
    """a guess that is the solution times 0.6 comes back as the solution: the
    energy-norm factor <u, rho> / <u, lap u> is exactly 1/0.6 there"""
    from pamr_amrd_gb300.learned import Net
    n, h = 65, 0.25
    x = np.arange(n) * h
    L = (n - 1) * h
    Z, Y, X = np.meshgrid(x, x, x, indexing="ij")
    u = np.sin(np.pi * X / L) * np.sin(2 * np.pi * Y / L) * np.sin(np.pi * Z / L) * (1 + 0.3 * X / L)
    u[0], u[-1], u[:, 0], u[:, -1], u[:, :, 0], u[:, :, -1] = 0, 0, 0, 0, 0, 0
    rho = np.zeros_like(u)
    c = u[1:-1, 1:-1, 1:-1]
    rho[1:-1, 1:-1, 1:-1] = (u[2:, 1:-1, 1:-1] + u[:-2, 1:-1, 1:-1] + u[1:-1, 2:, 1:-1] + u[1:-1, :-2, 1:-1]
                             + u[1:-1, 1:-1, 2:] + u[1:-1, 1:-1, :-2] - 6 * c) / h ** 2
    net = Net(n, seed=2)
    d_rho = torch.from_numpy(rho.reshape(-1).copy()).cuda()
    d_u = torch.from_numpy(0.6 * u.reshape(-1)).cuda()
    net.rescale(d_rho.data_ptr(), d_u.data_ptr(), h)
    torch.cuda.synchronize()
    got = d_u.cpu().numpy()
    assert np.abs(got - u.reshape(-1)).max() <= 1e-12 * np.abs(u).max()
    net.close()
