"""The warm-start network: the CPU oracle of its forward and backward pass is
pinned by finite differences and by an independent torch restatement, and the
GPU kernels (tensor-core convolutions,
pooling, upsampling, loss, Adam) are checked against that oracle on the same
BF16-rounded weights and inputs."""
import numpy as np
import pytest

from oracle import unet_oracle as uo
from glemur_gb300.warmstart import LAYERS, n_params


def rand_params(rng, scale=1.0):
    return {n: (rng.normal(0, scale * np.sqrt(2.0 / (27 * ci)), (27, co, ci)), rng.normal(0, 0.05, co))
            for n, ci, co, _ in LAYERS}


def test_param_count():
    """About 2 M parameters at base width 24 with a 192-channel bottleneck;
    a 96-channel bottleneck has 0.8 M."""
    assert 1_700_000 < n_params() < 1_900_000
    assert 750_000 < n_params(96) < 850_000


def test_oracle_gradients_by_finite_differences():
    rng = np.random.default_rng(0)
    P = rand_params(rng)
    x = rng.normal(size=(8, 4, 4, 3))
    tgt = rng.normal(size=(8, 4, 4, 3))
    a = uo.forward(P, x)
    L0, gy = uo.loss_grad(a["y"], tgt, 1.0)
    G = uo.backward(P, x, a, gy)
    h = 1e-6
    for name in ("e0a", "e1b", "bb", "d1a", "d0a", "head"):
        W, b = P[name]
        for _ in range(3):
            idx = tuple(rng.integers(s) for s in W.shape)
            W[idx] += h
            lp = uo.loss_grad(uo.forward(P, x)["y"], tgt, 1.0)[0]
            W[idx] -= 2 * h
            lm = uo.loss_grad(uo.forward(P, x)["y"], tgt, 1.0)[0]
            W[idx] += h
            fd = (lp - lm) / (2 * h)
            assert fd == pytest.approx(G[name][0][idx], rel=1e-4, abs=1e-7), (name, idx)
        o = rng.integers(b.shape[0])
        b[o] += h
        lp = uo.loss_grad(uo.forward(P, x)["y"], tgt, 1.0)[0]
        b[o] -= 2 * h
        lm = uo.loss_grad(uo.forward(P, x)["y"], tgt, 1.0)[0]
        b[o] += h
        assert (lp - lm) / (2 * h) == pytest.approx(G[name][1][o], rel=1e-4, abs=1e-7), (name, "bias")


def _torch_unet(P, x):
    """The network restated with torch.nn.functional in float64 on the CPU,
    independently of the oracle: conv3d on circularly padded x, y and
    zero-padded z (the oracle's tap t = 9 (dk+1) + 3 (dj+1) + (di+1) is the
    weight's (t // 9, t // 3 % 3, t % 3) entry), avg_pool3d, nearest
    upsampling, skips concatenated after the upsampled path."""
    import torch
    import torch.nn.functional as F
    Wt = {n: (torch.tensor(W.transpose(1, 2, 0).reshape(W.shape[1], W.shape[2], 3, 3, 3), requires_grad=True),
              torch.tensor(b, requires_grad=True)) for n, (W, b) in P.items()}

    def conv(n, a, act=True):
        a = F.pad(a, (1, 1, 1, 1, 0, 0), mode="circular")
        a = F.pad(a, (0, 0, 0, 0, 1, 1))
        y = F.conv3d(a, *Wt[n])
        return F.relu(y) if act else y

    up = lambda a: F.interpolate(a, scale_factor=2, mode="nearest")  # noqa: E731
    t = torch.tensor(x.transpose(3, 0, 1, 2)[None].copy())
    e0 = conv("e0b", conv("e0a", t))
    e1 = conv("e1b", conv("e1a", F.avg_pool3d(e0, 2)))
    bb = conv("bb", conv("ba", F.avg_pool3d(e1, 2)))
    d1 = conv("d1b", conv("d1a", torch.cat([up(bb), e1], 1)))
    d0 = conv("d0b", conv("d0a", torch.cat([up(d1), e0], 1)))
    y = conv("head", d0, act=False)
    return y, Wt


def test_oracle_matches_an_independent_torch_network():
    """Forward output and every layer's weight and bias gradient of the CPU
    oracle against the torch restatement (autograd) on a 8x8x8 grid."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(1)
    P = rand_params(rng)
    x = rng.normal(size=(8, 8, 8, 3))
    tgt = rng.normal(size=(8, 8, 8, 3))
    a = uo.forward(P, x)
    L0, gy = uo.loss_grad(a["y"], tgt, 0.5)
    G = uo.backward(P, x, a, gy)
    y, Wt = _torch_unet(P, x)
    yn = y[0].detach().numpy().transpose(1, 2, 3, 0)
    assert relerr(a["y"], yn) < 1e-12
    e = (y[0].permute(1, 2, 3, 0) - torch.tensor(tgt))[1:-1]
    loss = 0.5 * (e * e).sum()
    assert abs(float(loss.detach()) - L0) < 1e-10 * abs(L0)
    loss.backward()
    for n, (W, b) in Wt.items():
        gW = W.grad.numpy().reshape(W.shape[0], W.shape[1], 27).transpose(2, 0, 1)
        assert relerr(G[n][0], gW) < 1e-10, n
        assert relerr(G[n][1], b.grad.numpy()) < 1e-10, n


def bf16(a):
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def relerr(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


def frob(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.gpu
def test_gpu_network_matches_oracle():
    import torch
    from glemur_gb300.warmstart import UNet
    nx, ny, nz = 8, 8, 16
    net = UNet((nx, ny, nz), seed=3)
    rng = np.random.default_rng(1)
    for L in net.layers.values():
        L.b.copy_(torch.from_numpy(rng.normal(0, 0.05, L.co).astype(np.float32)))
    net.refresh_weights()
    x = rng.normal(size=(nz, ny, nx, 3))
    X0 = np.zeros((nx * ny * nz, 8), np.float32)
    X0[:, :3] = x.reshape(-1, 3)
    net.A["X0"].copy_(torch.from_numpy(X0).to(torch.bfloat16))
    tgt = rng.normal(size=(nz, ny, nx, 3)).astype(np.float32)
    tdev = torch.from_numpy(tgt.reshape(-1, 3)).cuda()
    net.zero_grad()
    y = net.forward()
    scale = 1.0 / (nx * ny * nz * 3)
    net.backward(tdev, scale)
    torch.cuda.synchronize()
    net.check_status()
    # oracle on the BF16 weights and input the GPU used
    P = {n: (bf16(W), b) for n, (W, b) in net.params_numpy().items()}
    xb = bf16(x)
    a = uo.forward(P, xb)
    yg = y[:, :3].float().cpu().numpy().reshape(nz, ny, nx, 3)
    assert relerr(yg, a["y"]) < 3e-2 and frob(yg, a["y"]) < 1.5e-2
    loss, gy = uo.loss_grad(a["y"], tgt.astype(np.float64), scale)
    assert float(net.loss_acc.item()) == pytest.approx(loss, rel=5e-2)
    G = uo.backward(P, xb, a, gy)
    g = net.grads_numpy()
    # end to end: the GPU rounds every activation and gradient buffer to BF16
    # (8-bit mantissa); through the 22 convolutions of the backward pass that
    # leaves up to ~6 % (Frobenius) on the first layer's gradient
    for name, _, _, _ in LAYERS:
        for q, what in ((0, "W"), (1, "b")):
            assert frob(g[name][q], G[name][q]) < 1e-1, (name, what, frob(g[name][q], G[name][q]))
    # layer by layer: each weight / bias gradient against numpy on the GPU's
    # own upstream gradient and input buffers (FP32 accumulation of BF16 products)
    def buf(name, c0, c, lvl):
        d = net.dims[lvl]
        a_ = net.A[name][:, c0:c0 + c].float().cpu().numpy().astype(np.float64)
        return a_.reshape(d[2], d[1], d[0], c)
    wb = net.wb
    pairs = {"head": (("dY", 0, 3, 0), ("D0b", 0, 24, 0)), "d0b": (("dD0b", 0, 24, 0), ("D0a", 0, 24, 0)),
             "d0a": (("dD0a", 0, 24, 0), ("CAT0", 0, 72, 0)), "d1b": (("dD1b", 0, 48, 1), ("D1a", 0, 48, 1)),
             "d1a": (("dD1a", 0, 48, 1), ("CAT1", 0, wb + 48, 1)), "bb": (("dBb", 0, wb, 2), ("Ba", 0, wb, 2)),
             "ba": (("dBa", 0, wb, 2), ("P2", 0, 48, 2)), "e1b": (("dCAT1", wb, 48, 1), ("E1a", 0, 48, 1)),
             "e1a": (("dE1a", 0, 48, 1), ("P1", 0, 24, 1)), "e0b": (("dCAT0", 48, 24, 0), ("E0a", 0, 24, 0)),
             "e0a": (("dE0a", 0, 24, 0), ("X0", 0, 3, 0))}
    for name, (dspec, ispec) in pairs.items():
        dpre, inp = buf(*dspec), buf(*ispec)
        W = P[name][0]
        _, dW, db = uo.conv_bwd(inp, W, dpre)
        assert frob(g[name][0], dW) < 3e-3, (name, "W kernel", frob(g[name][0], dW))
        assert frob(g[name][1], db) < 3e-3, (name, "b kernel", frob(g[name][1], db))
    # forward convolutions and input gradients, layer by layer, from GPU buffers
    fwd = {"e0b": ("E0a", 0, 24, 0, "CAT0", 48, 24), "d1a": ("CAT1", 0, wb + 48, 1, "D1a", 0, 48),
           "bb": ("Ba", 0, wb, 2, "Bb", 0, wb), "d0a": ("CAT0", 0, 72, 0, "D0a", 0, 24)}
    for name, (iname, i0, ic, lvl, oname, o0, oc) in fwd.items():
        ref = uo.relu(uo.conv(buf(iname, i0, ic, lvl), *P[name]))
        assert frob(buf(oname, o0, oc, lvl), ref) < 1e-2, (name, "forward kernel")
    # input gradient of d1a (the wb + 48 channel concatenation), before the pool / ReLU
    # updates of its skip part: the up part (channels 0..wb-1) is untouched afterwards
    dcat1 = uo.conv_bwd(buf("CAT1", 0, wb + 48, 1), P["d1a"][0], buf("dD1a", 0, 48, 1))[0]
    assert frob(buf("dCAT1", 0, wb, 1), dcat1[..., :wb]) < 1e-2, "input-gradient kernel"


@pytest.mark.gpu
def test_gpu_adam_step_reduces_loss():
    import torch
    from glemur_gb300.warmstart import UNet
    nx, ny, nz = 8, 8, 16
    net = UNet((nx, ny, nz), seed=4)
    rng = np.random.default_rng(2)
    X0 = np.zeros((nx * ny * nz, 8), np.float32)
    X0[:, :3] = rng.normal(size=(nx * ny * nz, 3))
    net.A["X0"].copy_(torch.from_numpy(X0).to(torch.bfloat16))
    tdev = torch.from_numpy(0.3 * rng.normal(size=(nx * ny * nz, 3)).astype(np.float32)).cuda()
    scale = 1.0 / (nx * ny * nz * 3)
    losses = []
    for it in range(30):
        net.zero_grad()
        net.forward()
        net.backward(tdev, scale)
        losses.append(float(net.loss_acc.item()))
        net.refresh_weights(lr=3e-3, step=True)
    net.check_status()
    assert losses[-1] < 0.5 * losses[0], losses


@pytest.mark.gpu
def test_gpu_input_and_loss_translation():
    """The augmentation: input and loss target read translated by whole cells."""
    import torch
    from glemur_gb300.warmstart import UNet
    nx, ny, nz = 8, 12, 16
    net = UNet((nx, ny, nz), seed=0)
    rng = np.random.default_rng(9)
    B0 = rng.normal(size=(nz + 2, ny + 2, nx + 2, 3)).astype(np.float32)
    sh = (3, 5)
    net.set_input_b0(torch.from_numpy(B0).cuda(), 32, sh)
    x = net.A["X0"][:, :3].float().cpu().numpy().reshape(nz, ny, nx, 3)
    ref = np.roll(B0[1:-1, 1:-1, 1:-1], (-sh[1], -sh[0]), axis=(1, 2)).astype(np.float64)
    ref[..., 2] -= 1.0
    assert np.abs(x - ref).max() < 1e-2 * np.abs(ref).max()
    tgt = rng.normal(size=(nz, ny, nx, 3)).astype(np.float32)
    net.zero_grad()
    net.forward()
    net.backward(torch.from_numpy(tgt.reshape(-1, 3)).cuda(), 1.0, sh)
    torch.cuda.synchronize()
    y = net.A["Y"][:, :3].float().cpu().numpy().reshape(nz, ny, nx, 3).astype(np.float64)
    e = y - np.roll(tgt, (-sh[1], -sh[0]), axis=(1, 2))
    e[0] = 0
    e[-1] = 0
    assert float(net.loss_acc.item()) == pytest.approx(float((e * e).sum()), rel=1e-3)


@pytest.mark.gpu
@pytest.mark.parametrize("smooth", [0, 2])
def test_gpu_warm_grid_matches_host_build(smooth):
    """gm_nn_warm_grid (smoothing, displacement, periodic images on the
    device) builds the grid the host path warm_grid builds, up to the float
    rounding of the smoothing (the host smooths in double)."""
    import torch
    from glemur_gb300 import configs
    from glemur_gb300.train_warmstart import DeviceWarmGrid, warm_grid
    from glemur_gb300.warmstart import UNet, load_weights, weights_width
    p = configs.random_braid(900003, shape=(64, 64, 128), precision=32)
    B0, xb0 = configs.init_state(p)
    w = load_weights()
    net = UNet((64, 64, 128), seed=0, wb=weights_width(w))
    net.load_state_dict(w)
    host = warm_grid(net, p, B0, smooth)
    dev = DeviceWarmGrid(p, xb0).build(net, torch.from_numpy(B0).cuda(), smooth).cpu().numpy()
    net.check_status()
    disp = np.abs(host.astype(np.float64) - xb0).max()
    assert disp > 0.1 * p.dx                       # the network moved the grid
    assert np.abs(dev.astype(np.float64) - host).max() <= 1e-5 * max(disp, 1.0)
    # line-tied z ghost planes and the held first / last inner planes stay at
    # the identity (away from the periodic images, which are recomputed)
    np.testing.assert_array_equal(dev[[0, 1, -2, -1], 1:-1, 1:-1], xb0[[0, 1, -2, -1], 1:-1, 1:-1])


def _sym_ref(a, sx, sy, sym):
    """numpy restatement of gm_nn_input's sample move on an inner array
    [nz][ny][nx][3]: cell (i, j) reads u = (i + sx) % nx, v = (j + sy) % ny,
    then 4: u <-> v, 2: v -> ny - 1 - v, 1: u -> nx - 1 - u; the x, y
    components negated (1, 2) and swapped (4)."""
    nz, ny, nx = a.shape[:3]
    i = np.arange(nx)[None, :].repeat(ny, 0)
    j = np.arange(ny)[:, None].repeat(nx, 1)
    u, v = (i + sx) % nx, (j + sy) % ny
    if sym & 4:
        u, v = v, u
    if sym & 2:
        v = ny - 1 - v
    if sym & 1:
        u = nx - 1 - u
    out = a[:, v, u].astype(np.float64)
    if sym & 1:
        out[..., 0] *= -1
    if sym & 2:
        out[..., 1] *= -1
    if sym & 4:
        out[..., [0, 1]] = out[..., [1, 0]]
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("sym", range(8))
def test_gpu_input_and_loss_symmetries(sym):
    """The mirror / swap augmentation of gm_nn_input and gm_nn_mse against
    numpy, with a translation: the input channels and the loss's target."""
    import torch
    from glemur_gb300.warmstart import UNet
    nx, ny, nz = 8, 8, 16
    net = UNet((nx, ny, nz), seed=0)
    rng = np.random.default_rng(10 + sym)
    B0 = rng.normal(size=(nz + 2, ny + 2, nx + 2, 3)).astype(np.float32)
    sh = (3, 5)
    net.set_input_b0(torch.from_numpy(B0).cuda(), 32, sh, sym)
    x = net.A["X0"][:, :3].float().cpu().numpy().reshape(nz, ny, nx, 3)
    ref = _sym_ref(B0[1:-1, 1:-1, 1:-1], sh[0], sh[1], sym)
    ref[..., 2] -= 1.0
    assert np.abs(x - ref).max() < 1e-2 * np.abs(ref).max()
    tgt = rng.normal(size=(nz, ny, nx, 3)).astype(np.float32)
    net.zero_grad()
    net.forward()
    net.backward(torch.from_numpy(tgt.reshape(-1, 3)).cuda(), 1.0, sh, sym)
    torch.cuda.synchronize()
    y = net.A["Y"][:, :3].float().cpu().numpy().reshape(nz, ny, nx, 3).astype(np.float64)
    e = y - _sym_ref(tgt, sh[0], sh[1], sym)
    e[0] = 0
    e[-1] = 0
    assert float(net.loss_acc.item()) == pytest.approx(float((e * e).sum()), rel=1e-3)


@pytest.mark.gpu
def test_gpu_input_refuses_swap_on_a_rectangle():
    import torch
    from glemur_gb300 import GlemurError
    from glemur_gb300.warmstart import UNet
    net = UNet((8, 12, 16), seed=0)
    B0 = torch.zeros((18, 14, 10, 3), dtype=torch.float32, device="cuda")
    with pytest.raises(GlemurError):
        net.set_input_b0(B0, 32, (0, 0), 4)
