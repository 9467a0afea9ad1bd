"""CPU oracle of the warm-start U-Net (test infrastructure only): forward and
backward of the same network as glemur_gb300/warmstart.py in float64 numpy,
for checking the GPU kernels' outputs and gradients.

Arrays are [nz, ny, nx, C]; convolutions are 3x3x3 with tap t = 9 (dk+1) +
3 (dj+1) + (di+1) reading x[k+dk, j+dj, i+di], periodic in x and y, zero
outside z; pooling is the 2x2x2 mean, upsampling nearest; the loss is
scale * sum over planes 1..nz-2 and channels 0..2 of (y - target)^2."""
import numpy as np

from glemur_gb300.warmstart import LAYERS


def shift(x, dk, dj, di):
    """x[k+dk, j+dj, i+di]: periodic in j, i; zero outside k."""
    y = np.roll(x, (-dj, -di), axis=(1, 2))
    out = np.zeros_like(y)
    nz = x.shape[0]
    if dk == 0:
        out[:] = y
    elif dk > 0:
        out[:nz - dk] = y[dk:]
    else:
        out[-dk:] = y[:nz + dk]
    return out


def taps():
    for t in range(27):
        yield t, t // 9 - 1, (t // 3) % 3 - 1, t % 3 - 1


def conv(x, W, b):
    out = np.zeros(x.shape[:3] + (W.shape[1],))
    for t, dk, dj, di in taps():
        out += shift(x, dk, dj, di) @ W[t].T
    return out + b


def conv_bwd(x, W, g):
    """Gradients of conv w.r.t. its input, weights and bias for upstream g."""
    dx = np.zeros_like(x)
    dW = np.zeros_like(W)
    for t, dk, dj, di in taps():
        xs = shift(x, dk, dj, di)
        dW[t] = np.einsum("zyxo,zyxi->oi", g, xs)
        dx += shift(g @ W[t], -dk, -dj, -di)
    return dx, dW, g.sum(axis=(0, 1, 2))


def pool(x):
    nz, ny, nx, c = x.shape
    return x.reshape(nz // 2, 2, ny // 2, 2, nx // 2, 2, c).mean(axis=(1, 3, 5))


def pool_bwd(g):
    return np.repeat(np.repeat(np.repeat(g, 2, 0), 2, 1), 2, 2) / 8.0


def up(x):
    return np.repeat(np.repeat(np.repeat(x, 2, 0), 2, 1), 2, 2)


def up_bwd(g):
    nz, ny, nx, c = g.shape
    return g.reshape(nz // 2, 2, ny // 2, 2, nx // 2, 2, c).sum(axis=(1, 3, 5))


def relu(x):
    return np.maximum(x, 0.0)


def forward(params, x):
    """params: name -> (W [27][co][ci], b [co]); x: [nz, ny, nx, 3]."""
    a = {}
    c = lambda n, inp, act=True: (relu if act else (lambda z: z))(conv(inp, *params[n]))
    a["e0a"] = c("e0a", x)
    a["e0b"] = c("e0b", a["e0a"])
    a["p1"] = pool(a["e0b"])
    a["e1a"] = c("e1a", a["p1"])
    a["e1b"] = c("e1b", a["e1a"])
    a["p2"] = pool(a["e1b"])
    a["ba"] = c("ba", a["p2"])
    a["bb"] = c("bb", a["ba"])
    a["cat1"] = np.concatenate([up(a["bb"]), a["e1b"]], axis=3)
    a["d1a"] = c("d1a", a["cat1"])
    a["d1b"] = c("d1b", a["d1a"])
    a["cat0"] = np.concatenate([up(a["d1b"]), a["e0b"]], axis=3)
    a["d0a"] = c("d0a", a["cat0"])
    a["d0b"] = c("d0b", a["d0a"])
    a["y"] = c("head", a["d0b"], act=False)
    return a


def loss_grad(y, target, scale):
    nz = y.shape[0]
    e = y - target
    e[0] = 0.0
    e[nz - 1] = 0.0
    return scale * float((e * e).sum()), 2.0 * scale * e


def backward(params, x, a, gy):
    g = {}
    def step(name, inp, gout, act_out=None):
        if act_out is not None:
            gout = gout * (act_out > 0)
        dx, dW, db = conv_bwd(inp, params[name][0], gout)
        g[name] = (dW, db)
        return dx
    d = step("head", a["d0b"], gy)
    d = step("d0b", a["d0a"], d, a["d0b"])
    dcat0 = step("d0a", a["cat0"], d, a["d0a"])
    c1 = a["d1b"].shape[3]
    d = up_bwd(dcat0[..., :c1])
    ds0 = dcat0[..., c1:]
    d = step("d1b", a["d1a"], d, a["d1b"])
    dcat1 = step("d1a", a["cat1"], d, a["d1a"])
    cb = a["bb"].shape[3]
    d = up_bwd(dcat1[..., :cb])
    ds1 = dcat1[..., cb:]
    d = step("bb", a["ba"], d, a["bb"])
    d = step("ba", a["p2"], d, a["ba"])
    ds1 = ds1 + pool_bwd(d)
    d = step("e1b", a["e1a"], ds1, a["e1b"])
    d = step("e1a", a["p1"], d, a["e1a"])
    ds0 = ds0 + pool_bwd(d)
    d = step("e0b", a["e0a"], ds0, a["e0b"])
    step("e0a", x, d, a["e0a"])
    return g


def layer_names():
    return [l[0] for l in LAYERS]
