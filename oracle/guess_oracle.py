"""CPU restatement (numpy, float64) of the pressure-guess network.

TEST INFRASTRUCTURE ONLY: imported by tests/ to check the CUDA network's
forward pass, gradients and Adam update; never called by the product path.

The reference has no learned component; this network is the one the CUDA
path builds (fluid-sim_gb300/csrc/fs_guess.cu), restated here so that its
gradients can be checked independently.  Both sides use:

* images NHWC, periodic 3x3 convolutions (x, y wrapped);
* channels 16/32/64/128 over four levels, 2x2 average pooling down,
  nearest-neighbour upsampling plus an additive skip up, ReLU after every
  convolution but the last;
* parameters flattened layer by layer, each layer as w[co][ci][3][3] then
  b[co];
* the loss, with e = out - target (pressure is defined up to a constant):
  L = w_p sum (e - mean_b e)^2 / (B H W) + w_r sum (lap e)^2 / (B H W),
  lap the periodic 5-point stencil l + r + b + t - 4c (unscaled: in the
  network's units lap p_n = div_n, so the second term is the initial residual
  of the projection the guess seeds).

``rnd`` (optional) rounds a tensor to the device's storage type at each point
where the device stores one in bf16 -- the convolution weights, every
activation and every activation gradient -- so the comparison can be tight.
(Biases stay f32 on the device and are not rounded.)
"""
from __future__ import annotations

import numpy as np

# (name, c_in, c_out, relu)
LAYERS = [
    ("A", 16, 16, True),    # input (2 real channels, padded to 16) -> 16, level 0
    ("B", 16, 16, True),    # level 0
    ("C", 16, 32, True),    # level 1, after pooling
    ("D", 32, 64, True),    # level 2
    ("E", 64, 128, True),   # level 3
    ("F", 128, 64, True),   # level 3, then up to level 2 + skip
    ("G", 64, 32, True),    # level 2, then up to level 1 + skip
    ("H", 32, 16, True),    # level 1, then up to level 0 + skip
    ("I", 16, 16, True),    # level 0
    ("J", 16, 16, False),   # level 0 output; channel 0 is the pressure guess
]
IN_CHANNELS = 16
REAL_IN = 2  # normalised divergence, solid mask


def layer_sizes():
    return [(n, ci * co * 9, co) for n, ci, co, _ in LAYERS]


def num_params():
    return sum(w + b for _, w, b in layer_sizes())


def unflatten(theta):
    out, k = {}, 0
    for n, ci, co, _ in LAYERS:
        w = theta[k:k + ci * co * 9].reshape(co, ci, 3, 3)
        k += ci * co * 9
        b = theta[k:k + co]
        k += co
        out[n] = (w, b)
    return out


def flatten(grads):
    return np.concatenate([np.concatenate([grads[n][0].ravel(), grads[n][1].ravel()]) for n, *_ in LAYERS])


def init_params(seed=0):
    """He-normal weights (the last layer scaled down), zero biases; float32."""
    rng = np.random.default_rng(seed)
    parts = []
    for n, ci, co, relu in LAYERS:
        fan_in = 9 * (REAL_IN if n == "A" else ci)
        std = np.sqrt(2.0 / fan_in) * (1.0 if relu else 0.1)
        w = rng.standard_normal((co, ci, 3, 3)) * std
        if n == "A":
            w[:, REAL_IN:] = 0.0
        parts += [w.ravel(), np.zeros(co)]
    return np.concatenate(parts).astype(np.float32)


# ----------------------------------------------------------------- operators
def conv(x, w, b):
    """out[b,y,x,o] = b[o] + sum_{ky,kx,c} w[o,c,ky,kx] x[b, y+ky-1, x+kx-1, c] (periodic)."""
    out = np.zeros(x.shape[:3] + (w.shape[0],))
    for ky in range(3):
        for kx in range(3):
            xs = np.roll(x, shift=(-(ky - 1), -(kx - 1)), axis=(1, 2))
            out += xs @ w[:, :, ky, kx].T
    return out + b


def conv_grad_input(g, w):
    dx = np.zeros(g.shape[:3] + (w.shape[1],))
    for ky in range(3):
        for kx in range(3):
            dx += np.roll(g @ w[:, :, ky, kx], shift=(ky - 1, kx - 1), axis=(1, 2))
    return dx


def conv_grad_weight(x, g):
    co, ci = g.shape[3], x.shape[3]
    dw = np.zeros((co, ci, 3, 3))
    gf = g.reshape(-1, co)
    for ky in range(3):
        for kx in range(3):
            xs = np.roll(x, shift=(-(ky - 1), -(kx - 1)), axis=(1, 2)).reshape(-1, ci)
            dw[:, :, ky, kx] = gf.T @ xs
    return dw, gf.sum(axis=0)


def pool(x):
    B, H, W, C = x.shape
    return x.reshape(B, H // 2, 2, W // 2, 2, C).mean(axis=(2, 4))


def up(x):
    return x.repeat(2, axis=1).repeat(2, axis=2)


def pool_sum(g):
    B, H, W, C = g.shape
    return g.reshape(B, H // 2, 2, W // 2, 2, C).sum(axis=(2, 4))


def _id(x):
    return x


# ------------------------------------------------------------------- network
def make_input(div_n, mask):
    """[B][H][W] normalised divergence and mask -> [B][H][W][16]."""
    x = np.zeros(div_n.shape + (IN_CHANNELS,))
    x[..., 0] = div_n
    x[..., 1] = mask
    return x


def _params(theta, rnd):
    P = unflatten(np.asarray(theta, np.float64))
    if rnd is not _id:
        P = {n: (rnd(w), b) for n, (w, b) in P.items()}
    return P


def forward(theta, x0, rnd=_id):
    P = _params(theta, rnd)
    relu = lambda t: np.maximum(t, 0.0)
    a = {"x0": rnd(x0)}
    a["a0"] = rnd(relu(conv(a["x0"], *P["A"])))
    a["a0b"] = rnd(relu(conv(a["a0"], *P["B"])))
    a["q1"] = rnd(pool(a["a0b"]))
    a["a1"] = rnd(relu(conv(a["q1"], *P["C"])))
    a["q2"] = rnd(pool(a["a1"]))
    a["a2"] = rnd(relu(conv(a["q2"], *P["D"])))
    a["q3"] = rnd(pool(a["a2"]))
    a["a3"] = rnd(relu(conv(a["q3"], *P["E"])))
    a["f3"] = rnd(relu(conv(a["a3"], *P["F"])))
    a["s2"] = rnd(up(a["f3"]) + a["a2"])
    a["g2"] = rnd(relu(conv(a["s2"], *P["G"])))
    a["s1"] = rnd(up(a["g2"]) + a["a1"])
    a["h1"] = rnd(relu(conv(a["s1"], *P["H"])))
    a["s0"] = rnd(up(a["h1"]) + a["a0b"])
    a["i0"] = rnd(relu(conv(a["s0"], *P["I"])))
    a["out"] = conv(a["i0"], *P["J"])[..., 0]
    return a["out"], a


def lap5(e):
    return (np.roll(e, 1, 1) + np.roll(e, -1, 1) + np.roll(e, 1, 2) + np.roll(e, -1, 2) - 4 * e)


def loss_and_seed(out, target, w_p=1.0, w_r=0.0):
    B = out.shape[0]
    n = out[0].size
    e = out - target
    ec = e - e.reshape(B, -1).mean(axis=1)[:, None, None]
    r = lap5(e)
    L = (w_p * (ec ** 2).sum() + w_r * (r ** 2).sum()) / (B * n)
    g = (w_p * 2.0 * ec + w_r * 2.0 * lap5(r)) / (B * n)
    return float(L), g


def backward(theta, acts, gout, rnd=_id):
    """Gradient of the loss w.r.t. the flattened parameters, given dL/dout."""
    P = _params(theta, rnd)
    a = acts
    G = {}
    mask = lambda g, t: g * (t > 0)
    gJ = np.zeros(gout.shape + (16,))
    gJ[..., 0] = gout
    gJ = rnd(gJ)
    G["J"] = conv_grad_weight(a["i0"], gJ)
    di0 = rnd(conv_grad_input(gJ, P["J"][0]))
    di0 = mask(di0, a["i0"])
    G["I"] = conv_grad_weight(a["s0"], di0)
    ds0 = rnd(conv_grad_input(di0, P["I"][0]))
    dh1 = mask(rnd(pool_sum(ds0)), a["h1"])
    G["H"] = conv_grad_weight(a["s1"], dh1)
    ds1 = rnd(conv_grad_input(dh1, P["H"][0]))
    dg2 = mask(rnd(pool_sum(ds1)), a["g2"])
    G["G"] = conv_grad_weight(a["s2"], dg2)
    ds2 = rnd(conv_grad_input(dg2, P["G"][0]))
    df3 = mask(rnd(pool_sum(ds2)), a["f3"])
    G["F"] = conv_grad_weight(a["a3"], df3)
    da3 = mask(rnd(conv_grad_input(df3, P["F"][0])), a["a3"])
    G["E"] = conv_grad_weight(a["q3"], da3)
    dq3 = rnd(conv_grad_input(da3, P["E"][0]))
    da2 = mask(rnd(ds2 + 0.25 * up(dq3)), a["a2"])
    G["D"] = conv_grad_weight(a["q2"], da2)
    dq2 = rnd(conv_grad_input(da2, P["D"][0]))
    da1 = mask(rnd(ds1 + 0.25 * up(dq2)), a["a1"])
    G["C"] = conv_grad_weight(a["q1"], da1)
    dq1 = rnd(conv_grad_input(da1, P["C"][0]))
    da0b = mask(rnd(ds0 + 0.25 * up(dq1)), a["a0b"])
    G["B"] = conv_grad_weight(a["a0"], da0b)
    da0 = mask(rnd(conv_grad_input(da0b, P["B"][0])), a["a0"])
    G["A"] = conv_grad_weight(a["x0"], da0)
    return flatten(G)


def loss_grad(theta, div_n, mask, target, rnd=_id, w_p=1.0, w_r=0.0):
    out, acts = forward(theta, make_input(div_n, mask), rnd)
    L, gout = loss_and_seed(out, target, w_p, w_r)
    return L, backward(theta, acts, gout, rnd), out


def adam(theta, grad, m, v, t, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam step (Kingma & Ba 2015) with bias correction; t starts at 1."""
    m = b1 * m + (1 - b1) * grad
    v = b2 * v + (1 - b2) * grad * grad
    mh = m / (1 - b1 ** t)
    vh = v / (1 - b2 ** t)
    return theta - lr * mh / (np.sqrt(vh) + eps), m, v
