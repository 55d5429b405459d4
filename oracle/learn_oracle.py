"""CPU restatement (float64 numpy) of the learned-correction network.

Test infrastructure only: the GPU library's forward, backward-data and
weight-gradient kernels (trans_bl_gb300/csrc/tb_learn.cu) are checked
against this file, and this file against finite differences.

The network has no counterpart in the reference, whose poi_uy starts from the
current v (poisson_par.f:6-30). Its definition:
  - four 3x3 convolutions with zero padding (cross-correlation, weights
    [cout][cin][ky][kx]), channels 4 -> 32 -> 32 -> 32 -> 1;
  - GELU(x) = x Phi(x) after the first three;
  - parameters packed layer by layer, weights then biases.
Training loss: mean squared error over the 64 x 64 interior of 72 x 72
crops; plane 4 of a crop is the target.
"""
import math

import numpy as np

LC, LIN, HALO, CROP = 32, 4, 4, 64
CW = CROP + 2 * HALO
SHAPES = [(LC, LIN), (LC, LC), (LC, LC), (1, LC)]


def param_count():
    return sum(o * i * 9 + o for o, i in SHAPES)


def unpack(w):
    w = np.asarray(w, dtype=np.float64)
    out, off = [], 0
    for o, i in SHAPES:
        W = w[off:off + o * i * 9].reshape(o, i, 3, 3)
        off += o * i * 9
        b = w[off:off + o]
        off += o
        out.append((W, b))
    assert off == w.size
    return out


def pack(layers):
    return np.concatenate([np.concatenate([W.ravel(), b.ravel()]) for W, b in layers])


_erf = np.vectorize(math.erf, otypes=[np.float64])


def gelu(x):
    return 0.5 * x * (1.0 + _erf(x / math.sqrt(2.0)))


def gelu_d(x):
    return 0.5 * (1.0 + _erf(x / math.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / math.sqrt(2.0 * math.pi)


def conv(x, W, b=None):
    """x (n, ci, H, Wd) -> (n, co, H, Wd): out[y, x] = sum W[ky, kx] in[y + ky - 1, x + kx - 1]."""
    n, ci, H, Wd = x.shape
    xp = np.pad(x, ((0, 0), (0, 0), (1, 1), (1, 1)))
    out = np.zeros((n, W.shape[0], H, Wd))
    for ky in range(3):
        for kx in range(3):
            out += np.einsum("nchw,oc->nohw", xp[:, :, ky:ky + H, kx:kx + Wd], W[:, :, ky, kx], optimize=True)
    if b is not None:
        out += b[None, :, None, None]
    return out


def conv_back_data(dp, W):
    """Gradient with respect to the input of conv(x, W)."""
    n, co, H, Wd = dp.shape
    dpp = np.pad(dp, ((0, 0), (0, 0), (1, 1), (1, 1)))
    dx = np.zeros((n, W.shape[1], H, Wd))
    for ky in range(3):
        for kx in range(3):
            dx += np.einsum("nohw,oc->nchw", dpp[:, :, 2 - ky:2 - ky + H, 2 - kx:2 - kx + Wd], W[:, :, ky, kx],
                            optimize=True)
    return dx


def conv_back_weights(x, dp):
    n, ci, H, Wd = x.shape
    xp = np.pad(x, ((0, 0), (0, 0), (1, 1), (1, 1)))
    dW = np.zeros((dp.shape[1], ci, 3, 3))
    for ky in range(3):
        for kx in range(3):
            dW[:, :, ky, kx] = np.einsum("nohw,nchw->oc", dp, xp[:, :, ky:ky + H, kx:kx + Wd], optimize=True)
    return dW, dp.sum(axis=(0, 2, 3))


def forward(w, x):
    """Output (n, H, Wd) and the cache of pre-activations and activations."""
    layers = unpack(w)
    acts, pres = [np.asarray(x, dtype=np.float64)], []
    for q, (W, b) in enumerate(layers):
        p = conv(acts[-1], W, b)
        pres.append(p)
        acts.append(gelu(p) if q < 3 else p)
    return acts[-1][:, 0], (acts, pres)


def interior_mask():
    m = np.zeros((CW, CW))
    m[HALO:HALO + CROP, HALO:HALO + CROP] = 1.0
    return m


def loss_grad(w, crops):
    """Mean squared error over the crop interiors and its gradient."""
    crops = np.asarray(crops, dtype=np.float64)
    x, t = crops[:, :LIN], crops[:, LIN]
    out, (acts, pres) = forward(w, x)
    m = interior_mask()[None]
    n = crops.shape[0] * CROP * CROP
    d = (out - t) * m
    loss = float((d * d).sum() / n)
    dp = (2.0 * d / n)[:, None]
    layers = unpack(w)
    grads = [None] * 4
    for q in range(3, -1, -1):
        W, _ = layers[q]
        grads[q] = conv_back_weights(acts[q], dp)
        if q > 0:
            dp = conv_back_data(dp, W) * gelu_d(pres[q - 1])
    return loss, pack(grads)


def init_weights(rng, last_scale=0.1):
    """He-normal weights, small biases; a nonzero last layer (for checks)."""
    layers = []
    for q, (o, i) in enumerate(SHAPES):
        s = math.sqrt(2.0 / (9 * i)) * (last_scale if q == 3 else 1.0)
        layers.append((rng.normal(0, s, (o, i, 3, 3)), rng.normal(0, 0.05, o)))
    return pack(layers)
