"""CPU restatement (float64 numpy) of the learned-correction network.

Test infrastructure only: the GPU library's forward, backward-data and
weight-gradient kernels (trans_bl_gb300/csrc/tb_learn.cu) are checked
against this file, and this file against finite differences.

The network has no counterpart in the reference, whose poi_uy starts from the
current v (poisson_par.f:6-30). Its definition:
  - four 3x3 convolutions with zero padding (cross-correlation, weights
    [cout][cin][ky][kx]), channels 4 -> 32 -> 32 -> 32 -> 1;
  - input plane p divided by an input scale a_p before the first layer;
  - GELU(x) = x Phi(x) after the first three;
  - the result times an output scale s;
  - parameters packed layer by layer, weights then biases, then a_0..a_3, s.
Training loss (defect_loss_grad): the defect a correction leaves, the
correction being e = s * output on the grid's interior,
  mean over the 64 x 64 crop interiors of (w_k (d0 - L e))^2,
with d0 = plane 2 / (1/|D|) (plane 2 holds D^-1 d0), L the finest FP32
operator of the mixed Poisson form (fine_terms, restating the residual kernel
of trans_bl_gb300/csrc/tb_mixed.cu, itself the defect of poisson_par.f:543-793)
and w_k the mode's smallest 1/|D|.  The scales are fixed during training
(their gradients are zero).
"""
import math

import numpy as np

LC, LIN, HALO, CROP = 32, 4, 4, 64
CW = CROP + 2 * HALO
SHAPES = [(LC, LIN), (LC, LC), (LC, LC), (1, LC)]


NSCALE = LIN + 1


def param_count():
    return sum(o * i * 9 + o for o, i in SHAPES) + NSCALE


def unpack(w):
    w = np.asarray(w, dtype=np.float64)
    out, off = [], 0
    for o, i in SHAPES:
        W = w[off:off + o * i * 9].reshape(o, i, 3, 3)
        off += o * i * 9
        b = w[off:off + o]
        off += o
        out.append((W, b))
    assert off + NSCALE == w.size
    return out


def out_scale(w):
    return float(np.asarray(w, dtype=np.float64)[-1])


def in_scales(w):
    return np.asarray(w, dtype=np.float64)[-NSCALE:-1]


def pack(layers, scale=1.0, iscale=(1.0, 1.0, 1.0, 1.0)):
    return np.concatenate([np.concatenate([W.ravel(), b.ravel()]) for W, b in layers] +
                          [np.asarray(iscale, dtype=np.float64), np.array([scale])])


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


def forward(w, x, scaled=True):
    """Output (n, H, Wd) and the cache of pre-activations and activations.
    scaled: x holds the raw planes, and the input and output scales apply;
    otherwise x is already divided by the input scales and the output is
    unscaled (the training form)."""
    layers = unpack(w)
    x = np.asarray(x, dtype=np.float64)
    if scaled:
        x = x / in_scales(w)[None, :, None, None]
    acts, pres = [x], []
    for q, (W, b) in enumerate(layers):
        p = conv(acts[-1], W, b)
        pres.append(p)
        acts.append(gelu(p) if q < 3 else p)
    out = acts[-1][:, 0]
    return (out * out_scale(w) if scaled else out), (acts, pres)


def init_weights(rng, last_scale=0.1, scale=1.0, iscale=(1.0, 1.0, 1.0, 1.0)):
    """He-normal weights, small biases; a nonzero last layer (for checks)."""
    layers = []
    for q, (o, i) in enumerate(SHAPES):
        s = math.sqrt(2.0 / (9 * i)) * (last_scale if q == 3 else 1.0)
        layers.append((rng.normal(0, s, (o, i, 3, 3)), rng.normal(0, 0.05, o)))
    return pack(layers, scale, iscale)


# ---- the finest operator and the defect loss -------------------------------
def split_tables(tab, ny):
    """Operator tables of one mode: den, ify, alpha2, k2b2, w_k, coef(24),
    qdy2(ny), invD(ny)."""
    tab = np.asarray(tab, dtype=np.float64)
    return dict(den=tab[0], ify=tab[1], alpha2=tab[2], k2=tab[3], wk=tab[4], coef=tab[5:29],
                qdy2=tab[29:29 + ny], invD=tab[29 + ny:29 + 2 * ny])


def fine_terms(T, nx, ny, i, j):
    """(i', j', c) of L e at interior point (i, j)."""
    SP, CP, PP, LP = T["coef"][0:7], T["coef"][7:15], T["coef"][15:19], T["coef"][19:24]
    den, ify, k2, q = T["den"], T["ify"], T["k2"], T["qdy2"]
    out = []

    def xs(jj, w):
        if i == 1 or i == nx - 2:
            e = 1 if i == 1 else -1
            for a, c in ((-e, 10.0), (0, -15.0), (e, -4.0), (2 * e, 14.0), (3 * e, -6.0), (4 * e, 1.0)):
                out.append((i + a, jj, c * w))
        else:
            for a, c in ((-2, -1.0), (-1, 16.0), (0, -30.0), (1, 16.0), (2, -1.0)):
                out.append((i + a, jj, c * w))
    n = ny
    if j == 1:
        q2 = q[0]
        xs(2, SP[2] * den); xs(1, SP[1] * den)
        out += [(i, 0, SP[3] * q2), (i, 1, SP[4] * q2 + k2 * SP[1] * ify), (i, 2, SP[5] * q2 + k2 * SP[2] * ify),
                (i, 3, SP[6] * q2)]
    elif j <= n - 3:
        q2 = q[j - 2]
        xs(j - 1, CP[0] * den); xs(j, CP[1] * den); xs(j + 1, CP[2] * den)
        out += [(i, j - 2, CP[3] * q2), (i, j - 1, CP[4] * q2 + k2 * CP[0] * ify), (i, j, CP[5] * q2 + k2 * CP[1] * ify),
                (i, j + 1, CP[6] * q2 + k2 * CP[2] * ify), (i, j + 2, CP[7] * q2)]
    elif j == n - 2:
        q2 = q[j - 1]
        xs(j, den)
        out += [(i, j - 1, PP[1] * q2), (i, j, PP[2] * q2 + k2 * ify), (i, j + 1, PP[3] * q2)]
    else:
        q2 = q[j - 2]
        top = LP[1] * math.sqrt((T["alpha2"] - k2) * ify) * math.sqrt(q2)
        xs(j, den)
        out += [(i, j, LP[2] * q2 + k2 * ify - top), (i, j - 1, LP[3] * q2), (i, j - 2, LP[4] * q2)]
    return out


def apply_L(T, nx, ny, e):
    """L e on the interior of an (nx, ny) field (0 elsewhere)."""
    out = np.zeros((nx, ny))
    for i in range(1, nx - 1):
        for j in range(1, ny):
            out[i, j] = sum(c * e[a, b] for a, b, c in fine_terms(T, nx, ny, i, j))
    return out


def _inner(nx, ny, i, j):
    return 1 <= i <= nx - 2 and 1 <= j <= ny - 1


def defect_loss_grad(w, crops, meta, tables, nx, ny):
    """Defect loss over crops (n, 5, CW, CW) with meta (n, 3) = image 2k+part,
    first row, first column, and per-mode tables; returns loss and gradient."""
    crops = np.asarray(crops, dtype=np.float64)
    isc = in_scales(w)
    x = crops[:, :LIN] / isc[None, :, None, None]
    out, (acts, pres) = forward(w, x, scaled=False)
    sc = out_scale(w)
    n = crops.shape[0]
    N = n * CROP * CROP
    loss = 0.0
    dout = np.zeros_like(out)
    for b in range(n):
        k, i0, j0 = int(meta[b][0]) >> 1, int(meta[b][1]), int(meta[b][2])
        T = tables[k]
        m = np.array([[1.0 if _inner(nx, ny, i0 + y, j0 + xx) else 0.0 for xx in range(CW)] for y in range(CW)])
        e = sc * out[b] * m
        g = np.zeros((CW, CW))
        for y in range(HALO, HALO + CROP):
            for xx in range(HALO, HALO + CROP):
                i, j = i0 + y, j0 + xx
                if not _inner(nx, ny, i, j):
                    continue
                terms = fine_terms(T, nx, ny, i, j)
                le = sum(c * e[a - i0, bb - j0] for a, bb, c in terms)
                rho = T["wk"] * (crops[b, 2, y, xx] / T["invD"][j] - le)
                loss += rho * rho / N
                for a, bb, c in terms:
                    g[a - i0, bb - j0] += c * T["wk"] * rho
        dout[b] = -2.0 * sc / N * m * g
    layers = unpack(w)
    dp = dout[:, None]
    grads = [None] * 4
    for q in range(3, -1, -1):
        W, _ = layers[q]
        grads[q] = conv_back_weights(acts[q], dp)
        if q > 0:
            dp = conv_back_data(dp, W) * gelu_d(pres[q - 1])
    return loss, pack(grads, 0.0, np.zeros(LIN))
