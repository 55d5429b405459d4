"""Shared test inputs: seeded synthetic states on the small parity grid."""
import numpy as np

from trans_bl_gb300 import api, configs

NAMES = ("ux", "uy", "uz", "wx", "wy", "wz")


def small_case(**kw):
    cfg = configs.small(**kw)
    coefs, base = configs.setup_inputs(cfg)
    return cfg, coefs, base


def smooth_random(shape, rng, scale=1.0):
    """Complex field with mode 0 real, smooth in x and y (sum of few waves)."""
    K, ny, nx = shape
    x = np.linspace(0, 1, nx)[None, :]
    y = np.linspace(0, 1, ny)[:, None]
    f = np.zeros(shape, dtype=np.complex128)
    for k in range(K):
        acc = np.zeros((ny, nx), dtype=np.complex128)
        for _ in range(3):
            a, b = rng.uniform(0.5, 4.0, 2)
            p = rng.uniform(0, 2 * np.pi, 2)
            c = rng.normal() + 1j * rng.normal()
            acc += c * np.sin(a * np.pi * x + p[0]) * np.cos(b * np.pi * y + p[1])
        f[k] = acc * scale / (1 + k)
    f[0] = f[0].real
    return f


def perturbed_state(cfg, base, rng, amp=1e-3):
    uxb, uyb, wzb = base
    st = {}
    for n in NAMES:
        st[n] = smooth_random((cfg.kfour, cfg.ny, cfg.nx), rng, amp)
    for n in ("ux", "uy", "uz"):   # no-slip wall row, as in every state of a run
        st[n][:, 0, :] = 0.0
    st["ux"][0] += uxb
    st["uy"][0] += uyb
    st["wz"][0] += wzb
    return st


def rel(a, b):
    """max |a - b| / max |b| (inf-norm relative error)."""
    d = np.max(np.abs(np.asarray(a) - np.asarray(b)))
    s = np.max(np.abs(np.asarray(b)))
    return d / s if s > 0 else d
