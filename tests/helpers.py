"""Shared test inputs: seeded synthetic states on the small parity grid."""
import numpy as np

from trans_bl_gb300 import api, configs

NAMES = configs.NAMES
smooth_random = configs.smooth_random


def small_case(**kw):
    cfg = configs.small(**kw)
    coefs, base = configs.setup_inputs(cfg)
    return cfg, coefs, base


def perturbed_state(cfg, base, rng, amp=1e-3):
    return configs.disturbed_state(cfg, base, rng, amp)


def rel(a, b):
    """max |a - b| / max |b| (inf-norm relative error)."""
    d = np.max(np.abs(np.asarray(a) - np.asarray(b)))
    s = np.max(np.abs(np.asarray(b)))
    return d / s if s > 0 else d
