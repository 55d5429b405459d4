"""tb_put_state / tb_get_state with page-locked host buffers the device can
address (moved by the SMs) against pageable numpy buffers (moved by the
copy engines): the same bytes both ways."""
import ctypes as C

import numpy as np
import pytest

from tests.helpers import NAMES, perturbed_state, small_case

pytestmark = pytest.mark.gpu


def test_pinned_and_pageable_copies_agree():
    torch = pytest.importorskip("torch")
    from trans_bl_gb300 import api
    cfg, coefs, base = small_case()
    g = api.Context(cfg, coefs, base)
    s1 = perturbed_state(cfg, base, np.random.default_rng(61))
    s2 = perturbed_state(cfg, base, np.random.default_rng(62))
    shape = (cfg.kfour, cfg.ny, cfg.nx, 2)
    pinned = {n: torch.empty(shape, dtype=torch.float64, pin_memory=True) for n in NAMES}
    D = C.POINTER(C.c_double)
    ptrs = [C.cast(pinned[n].data_ptr(), D) for n in NAMES]
    # pageable in, pinned out
    g.put_state(s1)
    api.check(g.lib.tb_get_state(g.h, *ptrs), "tb_get_state")
    for n in NAMES:
        got = pinned[n].numpy()
        assert np.array_equal(got[..., 0], s1[n].real) and np.array_equal(got[..., 1], s1[n].imag), n
    # pinned in, pageable out
    for n in NAMES:
        pinned[n].numpy()[...] = np.stack([s2[n].real, s2[n].imag], axis=-1)
    api.check(g.lib.tb_put_state(g.h, *ptrs), "tb_put_state")
    back = g.get_state()
    for n in NAMES:
        assert np.array_equal(back[n], s2[n]), n
    g.close()
