"""The allocation-free filter entry point (tb_filter_trid_noalloc).

It exists for hosts that cannot allocate GPU memory once their time loop
runs -- a memory manager that has taken every free byte of the device, or a
real-time section where an allocation may stall the device -- so it works on
the caller's device buffers and stages its lines in an array built into the
library.  Here it is
run through the C ABI on the device fields of one context and compared with
the context-based filter (tb_filter_trid) on an identical context, for two
calls in a row, within the single-sweep tolerance of the parity tests.
This file is collected last so that a stop-at-first-failure run has already
run every other test.
"""
import numpy as np
import pytest

from tests.helpers import perturbed_state, rel, small_case

pytestmark = pytest.mark.gpu

TOL_SWEEP = 1e-12


def test_noalloc_filter_matches_context_filter():
    from trans_bl_gb300 import api
    cfg, coefs, base = small_case()
    ref = api.Context(cfg, coefs, base)
    dev = api.Context(cfg, coefs, base)
    st = perturbed_state(cfg, base, np.random.default_rng(21))
    ref.put_state(st)
    dev.put_state(st)
    ptr = [dev.device_field(w) for w in (3, 4, 5)]  # wx, wy, wz
    lib = api.load()
    for call in range(2):
        ref.filter_trid()
        rc = lib.tb_filter_trid_noalloc(ptr[0], ptr[1], ptr[2], cfg.nx, cfg.ny, cfg.kfour, cfg.alphaf, dev.stream())
        api.check(rc, "tb_filter_trid_noalloc")
        dev.synchronize()
        a, b = dev.get_state(), ref.get_state()
        for n in ("wx", "wy", "wz"):
            assert rel(a[n], b[n]) < TOL_SWEEP, (call, n)
        for n in ("ux", "uy", "uz"):
            assert np.array_equal(a[n], b[n])


def test_noalloc_filter_rejects_oversize():
    from trans_bl_gb300 import api
    cfg, coefs, base = small_case()
    dev = api.Context(cfg, coefs, base)
    ptr = [dev.device_field(w) for w in (3, 4, 5)]
    lib = api.load()
    rc = lib.tb_filter_trid_noalloc(ptr[0], ptr[1], ptr[2], 1025, 193, 32, 0.48, dev.stream())
    assert rc == 1
    assert b"exceeds" in lib.tb_last_error()


def test_noalloc_filter_by_slices_of_modes():
    """A grid filtered one slice of Fourier modes per call (pointer offsets,
    a smaller kfour) gives the whole-field call's result."""
    from trans_bl_gb300 import api
    cfg, coefs, base = small_case()
    whole = api.Context(cfg, coefs, base)
    parts = api.Context(cfg, coefs, base)
    st = perturbed_state(cfg, base, np.random.default_rng(23))
    whole.put_state(st)
    parts.put_state(st)
    lib = api.load()
    pw = [whole.device_field(w) for w in (3, 4, 5)]
    pp = [parts.device_field(w) for w in (3, 4, 5)]
    api.check(lib.tb_filter_trid_noalloc(pw[0], pw[1], pw[2], cfg.nx, cfg.ny, cfg.kfour, cfg.alphaf,
                                         whole.stream()), "tb_filter_trid_noalloc")
    whole.synchronize()   # calls that overlap on the GPU race on the shared scratch array
    k1 = cfg.kfour // 2
    step = cfg.nx * cfg.ny * 16   # bytes per Fourier mode of a complex*16 field
    for k0, nk in ((0, k1), (k1, cfg.kfour - k1)):
        api.check(lib.tb_filter_trid_noalloc(pp[0] + k0 * step, pp[1] + k0 * step, pp[2] + k0 * step, cfg.nx,
                                             cfg.ny, nk, cfg.alphaf, parts.stream()), "tb_filter_trid_noalloc")
    whole.synchronize()
    parts.synchronize()
    a, b = parts.get_state(), whole.get_state()
    for n in ("wx", "wy", "wz"):
        assert np.array_equal(a[n], b[n]), n


def test_noalloc_filter_rejects_long_lines():
    from trans_bl_gb300 import api
    cfg, coefs, base = small_case()
    dev = api.Context(cfg, coefs, base)
    ptr = [dev.device_field(w) for w in (3, 4, 5)]
    lib = api.load()
    rc = lib.tb_filter_trid_noalloc(ptr[0], ptr[1], ptr[2], 4097, 2, 1, 0.48, dev.stream())
    assert rc == 1
    assert b"nx" in lib.tb_last_error()
