"""Spanwise transforms of the mixed nonlinear terms on the tensor cores.

The disturbance products go through two DFT-matrix GEMMs (tcgen05.mma,
three-part split-BF16 operands, FP32 accumulation); the mean terms stay in FP64.  The
result is checked against the FP64 oracle (nlterms_par.f) and against the
FP32 FFT passes, on grids whose point count is not a multiple of the
128-point tile, and through full mixed steps.
"""
import numpy as np
import pytest

from tests.helpers import NAMES, perturbed_state, rel, small_case

pytestmark = pytest.mark.gpu

GRIDS = [dict(nx=65, ny=33, kfour=16, kphys=32, msh=3),    # P = 32, 2145 points
         dict(nx=97, ny=49, kfour=32, kphys=64, msh=4)]    # P = 64, 4753 points


def pair(ora, grid, seed):
    from trans_bl_gb300 import api
    cfg, coefs, base = small_case(precision=api.FORM_MIXED, max_vcycles=40, **grid)
    g = api.Context(cfg, coefs, base)
    o = ora.Oracle(cfg, coefs, base)
    st = perturbed_state(cfg, base, np.random.default_rng(seed))
    g.put_state(st)
    o.put_state(st)
    return cfg, g, o


@pytest.mark.parametrize("grid", GRIDS)
def test_nlterms_tensor_cores(oracle_built, grid):
    cfg, g, o = pair(oracle_built, grid, 5)
    want = o.nlterms()
    got = g.nlterms()
    for a, b in zip(got, want):
        assert rel(a, b) < 1e-8
    # the quadratic disturbance term alone: tensor cores against the FP32 FFT
    g.nl_tensor_cores(False)
    fft = g.nlterms()
    for a, f, b in zip(got, fft, want):
        # the DFT as a 64-term dot product against the FFT's butterflies
        dq, dt = np.max(np.abs(f - b)), np.max(np.abs(a - b))
        print("\nP=%d quadratic-term error: FP32 FFT %.2e, tensor cores %.2e" % (cfg.kphys, dq, dt))
        assert dt < max(1024.0 * dq, 1e-14)
    g.close()
    o.close()


def test_steps_tensor_cores(oracle_built):
    cfg, g, o = pair(oracle_built, GRIDS[1], 9)
    t0 = cfg.stpp + 3
    for t in (t0, t0 + 1):
        g.step(t)
        o.step(t)
    a, b = g.get_state(), o.get_state()
    for n in NAMES:
        assert rel(a[n], b[n]) < 1e-6, n
    g.close()
    o.close()


def test_bounded_wait_times_out(oracle_built):
    """The tensor-core passes' wait for their MMAs is bounded: with the MMAs
    left unissued (a test switch) the wait runs out after a few thousand
    polls, the kernels free their tensor memory and return, the call reports
    TB_ERR_TIMEOUT, and the context computes correctly afterwards."""
    from trans_bl_gb300 import api
    cfg, g, o = pair(oracle_built, GRIDS[0], 5)
    api.check(g.lib.tb_tc_timeout_test(g.h, 1), "tb_tc_timeout_test")
    with pytest.raises(api.TbError, match="bounded wait"):
        g.nlterms()
    api.check(g.lib.tb_tc_timeout_test(g.h, 0), "tb_tc_timeout_test")
    for a, b in zip(g.nlterms(), o.nlterms()):
        assert rel(a, b) < 1e-8
    g.close()
    o.close()
