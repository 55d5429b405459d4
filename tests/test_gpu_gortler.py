"""Goertler form (my_form 1) against the CPU oracle.

drv_gv (main_par.f:1338-1401) with lterms_gv (nlterms_par.f:89-112): every
Fourier mode is a linear disturbance about the 2D base flow, with the wall
curvature terms of varg = Go^2 / sqrt(Re); the wall forcing is gv_pert
(main_par.f:1577-1610), the third mode's buffer ramp init_gv's second row
(main_par.f:991-996).  Compared term by term and through full RK4 steps, in
both precision forms, and replayed against host-launched steps.
"""
import numpy as np
import pytest

from tests.helpers import NAMES, rel

pytestmark = pytest.mark.gpu

TOL_TERMS = 1e-11
TOL_STEP = 1e-9
TOL_MIXED_STEP = 1e-6


def pair(oracle_built, go, seed, **kw):
    from trans_bl_gb300 import api, configs
    cfg = configs.gortler(go_number=go, **kw)
    coefs, base = configs.setup_inputs(cfg)
    g = api.Context(cfg, coefs, base)
    o = oracle_built.Oracle(cfg, coefs, base)
    st = configs.disturbance_state(cfg, np.random.default_rng(seed))
    g.put_state(st)
    o.put_state(st)
    return cfg, g, o


@pytest.mark.parametrize("go", [0.0, 8.0])
def test_drv_gv(oracle_built, go):
    cfg, g, o = pair(oracle_built, go, 51)
    for a, b in zip(g.drv(), o.drv()):
        assert np.max(np.abs(b)) > 0
        assert rel(a, b) < TOL_TERMS
    g.close()
    o.close()


def test_gv_pert_strip(oracle_built):
    """The strip goes into the wall row of modes k >= 1 only, ramped in the
    first period (t < stpp) and steady after it."""
    cfg, g, o = pair(oracle_built, 0.0, 52)
    for t in (cfg.stpp // 3, cfg.stpp + 7):
        g.ts_pert(t, 0.5)
        o.ts_pert(t, 0.5)
        a, b = g.get_state()["uy"], o.get_state()["uy"]
        assert rel(a, b) < 1e-15
        assert np.all(a[0, 0, :] == 0)           # mode 0 is not forced
        assert np.max(np.abs(b[1:, 0, :])) > 0
        assert rel(g.get_wall(), o.get_wall()) < 1e-15
    g.close()
    o.close()


@pytest.mark.parametrize("go", [0.0, 8.0])
def test_steps_gortler_plain(oracle_built, go):
    """Two RK4 steps in the ramp of the forcing and two after it."""
    cfg, g, o = pair(oracle_built, go, 53)
    for t in (cfg.stpp // 2, cfg.stpp // 2 + 1, cfg.stpp + 3, cfg.stpp + 4):
        g.step(t)
        o.step(t)
    a, b = g.get_state(), o.get_state()
    for n in NAMES:
        assert rel(a[n], b[n]) < TOL_STEP, n
    g.close()
    o.close()


def test_steps_gortler_mixed(oracle_built):
    from trans_bl_gb300 import api
    cfg, g, o = pair(oracle_built, 8.0, 54, precision=api.FORM_MIXED, max_vcycles=40)
    for t in (cfg.stpp + 3, cfg.stpp + 4):
        g.step(t)
        o.step(t)
    a, b = g.get_state(), o.get_state()
    for n in NAMES:
        assert rel(a[n], b[n]) < TOL_MIXED_STEP, n
    g.close()
    o.close()


def test_gortler_graph_matches_host_launched():
    """Recorded steps (the forcing amplitude of the ramp uploaded before each
    replay) equal host-launched ones bit for bit."""
    from trans_bl_gb300 import api, configs
    cfg = configs.gortler(go_number=8.0, precision=api.FORM_MIXED, max_vcycles=40)
    coefs, base = configs.setup_inputs(cfg)
    cfg_e = api.TbConfig.from_buffer_copy(cfg)
    cfg_e.step_graph = 0
    g = api.Context(cfg, coefs, base)
    e = api.Context(cfg_e, coefs, base)
    st = configs.disturbance_state(cfg, np.random.default_rng(55))
    for c in (g, e):
        c.put_state(st)
    for t in range(cfg.stpp - 2, cfg.stpp + 2):
        g.step(t)
        e.step(t)
        a, b = g.get_state(), e.get_state()
        for n in NAMES:
            assert np.array_equal(a[n], b[n]), (t, n)
    g.close()
    e.close()
