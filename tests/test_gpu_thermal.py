"""Thermal form (my_form 2) against the CPU oracle.

drv_gvth with nlterms_th (main_par.f:1404-1484, nlterms_par.f:216-300): the
disturbance with its full nonlinear products about the 2D base flow (uxb,
uyb, wzb) and base temperature thb, the momentum terms of drv_gv, and a
transported temperature th with its own RK update (main_par.f:354-445) and
buffer zone (loop_par.f:36-39); ts2d_pert forces it.  Full RK4 steps in both
precision forms, replayed against host-launched steps, and the API's form
checks.
"""
import numpy as np
import pytest

from tests.helpers import NAMES, rel

pytestmark = pytest.mark.gpu


def thermal_pair(oracle_built, seed, **kw):
    from trans_bl_gb300 import api, configs
    cfg = configs.thermal(**kw)
    coefs, base = configs.setup_inputs(cfg)
    thb = configs.base_temperature(cfg, base)
    rng = np.random.default_rng(seed)
    st = configs.disturbance_state(cfg, rng)
    th = configs.smooth_random((cfg.kfour, cfg.ny, cfg.nx), rng, 1e-3)
    th[:, 0, :] = 0.0
    th[:, -1, :] = 0.0
    g = api.Context(cfg, coefs, base)
    o = oracle_built.Oracle(cfg, coefs, base)
    for c in (g, o):
        c.set_baseflow_th(thb)
        c.put_state(st)
        c.put_th(th)
    return cfg, g, o


def test_steps_thermal_plain(oracle_built):
    cfg, g, o = thermal_pair(oracle_built, 71)
    for t in (cfg.stpp + 3, cfg.stpp + 4):
        g.step(t)
        o.step(t)
    a, b = g.get_state(), o.get_state()
    for n in NAMES:
        assert rel(a[n], b[n]) < 1e-9, n
    assert rel(g.get_th(), o.get_th()) < 1e-9
    g.close()
    o.close()


def test_steps_thermal_mixed(oracle_built):
    from trans_bl_gb300 import api
    cfg, g, o = thermal_pair(oracle_built, 72, precision=api.FORM_MIXED, max_vcycles=40)
    for t in (cfg.stpp + 3, cfg.stpp + 4):
        g.step(t)
        o.step(t)
    a, b = g.get_state(), o.get_state()
    for n in NAMES:
        assert rel(a[n], b[n]) < 1e-6, n
    assert rel(g.get_th(), o.get_th()) < 1e-6
    g.close()
    o.close()


def test_thermal_graph_matches_host_launched():
    from trans_bl_gb300 import api, configs
    cfg = configs.thermal(precision=api.FORM_MIXED, max_vcycles=40)
    coefs, base = configs.setup_inputs(cfg)
    thb = configs.base_temperature(cfg, base)
    rng = np.random.default_rng(73)
    st = configs.disturbance_state(cfg, rng)
    th = configs.smooth_random((cfg.kfour, cfg.ny, cfg.nx), rng, 1e-3)
    cfg_e = api.TbConfig.from_buffer_copy(cfg)
    cfg_e.step_graph = 0
    g = api.Context(cfg, coefs, base)
    e = api.Context(cfg_e, coefs, base)
    for c in (g, e):
        c.set_baseflow_th(thb)
        c.put_state(st)
        c.put_th(th)
    for t in range(cfg.stpp + 1, cfg.stpp + 4):
        g.step(t)
        e.step(t)
        a, b = g.get_state(), e.get_state()
        for n in NAMES:
            assert np.array_equal(a[n], b[n]), (t, n)
        assert np.array_equal(g.get_th(), e.get_th()), t
    g.close()
    e.close()


def test_temperature_only_in_the_thermal_form():
    from trans_bl_gb300 import api, configs
    cfg = configs.small()
    coefs, base = configs.setup_inputs(cfg)
    g = api.Context(cfg, coefs, base)
    with pytest.raises(api.TbError):
        g.put_th(np.zeros((cfg.kfour, cfg.ny, cfg.nx), dtype=np.complex128))
    g.close()


def test_thermal_checkpoint(tmp_path):
    """escreve's form-2 record (escreve_par.f:11-17): the step, then ux uy
    uz wx wy wz th in one record; a fresh context reads the same state."""
    import struct
    from trans_bl_gb300 import api, configs
    cfg = configs.thermal()
    coefs, base = configs.setup_inputs(cfg)
    rng = np.random.default_rng(74)
    st = configs.disturbance_state(cfg, rng)
    th = configs.smooth_random((cfg.kfour, cfg.ny, cfg.nx), rng, 1e-3)
    g = api.Context(cfg, coefs, base)
    g.put_state(st)
    g.put_th(th)
    path = str(tmp_path / "data_00.bin")
    g.write_checkpoint(path, 17)
    data = open(path, "rb").read()
    n3 = cfg.nx * cfg.ny * cfg.kfour
    assert struct.unpack("<i", data[:4])[0] == 4
    assert struct.unpack("<i", data[12:16])[0] == 7 * n3 * 16
    h = api.Context(cfg, coefs, base)
    assert h.read_checkpoint(path) == 17
    a = h.get_state()
    for n in NAMES:
        assert np.array_equal(a[n], st[n]), n
    assert np.array_equal(h.get_th(), th)
    g.close()
    h.close()
