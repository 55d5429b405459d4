"""Steps replayed as CUDA graphs, and ensembles, against host-launched steps.

A recorded step runs the kernels of the host-launched step with the same
arguments in the same order; only the decision to run another Poisson
correction moves to the device (a conditional WHILE node).  So replayed
steps must give bit-identical fields, the same per-mode correction counts
and the same number of kernel launches, including across the warm-start
bookkeeping (consecutive steps, a gap in the step index, a new state).  An
ensemble of uneven runs replays every member's step in one graph and must
match each member stepped on its own.
"""
import numpy as np
import pytest

from tests.helpers import NAMES, perturbed_state, small_case

pytestmark = pytest.mark.gpu


def ctx_pair(seed=7, **kw):
    from trans_bl_gb300 import api
    cfg, coefs, base = small_case(precision=api.FORM_MIXED, **kw)
    cfg_e = api.TbConfig.from_buffer_copy(cfg)
    cfg_e.step_graph = 0
    g = api.Context(cfg, coefs, base)
    e = api.Context(cfg_e, coefs, base)
    st = perturbed_state(cfg, base, np.random.default_rng(seed))
    g.put_state(st)
    e.put_state(st)
    return cfg, g, e


def same(a, b):
    for n in NAMES:
        assert np.array_equal(a[n], b[n]), n


def stats(ctx):
    s = ctx.poisson_stats()
    return list(s["vcycles"]), s["total_vcycles"], s["solves"]


@pytest.mark.parametrize("grid", [dict(), dict(nx=97, ny=49, kfour=2, kphys=4, msh=4)])
def test_graph_matches_host_launched(grid):
    cfg, g, e = ctx_pair(**grid)
    t0 = cfg.stpp + 1
    # consecutive steps (the warm start engages), a gap (history dropped),
    # then steps from the ramp (forcing amplitudes change every step)
    for t in [t0, t0 + 1, t0 + 2, t0 + 3, t0 + 9, t0 + 10, 3, 4]:
        n_g, n_e = g.launch_count(), e.launch_count()
        g.step(t)
        e.step(t)
        same(g.get_state(), e.get_state())
        assert stats(g) == stats(e)
        assert g.launch_count() - n_g == e.launch_count() - n_e
    g.close()
    e.close()


def test_graph_after_new_state():
    from trans_bl_gb300 import api
    cfg, g, e = ctx_pair(seed=8)
    t = cfg.stpp + 1
    for q in range(3):
        g.step(t + q)
        e.step(t + q)
    st = perturbed_state(cfg, api.baseflow_fs(cfg, 0.0), np.random.default_rng(9))
    g.put_state(st)
    e.put_state(st)
    g.init_fields()
    e.init_fields()
    g.put_state(st)
    e.put_state(st)
    for q in range(3, 6):
        g.step(t + q)
        e.step(t + q)
        same(g.get_state(), e.get_state())
    g.close()
    e.close()


def test_ensemble_matches_members():
    from trans_bl_gb300 import api, configs
    grids = [dict(nx=65, ny=33, kfour=4, kphys=8, msh=3, F=0.8e-4),
             dict(nx=97, ny=49, kfour=2, kphys=4, msh=4, F=1.2e-4),
             dict(nx=129, ny=33, kfour=1, kphys=2, msh=3, F=1.0e-4)]
    ens_ctx, solo = [], []
    for q, kw in enumerate(grids):
        cfg = configs.small(precision=api.FORM_MIXED, **kw)
        coefs, base = configs.setup_inputs(cfg)
        st = perturbed_state(cfg, base, np.random.default_rng(20 + q))
        a = api.Context(cfg, coefs, base)
        cfg_e = api.TbConfig.from_buffer_copy(cfg)
        cfg_e.step_graph = 0
        b = api.Context(cfg_e, coefs, base)
        a.put_state(st)
        b.put_state(st)
        ens_ctx.append((cfg, a))
        solo.append(b)
    ens = api.Ensemble([a for _, a in ens_ctx])
    t = [c.stpp + 1 + 5 * q for q, (c, _) in enumerate(ens_ctx)]
    for step in range(4):
        ens.step([v + step for v in t])
        for q, b in enumerate(solo):
            b.step(t[q] + step)
    for (cfg, a), b in zip(ens_ctx, solo):
        same(a.get_state(), b.get_state())
        assert stats(a) == stats(b)
    # a member stays usable alone between ensemble steps
    a0 = ens_ctx[0][1]
    a0.step(t[0] + 4)
    solo[0].step(t[0] + 4)
    same(a0.get_state(), solo[0].get_state())
    ens.step([v + 5 for v in t])
    solo[0].step(t[0] + 5)
    same(a0.get_state(), solo[0].get_state())
    ens.close()
    for _, a in ens_ctx:
        a.close()
    for b in solo:
        b.close()


def test_ensemble_rejects_plain_member():
    from trans_bl_gb300 import api
    cfg, coefs, base = small_case()
    g = api.Context(cfg, coefs, base)
    with pytest.raises(api.TbError):
        api.Ensemble([g])
    g.close()


def test_autotune_keeps_results():
    """Tuned launch shapes move work between blocks, not between threads:
    an autotuned context steps bit-identically to an untuned one."""
    from trans_bl_gb300 import api
    cfg, coefs, base = small_case(precision=api.FORM_MIXED, nx=65, ny=33, kfour=16, kphys=32, msh=3)
    a = api.Context(cfg, coefs, base)
    b = api.Context(cfg, coefs, base)
    st = perturbed_state(cfg, base, np.random.default_rng(17))
    a.put_state(st)
    b.put_state(st)
    r = a.autotune()
    assert r["xline_warps"] in (1, 2) and r["yline_threads"] in (32, 64, 128)
    assert r["nl_blocks_per_sm"] in (1, 2, 4, 8)
    assert same_state_after(a, b, cfg.stpp + 1, 3)
    a.close()
    b.close()


def same_state_after(a, b, t0, n):
    for t in range(t0, t0 + n):
        a.step(t)
        b.step(t)
    x, y = a.get_state(), b.get_state()
    return all(np.array_equal(x[f], y[f]) for f in NAMES)
