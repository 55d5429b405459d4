"""Learned first correction of the mixed solve.

  (a) the library's training kernels (forward, backward data, weight
      gradient, defect loss) against the float64 CPU restatement of the
      network, and the loss's operator against the solver's own;
  (b) the solver with the trained network: same fields as without it (both
      iterate to the tolerance), bit-identical host-launched and replayed
      steps, and what the network gains: corrections per step with and
      without it, and the share of solves where it was kept.
"""
import os
import sys

import numpy as np
import pytest

from tests.helpers import NAMES, perturbed_state, rel

pytestmark = pytest.mark.gpu

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import learn_oracle as lo  # noqa: E402


@pytest.fixture(scope="module")
def small_mixed():
    from trans_bl_gb300 import api, configs
    cfg = configs.small(nx=97, ny=49, kfour=2, kphys=4, msh=4, precision=api.FORM_MIXED)
    coefs, base = configs.setup_inputs(cfg)
    g = api.Context(cfg, coefs, base)
    yield cfg, g
    g.close()


def test_operator_matches_solver(small_mixed):
    """The loss's operator (stencil restated in the oracle) is the solver's."""
    cfg, g = small_mixed
    rng = np.random.default_rng(10)
    for k in range(cfg.kfour):
        T = lo.split_tables(g.learn_op_tables(k), cfg.ny)
        e = rng.normal(0, 1, (cfg.nx, cfg.ny))
        e[0], e[-1], e[:, 0] = 0, 0, 0
        want = lo.apply_L(T, cfg.nx, cfg.ny, e)
        got = -g.learn_op_apply(k, e.astype(np.float32))
        assert np.max(np.abs(got - want)) <= 1e-5 * np.max(np.abs(want)), k


def test_grad_matches_oracle(small_mixed):
    cfg, g = small_mixed
    rng = np.random.default_rng(11)
    w = lo.init_weights(rng, last_scale=1.0, scale=0.7, iscale=(0.5, 2.0, 1.5, 0.8)).astype(np.float32)
    crops = rng.normal(0, 1, (3, lo.LIN + 1, lo.CW, lo.CW)).astype(np.float32)
    meta = np.array([[0, -4, -4], [3, 20, -30], [1, 30, 2]], dtype=np.int32)   # crops over every edge
    tables = [lo.split_tables(g.learn_op_tables(k), cfg.ny) for k in range(cfg.kfour)]
    loss_g, g_g = g.learn_grad(w, crops, meta)
    loss_o, g_o = lo.defect_loss_grad(w.astype(np.float64), crops.astype(np.float64), meta, tables, cfg.nx, cfg.ny)
    assert abs(loss_g - loss_o) <= 1e-4 * loss_o
    assert np.all(g_g[-lo.NSCALE:] == 0.0)
    sizes = [o * i * 9 + o for o, i in lo.SHAPES]
    off = 0
    for n in sizes:   # per layer, relative to the layer's gradient norm
        a, b = g_g[off:off + n], g_o[off:off + n]
        assert np.linalg.norm(a - b) <= 1e-4 * np.linalg.norm(b), off
        off += n


def test_forward_matches_oracle():
    from trans_bl_gb300 import api
    rng = np.random.default_rng(12)
    w = lo.init_weights(rng, last_scale=1.0, scale=1.3, iscale=(0.5, 2.0, 1.5, 0.8)).astype(np.float32)
    x = rng.normal(0, 1, (2, lo.LIN, 45, 37)).astype(np.float32)
    out = api.learn_forward(w, x)
    ref, _ = lo.forward(w.astype(np.float64), x.astype(np.float64))
    assert np.max(np.abs(out - ref)) <= 1e-5 * np.max(np.abs(ref))


def corrections(ctx, t0, n):
    v0 = ctx.poisson_stats()["total_vcycles"]
    for q in range(n):
        ctx.step(t0 + q)
    return ctx.poisson_stats()["total_vcycles"] - v0


@pytest.fixture(scope="module")
def trained():
    from trans_bl_gb300 import api, configs
    cfg = configs.blasius_ts_config(257, 97, 8, 16, 4, precision=api.FORM_MIXED, amp2d=1e-4, amp3d=1e-5,
                                    n_lambda=6.0, strip=(1.0, 1.6))
    cfg.stpp = configs.stable_steps_per_period(cfg)
    coefs, base = configs.setup_inputs(cfg)
    g = api.Context(cfg, coefs, base)
    st = perturbed_state(cfg, base, np.random.default_rng(31))
    g.put_state(st)
    t = cfg.stpp + 1
    g.learn_init(7)
    g.learn_sample(4096, crops_per_solve=16, seed=5)
    for q in range(64):
        g.step(t + q)
    g.learn_sample(0)
    n = g.learn_stats()["samples"]
    ntr = int(0.75 * n)          # train on the earlier steps, hold out the later ones
    g.learn_train(1, batch=32, lr=1e-12, n_train=ntr)   # sets the scales; weights stay as initialised
    loss0, base_loss = g.learn_eval(ntr, n - ntr)
    g.learn_train(1500, batch=32, lr=1e-3, n_train=ntr)
    loss1, _ = g.learn_eval(ntr, n - ntr)
    w = g.learn_weights()
    state = g.get_state()
    g.close()
    return cfg, coefs, base, state, t + 64, w, loss0 / base_loss, loss1 / base_loss


def test_learned_solve(trained):
    from trans_bl_gb300 import api
    cfg, coefs, base, state, t, w, rel0, rel1 = trained
    # defect left on held-out steps relative to the extrapolated guess's: 1 for
    # the untrained network (zero output), below 1 after training
    assert abs(rel0 - 1.0) < 1e-6
    assert rel1 < 1.0
    plain = api.Context(cfg, coefs, base)
    learned = api.Context(cfg, coefs, base)
    learned.learn_set_weights(w)
    learned.learn_enable(True)
    for c in (plain, learned):
        c.put_state(state)
        corrections(c, t - 2, 2)   # rebuild the warm-start history
    n = 16
    c_plain = corrections(plain, t, n)
    c_learned = corrections(learned, t, n)
    st = learned.learn_stats()
    a, b = learned.get_state(), plain.get_state()
    for f in NAMES:
        assert rel(a[f], b[f]) < 1e-6, f
    assert st["tried"] == 4 * n * cfg.kfour
    print("\nlearned correction: held-out relative defect %.3f -> %.3f; corrections over %d steps %d -> %d; "
          "kept %d of %d" % (rel0, rel1, n, c_plain, c_learned, st["kept"], st["tried"]))
    # what the network gains: on held-out steps its correction leaves less
    # than 0.6 of the guess's mean-square defect (measured 0.23); it is kept
    # where it lowers a mode's max defect.  The multigrid contracts the
    # defect ~1e3 per correction, so the count of corrections moves little
    # either way: it is reported, and the gated form (below) removes the
    # network's cost where it does not help
    assert rel1 < 0.6
    plain.close()
    learned.close()


def test_learned_other_frequency(trained):
    """Weights trained at F = 1e-4 applied to a run at F = 1.2e-4: the
    fields still agree with the run without the network (both iterate to the
    tolerance); the share of kept corrections and the corrections per step
    are reported."""
    from trans_bl_gb300 import api, configs
    cfg0, coefs, base, state, t, w, _, _ = trained
    cfg = configs.blasius_ts_config(257, 97, 8, 16, 4, precision=api.FORM_MIXED, amp2d=1e-4, amp3d=1e-5,
                                    n_lambda=6.0, strip=(1.0, 1.6), F=1.2e-4)
    cfg.stpp = configs.stable_steps_per_period(cfg)
    coefs, base = configs.setup_inputs(cfg)
    st = perturbed_state(cfg, base, np.random.default_rng(32))
    plain = api.Context(cfg, coefs, base)
    learned = api.Context(cfg, coefs, base)
    learned.learn_set_weights(w)
    learned.learn_enable(True)
    t1 = cfg.stpp + 1
    for c in (plain, learned):
        c.put_state(st)
        corrections(c, t1, 2)
    n = 16
    c_plain = corrections(plain, t1 + 2, n)
    c_learned = corrections(learned, t1 + 2, n)
    s = learned.learn_stats()
    a, b = learned.get_state(), plain.get_state()
    for f in NAMES:
        assert rel(a[f], b[f]) < 1e-6, f
    print("\nF = 1.2e-4 with weights from F = 1e-4: corrections over %d steps %d -> %d; kept %d of %d"
          % (n, c_plain, c_learned, s["kept"], s["tried"]))
    assert s["tried"] == 4 * n * cfg.kfour
    plain.close()
    learned.close()


@pytest.mark.parametrize("gated", [False, True])
def test_learned_graph_matches_host_launched(trained, gated):
    from trans_bl_gb300 import api
    cfg, coefs, base, state, t, w, _, _ = trained
    cfg_e = api.TbConfig.from_buffer_copy(cfg)
    cfg_e.step_graph = 0
    g = api.Context(cfg, coefs, base)
    e = api.Context(cfg_e, coefs, base)
    for c in (g, e):
        c.learn_set_weights(w)
        c.learn_enable(True, gated=gated)
        c.put_state(state)
    for q in range(6):
        g.step(t + q)
        e.step(t + q)
        a, b = g.get_state(), e.get_state()
        for f in NAMES:
            assert np.array_equal(a[f], b[f]), f
    assert g.learn_stats()["kept"] == e.learn_stats()["kept"]
    if gated:
        assert g.learn_stats()["evaluated"] == e.learn_stats()["evaluated"]
        assert g.learn_stats()["solves"] == e.learn_stats()["solves"] == 4 * 6
    g.close()
    e.close()


@pytest.mark.parametrize("graph", [1, 0])
def test_gated_falls_back(trained, graph):
    """A network that never helps (zero output: the last layer starts at
    zero) runs only in a stage's first solve and then once every 32 solves;
    the fields are those of the form without it, bit for bit."""
    from trans_bl_gb300 import api
    cfg0, coefs, base, state, t, w, _, _ = trained
    cfg = api.TbConfig.from_buffer_copy(cfg0)
    cfg.step_graph = graph
    g = api.Context(cfg, coefs, base)
    ref = api.Context(cfg, coefs, base)
    g.learn_init(3)
    g.learn_enable(True, gated=True)
    for c in (g, ref):
        c.put_state(state)
    n = 36
    for q in range(n):
        g.step(t + q)
        ref.step(t + q)
    st = g.learn_stats()
    assert st["solves"] == 4 * n
    assert st["evaluated"] == 4 * 2          # solves 1 and 33 of each stage
    assert st["kept"] == 0
    a, b = g.get_state(), ref.get_state()
    for f in NAMES:
        assert np.array_equal(a[f], b[f]), f
    g.close()
    ref.close()
