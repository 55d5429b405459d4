"""Learned first correction of the mixed solve.

  (a) the library's training kernels (forward, backward data, weight
      gradient, loss) against the float64 CPU restatement of the network;
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


def test_grad_matches_oracle():
    from trans_bl_gb300 import api
    rng = np.random.default_rng(11)
    w = lo.init_weights(rng, last_scale=1.0).astype(np.float32)
    crops = rng.normal(0, 1, (3, lo.LIN + 1, lo.CW, lo.CW)).astype(np.float32)
    loss_g, g_g = api.learn_grad(w, crops)
    loss_o, g_o = lo.loss_grad(w.astype(np.float64), crops.astype(np.float64))
    assert abs(loss_g - loss_o) <= 1e-5 * loss_o
    sizes = [o * i * 9 + o for o, i in lo.SHAPES]
    off = 0
    for n in sizes:   # per layer, relative to the layer's gradient norm
        a, b = g_g[off:off + n], g_o[off:off + n]
        assert np.linalg.norm(a - b) <= 1e-4 * np.linalg.norm(b), off
        off += n


def test_forward_matches_oracle():
    from trans_bl_gb300 import api
    rng = np.random.default_rng(12)
    w = lo.init_weights(rng, last_scale=1.0).astype(np.float32)
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
    loss0 = g.learn_train(1, batch=32, lr=1e-12)      # the untrained (zero-output) loss
    loss = g.learn_train(1500, batch=32, lr=1e-3)
    w = g.learn_weights()
    state = g.get_state()
    g.close()
    return cfg, coefs, base, state, t + 64, w, loss0, loss


def test_learned_solve(trained):
    from trans_bl_gb300 import api
    cfg, coefs, base, state, t, w, loss0, loss = trained
    assert loss < loss0
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
    print("\nlearned correction: loss %.3e -> %.3e; corrections over %d steps %d -> %d; kept %d of %d"
          % (loss0, loss, n, c_plain, c_learned, st["kept"], st["tried"]))
    assert c_learned <= c_plain
    plain.close()
    learned.close()


def test_learned_graph_matches_host_launched(trained):
    from trans_bl_gb300 import api
    cfg, coefs, base, state, t, w, _, _ = trained
    cfg_e = api.TbConfig.from_buffer_copy(cfg)
    cfg_e.step_graph = 0
    g = api.Context(cfg, coefs, base)
    e = api.Context(cfg_e, coefs, base)
    for c in (g, e):
        c.learn_set_weights(w)
        c.learn_enable(True)
        c.put_state(state)
    for q in range(6):
        g.step(t + q)
        e.step(t + q)
        a, b = g.get_state(), e.get_state()
        for f in NAMES:
            assert np.array_equal(a[f], b[f]), f
    assert g.learn_stats()["kept"] == e.learn_stats()["kept"]
    g.close()
    e.close()
