"""The CPU restatement of the learned-correction network against finite
differences (its gradients are then the reference for the GPU kernels)."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import learn_oracle as lo  # noqa: E402


def test_param_count_matches_library():
    from trans_bl_gb300 import api
    assert lo.param_count() == api.learn_param_count()
    assert lo.CW == api.learn_crop_size()


def test_gradient_finite_differences():
    rng = np.random.default_rng(3)
    w = lo.init_weights(rng, last_scale=1.0)
    crops = rng.normal(0, 1, (2, lo.LIN + 1, lo.CW, lo.CW))
    loss, g = lo.loss_grad(w, crops)
    assert loss > 0
    # a few parameters of every layer
    sizes = [o * i * 9 + o for o, i in lo.SHAPES]
    starts = np.cumsum([0] + sizes[:-1])
    idx = []
    for s, n in zip(starts, sizes):
        idx += list(rng.choice(np.arange(s, s + n), 4, replace=False))
    h = 1e-5
    for q in idx:
        wp, wm = w.copy(), w.copy()
        wp[q] += h
        wm[q] -= h
        fd = (lo.loss_grad(wp, crops)[0] - lo.loss_grad(wm, crops)[0]) / (2 * h)
        assert abs(fd - g[q]) <= 1e-6 * max(1.0, abs(g[q])) + 1e-5 * abs(g[q]), (q, fd, g[q])
