"""The CPU restatement of the learned-correction network and its defect loss
against finite differences (its gradients are then the reference for the
GPU kernels)."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import learn_oracle as lo  # noqa: E402


def test_param_count_matches_library():
    from trans_bl_gb300 import api
    assert lo.param_count() == api.learn_param_count()
    assert lo.CW == api.learn_crop_size()


def synthetic_tables(rng, K, ny):
    tabs = []
    for k in range(K):
        t = np.concatenate([[rng.uniform(0.5, 2.0), 1.0, 4.0, 0.5 * k, rng.uniform(0.1, 0.5)],
                            rng.uniform(-1, 1, 24), rng.uniform(0.5, 3.0, ny), rng.uniform(0.2, 1.0, ny)])
        tabs.append(lo.split_tables(t, ny))
    return tabs


def test_defect_gradient_finite_differences():
    rng = np.random.default_rng(3)
    nx, ny = 80, 40   # crops straddle every edge of the grid
    tables = synthetic_tables(rng, 2, ny)
    w = lo.init_weights(rng, last_scale=1.0, scale=0.7, iscale=(0.5, 2.0, 1.5, 0.8))
    crops = rng.normal(0, 1, (2, lo.LIN + 1, lo.CW, lo.CW))
    meta = np.array([[1, -4, -4], [2, 10, -20]])
    loss, g = lo.defect_loss_grad(w, crops, meta, tables, nx, ny)
    assert loss > 0
    assert np.all(g[-lo.NSCALE:] == 0.0)   # the scales are not trained
    sizes = [o * i * 9 + o for o, i in lo.SHAPES]
    starts = np.cumsum([0] + sizes[:-1])
    idx = []
    for s, n in zip(starts, sizes):
        idx += list(rng.choice(np.arange(s, s + n), 3, replace=False))
    h = 1e-5
    for q in idx:
        wp, wm = w.copy(), w.copy()
        wp[q] += h
        wm[q] -= h
        fd = (lo.defect_loss_grad(wp, crops, meta, tables, nx, ny)[0] -
              lo.defect_loss_grad(wm, crops, meta, tables, nx, ny)[0]) / (2 * h)
        assert abs(fd - g[q]) <= 1e-6 * max(1.0, abs(g[q])) + 1e-5 * abs(g[q]), (q, fd, g[q])
