"""TS-wave growth of a 2D run against linear stability theory.

A 2D run of the config-1 flat plate (385 x 129, Re_delta* = 1000 at the
inflow, F = 1e-4, wall strip at 3-4 TS wavelengths) is forced for 24
periods; the ux amplitude at the forcing frequency is taken from 16
snapshots of the last period and its streamwise growth rate d ln A/dx is
compared with the spatial LST growth rate at the same stations, between the
strip and the outflow damping zone.

The run is non-parallel and measures the amplitude by max_y |u|, while the
LST is parallel: their growth rates differ by a near-constant offset (the
DNS decays more slowly past branch II, ~0.3 in units of 1/x0 here), so the
test bounds that offset and checks that the two curves have the same shape
and cross zero (branch II) within one TS wavelength of each other.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PERIODS = 24


@pytest.fixture(scope="module")
def growth():
    from trans_bl_gb300 import api, configs, tsval
    cfg = configs.config1(tol=1e-10, precision=api.FORM_MIXED)
    coefs, base = configs.setup_inputs(cfg)
    g = api.Context(cfg, coefs, base)
    amax = tsval.amplitude_along_x(g, cfg, base[0], 1, PERIODS)
    g.close()
    with np.errstate(divide="ignore"):               # A = 0 inside the outflow damping zone
        gr = tsval.growth_rate(np.log(amax), cfg.dx)
    x, gl = tsval.lst_growth(cfg)
    lam = 2 * np.pi / cfg.alpha
    w = slice(cfg.i2 + 20, cfg.i3 - 8)           # past the strip, before the damping zone
    return x[w], gr[w], gl[w], lam


def test_growth_tracks_lst(growth):
    x, gr, gl, lam = growth
    assert np.all(np.isfinite(gr))
    assert np.corrcoef(gr, gl)[0, 1] > 0.95
    off = gr - gl
    assert abs(off.mean()) < 0.4
    assert off.std() < 0.25


def test_branch_two(growth):
    x, gr, gl, lam = growth
    def crossing(g):
        s = np.where(np.diff(np.sign(g)) < 0)[0]
        assert len(s) == 1, "one branch-II crossing in the window"
        i = s[0]
        return x[i] - g[i] * (x[i + 1] - x[i]) / (g[i + 1] - g[i])
    assert abs(crossing(gr) - crossing(gl)) < lam
