"""TS wave of a 2D run against the repository's linear stability solver.

A 2D run of the config-1 flat plate (385 x 129, Re_delta* = 1000 at the
inflow, F = 1e-4, wall strip at 3-4 TS wavelengths) is forced for 24
periods; the ux disturbance at the forcing frequency is taken from 32
snapshots of the last period (temporal DFT, ftanalysis_par.f:23-38).  Between
the strip and the outflow damping zone it is compared with the spatial LST
of the same Blasius layer (tb_lst_march, lst_ts/ose_bl.f) at the same
stations:

- the streamwise wavenumber alpha_r (x-derivative of the phase at the height
  of max |u|) must agree with the LST's within 2% at every station;
- the growth rate d ln(max_y |u|)/dx follows the LST's curve with a
  near-constant positive offset: the LST is parallel, the run is not, and
  max_y |u| of a growing boundary layer grows faster than the parallel
  eigenvalue says, by O(1/R) in units of the local length sqrt(nu x / U).
  Measured: 0.30 in units of 1/x0, i.e. 0.44/R at R = 700, the size of the
  non-parallel corrections of the literature, varying by 0.14 (standard
  deviation) along the window.  The test bounds the offset to that physics
  (mean 0.2-0.45, spread below 0.2) and the branch-II crossing to within one
  TS wavelength of the LST's (measured 0.61).

The run uses the mixed form (its fields agree with the plain FP64 form to
1e-6); 24 periods of config 1 take about a minute there.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PERIODS = 24
SNAPS = 32


@pytest.fixture(scope="module")
def wave():
    from trans_bl_gb300 import api, configs, tsval
    cfg = configs.config1(tol=1e-10, precision=api.FORM_MIXED)
    coefs, base = configs.setup_inputs(cfg)
    g = api.Context(cfg, coefs, base)
    stride = cfg.stpp // SNAPS
    nsteps = PERIODS * cfg.stpp
    snaps = []
    for q in range(nsteps):
        g.step(1 + q)
        if q >= nsteps - cfg.stpp and (q - (nsteps - cfg.stpp)) % stride == stride - 1:
            snaps.append(g.get_state()["ux"][0].real - base[0])
    g.close()
    u = np.array(snaps)
    c = np.fft.fft(u, axis=0)[1] * 2.0 / u.shape[0]     # complex amplitude at the forcing frequency
    y = tsval.y_coordinates(cfg)
    amax = tsval.wall_normal_max(np.abs(c), y)
    with np.errstate(divide="ignore"):                  # A = 0 inside the outflow damping zone
        gr = tsval.growth_rate(np.log(amax), cfg.dx)
    jm = np.argmax(np.abs(c), axis=0)
    phase = np.unwrap(np.angle(c[jm, np.arange(cfg.nx)]))
    ar = -np.gradient(phase, cfg.dx)
    x, gl, al = tsval.lst_growth(cfg, with_alpha=True)
    lam = 2 * np.pi / cfg.alpha
    w = slice(cfg.i2 + 20, cfg.i3 - 8)                  # past the strip, before the damping zone
    return dict(x=x[w], gr=gr[w], gl=gl[w], ar=ar[w], al=al[w], lam=lam)


def test_wavenumber_matches_lst(wave):
    rel = np.abs(wave["ar"] / wave["al"] - 1.0)
    print("\nalpha_r vs LST: mean %.2e, max %.2e relative" % (rel.mean(), rel.max()))
    assert rel.max() < 0.02


def test_growth_rate_tracks_lst(wave):
    gr, gl = wave["gr"], wave["gl"]
    assert np.all(np.isfinite(gr))
    off = gr - gl
    print("\ngrowth rate - LST: mean %.3f, spread %.3f (1/x0)" % (off.mean(), off.std()))
    assert np.corrcoef(gr, gl)[0, 1] > 0.97
    assert 0.2 < off.mean() < 0.45
    assert off.std() < 0.2


def test_branch_two(wave):
    x, lam = wave["x"], wave["lam"]

    def crossing(g):
        s = np.where(np.diff(np.sign(g)) < 0)[0]
        assert len(s) == 1, "one branch-II crossing in the window"
        i = s[0]
        return x[i] - g[i] * (x[i + 1] - x[i]) / (g[i + 1] - g[i])

    d = crossing(wave["gr"]) - crossing(wave["gl"])
    print("\nbranch II: run - LST = %.3f wavelengths" % (d / lam))
    assert abs(d) < lam
