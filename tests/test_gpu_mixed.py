"""Mixed-precision form of poi_uy against the FP64 oracle.

The mixed form (FP64 defect correction on the reference's fine operator
around an FP32 multigrid with coloured y-line relaxation) solves the
reference's discrete v-Poisson problem with the reference's stopping rule
(max |defect| < tol over the fine interior) through different iterates.  So
it is compared with the oracle
  (a) on one poi_uy call solved far below a run's tolerance, where both
      iterates sit within the solve tolerance of the same discrete solution;
  (b) after full RK4 steps at the run's tolerance, to 1e-6 relative: the
      accuracy the mixed form is specified for.
"""
import numpy as np
import pytest

from tests.helpers import NAMES, perturbed_state, rel, small_case

pytestmark = pytest.mark.gpu

TOL_MIXED_STEP = 1e-6    # full steps, mixed form vs the oracle's FP64 iterates
TOL_MIXED_SOLVE = 1e-8   # one solve at erro = 1e-9 (both far below run tolerance)


def make_case(ora, **kw):
    from trans_bl_gb300 import api
    cfg, coefs, base = small_case(precision=api.FORM_MIXED, max_vcycles=40, **kw)
    return cfg, coefs, base, ora, api


@pytest.fixture(scope="module")
def mcase(oracle_built):
    return make_case(oracle_built)


def pair(case, seed):
    cfg, coefs, base, ora, api = case
    g = api.Context(cfg, coefs, base)
    o = ora.Oracle(cfg, coefs, base)
    st = perturbed_state(cfg, base, np.random.default_rng(seed))
    g.put_state(st)
    o.put_state(st)
    return g, o


@pytest.mark.parametrize("grid", [dict(), dict(nx=97, ny=49, kfour=2, kphys=4, msh=4),
                                  dict(nx=81, ny=129, kfour=3, kphys=8, msh=3)])
def test_poi_uy_mixed_tight(oracle_built, grid):
    case = make_case(oracle_built, **grid)
    g, o = pair(case, 3)
    d = o.outuy()
    g.outuy()
    erro = 1e-9
    g.poi_uy(d, erro)
    o.poi_uy(d, erro)
    st = g.poisson_stats()
    assert st["noconv"] == 0
    assert max(st["residual"][:case[0].kfour]) < erro
    assert rel(g.get_state()["uy"], o.get_state()["uy"]) < TOL_MIXED_SOLVE


def test_poi_uy_mixed_corrections(mcase):
    """Loose tolerances take fewer FP64 corrections than tight ones; each
    solve ends below its tolerance."""
    counts = []
    for erro in (1e-3, 1e-7, 1e-11):
        g, o = pair(mcase, 4)
        d = o.outuy()
        g.outuy()
        g.poi_uy(d, erro)
        st = g.poisson_stats()
        k = mcase[0].kfour
        assert st["noconv"] == 0, erro
        assert max(st["residual"][:k]) < erro
        counts.append(sum(st["vcycles"][:k]))
    assert counts[0] <= counts[1] <= counts[2]
    assert counts[2] > 0


def test_nlterms_mixed(mcase):
    """Mean part exact in FP64, disturbance products through FP32 transforms:
    the error is FP32 rounding of the quadratic disturbance term only."""
    g, o = pair(mcase, 7)
    for a, b in zip(g.nlterms(), o.nlterms()):
        assert rel(a, b) < 1e-8


def test_full_steps_mixed(mcase):
    cfg, coefs, base, ora, api = mcase
    g, o = pair(mcase, 11)
    t0 = cfg.stpp + 5
    for t in (t0, t0 + 1):
        g.step(t)
        o.step(t)
    a, b = g.get_state(), o.get_state()
    for n in NAMES:
        assert rel(a[n], b[n]) < TOL_MIXED_STEP, n


def test_perturbation_parity_mixed(mcase):
    """The disturbance (state minus start) after 3 steps, mixed vs oracle."""
    cfg, coefs, base, ora, api = mcase
    g, o = pair(mcase, 12)
    s0 = g.get_state()
    for t in (cfg.stpp + 1, cfg.stpp + 2, cfg.stpp + 3):
        g.step(t)
        o.step(t)
    a, b = g.get_state(), o.get_state()
    for n in NAMES:
        da, db = a[n] - s0[n], b[n] - s0[n]
        if np.max(np.abs(db)) > 0:
            assert rel(da, db) < TOL_MIXED_STEP, n


def test_mixed_rejects_tiny_coarse_grid(oracle_built):
    from trans_bl_gb300 import api
    cfg, coefs, base = small_case(nx=33, precision=api.FORM_MIXED)   # coarsest level 9 points in x
    with pytest.raises(api.TbError):
        api.Context(cfg, coefs, base)


def test_fp32_lines(mcase):
    """x-line operators of modes k >= 1 in FP32 against FP64: the modes hold
    only the disturbance (1e-3 of the base flow here), so the difference sits
    at FP32 rounding of the disturbance."""
    cfg, coefs, base, ora, api = mcase
    g32 = api.Context(cfg, coefs, base)
    g64 = api.Context(cfg, coefs, base)
    g32.fp32_lines(True)
    st = perturbed_state(cfg, base, np.random.default_rng(13))
    for g in (g32, g64):
        g.put_state(st)
    t0 = cfg.stpp + 5
    for t in (t0, t0 + 1):
        g32.step(t)
        g64.step(t)
    a, b = g32.get_state(), g64.get_state()
    for n in NAMES:
        d = np.max(np.abs(a[n][1:] - b[n][1:]))        # modes k >= 1
        s = np.max(np.abs(b[n][1:]))
        assert d <= 1e-5 * s, n                        # FP32 differencing of the disturbance
        assert np.array_equal(a[n][0], b[n][0]) or rel(a[n][0], b[n][0]) < 1e-8, n
    g32.close()
    g64.close()
