"""GPU library vs the CPU oracle, subroutine by subroutine, through the C ABI.

Every case runs both on the same seeded inputs of a small grid and compares
the results in the max norm relative to the field's maximum.  The tolerances
are stated per operator: the GPU computes in FP64 with fused multiply-adds,
reciprocal pivots and exact twiddles where the oracle follows the reference's
operation order, so results agree to rounding (1e-12) for single sweeps and
to the Poisson tolerance times a small factor after iterative solves.
"""
import numpy as np
import pytest

from tests.helpers import NAMES, perturbed_state, rel, small_case

pytestmark = pytest.mark.gpu

TOL_SWEEP = 1e-12     # one explicit or tridiagonal line pass
TOL_SPECTRAL = 1e-12  # FFT-based transforms and products
TOL_SOLVE = 1e-9      # multigrid solve (iterates agree to rounding, amplified by the V-cycles)


@pytest.fixture(scope="module")
def case(oracle_built):
    from trans_bl_gb300 import api
    cfg, coefs, base = small_case()
    return cfg, coefs, base, oracle_built, api


def pair(case, state_seed=3):
    cfg, coefs, base, ora, api = case
    g = api.Context(cfg, coefs, base)
    o = ora.Oracle(cfg, coefs, base)
    if state_seed is not None:
        st = perturbed_state(cfg, base, np.random.default_rng(state_seed))
        g.put_state(st)
        o.put_state(st)
    return g, o


@pytest.mark.parametrize("op", ["derparx", "derparxx", "dery", "deryfv", "deryy"])
def test_line_derivatives(case, op):
    g, o = pair(case, None)
    cfg = case[0]
    rng = np.random.default_rng(7)
    f = rng.normal(size=g.shape) + 1j * rng.normal(size=g.shape)
    a = getattr(g, op)(f)
    b = getattr(o, op)(f)
    assert rel(a, b) < TOL_SWEEP, op


def test_spanwise_transforms(case):
    g, o = pair(case, None)
    rng = np.random.default_rng(8)
    c = rng.normal(size=g.shape) + 1j * rng.normal(size=g.shape)
    assert rel(g.f_to_p(c), o.f_to_p(c)) < TOL_SPECTRAL
    p = rng.normal(size=(case[0].kphys,) + g.shape[1:])
    assert rel(g.p_to_f(p), o.p_to_f(p)) < TOL_SPECTRAL


def test_nlterms(case):
    g, o = pair(case)
    for x, y in zip(g.nlterms(), o.nlterms()):
        assert rel(x, y) < TOL_SPECTRAL


def test_drv(case):
    g, o = pair(case)
    for x, y in zip(g.drv(), o.drv()):
        # rows j >= 2 are defined (main_par.f:1313)
        assert rel(x[:, 1:], y[:, 1:]) < 1e-11


def test_filter_and_buffers(case):
    g, o = pair(case)
    for op in ("filter_trid", "bzone", "bzonew"):
        getattr(g, op)()
        getattr(o, op)()
        a, b = g.get_state(), o.get_state()
        for n in ("wx", "wy", "wz"):
            assert rel(a[n], b[n]) < TOL_SWEEP, (op, n)


def test_outuy(case):
    g, o = pair(case)
    assert rel(g.outuy(), o.outuy()) < TOL_SWEEP
    assert rel(g.get_state()["uy"], o.get_state()["uy"]) < TOL_SWEEP


@pytest.mark.parametrize("erro", [1e-3, 1e-10])
def test_poi_uy(case, erro):
    g, o = pair(case)
    d = o.outuy()
    g.outuy()
    g.poi_uy(d, erro)
    o.poi_uy(d, erro)
    assert rel(g.get_state()["uy"], o.get_state()["uy"]) < TOL_SOLVE
    vg = g.poisson_stats()["vcycles"]
    vo, ro = o.poisson_stats()
    assert vg == vo, (vg, vo)


def test_poi_ux_uz(case):
    g, o = pair(case)
    a = g.poi_ux()
    b = o.poi_ux()
    assert rel(a, b) < TOL_SWEEP
    assert rel(g.get_state()["ux"], o.get_state()["ux"]) < 1e-11
    g.poi_uz(b)
    o.poi_uz(b)
    assert rel(g.get_state()["uz"], o.get_state()["uz"]) < 1e-11


def test_wall_vorticity(case):
    g, o = pair(case)
    rng = np.random.default_rng(9)
    w = rng.normal(size=(case[0].kfour, case[0].nx)) * 1e-3 + 0j
    g.put_wall(w)
    o.put_wall(w)
    la = g.wx_wall()
    lb = o.wx_wall()
    assert rel(la, lb) < 1e-11
    assert rel(g.get_state()["wx"][:, 0], o.get_state()["wx"][:, 0]) < 1e-11
    g.wz_wall(lb)
    o.wz_wall(lb)
    assert rel(g.get_state()["wz"][:, 0], o.get_state()["wz"][:, 0]) < 1e-11


def test_ts_forcing(case):
    g, o = pair(case)
    for t, tau in ((1, 0.5), (300, 1.0)):
        g.ts_pert(t, tau)
        o.ts_pert(t, tau)
        assert rel(g.get_state()["uy"][:, 0], o.get_state()["uy"][:, 0]) < 1e-14
        assert rel(g.get_wall(), o.get_wall()) < 1e-14


def test_full_steps(case):
    """Four RK stages (drv, RK update, forcing, loop with filter) for two
    steps from a disturbed state, with the wall forcing at full amplitude
    (t past the one-period smooth start)."""
    cfg, coefs, base, ora, api = case
    g, o = pair(case, state_seed=11)
    t0 = cfg.stpp + 5
    for t in (t0, t0 + 1):
        g.step(t)
        o.step(t)
    a, b = g.get_state(), o.get_state()
    for n in NAMES:
        assert rel(a[n], b[n]) < 1e-9, n
    assert g.launch_count() > 0


def test_perturbation_parity_after_steps(case):
    """Parity of the disturbance (not just the base flow) over 3 steps."""
    cfg, coefs, base, ora, api = case
    g, o = pair(case, state_seed=12)
    s0 = g.get_state()
    for t in (cfg.stpp + 1, cfg.stpp + 2, cfg.stpp + 3):
        g.step(t)
        o.step(t)
    a, b = g.get_state(), o.get_state()
    for n in NAMES:
        da, db = a[n] - s0[n], b[n] - s0[n]
        if np.max(np.abs(db)) > 0:
            assert rel(da, db) < 1e-7, n
