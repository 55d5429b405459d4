"""LES (form 4) and immersed-boundary forcing against the CPU oracle.

les_terms (les_par.f:6-211) and cvirt (immersed_par.f:98-313) run through
the spanwise transforms, compact line operators and pointwise products of
the stage, so they are compared at the spectral tolerance; full RK steps of
form 4 with the roughness element switched on are compared at the step
tolerance of the plain form.
"""
import math

import numpy as np
import pytest

from tests.helpers import NAMES, perturbed_state, rel, small_case

pytestmark = pytest.mark.gpu

TOL_TERMS = 1e-11   # transforms + line operators + products (rounding of sums of 8-64 terms)
TOL_STEP = 1e-9     # whole RK steps including the multigrid solve


def les_ibm_case(damping=0, ibm=1, my_form=4):
    cfg, coefs, base = small_case(my_form=my_form)
    dstar = 1.7208 / math.sqrt(cfg.Re)
    cfg.C_s = 0.1
    cfg.A_plus = 26.0
    cfg.les_damping = damping
    cfg.ibm = ibm
    lx = (cfg.nx - 1) * cfg.dx
    cfg.ibm_xc = cfg.x0 + 0.25 * lx
    cfg.ibm_zc = 0.5 * 2.0 * math.pi / cfg.beta
    cfg.ibm_h = 3.0 * dstar     # a few wall rows of the 33-point grid
    cfg.ibm_R = 8.0 * dstar     # a few spanwise points of the 8-point grid
    # the feedback force irf*delta*u is integrated explicitly: RK4 needs
    # |irf| dt < 2.78, so the reference's -0.1 Re (with Re = U x0 / nu
    # = 3.4e5 here) would diverge; -500 gives |irf| dt = 0.37
    cfg.irf = -500.0
    return cfg, coefs, base


def pair(oracle_built, case, seed):
    from trans_bl_gb300 import api
    cfg, coefs, base = case
    g = api.Context(cfg, coefs, base)
    o = oracle_built.Oracle(cfg, coefs, base)
    st = perturbed_state(cfg, base, np.random.default_rng(seed))
    g.put_state(st)
    o.put_state(st)
    return g, o


@pytest.mark.parametrize("damping", [0, 1, 2, 3])
def test_les_terms(oracle_built, damping):
    g, o = pair(oracle_built, les_ibm_case(damping=damping, ibm=0), 31)
    for a, b in zip(g.les_terms(), o.les_terms()):
        assert np.max(np.abs(b)) > 0
        assert rel(a, b) < TOL_TERMS


@pytest.mark.parametrize("damping", [0, 1, 2, 3])
def test_les_terms_reversed_wall_shear(oracle_built, damping):
    """Mean wall vorticity negative over a band of stations, where the
    reference's y+ = sqrt(Re wz_wall) y is NaN: the cubic damping's
    min(y+/A, 100) takes 100 (IEEE minNum) and van Driest's exponential
    carries the NaN, in both implementations; with y+ from |wz_wall|
    (damping 2, 3) both give the same finite terms."""
    from trans_bl_gb300 import api
    cfg, coefs, base = les_ibm_case(damping=damping, ibm=0)
    st = perturbed_state(cfg, base, np.random.default_rng(35))
    band = slice(cfg.nx // 3, cfg.nx // 3 + 6)
    st["wz"][0, 0, band] = -np.abs(st["wz"][0, 0, band])
    g = api.Context(cfg, coefs, base)
    o = oracle_built.Oracle(cfg, coefs, base)
    g.put_state(st)
    o.put_state(st)
    ga, oa = g.les_terms(), o.les_terms()
    if damping == 1:
        assert not all(np.all(np.isfinite(a)) for a in ga)
        assert not all(np.all(np.isfinite(a)) for a in oa)
    else:
        for a, b in zip(ga, oa):
            assert np.all(np.isfinite(a)) and np.all(np.isfinite(b))
            assert rel(a, b) < TOL_TERMS


# Form 4 with the roughness element runs with y+ from |wz_wall| (damping
# 3): the roughness reverses the wall shear within two steps, where the
# reference's y+ = sqrt(Re wz(i,1,1)) y (les_par.f:194) is NaN, in its
# formula as in both implementations.
@pytest.mark.parametrize("damping,ibm,form", [(0, 0, 4), (1, 0, 4), (0, 1, 0), (3, 1, 4)])
def test_steps_les_ibm(oracle_built, damping, ibm, form):
    case = les_ibm_case(damping=damping, ibm=ibm, my_form=form)
    g, o = pair(oracle_built, case, 34)
    t0 = case[0].stpp + 5
    for t in (t0, t0 + 1):
        g.step(t)
        o.step(t)
    a, b = g.get_state(), o.get_state()
    for n in NAMES:
        assert rel(a[n], b[n]) < TOL_STEP, n
