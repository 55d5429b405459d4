"""Properties of the CPU oracle (the checker of the GPU library)."""
import numpy as np
import pytest

from tests.helpers import perturbed_state, rel, small_case


@pytest.fixture(scope="module")
def case(lib_built, oracle_built):
    cfg, coefs, base = small_case()
    return cfg, coefs, base, oracle_built


def test_x_derivatives_exact_on_polynomials(case):
    cfg, coefs, base, ora = case
    o = ora.Oracle(cfg, coefs, base)
    x = cfg.x0 + cfg.dx * np.arange(cfg.nx)
    f = np.zeros(o.shape, complex)
    f[:] = (x ** 4 - 2 * x ** 3 + x)[None, None, :]
    d1 = o.derparx(f)
    d2 = o.derparxx(f)
    assert rel(d1[0, 3], 4 * x ** 3 - 6 * x ** 2 + 1) < 1e-9
    assert rel(d2[0, 3], 12 * x ** 2 - 12 * x) < 1e-8


def test_y_derivatives_exact_on_polynomials(case):
    cfg, coefs, base, ora = case
    o = ora.Oracle(cfg, coefs, base)
    j = np.arange(cfg.ny)
    y = cfg.dy * (cfg.stf ** j - 1) / (cfg.stf - 1)
    f = np.zeros(o.shape, complex)
    f[:] = (y ** 3 - y ** 2)[None, :, None]
    d1 = o.dery(f)
    d2 = o.deryy(f)
    assert rel(d1[0, :, 5], 3 * y ** 2 - 2 * y) < 1e-8
    assert rel(d2[0, :, 5], 6 * y - 2) < 1e-8


def test_spanwise_transform_convention_and_roundtrip(case):
    cfg, coefs, base, ora = case
    o = ora.Oracle(cfg, coefs, base)
    rng = np.random.default_rng(1)
    c = rng.normal(size=o.shape) + 1j * rng.normal(size=o.shape)
    c[0] = c[0].real
    p = o.f_to_p(c)
    P, K = cfg.kphys, cfg.kfour
    n = np.arange(P)
    ref = np.zeros((P,) + c.shape[1:])
    for k in range(K):
        w = np.exp(-2j * np.pi * k * n / P)[:, None, None]
        ref += (c[k][None] * w).real
    assert rel(p, ref) < 1e-13
    back = o.p_to_f(p)
    assert rel(back, c) < 1e-12


def test_poisson_reaches_tolerance(case):
    cfg, coefs, base, ora = case
    o = ora.Oracle(cfg, coefs, base)
    rng = np.random.default_rng(2)
    o.put_state(perturbed_state(cfg, base, rng))
    dwzdx = o.outuy()
    o.poi_uy(dwzdx, 1e-3)
    v, r = o.poisson_stats()
    assert all(x < cfg.max_vcycles for x in v), v
    assert np.all(r < 1e-3)


def test_stage_runs_finite(case):
    cfg, coefs, base, ora = case
    o = ora.Oracle(cfg, coefs, base)
    for t in (1, 2):
        o.step(t)
    s = o.get_state()
    for n, f in s.items():
        assert np.all(np.isfinite(f)), n
    assert np.max(np.abs(s["uy"][0, 0])) > 0  # the wall forcing is on


@pytest.mark.parametrize("damping", [0, 1])
def test_les_damping_reversed_wall_shear(lib_built, oracle_built, damping):
    """les_par.f:194 takes y+ = sqrt(Re wz_wall) y, NaN at stations with a
    negative mean wall vorticity.  The cubic damping's min(y+/A, 100) takes
    the number (IEEE minNum: full eddy viscosity there); van Driest's
    exponential carries the NaN.  With y+ from |wz_wall| (damping + 2) the
    terms are finite, and equal the reference's where wz_wall > 0."""
    cfg, coefs, base = small_case(my_form=4)
    cfg.C_s, cfg.A_plus = 0.1, 26.0
    st = perturbed_state(cfg, base, np.random.default_rng(36))
    band = slice(cfg.nx // 3, cfg.nx // 3 + 6)
    out = {}
    for d in (damping, damping + 2):
        cfg.les_damping = d
        o = oracle_built.Oracle(cfg, coefs, base)
        o.put_state(st)
        out[d, "pos"] = o.les_terms()
        s2 = {n: f.copy() for n, f in st.items()}
        s2["wz"][0, 0, band] = -np.abs(s2["wz"][0, 0, band])
        o.put_state(s2)
        out[d, "neg"] = o.les_terms()
    for a, b in zip(out[damping, "pos"], out[damping + 2, "pos"]):
        assert np.array_equal(a, b)
    finite = all(np.all(np.isfinite(a)) for a in out[damping, "neg"])
    assert finite == (damping == 0)
    assert all(np.all(np.isfinite(a)) for a in out[damping + 2, "neg"])


def test_gortler_form_is_linear(lib_built, oracle_built):
    """drv_gv is linear in the disturbance (the base flow is fixed): drv of
    2s is twice drv of s; the curvature terms enter dvx and dvz only; the
    form starts from zero fields and gv_pert forces modes k >= 1 only."""
    from trans_bl_gb300 import configs
    out = {}
    for go in (0.0, 8.0):
        cfg = configs.gortler(go_number=go, make_default=oracle_built.default_config)
        coefs, base = oracle_built.setup_inputs(cfg)
        o = oracle_built.Oracle(cfg, coefs, base)
        s = configs.disturbance_state(cfg, np.random.default_rng(56))
        o.put_state(s)
        d1 = o.drv()
        o.put_state({n: 2.0 * f for n, f in s.items()})
        d2 = o.drv()
        for a, b in zip(d1, d2):
            assert rel(b, 2.0 * a) < 1e-12
        out[go] = d1
        o.init_fields()
        z = o.get_state()
        assert all(np.all(f == 0) for f in z.values())
        o.ts_pert(cfg.stpp + 1, 0.5)
        uy = o.get_state()["uy"]
        assert np.all(uy[0] == 0) and np.max(np.abs(uy[1:, 0, :])) > 0
    assert np.array_equal(out[0.0][1], out[8.0][1])
    assert not np.array_equal(out[0.0][0], out[8.0][0]) and not np.array_equal(out[0.0][2], out[8.0][2])


def test_thermal_form_passive_and_linear(lib_built, oracle_built):
    """drv_gvth: the temperature does not act on the momentum terms; without
    a velocity disturbance and forcing the velocities stay zero and one step
    of th is linear in th (doubling th doubles it); th keeps its zero wall
    and top rows."""
    from trans_bl_gb300 import configs
    cfg = configs.thermal(make_default=oracle_built.default_config)
    coefs, base = oracle_built.setup_inputs(cfg)
    thb = configs.base_temperature(cfg, base)
    rng = np.random.default_rng(57)
    s = configs.disturbance_state(cfg, rng)
    th = configs.smooth_random((cfg.kfour, cfg.ny, cfg.nx), rng, 1e-3)
    th[:, 0, :] = 0.0
    th[:, -1, :] = 0.0
    o = oracle_built.Oracle(cfg, coefs, base)
    o.set_baseflow_th(thb)
    o.put_state(s)
    o.put_th(np.zeros_like(th))
    d0 = o.drv()
    o.put_th(th)
    d1 = o.drv()
    for a, b in zip(d0, d1):
        assert np.array_equal(a, b)
    cfg.n_forced = 0
    outs = []
    for scale in (1.0, 2.0):
        o = oracle_built.Oracle(cfg, coefs, base)
        o.set_baseflow_th(thb)
        o.put_th(scale * th)
        o.step(cfg.stpp + 1)
        outs.append(o.get_th())
        assert all(np.max(np.abs(f)) == 0 for f in o.get_state().values())
    assert rel(outs[1], 2.0 * outs[0]) < 1e-12
    assert np.all(outs[0][:, 0, :] == 0) and np.all(outs[0][:, -1, :] == 0)
    assert np.max(np.abs(outs[0] - th)) > 0
