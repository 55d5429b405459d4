"""Workload definitions: the seeded ensemble and the viscous step-size rule."""
import math

from trans_bl_gb300 import api, configs


def test_stable_steps_per_period():
    cfg = configs.config2()
    n = configs.stable_steps_per_period(cfg)
    assert n == cfg.stpp == 1024
    # nu dt lambda_max below the bound, and above it at half the steps
    def nudt(c, steps):
        return 6.86 / (c.Re * c.fac_y * c.dy ** 2) * 2.0 * math.pi / c.omega / steps
    assert nudt(cfg, n) <= 1.3
    assert n == 256 or nudt(cfg, n // 2) > 1.3   # the smallest power of two that is stable


def test_ensemble_members():
    a = configs.config3(precision=api.FORM_MIXED)
    b = configs.config3(precision=api.FORM_MIXED)
    assert len(a) == 12
    for x, y in zip(a, b):   # seeded: the same members every time
        assert (x.nx, x.ny, x.kfour, x.stpp, x.omega, x.forced_amp[0]) == (y.nx, y.ny, y.kfour, y.stpp, y.omega,
                                                                           y.forced_amp[0])
    for c in a:
        assert c.nx in (257, 513, 769, 1025) and c.ny in (97, 129, 193) and c.kfour in (8, 16, 32)
        assert c.kphys == 2 * c.kfour and c.precision == api.FORM_MIXED
        F = c.omega / c.Re
        assert 0.6e-4 <= F <= 1.4e-4
        assert 1e-6 <= c.forced_amp[0] <= 1e-4
        assert configs.stable_steps_per_period(c) == c.stpp
    assert len({(c.nx, c.ny, c.kfour) for c in a}) > 6   # uneven sizes
    other = configs.config3(seed=7, precision=api.FORM_MIXED)
    assert [(c.nx, c.ny, c.kfour) for c in other] != [(c.nx, c.ny, c.kfour) for c in a]


def test_config5():
    """2049 x 257 x 64 (P = 128), LES with y+ from |wall vorticity|, the
    roughness element at a quarter of the domain (0.5 delta* high, 2 delta*
    across) mid-span, tolerance 1e-8, the step its first cell needs and the
    immersed-boundary gain below the explicit RK4 limit; nx = 1025 keeps
    the 12 wavelengths (the FP64 check's grid)."""
    c = configs.config5(precision=api.FORM_MIXED)
    assert (c.nx, c.ny, c.kfour, c.kphys, c.msh, c.my_form) == (2049, 257, 64, 128, 4, 4)
    assert c.les_damping == 3 and c.C_s == 0.1 and c.A_plus == 26.0
    assert c.tol_stage == c.tol_final == 1e-8
    assert c.stpp == configs.stable_steps_per_period(c) == 16384
    dstar = configs.BLASIUS_DSTAR / math.sqrt(c.Re)
    assert c.ibm == 1 and abs(c.ibm_h - 0.5 * dstar) < 1e-15 and abs(c.ibm_R - dstar) < 1e-15
    assert abs(c.ibm_xc - (c.x0 + 0.25 * (c.nx - 1) * c.dx)) < 1e-12 and abs(c.ibm_zc - math.pi / c.beta) < 1e-12
    dt = 2.0 * math.pi / c.omega / c.stpp
    assert c.irf == -0.1 * c.Re and abs(c.irf) * dt < 2.0
    assert c.forced_amp[0] == c.forced_amp[1] == 3e-3
    h = configs.config5(nx=1025, precision=api.FORM_MIXED)
    assert abs(h.dx - 2.0 * c.dx) < 1e-15 and h.ny == c.ny and h.dy == c.dy


def test_gortler_config():
    """The Goertler form's helper: my_form 1, the curvature's Goertler
    number, no immersed boundary."""
    c = configs.gortler(go_number=8.0)
    assert c.my_form == 1 and c.go_number == 8.0 and c.ibm == 0
