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
