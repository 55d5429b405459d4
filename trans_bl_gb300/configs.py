"""Workload definitions: synthetic Blasius/TS set-ups of the benchmark sizes.

No dataset is involved: every input is generated -- the Blasius base flow by
the Falkner-Skan shooting of the library (pre_processing/fs_sch.f90), the
compact-scheme tables by the library's coefficient generator
(pre_processing/derivative.f90), and the wall forcing (ts2d_pert/ts3d_pert,
main_par.f:1613-1685) with phases drawn from a seeded generator.

Non-dimensionalisation follows the reference with fac_y = 1: lengths in units
of L = x0 (the inflow station), Re = U L / nu, time in L / U.  At the inflow
Re_delta* = 1.7208 sqrt(Re) (Blasius).
"""
import math

import numpy as np

from . import api

BLASIUS_DSTAR = 1.7208  # delta* sqrt(U/(nu x)) of the Blasius profile


def blasius_ts_config(nx, ny, kfour, kphys, msh, stf=1.02, re_dstar=1000.0, F=1e-4, n_lambda=12.0,
                      y_top_dstar=40.0, steps_per_period=256, beta_dstar=0.2, amp2d=1e-5, amp3d=0.0,
                      seed=20261203, tol=1e-10, max_vcycles=11, precision=api.FORM_PLAIN_FP64, my_form=0,
                      strip=(3.0, 4.0), make_default=None):
    """tb_config of a flat-plate TS forcing case on an (nx, ny, kfour) grid.

    make_default(**fields) builds the tb_config from its defaults; the
    library's tb_config_default unless given (the CPU baseline passes one that
    does not load the library)."""
    Re = (re_dstar / BLASIUS_DSTAR) ** 2
    dstar = BLASIUS_DSTAR / math.sqrt(Re)          # at x0 = 1
    omega = F * Re                                 # F = omega nu / U^2
    alpha = 0.26 / dstar                           # TS wavenumber estimate (alpha_r delta* ~ 0.26)
    lam = 2.0 * math.pi / alpha
    dx = n_lambda * lam / (nx - 1)
    y_top = y_top_dstar * dstar
    dy0 = y_top * (stf - 1.0) / (stf ** (ny - 1) - 1.0) if stf != 1.0 else y_top / (ny - 1)
    i1 = int(round(1 + strip[0] * lam / dx))
    i2 = int(round(1 + strip[1] * lam / dx))
    i0 = max(5, int(round(0.025 * nx)))
    i3 = int(round(0.80 * nx))
    i4 = int(round(0.90 * nx))
    rng = np.random.default_rng(seed)
    modes, amps, phases = [0], [amp2d], [float(rng.uniform(0, 2 * math.pi))]
    if amp3d > 0 and kfour > 1:
        modes.append(1); amps.append(amp3d); phases.append(float(rng.uniform(0, 2 * math.pi)))
    cfg = (make_default or api.default_config)(
        nx=nx, ny=ny, kfour=kfour, kphys=kphys, msh=msh, my_form=my_form, i0=i0, i1=i1, i2=i2, i3=i3, i4=i4,
        stpp=steps_per_period, max_vcycles=max_vcycles, precision=precision,
        Re=Re, dx=dx, dy=dy0, stf=stf, x0=1.0, alpha=alpha, omega=omega, beta=beta_dstar / dstar, fac_y=1.0,
        alphaf=0.48, tol_stage=tol, tol_final=tol, irf=-0.1 * Re, n_forced=len(modes),
        forced_mode=modes, forced_amp=amps, forced_phase=phases)
    return cfg


# Benchmark workloads (grid sizes of the reference's headline configurations).
def config1(**kw):
    """2D: nx=385, ny=129, one Fourier mode (P=2), 3-level multigrid."""
    return blasius_ts_config(385, 129, 1, 2, 3, **kw)


def config2(**kw):
    """3D: nx=1025, ny=193, 32 modes (P=64), 2D TS + oblique pair, 4-level multigrid.

    1024 steps per forcing period: with the 1.02 stretching to 40 delta* over
    193 points the first wall cell is dy0 = 5.4e-5 L, and the explicit RK4
    viscous term is stable only for nu dt lambda_max < 2.78 with lambda_max =
    6.86 / dy0^2 (compact 6th-order second derivative at the grid scale).  At
    256 steps per period nu dt lambda_max = 5.0 and the run diverges within
    ten steps from the undisturbed base flow; at 1024 it is 1.26."""
    kw.setdefault("steps_per_period", 1024)
    kw.setdefault("amp2d", 1e-4)
    kw.setdefault("amp3d", 1e-5)
    return blasius_ts_config(1025, 193, 32, 64, 4, **kw)


def config5(nx=2049, **kw):
    """Large 3D run with a roughness element and LES: nx=2049, ny=257 (1.02
    stretching to 40 delta*), 64 modes (P=128), 4-level multigrid; 2D TS wave
    plus the oblique pair at amplitude 3e-3; Smagorinsky LES (drv_les,
    les_par.f:6-211) with C_s = 0.1 and van Driest damping A+ = 26; and the
    reference's immersed-boundary roughness element (delta/cvirt,
    immersed_par.f:98-313): an edge-smoothed cylinder of height 0.5 delta* and
    diameter 2 delta* centred at 25% of the domain length (the 0.5 delta*
    high, 2 delta* wide bump).  The steps per period keep the explicit viscous
    term stable (as config 2): the first cell of the 257-point grid is
    0.005 delta*, which takes 16384 steps per forcing period.  The
    immersed-boundary gain is the reference's -0.1 Re (par.for:123), capped
    at |irf| dt = 2 for explicit RK4 stability (|irf| dt = 0.38 at this step,
    so the cap does not act).

    The damping's friction velocity is taken from |wall vorticity|
    (les_damping 3, van Driest [1 - e^{-y+/A+}]^2): the TS strip at this
    amplitude and the end of the damping ramp turn the mean wall vorticity
    negative within the first step, where the reference's sqrt(Re wz_wall)
    (les_par.f:194) is NaN.  The Poisson tolerance defaults to 1e-8: on this
    grid the FP64 defect itself carries round-off of ~6e-9 (first cell
    0.005 delta*), so 1e-10 is not reachable in FP64.

    nx other than 2049 keeps the 12 wavelengths (nx=1025: config 2's x
    spacing, where the reference's plain multigrid still converges on this
    wall-normal grid; at 2049 points it diverges on the low modes)."""
    kw.setdefault("tol", 1e-8)
    kw.setdefault("amp2d", 3e-3)
    kw.setdefault("amp3d", 3e-3)
    kw.setdefault("my_form", 4)
    cfg = blasius_ts_config(nx, 257, 64, 128, 4, **kw)
    if "steps_per_period" not in kw:
        cfg.stpp = stable_steps_per_period(cfg)
    dstar = BLASIUS_DSTAR / math.sqrt(cfg.Re)
    cfg.ibm = 1
    cfg.ibm_xc = cfg.x0 + 0.25 * (cfg.nx - 1) * cfg.dx
    cfg.ibm_zc = math.pi / cfg.beta          # mid-span
    cfg.ibm_h = 0.5 * dstar
    cfg.ibm_R = 1.0 * dstar
    dt = 2.0 * math.pi / cfg.omega / cfg.stpp
    cfg.irf = -min(0.1 * cfg.Re, 2.0 / dt)
    cfg.C_s = 0.1
    cfg.A_plus = 26.0
    cfg.les_damping = 3
    return cfg


def stable_steps_per_period(cfg, limit=1.3):
    """Smallest power of two (>= 256) of steps per forcing period keeping the
    explicit RK4 viscous term at nu dt lambda_max <= limit, lambda_max =
    6.86 / dy0^2 (stability bound 2.78)."""
    period = 2.0 * math.pi / cfg.omega
    need = period * 6.86 / (cfg.Re * cfg.fac_y * cfg.dy ** 2 * limit)
    n = 256
    while n < need:
        n *= 2
    return n


def config3(seed=20261203, members=12, **kw):
    """Ensemble of independent runs of uneven sizes: nx in {257, 513, 769,
    1025}, ny in {97, 129, 193}, kfour in {8, 16, 32} (P = 2 kfour),
    F ~ U[0.6e-4, 1.4e-4], 2D TS amplitude ~ log-U[1e-6, 1e-4] with an
    oblique pair at a tenth of it; each member at the steps per period its
    first cell needs.  Drawn from numpy's PCG64 seeded with `seed`."""
    rng = np.random.default_rng(seed)
    out = []
    for m in range(members):
        nx = int(rng.choice([257, 513, 769, 1025]))
        ny = int(rng.choice([97, 129, 193]))
        K = int(rng.choice([8, 16, 32]))
        F = float(rng.uniform(0.6e-4, 1.4e-4))
        A = float(math.exp(rng.uniform(math.log(1e-6), math.log(1e-4))))
        args = dict(F=F, amp2d=A, amp3d=0.1 * A, seed=seed + 1 + m)
        args.update(kw)
        cfg = blasius_ts_config(nx, ny, K, 2 * K, 4, **args)
        if "steps_per_period" not in kw:
            cfg.stpp = stable_steps_per_period(cfg)
        out.append(cfg)
    return out


def small(nx=65, ny=33, kfour=4, kphys=8, msh=3, **kw):
    """A small grid for parity tests (seconds on the CPU oracle)."""
    kw.setdefault("amp3d", 1e-5)
    kw.setdefault("n_lambda", 4.0)
    kw.setdefault("strip", (1.0, 1.6))
    return blasius_ts_config(nx, ny, kfour, kphys, msh, **kw)


def gortler(nx=65, ny=33, kfour=4, kphys=8, msh=3, go_number=0.0, **kw):
    """Goertler form (my_form 1, drv_gv, main_par.f:1338-1401): every Fourier
    mode a linear disturbance about the 2D base flow, forced by the steady
    wall strip of gv_pert (modes k >= 1, amplitude 1e-6) over i1..i2, with
    the wall curvature of Goertler number go_number (0 in the reference).
    The ramp of the third mode's buffer zone, over i = 1 .. 2 (i1 + i2), is
    clamped to nx."""
    cfg = small(nx=nx, ny=ny, kfour=kfour, kphys=kphys, msh=msh, my_form=1, **kw)
    cfg.go_number = go_number
    return cfg


def thermal(nx=65, ny=33, kfour=4, kphys=8, msh=3, **kw):
    """Thermal form (my_form 2, drv_gvth, main_par.f:1404-1484): the
    disturbance with its full nonlinear products about the 2D base flow and
    a transported temperature th (Prandtl number Pr, 0.72), forced by the TS
    strip of ts2d_pert."""
    return small(nx=nx, ny=ny, kfour=kfour, kphys=kphys, msh=msh, my_form=2, **kw)


def base_temperature(cfg, base):
    """A base temperature for the thermal form: thb = 1 - uxb / U_e, the
    profile of a heated wall by Reynolds' analogy.  The reference reads its
    thb from the 2D thermal base-flow marcher's output, which it does not
    ship."""
    uxb = base[0]
    return 1.0 - uxb / uxb[-1:, :]


NAMES = ("ux", "uy", "uz", "wx", "wy", "wz")


def smooth_random(shape, rng, scale=1.0):
    """Complex field with mode 0 real, smooth in x and y (sum of few waves)."""
    K, ny, nx = shape
    x = np.linspace(0, 1, nx)[None, :]
    y = np.linspace(0, 1, ny)[:, None]
    f = np.zeros(shape, dtype=np.complex128)
    for k in range(K):
        acc = np.zeros((ny, nx), dtype=np.complex128)
        for _ in range(3):
            a, b = rng.uniform(0.5, 4.0, 2)
            p = rng.uniform(0, 2 * np.pi, 2)
            c = rng.normal() + 1j * rng.normal()
            acc += c * np.sin(a * np.pi * x + p[0]) * np.cos(b * np.pi * y + p[1])
        f[k] = acc * scale / (1 + k)
    f[0] = f[0].real
    return f


def disturbed_state(cfg, base, rng, amp=1e-3):
    """Base flow plus a smooth seeded disturbance of relative size amp in
    every field and mode; velocities keep the no-slip wall row."""
    uxb, uyb, wzb = base
    st = {}
    for n in NAMES:
        st[n] = smooth_random((cfg.kfour, cfg.ny, cfg.nx), rng, amp)
    for n in ("ux", "uy", "uz"):
        st[n][:, 0, :] = 0.0
    st["ux"][0] += uxb
    st["uy"][0] += uyb
    st["wz"][0] += wzb
    return st


def disturbance_state(cfg, rng, amp=1e-3):
    """A smooth seeded disturbance of size amp in every field and mode, no
    base flow (the Goertler form's state); velocities keep the no-slip wall
    row."""
    st = {n: smooth_random((cfg.kfour, cfg.ny, cfg.nx), rng, amp) for n in NAMES}
    for n in ("ux", "uy", "uz"):
        st[n][:, 0, :] = 0.0
    return st


def setup_inputs(cfg):
    """Coefficient blob and Blasius base flow for cfg (the library's generators)."""
    coefs = api.generate_coefs(cfg.stf, cfg.msh)
    base = api.baseflow_fs(cfg, 0.0)
    return coefs, base
