"""TS-wave amplification of a run against linear stability theory.

The analysis of the reference's ftanalysis_par.f, on snapshots of ux:
  - temporal Fourier transform over one forcing period of N equally spaced
    snapshots (fft1d, ftanalysis_par.f:23-38): amplitude of harmonic f,
  - its wall-normal maximum from the parabola through the three points
    around the discrete maximum (polcoe, ftanalysis_par.f:40-60; here on the
    exact stretched y of those points),
  - the streamwise growth rate d ln(A_max)/dx by the 6th-order central
    difference of derfax (ftanalysis_par.f:171-190),
and the growth rate of the spatial LST (tb_lst_march, lst_ts/ose_bl.f) at the
same stations, -Im(alpha0) Re / Re^(1/2) in units of the run (x0 = 1).
"""
import numpy as np

from . import api


def fourier_amplitude(snaps, harmonic=1):
    """|DFT coefficient| of the given harmonic over N snapshots of one period
    (snaps: array (N, ...)); the one-sided amplitude of a real signal."""
    n = snaps.shape[0]
    c = np.fft.fft(snaps, axis=0) / n
    return 2.0 * np.abs(c[harmonic])


def wall_normal_max(a, y):
    """Max over y (axis -2 of a (..., ny, nx)) by a parabola through the
    discrete maximum and its neighbours."""
    ny = a.shape[-2]
    jj = np.clip(np.argmax(a, axis=-2), 1, ny - 2)
    out = np.empty(a.shape[:-2] + a.shape[-1:])
    for idx in np.ndindex(*out.shape):
        i = idx[-1]
        j = jj[idx]
        col = a[idx[:-1] + (slice(None), i)]
        xs, ys = y[j - 1:j + 2], col[j - 1:j + 2]
        c2, c1, c0 = np.polyfit(xs, ys, 2)
        out[idx] = c0 - 0.25 * c1 * c1 / c2 if c2 < 0 else ys.max()
    return out


def growth_rate(f, dx):
    """d f / dx by the 6-point central difference of derfax; NaN at the 3
    points next to each end."""
    g = np.full_like(f, np.nan)
    g[3:-3] = (-f[:-6] + 9 * f[1:-5] - 45 * f[2:-4] + 45 * f[4:-2] - 9 * f[5:-1] + f[6:]) / (60.0 * dx)
    return g


def y_coordinates(cfg):
    j = np.arange(cfg.ny)
    if cfg.stf == 1.0:
        return j * cfg.dy
    return cfg.dy * (cfg.stf ** j - 1.0) / (cfg.stf - 1.0)


def lst_growth(cfg, steps=1000, with_alpha=False):
    """LST growth rate at the stations x = x0 + i dx of a run of cfg (2D
    wave, Blasius wall shear), in units of the run; starts from the
    reference's namelist point of lst_ts/ose3d.in.  with_alpha: also the
    streamwise wavenumber alpha_r in the same units."""
    rein = np.sqrt(cfg.Re * cfg.x0)
    w0in = 2.6134e-2
    w_target = cfg.omega / cfg.Re * rein
    # the continuation stops one step short of its target (ose_bl.f:55-58)
    omega_dns = w0in + (w_target - w0in) / ((steps - 1.0) / steps)
    out = api.lst_march(751.50, w0in, complex(0.08658, 1.9598e-5), rein, omega_dns, 0.0, cfg.nx, cfg.dx / cfg.x0,
                        0.33205733621540984, steps=steps)
    x, sigma = cfg.x0 * out["x"], -out["alpha"].imag * cfg.Re / out["re0"]
    if with_alpha:
        return x, sigma, out["alpha"].real * cfg.Re / out["re0"]
    return x, sigma


def amplitude_along_x(ctx, cfg, base_ux, t0, periods, n_snap=16):
    """Advance ctx for `periods` forcing periods from step t0 and return
    A_max(x), the wall-normal maximum of the ux amplitude at the forcing
    frequency from n_snap snapshots over the last period (2D wave, mode 0)."""
    stride = cfg.stpp // n_snap
    nsteps = periods * cfg.stpp
    snaps = []
    for q in range(nsteps):
        ctx.step(t0 + q)
        left = nsteps - 1 - q
        if left < cfg.stpp and (cfg.stpp - 1 - left) % stride == stride - 1:
            snaps.append(ctx.get_state()["ux"][0].real - base_ux)
    a = fourier_amplitude(np.array(snaps[-n_snap:]))
    return wall_normal_max(a, y_coordinates(cfg))
