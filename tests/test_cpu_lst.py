"""Linear stability (lst_ts/ose_bl.f) against the reference's own station log.

lst_ts/saida records, for each of 665 stations of the reference's LST march,
x, Re^(1/2), the scaled frequency and the converged eigenvalue alpha0.  The
run started from the namelist of lst_ts/ose3d.in (Re^(1/2) = 751.5,
w0 = 2.6134e-2, alpha0 = 0.08658 + 1.9598e-5 i, beta = 0) and continued to
Re^(1/2) = 604.15 in 1000 steps per parameter; its target frequency follows
from the logged frequency at x = 1, which the continuation reaches at step
999 of 1000 (ose_bl.f:55-58).  The restatement follows the same path, so the
eigenvalues agree to the secant tolerance of the reference (ose_bl.f:406-412).
"""
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def march(lib_built):
    from trans_bl_gb300 import api
    g = json.load(open(os.path.join(HERE, "golden", "lst_saida.json")))
    rows = np.array(g["rows_x_re0_w0_alpha_re_alpha_im"])
    nml = g["osedata"]
    f = lambda s: float(s.replace("d", "e"))
    a0 = [float(t.replace("d", "e")) for t in nml["alfa0"].strip("()").split(",")]
    w0in = f(nml["w0"])
    re_dns, w0_x1 = rows[0, 1], rows[0, 2]
    omega_dns = w0in + (w0_x1 - w0in) / 0.999
    out = api.lst_march(f(nml["re0"]), w0in, complex(*a0), re_dns, omega_dns, f(nml["beta"]), g["stations"], 6.25e-3,
                        0.33205733621540984, jedge=int(nml["jedge"]), bl=f(nml["bl"]), etamax=f(nml["etamax"]),
                        wslope=f(nml["wslope"]))
    return out, rows, np.array(g["index"])


def test_stations(march):
    out, rows, idx = march
    assert np.allclose(out["x"][idx], rows[:, 0], rtol=1e-12)
    assert np.allclose(out["re0"][idx], rows[:, 1], rtol=1e-12)
    assert np.allclose(out["w0"][idx], rows[:, 2], rtol=1e-12)


def test_eigenvalues(march):
    out, rows, idx = march
    a = out["alpha"][idx]
    assert np.max(np.abs(a.real - rows[:, 3]) / np.abs(rows[:, 3])) < 1e-5
    assert np.max(np.abs(a.imag - rows[:, 4])) < 1e-6          # growth rate -Im(alpha0)
    # branch I/II: the growth rate changes sign where the reference's does
    assert np.array_equal(np.sign(a.imag), np.sign(rows[:, 4]))
