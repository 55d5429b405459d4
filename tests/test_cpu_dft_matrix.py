"""The DFT matrices of the tensor-core nonlinear-term passes against the
oracle's FP64 spectral transforms (nlterms_par.f's realft convention)."""
import numpy as np
import pytest

from tests.helpers import small_case


@pytest.mark.parametrize("P", [16, 32, 64])
def test_dft_matrices_match_oracle(oracle_built, P):
    from trans_bl_gb300 import api
    cfg, coefs, base = small_case(nx=65, ny=33, kfour=P // 2, kphys=P, msh=3)
    o = oracle_built.Oracle(cfg, coefs, base)
    rng = np.random.default_rng(P)
    K = P // 2
    four = rng.normal(0, 1, (K, cfg.ny, cfg.nx)) + 1j * rng.normal(0, 1, (K, cfg.ny, cfg.nx))
    four[0] = 1j * four[0].imag            # the mean (Re c0) stays out of the matrices
    phys = o.f_to_p(four)                  # (P, ny, nx)
    slots = np.zeros((P, cfg.ny, cfg.nx))
    slots[1] = four[0].imag
    for k in range(1, K):
        slots[2 * k], slots[2 * k + 1] = four[k].real, four[k].imag
    Ti = api.dft_matrix(P, False)
    got = np.einsum("zs,sji->zji", Ti, slots)
    assert np.max(np.abs(got - phys)) <= 1e-12 * np.max(np.abs(phys))
    Tf = api.dft_matrix(P, True)
    back = o.p_to_f(phys)                  # Im c0 = 0 as nlterms does
    s2 = np.einsum("sz,zji->sji", Tf, phys)
    want = np.zeros_like(s2)
    want[0] = back[0].real
    for k in range(1, K):
        want[2 * k], want[2 * k + 1] = back[k].real, back[k].imag
    assert np.max(np.abs(s2 - want)) <= 1e-12 * np.max(np.abs(want))
    o.close()
