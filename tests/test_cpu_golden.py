"""Known-answer tests against the reference's own data files (CPU only).

Fixtures in tests/golden/ were extracted from the reference by
tests/golden/make_golden.py: pre_processing/coefs.bin (compact-scheme,
Poisson and wall coefficients at stretching 1.01, 4 levels) and
lst_ts/fpp.dat (Blasius wall shear).
"""
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")

ORDER = [("fp_fd_e", 6), ("sp_fd", 9), ("cp_fd", 8), ("pp_fd", 9), ("lp_fd", 7), ("fp_sd", 8), ("sp_sd", 10),
         ("cp_sd", 8), ("pp_sd", 10), ("lp_sd", 8), ("sp_poi", 28), ("cp_poi", 32), ("pp_poi", 16),
         ("lp_poi", 20), ("w_at_w", 9), ("dwydy", 8)]


@pytest.fixture(scope="module")
def golden():
    return json.load(open(os.path.join(GOLD, "coefs_stf1.01_lvl4.json")))["records"]


def test_coefficient_generator_matches_coefs_bin(lib_built, golden):
    from trans_bl_gb300 import api
    blob = api.generate_coefs(1.01, 4)
    off = 0
    for name, n in ORDER:
        v = blob[off:off + n]
        off += n
        if name == "fp_fd_e":
            continue  # not stored in coefs.bin (its record 1 holds fp_fd, tested below)
        ref = np.array(golden[name])
        np.testing.assert_allclose(v, ref, rtol=1e-12, atol=1e-13, err_msg=name)
    assert off == api.coef_count(4)


def test_first_record_is_compact_first_point(lib_built, golden):
    from trans_bl_gb300 import api
    np.testing.assert_allclose(api.generate_fp_fd(1.01), golden["record1_stale_fp_fd"], rtol=1e-12)


def test_explicit_first_point_uniform_limit(lib_built):
    # stretching 1: the explicit wall derivative is the 5-point one-sided rule
    # of rhsx row 1 (derivs_par.f:269-271): (-25, 48, -36, 16, -3) / 12
    from trans_bl_gb300 import api
    blob = api.generate_coefs(1.0, 2)
    np.testing.assert_allclose(blob[:6], [12, -25, 48, -36, 16, -3], rtol=1e-13, atol=1e-12)


def test_blasius_wall_shear_matches_fpp_dat(lib_built):
    from trans_bl_gb300 import api
    fpp = json.load(open(os.path.join(GOLD, "fpp.json")))["fpp"]
    assert len(set(fpp)) == 1
    got = api.fs_wall_shear(0.0) * np.sqrt(0.5)
    assert abs(got - fpp[0]) <= 1e-13 * fpp[0]


def test_blasius_profile_properties(lib_built):
    from trans_bl_gb300 import api, configs
    cfg = configs.small()
    ux, uy, wz = api.baseflow_fs(cfg, 0.0)
    assert ux.shape == (cfg.ny, cfg.nx)
    assert np.all(ux[0] == 0.0) and abs(ux[-1, 0] - 1.0) < 1e-6
    assert np.all(np.diff(ux[:, 0]) > -1e-12)
    assert np.all(wz[0] > 0)


# The oracle's own restatement of the pre-processing (oracle/tb_inputs.cpp),
# which builds the CPU baseline's inputs without the GPU library, against the
# same golden data and against the library's generator.
def test_oracle_coefficient_generator_matches_coefs_bin(oracle_built, golden):
    blob = oracle_built.generate_coefs(1.01, 4)
    off = 0
    for name, n in ORDER:
        v = blob[off:off + n]
        off += n
        if name == "fp_fd_e":
            continue
        np.testing.assert_allclose(v, np.array(golden[name]), rtol=1e-12, atol=1e-13, err_msg=name)
    np.testing.assert_allclose(oracle_built.generate_fp_fd(1.01), golden["record1_stale_fp_fd"], rtol=1e-12)


def test_oracle_inputs_match_library(lib_built, oracle_built):
    from trans_bl_gb300 import api, configs
    for stf, msh in ((1.02, 3), (1.02, 4), (1.0, 2)):
        np.testing.assert_allclose(oracle_built.generate_coefs(stf, msh), api.generate_coefs(stf, msh),
                                   rtol=1e-13, atol=1e-14)
    cfg = configs.small(make_default=oracle_built.default_config)
    assert cfg.as_dict() == configs.small().as_dict()
    fpp = oracle_built.fs_wall_shear(0.0)
    gold = json.load(open(os.path.join(GOLD, "fpp.json")))["fpp"][0]
    assert abs(fpp * np.sqrt(0.5) - gold) <= 1e-13 * gold
    for a, b in zip(oracle_built.baseflow_fs(cfg), api.baseflow_fs(cfg)):
        np.testing.assert_allclose(a, b, rtol=0, atol=1e-14 * np.max(np.abs(b)))
