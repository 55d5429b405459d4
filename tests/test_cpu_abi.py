"""The C ABI: every entry point of include/transbl.h is exported, and
configuration errors are reported without touching a GPU."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    src = open(os.path.join(ROOT, "include", "transbl.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(tb_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_entry_points():
    names = header_functions()
    assert "tb_create" in names and "tb_poi_uy" in names and len(names) > 40


def test_library_exports_every_declared_symbol(lib_built):
    missing = [n for n in header_functions() if not hasattr(lib_built, n)]
    assert not missing, missing


def test_bad_configs_are_rejected(lib_built):
    from trans_bl_gb300 import api
    bad = [dict(nx=66), dict(ny=30), dict(kphys=12), dict(kfour=9, kphys=16), dict(msh=1), dict(i2=5),
           dict(precision=7), dict(my_form=3), dict(my_form=2, ibm=1), dict(my_form=2, Pr=0.0)]
    for b in bad:
        cfg = api.default_config(**b)
        h = C.c_void_p()
        rc = lib_built.tb_create(C.byref(cfg), C.byref(h))
        assert rc == 1, (b, rc)
        assert lib_built.tb_last_error()


def test_coef_count(lib_built):
    assert lib_built.tb_coef_count(4) == 100 + 24 * 4


def header_prototypes():
    src = open(os.path.join(ROOT, "include", "transbl.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return {m.group(1): m.group(2) for m in re.finditer(r"\b(tb_[a-z0-9_]+)\s*\(([^)]*)\)\s*;", src)}


def test_pointer_arguments_have_ctypes_prototypes():
    """ctypes passes undeclared arguments as C int: a function taking a
    pointer must have argtypes in api.load(), or its pointers get truncated."""
    from trans_bl_gb300 import api
    lib = api.load()
    missing = [n for n, args in header_prototypes().items() if "*" in args and getattr(lib, n).argtypes is None]
    assert not missing, missing


def test_dft_matrix_sizes():
    import numpy as np
    from trans_bl_gb300 import api
    for P in (16, 128):
        Ti, Tf = api.dft_matrix(P, False), api.dft_matrix(P, True)
        # forward after inverse is the identity on the slots the transforms keep
        # (Re c0 is the mean, carried outside the matrices; Im c0 is dropped forward)
        M = Tf @ Ti
        keep = np.arange(2, P)
        assert np.max(np.abs(M[np.ix_(keep, keep)] - np.eye(P - 2))) < 1e-12
    with pytest.raises(api.TbError):
        api.dft_matrix(12, False)
