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
           dict(precision=7), dict(my_form=2)]
    for b in bad:
        cfg = api.default_config(**b)
        h = C.c_void_p()
        rc = lib_built.tb_create(C.byref(cfg), C.byref(h))
        assert rc == 1, (b, rc)
        assert lib_built.tb_last_error()


def test_coef_count(lib_built):
    assert lib_built.tb_coef_count(4) == 100 + 24 * 4
