"""ctypes binding of the CPU oracle (oracle/tb_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by the test suite, the smoke check and
the CPU-baseline leg of bench.py, to compare against; never by the library.
Array conventions follow trans_bl_gb300.api (complex128, shape (K, ny, nx)).
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libtb_oracle.so")
_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB):
        build()
    from trans_bl_gb300.api import TbConfig
    lib = C.CDLL(LIB)
    P, D = C.c_void_p, C.POINTER(C.c_double)
    lib.ora_create.restype = P
    lib.ora_create.argtypes = [C.POINTER(TbConfig)]
    lib.ora_destroy.argtypes = [P]
    lib.ora_set_coefs.argtypes = [P, D]
    lib.ora_set_baseflow.argtypes = [P, D, D, D]
    lib.ora_init_fields.argtypes = [P]
    lib.ora_put_state.argtypes = [P] + [D] * 6
    lib.ora_get_state.argtypes = [P] + [D] * 6
    lib.ora_put_wall.argtypes = [P, D]
    lib.ora_get_wall.argtypes = [P, D]
    for n in ("ora_derparx", "ora_derparxx", "ora_dery", "ora_deryfv", "ora_deryy", "ora_f_to_p", "ora_p_to_f"):
        getattr(lib, n).argtypes = [P, D, D]
    for n in ("ora_nlterms", "ora_drv", "ora_les_terms", "ora_cvirt"):
        getattr(lib, n).argtypes = [P, D, D, D]
    for n in ("ora_filter_trid", "ora_bzone", "ora_bzonew"):
        getattr(lib, n).argtypes = [P]
    lib.ora_outuy.argtypes = [P, D]
    lib.ora_poi_uy.argtypes = [P, D, C.c_double]
    lib.ora_poi_ux.argtypes = [P, D]
    lib.ora_poi_uz.argtypes = [P, D]
    lib.ora_wx_wall.argtypes = [P, D]
    lib.ora_wz_wall.argtypes = [P, D]
    lib.ora_ts_pert.argtypes = [P, C.c_int, C.c_double]
    for n in ("ora_set_baseflow_th", "ora_put_th", "ora_get_th"):
        getattr(lib, n).argtypes = [P, D]
    lib.ora_loop.argtypes = [P, C.c_double]
    lib.ora_rk_stage.argtypes = [P, C.c_int, C.c_int]
    lib.ora_step.argtypes = [P, C.c_int]
    lib.ora_poisson_stats.argtypes = [P, C.POINTER(C.c_int), D]
    lib.ora_set_threads.argtypes = [C.c_int]
    lib.ora_set_threads.restype = C.c_int
    lib.ora_generate_coefs.argtypes = [C.c_double, C.c_int, D]
    lib.ora_generate_fp_fd.argtypes = [C.c_double, D]
    lib.ora_fs_wall_shear.argtypes = [C.c_double, D]
    lib.ora_baseflow_fs.argtypes = [C.POINTER(TbConfig), C.c_double, D, D, D]
    _lib = lib
    return lib


def default_config(**kw):
    """A tb_config with the reference's par.for constants (par.for:34-129)
    and the given fields, built without the GPU library."""
    from trans_bl_gb300.api import TbConfig, FORM_PLAIN_FP64
    cfg = TbConfig()
    d = dict(nx=129, ny=65, kfour=4, kphys=8, msh=3, my_form=0, i0=10, i1=22, i2=36, i3=100, i4=115, stpp=368,
             max_vcycles=11, ibm=0, precision=FORM_PLAIN_FP64, les_damping=0, warm_start=2, step_graph=1,
             Re=5.0 * 0.1 / 1.509479531e-5, dx=0.02962963, dy=0.15 / 182.0, stf=1.0, x0=1.0, alpha=0.45723605,
             omega=2.6, beta=34.9, fac_y=1.0, alphaf=0.48, tol_stage=1e-5, tol_final=1e-6, C_s=0.032, A_plus=25.0,
             ibm_xc=1.7, ibm_zc=0.0, ibm_h=0.0, ibm_R=1e-2 / 0.1, n_forced=1, forced_mode=[0], forced_amp=[1e-5],
             forced_phase=[0.0], go_number=0.0, Pr=0.72)
    d["irf"] = -0.1 * d["Re"]
    d.update(kw)
    for k, v in d.items():
        if k in ("forced_mode", "forced_amp", "forced_phase"):
            arr = getattr(cfg, k)
            for q in range(4):
                arr[q] = v[q] if q < len(v) else 0
        else:
            setattr(cfg, k, v)
    return cfg


def generate_coefs(stf, msh):
    """The coefficient blob of tb_set_coefs (100 + 24 msh doubles)."""
    blob = np.zeros(100 + 24 * msh)
    if load().ora_generate_coefs(float(stf), int(msh), _d(blob)) != 0:
        raise ValueError("oracle coefficient generator failed")
    return blob


def generate_fp_fd(stf):
    out = np.zeros(7)
    if load().ora_generate_fp_fd(float(stf), _d(out)) != 0:
        raise ValueError("oracle coefficient generator failed")
    return out


def fs_wall_shear(beta_fs=0.0):
    v = np.zeros(1)
    if load().ora_fs_wall_shear(float(beta_fs), _d(v)) != 0:
        raise ValueError("Falkner-Skan shooting failed")
    return float(v[0])


def baseflow_fs(cfg, beta_fs=0.0):
    """(uxb, uyb, wzb), each (ny, nx)."""
    shape = (cfg.ny, cfg.nx)
    ux, uy, wz = np.zeros(shape), np.zeros(shape), np.zeros(shape)
    if load().ora_baseflow_fs(C.byref(cfg), float(beta_fs), _d(ux), _d(uy), _d(wz)) != 0:
        raise ValueError("Falkner-Skan base flow failed")
    return ux, uy, wz


def setup_inputs(cfg):
    """Coefficient blob and Blasius base flow for cfg, from the oracle alone."""
    return generate_coefs(cfg.stf, cfg.msh), baseflow_fs(cfg, 0.0)


def _d(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Oracle:
    """Mirror of trans_bl_gb300.api.Context running the CPU restatement."""

    NAMES = ("ux", "uy", "uz", "wx", "wy", "wz")

    def __init__(self, cfg, coefs, baseflow, init=True):
        self.lib = load()
        self.cfg = cfg
        self.h = self.lib.ora_create(C.byref(cfg))
        if not self.h:
            raise ValueError("oracle rejected the configuration")
        self.shape = (cfg.kfour, cfg.ny, cfg.nx)
        blob = np.ascontiguousarray(coefs, dtype=np.float64)
        self.lib.ora_set_coefs(self.h, _d(blob))
        b = [np.ascontiguousarray(x, dtype=np.float64) for x in baseflow]
        self.lib.ora_set_baseflow(self.h, *[_d(x) for x in b])
        if init:
            self.lib.ora_init_fields(self.h)

    def init_fields(self):
        self.lib.ora_init_fields(self.h)

    def set_baseflow_th(self, thb):
        a = np.ascontiguousarray(thb, dtype=np.float64)
        self.lib.ora_set_baseflow_th(self.h, _d(a))

    def put_th(self, th):
        a = np.ascontiguousarray(th, dtype=np.complex128)
        self.lib.ora_put_th(self.h, _d(a.view(np.float64)))

    def get_th(self):
        a = self.field()
        self.lib.ora_get_th(self.h, _d(a.view(np.float64)))
        return a

    def close(self):
        if self.h:
            self.lib.ora_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def field(self):
        return np.zeros(self.shape, dtype=np.complex128)

    def put_state(self, s):
        a = [np.ascontiguousarray(s[n], dtype=np.complex128) for n in self.NAMES]
        self.lib.ora_put_state(self.h, *[_d(x.view(np.float64)) for x in a])

    def get_state(self):
        out = {n: self.field() for n in self.NAMES}
        self.lib.ora_get_state(self.h, *[_d(out[n].view(np.float64)) for n in self.NAMES])
        return out

    def put_wall(self, w):
        a = np.ascontiguousarray(w, dtype=np.complex128)
        self.lib.ora_put_wall(self.h, _d(a.view(np.float64)))

    def get_wall(self):
        a = np.zeros((self.cfg.kfour, self.cfg.nx), dtype=np.complex128)
        self.lib.ora_get_wall(self.h, _d(a.view(np.float64)))
        return a

    def _unary(self, name, f):
        f = np.ascontiguousarray(f, dtype=np.complex128)
        out = self.field()
        getattr(self.lib, name)(self.h, _d(out.view(np.float64)), _d(f.view(np.float64)))
        return out

    def derparx(self, f): return self._unary("ora_derparx", f)
    def derparxx(self, f): return self._unary("ora_derparxx", f)
    def dery(self, f): return self._unary("ora_dery", f)
    def deryfv(self, f): return self._unary("ora_deryfv", f)
    def deryy(self, f): return self._unary("ora_deryy", f)

    def f_to_p(self, four):
        four = np.ascontiguousarray(four, dtype=np.complex128)
        out = np.zeros((self.cfg.kphys, self.cfg.ny, self.cfg.nx))
        self.lib.ora_f_to_p(self.h, _d(out), _d(four.view(np.float64)))
        return out

    def p_to_f(self, phys):
        phys = np.ascontiguousarray(phys, dtype=np.float64)
        out = self.field()
        self.lib.ora_p_to_f(self.h, _d(out.view(np.float64)), _d(phys))
        return out

    def _three(self, name):
        a, b, c = self.field(), self.field(), self.field()
        getattr(self.lib, name)(self.h, *[_d(x.view(np.float64)) for x in (a, b, c)])
        return a, b, c

    def nlterms(self): return self._three("ora_nlterms")
    def drv(self): return self._three("ora_drv")
    def les_terms(self): return self._three("ora_les_terms")
    def cvirt(self): return self._three("ora_cvirt")
    def filter_trid(self): self.lib.ora_filter_trid(self.h)
    def bzone(self): self.lib.ora_bzone(self.h)
    def bzonew(self): self.lib.ora_bzonew(self.h)
    def loop(self, erro): self.lib.ora_loop(self.h, float(erro))
    def rk_stage(self, stage, t): self.lib.ora_rk_stage(self.h, int(stage), int(t))
    def step(self, t): self.lib.ora_step(self.h, int(t))
    def ts_pert(self, t, tempt): self.lib.ora_ts_pert(self.h, int(t), float(tempt))

    def outuy(self):
        out = self.field()
        self.lib.ora_outuy(self.h, _d(out.view(np.float64)))
        return out

    def poi_uy(self, dwzdx, erro):
        a = np.ascontiguousarray(dwzdx, dtype=np.complex128)
        self.lib.ora_poi_uy(self.h, _d(a.view(np.float64)), float(erro))

    def poi_ux(self):
        out = self.field()
        self.lib.ora_poi_ux(self.h, _d(out.view(np.float64)))
        return out

    def poi_uz(self, duydy):
        a = np.ascontiguousarray(duydy, dtype=np.complex128)
        self.lib.ora_poi_uz(self.h, _d(a.view(np.float64)))

    def wx_wall(self):
        out = np.zeros((self.cfg.kfour, self.cfg.nx), dtype=np.complex128)
        self.lib.ora_wx_wall(self.h, _d(out.view(np.float64)))
        return out

    def wz_wall(self, lapv):
        a = np.ascontiguousarray(lapv, dtype=np.complex128)
        self.lib.ora_wz_wall(self.h, _d(a.view(np.float64)))

    def poisson_stats(self):
        K = self.cfg.kfour
        v = (C.c_int * K)()
        r = np.zeros(K)
        self.lib.ora_poisson_stats(self.h, v, _d(r))
        return list(v), r


def set_threads(n):
    """Host threads of the oracle's parallel loops; returns the count in use."""
    return int(load().ora_set_threads(int(n)))
