"""ctypes binding of the C ABI in include/transbl.h.

Fields are numpy complex128 arrays of shape (kfour, ny, nx), C-contiguous:
the same memory as the reference's Fortran complex*16 f(nx, ny, kfour).
The library is the CUDA build in this package directory; there is no CPU
fallback -- loading fails loudly when it is missing.
"""
import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libtransbl.so")

TB_OK = 0
TB_ERR = {1: "TB_ERR_ARG", 2: "TB_ERR_CUDA", 3: "TB_ERR_NOCONV", 4: "TB_ERR_NONFINITE",
          5: "TB_ERR_TIMEOUT", 6: "TB_ERR_STATE", 7: "TB_ERR_NOMEM"}
FORM_PLAIN_FP64 = 0
FORM_MIXED = 1


class TbConfig(C.Structure):
    """Mirror of struct tb_config (runtime replacement of par.for)."""
    _fields_ = [(n, C.c_int) for n in (
        "nx", "ny", "kfour", "kphys", "msh", "my_form", "i0", "i1", "i2", "i3", "i4", "stpp",
        "max_vcycles", "ibm", "precision", "les_damping", "warm_start", "step_graph")] + \
        [(n, C.c_double) for n in (
            "Re", "dx", "dy", "stf", "x0", "alpha", "omega", "beta", "fac_y", "alphaf", "tol_stage",
            "tol_final", "C_s", "A_plus", "irf", "ibm_xc", "ibm_zc", "ibm_h", "ibm_R")] + \
        [("n_forced", C.c_int), ("forced_mode", C.c_int * 4), ("forced_amp", C.c_double * 4),
         ("forced_phase", C.c_double * 4), ("go_number", C.c_double), ("Pr", C.c_double)]

    def as_dict(self):
        d = {}
        for n, _ in self._fields_:
            v = getattr(self, n)
            d[n] = list(v) if hasattr(v, "__len__") else v
        return d


class PoissonStats(C.Structure):
    _fields_ = [("vcycles", C.c_int * 256), ("residual", C.c_double * 256), ("total_vcycles", C.c_int),
                ("solves", C.c_int), ("noconv", C.c_int)]


class LstConfig(C.Structure):
    """struct tb_lst_config (include/transbl.h)."""
    _fields_ = [(n, C.c_double) for n in ("re0", "w0", "alfa0_re", "alfa0_im")] + [("jedge", C.c_int)] + \
        [(n, C.c_double) for n in ("bl", "etamax", "beta", "wslope", "re_dns", "omega_dns", "beta_dns")] + \
        [("imax", C.c_int), ("dx", C.c_double), ("steps", C.c_int)]


class LearnStats(C.Structure):
    _fields_ = [("samples", C.c_longlong), ("capacity", C.c_longlong), ("tried", C.c_longlong),
                ("kept", C.c_longlong), ("loss", C.c_double), ("solves", C.c_longlong), ("evaluated", C.c_longlong)]


class TuneResult(C.Structure):
    _fields_ = [("xline_warps", C.c_int), ("yline_threads", C.c_int), ("nl_blocks_per_sm", C.c_int),
                ("xline_ms", C.c_float), ("yline_ms", C.c_float), ("nl_ms", C.c_float),
                ("plain_line_warps_multi", C.c_int), ("plain_line_warps_single", C.c_int),
                ("plain_multi_ms", C.c_float), ("plain_single_ms", C.c_float)]


class TbError(RuntimeError):
    pass


_lib = None


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise TbError("CUDA library %s is missing: build it with `python -m trans_bl_gb300.build`" % LIB_PATH)
    lib = C.CDLL(LIB_PATH)
    P = C.c_void_p
    D = C.POINTER(C.c_double)
    lib.tb_last_error.restype = C.c_char_p
    lib.tb_dt.restype = C.c_double
    lib.tb_dt.argtypes = [C.POINTER(TbConfig)]
    lib.tb_launch_count.restype = C.c_longlong
    lib.tb_launch_count.argtypes = [P]
    lib.tb_create.argtypes = [C.POINTER(TbConfig), C.POINTER(P)]
    lib.tb_config_default.argtypes = [C.POINTER(TbConfig)]
    lib.tb_coef_count.argtypes = [C.c_int]
    lib.tb_generate_coefs.argtypes = [C.c_double, C.c_int, D]
    lib.tb_generate_fp_fd.argtypes = [C.c_double, D]
    lib.tb_fs_wall_shear.argtypes = [C.c_double, D]
    lib.tb_baseflow_fs.argtypes = [C.POINTER(TbConfig), C.c_double, D, D, D]
    for n in ("tb_destroy", "tb_init_fields", "tb_synchronize", "tb_filter_trid", "tb_bzone", "tb_bzonew"):
        getattr(lib, n).argtypes = [P]
    lib.tb_set_coefs.argtypes = [P, D]
    lib.tb_set_baseflow.argtypes = [P, D, D, D]
    lib.tb_put_state.argtypes = [P] + [D] * 6
    lib.tb_get_state.argtypes = [P] + [D] * 6
    lib.tb_put_wall.argtypes = [P, D]
    for n in ("tb_set_baseflow_th", "tb_put_th", "tb_get_th"):
        getattr(lib, n).argtypes = [P, D]
    lib.tb_get_wall.argtypes = [P, D]
    lib.tb_rk_stage.argtypes = [P, C.c_int, C.c_int]
    lib.tb_step.argtypes = [P, C.c_int]
    lib.tb_steps.argtypes = [P, C.c_int, C.c_int]
    lib.tb_get_poisson_stats.argtypes = [P, C.POINTER(PoissonStats)]
    for n in ("tb_derparx", "tb_derparxx", "tb_dery", "tb_deryfv", "tb_deryy", "tb_f_to_p", "tb_p_to_f"):
        getattr(lib, n).argtypes = [P, D, D]
    for n in ("tb_nlterms", "tb_drv", "tb_les_terms", "tb_cvirt"):
        getattr(lib, n).argtypes = [P, D, D, D]
    lib.tb_loop.argtypes = [P, C.c_double]
    lib.tb_outuy.argtypes = [P, D]
    lib.tb_poi_uy.argtypes = [P, D, C.c_double]
    lib.tb_poi_ux.argtypes = [P, D]
    lib.tb_poi_uz.argtypes = [P, D]
    lib.tb_wx_wall.argtypes = [P, D]
    lib.tb_wz_wall.argtypes = [P, D]
    lib.tb_ts_pert.argtypes = [P, C.c_int, C.c_double]
    lib.tb_device_field.argtypes = [P, C.c_int, C.POINTER(P)]
    lib.tb_stream.argtypes = [P, C.POINTER(P)]
    lib.tb_filter_trid_noalloc.argtypes = [P, P, P, C.c_int, C.c_int, C.c_int, C.c_double, P]
    lib.tb_profile.argtypes = [P, C.c_int]
    lib.tb_profile_read.argtypes = [P, C.c_int, D, C.POINTER(C.c_longlong)]
    lib.tb_lst_march.argtypes = [C.POINTER(LstConfig), D, D, D, D, D, D]
    lib.tb_write_checkpoint.argtypes = [P, C.c_char_p, C.c_int]
    lib.tb_read_checkpoint.argtypes = [P, C.c_char_p, C.POINTER(C.c_int)]
    lib.tb_write_pert.argtypes = [P, C.c_char_p]
    lib.tb_io_set_subrecord_limit.argtypes = [C.c_longlong]
    F = C.POINTER(C.c_float)
    lib.tb_nl_tensor_cores.argtypes = [P, C.c_int]
    lib.tb_tc_timeout_test.argtypes = [P, C.c_int]
    lib.tb_autotune.argtypes = [P, C.POINTER(TuneResult)]
    lib.tb_fp64_peak.argtypes = [D]
    lib.tb_mixed_fp32_lines.argtypes = [P, C.c_int]
    lib.tb_dft_matrix.argtypes = [C.c_int, C.c_int, D]
    lib.tb_learn_init.argtypes = [P, C.c_ulonglong]
    lib.tb_learn_set_weights.argtypes = [P, F]
    lib.tb_learn_get_weights.argtypes = [P, F]
    lib.tb_learn_enable.argtypes = [P, C.c_int]
    lib.tb_learn_sample.argtypes = [P, C.c_longlong, C.c_int, C.c_ulonglong]
    lib.tb_learn_train.argtypes = [P, C.c_longlong, C.c_int, C.c_int, C.c_float, C.c_ulonglong, D]
    lib.tb_learn_eval.argtypes = [P, C.c_longlong, C.c_longlong, D, D]
    lib.tb_learn_get_stats.argtypes = [P, C.POINTER(LearnStats)]
    lib.tb_learn_get_samples.argtypes = [P, C.c_longlong, C.c_longlong, F]
    lib.tb_learn_grad.argtypes = [P, F, F, C.POINTER(C.c_int), C.c_int, D, F]
    lib.tb_learn_op_tables.argtypes = [P, C.c_int, F]
    lib.tb_learn_op_apply.argtypes = [P, C.c_int, F, F]
    lib.tb_learn_forward.argtypes = [F, F, C.c_int, C.c_int, C.c_int, F]
    lib.tb_ensemble_create.argtypes = [C.POINTER(P), C.c_int, C.POINTER(P)]
    lib.tb_ensemble_step.argtypes = [P, C.POINTER(C.c_int)]
    lib.tb_ensemble_destroy.argtypes = [P]
    _lib = lib
    return lib


def check(rc, what=""):
    if rc != TB_OK:
        msg = load().tb_last_error().decode(errors="replace")
        raise TbError("%s failed: %s (%s)" % (what, TB_ERR.get(rc, rc), msg))


def dptr(a):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(C.c_double))


def default_config(**kw):
    cfg = TbConfig()
    check(load().tb_config_default(C.byref(cfg)), "tb_config_default")
    for k, v in kw.items():
        if k in ("forced_mode", "forced_amp", "forced_phase"):
            arr = getattr(cfg, k)
            for q in range(4):
                arr[q] = v[q] if q < len(v) else 0
        else:
            setattr(cfg, k, v)
    return cfg


def fptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def dft_matrix(P, forward):
    """The tensor-core passes' DFT matrix (P x P, double): forward False maps
    slots to physical z, True physical z to slots."""
    out = np.zeros((P, P))
    check(load().tb_dft_matrix(int(P), 1 if forward else 0, dptr(out)), "tb_dft_matrix")
    return out


def learn_param_count():
    return int(load().tb_learn_param_count())


def learn_crop_size():
    return int(load().tb_learn_crop_size())


def learn_forward(w, x):
    """The network's output (n, H, W) on inputs x (n, 4, H, W) float32."""
    w = np.ascontiguousarray(w, dtype=np.float32)
    x = np.ascontiguousarray(x, dtype=np.float32)
    n, _, H, W = x.shape
    out = np.zeros((n, H, W), dtype=np.float32)
    check(load().tb_learn_forward(fptr(w), fptr(x), n, H, W, fptr(out)), "tb_learn_forward")
    return out


def fp64_peak():
    """Measured FP64 throughput of the current device, TFLOP/s (FMA = 2 flops)."""
    v = np.zeros(1)
    check(load().tb_fp64_peak(dptr(v)), "tb_fp64_peak")
    return float(v[0])


def coef_count(msh):
    return load().tb_coef_count(msh)


def generate_coefs(stf, msh):
    blob = np.zeros(coef_count(msh))
    check(load().tb_generate_coefs(float(stf), int(msh), dptr(blob)), "tb_generate_coefs")
    return blob


def generate_fp_fd(stf):
    out = np.zeros(7)
    check(load().tb_generate_fp_fd(float(stf), dptr(out)), "tb_generate_fp_fd")
    return out


def fs_wall_shear(beta_fs=0.0):
    v = np.zeros(1)
    check(load().tb_fs_wall_shear(float(beta_fs), dptr(v)), "tb_fs_wall_shear")
    return float(v[0])


def baseflow_fs(cfg, beta_fs=0.0):
    shape = (cfg.ny, cfg.nx)
    ux, uy, wz = np.zeros(shape), np.zeros(shape), np.zeros(shape)
    check(load().tb_baseflow_fs(C.byref(cfg), float(beta_fs), dptr(ux), dptr(uy), dptr(wz)), "tb_baseflow_fs")
    return ux, uy, wz


class Context:
    """One simulation resident on the current CUDA device (tb_ctx)."""

    def __init__(self, cfg, coefs=None, baseflow=None, init=True):
        self.lib = load()
        self.cfg = cfg
        h = C.c_void_p()
        check(self.lib.tb_create(C.byref(cfg), C.byref(h)), "tb_create")
        self.h = h
        self.shape = (cfg.kfour, cfg.ny, cfg.nx)
        if coefs is not None:
            self.set_coefs(coefs)
        if baseflow is not None:
            self.set_baseflow(*baseflow)
            if init and coefs is not None:
                self.init_fields()

    def close(self):
        if self.h:
            self.lib.tb_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _c(self, rc, what):
        check(rc, what)

    def field(self):
        return np.zeros(self.shape, dtype=np.complex128)

    def set_coefs(self, blob):
        blob = np.ascontiguousarray(blob, dtype=np.float64)
        self._c(self.lib.tb_set_coefs(self.h, dptr(blob)), "tb_set_coefs")

    def set_baseflow(self, uxb, uyb, wzb):
        a = [np.ascontiguousarray(x, dtype=np.float64) for x in (uxb, uyb, wzb)]
        self._c(self.lib.tb_set_baseflow(self.h, *[dptr(x) for x in a]), "tb_set_baseflow")

    def init_fields(self):
        self._c(self.lib.tb_init_fields(self.h), "tb_init_fields")

    def put_state(self, state):
        a = [np.ascontiguousarray(state[n], dtype=np.complex128) for n in ("ux", "uy", "uz", "wx", "wy", "wz")]
        self._c(self.lib.tb_put_state(self.h, *[dptr(x.view(np.float64)) for x in a]), "tb_put_state")

    def get_state(self):
        out = {n: self.field() for n in ("ux", "uy", "uz", "wx", "wy", "wz")}
        self._c(self.lib.tb_get_state(self.h, *[dptr(out[n].view(np.float64)) for n in
                                                ("ux", "uy", "uz", "wx", "wy", "wz")]), "tb_get_state")
        return out

    def set_baseflow_th(self, thb):
        """Base temperature thb(ny, nx) of the thermal form (tb_set_baseflow_th)."""
        a = np.ascontiguousarray(thb, dtype=np.float64)
        self._c(self.lib.tb_set_baseflow_th(self.h, dptr(a)), "tb_set_baseflow_th")

    def put_th(self, th):
        a = np.ascontiguousarray(th, dtype=np.complex128)
        self._c(self.lib.tb_put_th(self.h, dptr(a.view(np.float64))), "tb_put_th")

    def get_th(self):
        out = self.field()
        self._c(self.lib.tb_get_th(self.h, dptr(out.view(np.float64))), "tb_get_th")
        return out

    def put_wall(self, d2uydx2):
        a = np.ascontiguousarray(d2uydx2, dtype=np.complex128)
        self._c(self.lib.tb_put_wall(self.h, dptr(a.view(np.float64))), "tb_put_wall")

    def get_wall(self):
        a = np.zeros((self.cfg.kfour, self.cfg.nx), dtype=np.complex128)
        self._c(self.lib.tb_get_wall(self.h, dptr(a.view(np.float64))), "tb_get_wall")
        return a

    def rk_stage(self, stage, t):
        self._c(self.lib.tb_rk_stage(self.h, stage, t), "tb_rk_stage")

    def step(self, t):
        self._c(self.lib.tb_step(self.h, t), "tb_step")

    def steps(self, t0, n):
        self._c(self.lib.tb_steps(self.h, t0, n), "tb_steps")

    def synchronize(self):
        self._c(self.lib.tb_synchronize(self.h), "tb_synchronize")

    def poisson_stats(self):
        st = PoissonStats()
        self._c(self.lib.tb_get_poisson_stats(self.h, C.byref(st)), "tb_get_poisson_stats")
        K = self.cfg.kfour
        return {"vcycles": list(st.vcycles[:K]), "residual": list(st.residual[:K]),
                "total_vcycles": st.total_vcycles, "solves": st.solves, "noconv": st.noconv}

    def launch_count(self):
        return int(self.lib.tb_launch_count(self.h))

    def device_field(self, which):
        p = C.c_void_p()
        self._c(self.lib.tb_device_field(self.h, int(which), C.byref(p)), "tb_device_field")
        return p.value

    def stream(self):
        p = C.c_void_p()
        self._c(self.lib.tb_stream(self.h, C.byref(p)), "tb_stream")
        return p.value

    PROF = {"sor": 0, "poi_uy": 1, "nlterms": 2, "xlines": 3, "ylines": 4, "stage": 5, "penta": 6, "defect": 7,
            "relax0": 8}

    # on-disk formats of the reference (escreve_par.f)
    def write_checkpoint(self, path, t):
        self._c(self.lib.tb_write_checkpoint(self.h, os.fsencode(path), int(t)), "tb_write_checkpoint")

    def read_checkpoint(self, path):
        t = C.c_int(0)
        self._c(self.lib.tb_read_checkpoint(self.h, os.fsencode(path), C.byref(t)), "tb_read_checkpoint")
        return t.value

    def write_pert(self, path):
        self._c(self.lib.tb_write_pert(self.h, os.fsencode(path)), "tb_write_pert")

    def autotune(self):
        """Time the candidate launch shapes on this grid and keep the fastest (tb_autotune)."""
        r = TuneResult()
        self._c(self.lib.tb_autotune(self.h, C.byref(r)), "tb_autotune")
        return {n: getattr(r, n) for n, _ in TuneResult._fields_}

    def fp32_lines(self, on=True):
        self._c(self.lib.tb_mixed_fp32_lines(self.h, 1 if on else 0), "tb_mixed_fp32_lines")

    def nl_tensor_cores(self, on=True):
        self._c(self.lib.tb_nl_tensor_cores(self.h, 1 if on else 0), "tb_nl_tensor_cores")

    # learned first correction ----------------------------------------------
    def learn_init(self, seed=1):
        self._c(self.lib.tb_learn_init(self.h, seed), "tb_learn_init")

    def learn_weights(self):
        w = np.zeros(learn_param_count(), dtype=np.float32)
        self._c(self.lib.tb_learn_get_weights(self.h, fptr(w)), "tb_learn_get_weights")
        return w

    def learn_set_weights(self, w):
        w = np.ascontiguousarray(w, dtype=np.float32)
        if w.size != learn_param_count():
            raise ValueError("expected %d weights" % learn_param_count())
        self._c(self.lib.tb_learn_set_weights(self.h, fptr(w)), "tb_learn_set_weights")

    def learn_enable(self, on=True, gated=False):
        """Apply the learned correction in every solve (on), or gated: once
        every 32 solves of a stage, and on while it saves corrections (gated)."""
        mode = (2 if gated else 1) if on else 0
        self._c(self.lib.tb_learn_enable(self.h, mode), "tb_learn_enable")

    def learn_sample(self, capacity, crops_per_solve=16, seed=1):
        self._c(self.lib.tb_learn_sample(self.h, int(capacity), int(crops_per_solve), seed), "tb_learn_sample")

    def learn_train(self, iters, batch=32, lr=1e-3, seed=1, n_train=0):
        """Adam on the first n_train crops (all when 0); returns the mean batch
        loss over the last tenth of the iterations."""
        loss = np.zeros(1)
        self._c(self.lib.tb_learn_train(self.h, int(n_train), int(iters), int(batch), float(lr), seed, dptr(loss)),
                "tb_learn_train")
        return float(loss[0])

    def learn_eval(self, first, n):
        """(mean squared error, mean squared target) over crops first .. first+n-1."""
        a, b = np.zeros(1), np.zeros(1)
        self._c(self.lib.tb_learn_eval(self.h, int(first), int(n), dptr(a), dptr(b)), "tb_learn_eval")
        return float(a[0]), float(b[0])

    def learn_samples(self, first, n):
        cw = learn_crop_size()
        out = np.zeros((int(n), 5, cw, cw), dtype=np.float32)
        self._c(self.lib.tb_learn_get_samples(self.h, int(first), int(n), fptr(out)), "tb_learn_get_samples")
        return out

    def learn_grad(self, w, crops, meta):
        """Defect loss and gradient of the network on crops (n, 5, 72, 72) with
        meta (n, 3), by the library's training kernels on this grid."""
        w = np.ascontiguousarray(w, dtype=np.float32)
        crops = np.ascontiguousarray(crops, dtype=np.float32)
        meta = np.ascontiguousarray(meta, dtype=np.int32)
        g = np.zeros(learn_param_count(), dtype=np.float32)
        loss = np.zeros(1)
        self._c(self.lib.tb_learn_grad(self.h, fptr(w), fptr(crops), meta.ctypes.data_as(C.POINTER(C.c_int)),
                                       crops.shape[0], dptr(loss), fptr(g)), "tb_learn_grad")
        return float(loss[0]), g

    def learn_op_tables(self, k):
        tab = np.zeros(29 + 2 * self.cfg.ny, dtype=np.float32)
        self._c(self.lib.tb_learn_op_tables(self.h, int(k), fptr(tab)), "tb_learn_op_tables")
        return tab

    def learn_op_apply(self, k, e):
        """-L e of mode k (e: (nx, ny) float32) by the solver's residual kernel."""
        e = np.ascontiguousarray(e, dtype=np.float32)
        out = np.zeros_like(e)
        self._c(self.lib.tb_learn_op_apply(self.h, int(k), fptr(e), fptr(out)), "tb_learn_op_apply")
        return out

    def learn_stats(self):
        st = LearnStats()
        self._c(self.lib.tb_learn_get_stats(self.h, C.byref(st)), "tb_learn_get_stats")
        return {n: getattr(st, n) for n, _ in LearnStats._fields_}

    def profile(self, enable):
        self._c(self.lib.tb_profile(self.h, 1 if enable else 0), "tb_profile")

    def profile_read(self, family):
        ms = np.zeros(1)
        n = C.c_longlong()
        self._c(self.lib.tb_profile_read(self.h, self.PROF[family], dptr(ms), C.byref(n)), "tb_profile_read")
        return float(ms[0]), int(n.value)

    # per-subroutine mirrors -------------------------------------------------
    def _unary(self, name, f):
        f = np.ascontiguousarray(f, dtype=np.complex128)
        out = self.field()
        self._c(getattr(self.lib, name)(self.h, dptr(out.view(np.float64)), dptr(f.view(np.float64))), name)
        return out

    def derparx(self, f): return self._unary("tb_derparx", f)
    def derparxx(self, f): return self._unary("tb_derparxx", f)
    def dery(self, f): return self._unary("tb_dery", f)
    def deryfv(self, f): return self._unary("tb_deryfv", f)
    def deryy(self, f): return self._unary("tb_deryy", f)

    def _three(self, name):
        a, b, c = self.field(), self.field(), self.field()
        self._c(getattr(self.lib, name)(self.h, *[dptr(x.view(np.float64)) for x in (a, b, c)]), name)
        return a, b, c

    def nlterms(self): return self._three("tb_nlterms")
    def drv(self): return self._three("tb_drv")
    def les_terms(self): return self._three("tb_les_terms")
    def cvirt(self): return self._three("tb_cvirt")

    def loop(self, erro): self._c(self.lib.tb_loop(self.h, float(erro)), "tb_loop")
    def filter_trid(self): self._c(self.lib.tb_filter_trid(self.h), "tb_filter_trid")
    def bzone(self): self._c(self.lib.tb_bzone(self.h), "tb_bzone")
    def bzonew(self): self._c(self.lib.tb_bzonew(self.h), "tb_bzonew")

    def outuy(self):
        out = self.field()
        self._c(self.lib.tb_outuy(self.h, dptr(out.view(np.float64))), "tb_outuy")
        return out

    def poi_uy(self, dwzdx, erro):
        a = np.ascontiguousarray(dwzdx, dtype=np.complex128)
        self._c(self.lib.tb_poi_uy(self.h, dptr(a.view(np.float64)), float(erro)), "tb_poi_uy")

    def poi_ux(self):
        out = self.field()
        self._c(self.lib.tb_poi_ux(self.h, dptr(out.view(np.float64))), "tb_poi_ux")
        return out

    def poi_uz(self, duydy):
        a = np.ascontiguousarray(duydy, dtype=np.complex128)
        self._c(self.lib.tb_poi_uz(self.h, dptr(a.view(np.float64))), "tb_poi_uz")

    def wx_wall(self):
        out = np.zeros((self.cfg.kfour, self.cfg.nx), dtype=np.complex128)
        self._c(self.lib.tb_wx_wall(self.h, dptr(out.view(np.float64))), "tb_wx_wall")
        return out

    def wz_wall(self, lapv):
        a = np.ascontiguousarray(lapv, dtype=np.complex128)
        self._c(self.lib.tb_wz_wall(self.h, dptr(a.view(np.float64))), "tb_wz_wall")

    def ts_pert(self, t, tempt):
        self._c(self.lib.tb_ts_pert(self.h, int(t), float(tempt)), "tb_ts_pert")

    def f_to_p(self, four):
        four = np.ascontiguousarray(four, dtype=np.complex128)
        out = np.zeros((self.cfg.kphys, self.cfg.ny, self.cfg.nx))
        self._c(self.lib.tb_f_to_p(self.h, dptr(out), dptr(four.view(np.float64))), "tb_f_to_p")
        return out

    def p_to_f(self, phys):
        phys = np.ascontiguousarray(phys, dtype=np.float64)
        out = self.field()
        self._c(self.lib.tb_p_to_f(self.h, dptr(out.view(np.float64)), dptr(phys)), "tb_p_to_f")
        return out


def lst_march(re0, w0, alfa0, re_dns, omega_dns, beta_dns, imax, dx, fpp, betafs=None, jedge=251, bl=0.7,
              etamax=7.0, beta=0.0, wslope=0.3320548, steps=1000):
    """Spatial LST of the Falkner-Skan layer (tb_lst_march): continuation from
    (re0, w0, alfa0) to the target, then the station march; returns x, Re^(1/2),
    scaled frequency and the complex eigenvalue alpha0 per station."""
    cfg = LstConfig(re0=re0, w0=w0, alfa0_re=alfa0.real, alfa0_im=alfa0.imag, jedge=jedge, bl=bl, etamax=etamax,
                    beta=beta, wslope=wslope, re_dns=re_dns, omega_dns=omega_dns, beta_dns=beta_dns, imax=imax,
                    dx=dx, steps=steps)
    fpp = np.ascontiguousarray(np.broadcast_to(np.asarray(fpp, dtype=np.float64), (imax,)))
    betafs = np.zeros(imax) if betafs is None else np.ascontiguousarray(np.broadcast_to(
        np.asarray(betafs, dtype=np.float64), (imax,)))
    x, r, w = np.zeros(imax), np.zeros(imax), np.zeros(imax)
    a = np.zeros(2 * imax)
    check(load().tb_lst_march(C.byref(cfg), dptr(fpp), dptr(betafs), dptr(x), dptr(r), dptr(w), dptr(a)), "tb_lst_march")
    return {"x": x, "re0": r, "w0": w, "alpha": a[0::2] + 1j * a[1::2]}


class Ensemble:
    """Independent runs (mixed-form Contexts of any sizes) advanced together:
    one recorded CUDA graph per step holds every member's four stages
    (tb_ensemble_*).  The members stay usable on their own between steps;
    close the ensemble before them."""

    def __init__(self, members):
        self.lib = load()
        self.members = list(members)
        arr = (C.c_void_p * len(self.members))(*[m.h.value if hasattr(m.h, "value") else m.h for m in self.members])
        h = C.c_void_p()
        check(self.lib.tb_ensemble_create(arr, len(self.members), C.byref(h)), "tb_ensemble_create")
        self.h = h

    def step(self, t):
        """Advance member i by its step t[i] (an int applies to every member)."""
        if isinstance(t, int):
            t = [t] * len(self.members)
        ts = (C.c_int * len(self.members))(*[int(v) for v in t])
        check(self.lib.tb_ensemble_step(self.h, ts), "tb_ensemble_step")

    def close(self):
        if self.h:
            self.lib.tb_ensemble_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
