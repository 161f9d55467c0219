"""ctypes binding of libmappg.so (include/mappg.h).

The library is built in-tree (mapp4py_gb300/build.py).  Loading fails loudly
when it is missing: there is no CPU fallback for the EAM path.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmappg.so")

FP64 = 0
MIXED = 1

_D = C.POINTER(C.c_double)
_F = C.POINTER(C.c_float)
_I = C.POINTER(C.c_int)
_U8 = C.POINTER(C.c_ubyte)
_LL = C.POINTER(C.c_longlong)
_VP = C.c_void_p
_HOOK = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_longlong)

# every exported entry point and its argument types (include/mappg.h)
SIGNATURES = {
    "mappg_last_error": (C.c_char_p, []),
    "mappg_device_info": (C.c_int, [C.c_char_p, C.c_int, _I]),
    "mappg_batch_autotune": (C.c_int, [_VP, _I, _I, _I, _D]),
    "mappg_mlp_set_refresh": (C.c_int, [_VP, C.c_int]),
    "mappg_fp64_fma_rate": (C.c_int, [C.c_int, C.c_int, _D]),
    "mappg_ff_setfl": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(C.c_char_p), C.POINTER(_VP)]),
    "mappg_ff_fs": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(C.c_char_p), C.POINTER(_VP)]),
    "mappg_ff_funcfl": (C.c_int, [C.c_int, C.POINTER(C.c_char_p), C.POINTER(_VP)]),
    "mappg_ff_from_knots": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, _D, _D, _D,
                                      C.POINTER(_VP)]),
    "mappg_ff_info": (C.c_int, [_VP, _I, _I, _I, _D, _D]),
    "mappg_ff_tables": (C.c_int, [_VP, _D, _D, _D, _D]),
    "mappg_ff_element_name": (C.c_int, [_VP, C.c_int, C.c_char_p, C.c_int]),
    "mappg_ff_destroy": (None, [_VP]),
    "mappg_sys_create": (C.c_int, [_VP, C.c_int, _D, _D, _U8, _D, C.c_double, C.c_int, C.POINTER(_VP)]),
    "mappg_sys_destroy": (None, [_VP]),
    "mappg_sys_natoms": (C.c_int, [_VP]),
    "mappg_sys_set_x": (C.c_int, [_VP, _D]),
    "mappg_sys_get_x": (C.c_int, [_VP, _D]),
    "mappg_sys_set_v": (C.c_int, [_VP, _D]),
    "mappg_sys_get_v": (C.c_int, [_VP, _D]),
    "mappg_sys_get_f": (C.c_int, [_VP, _D]),
    "mappg_sys_set_box": (C.c_int, [_VP, _D]),
    "mappg_sys_build": (C.c_int, [_VP]),
    "mappg_sys_update": (C.c_int, [_VP, _I]),
    "mappg_sys_force": (C.c_int, [_VP, _D, _D]),
    "mappg_sys_force_noalloc": (C.c_int, [_VP, _VP, _VP]),
    "mappg_sys_energy": (C.c_int, [_VP, _D]),
    "mappg_sys_energy_delta": (C.c_int, [_VP, _D, C.c_double, _D]),
    "mappg_sys_get_rho": (C.c_int, [_VP, _D, _D]),
    "mappg_sys_neighbors": (C.c_int, [_VP, _I, _I, _LL]),
    "mappg_sys_stats": (C.c_int, [_VP, _LL]),
    "mappg_create_temp": (C.c_int, [C.c_int, _U8, _D, C.c_double, C.c_double, C.c_int, _D]),
    "mappg_nvt_run_host": (C.c_int, [_VP, _D, _D, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int,
                                     C.c_int, _D, _D, _D, _D, _D]),
    "mappg_nvt_run": (C.c_int, [_VP, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int, C.c_int,
                                _D, _D]),
    "mappg_nvt_begin": (C.c_int, [_VP, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int,
                                  C.c_longlong, _D, C.c_int]),
    "mappg_nvt_steps": (C.c_int, [_VP, C.c_longlong]),
    "mappg_nvt_end": (C.c_int, [_VP, _D, _D]),
    "mappg_nvt_snapshot": (C.c_int, [_VP, _D, _D]),
    "mappg_sys_set_hook": (C.c_int, [_VP, _VP, _VP, C.c_int]),
    "mappg_lbfgs_run_ls": (C.c_int, [_VP, C.c_int, C.c_double, C.c_double, C.c_double, _VP, C.c_int, _D]),
    "mappg_min_box_run": (C.c_int, [_VP, C.c_int, C.c_int, C.c_double, C.c_double, _I, C.c_int, _VP, C.c_int,
                                    _D]),
    "mappg_sys_get_box": (C.c_int, [_VP, _D]),
    "mappg_sys_set_dof": (C.c_int, [_VP, _U8]),
    "mappg_create_temp_dof": (C.c_int, [C.c_int, _U8, _D, _U8, C.c_double, C.c_double, C.c_int, _D]),
    "mappg_sys_init_xchng": (C.c_int, [_VP]),
    "mappg_sys_fin_xchng": (C.c_int, [_VP]),
    "mappg_sys_pre_xchng_energy": (C.c_int, [_VP, _VP]),
    "mappg_sys_xchng_energy": (C.c_int, [_VP, _VP, _D]),
    "mappg_sys_post_xchng_energy": (C.c_int, [_VP, _VP]),
    "mappg_nst_run": (C.c_int, [_VP, _D, _D, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int,
                                C.c_double, C.c_int, C.c_int, C.c_int, C.c_int, _D, _D, _D, _D]),
    "mappg_cg_run_ls": (C.c_int, [_VP, C.c_double, C.c_double, C.c_double, _VP, C.c_int, _D]),
    "mappg_cfg_read": (C.c_int, [C.c_char_p, C.POINTER(_VP)]),
    "mappg_cfg_info": (C.c_int, [_VP, _I, _I, _I, _D]),
    "mappg_cfg_element": (C.c_int, [_VP, C.c_int, _D, C.c_char_p, C.c_int]),
    "mappg_cfg_atoms": (C.c_int, [_VP, _D, _D, _U8]),
    "mappg_cfg_destroy": (C.c_int, [_VP]),
    "mappg_cfg_write": (C.c_int, [C.c_char_p, C.c_int, _D, _D, _U8, C.c_int, _D, C.POINTER(C.c_char_p), C.c_int,
                                  C.POINTER(C.c_char_p), _I, C.POINTER(_D)]),
    "mappg_sys_stream": (C.c_int, [_VP, C.POINTER(_VP)]),
    "mappg_sys_sync": (C.c_int, [_VP]),
    "mappg_sys_enqueue": (C.c_int, [_VP, C.c_int]),
    "mappg_lbfgs_run": (C.c_int, [_VP, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                                  C.c_double, C.c_int, _D]),
    "mappg_sys_autotune": (C.c_int, [_VP, _I, _I, _D]),
    "mappg_sys_force_tables": (C.c_int, [_VP, C.c_int, _I]),
    "mappg_sys_tuning": (C.c_int, [_VP, _I]),
    "mappg_lbfgs_run_diag": (C.c_int, [_VP, _D, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                       C.c_double, C.c_double, C.c_int, _D]),
    "mappg_cg_run": (C.c_int, [_VP, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                               C.c_int, _D]),
    "mappg_batch_lbfgs_run": (C.c_int, [_VP, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                                        C.c_double, C.c_int, _D]),
    "mappg_batch_lbfgs_run_precond": (C.c_int, [_VP, _VP, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                                C.c_double, C.c_double, C.c_int, _D]),
    "mappg_tc_gemm_check": (C.c_int, [_VP, _VP, _VP]),
    "mappg_mlp_nparams": (C.c_int, []),
    "mappg_mlp_create": (C.c_int, [C.c_int, C.POINTER(_VP)]),
    "mappg_mlp_destroy": (None, [_VP]),
    "mappg_mlp_set_data": (C.c_int, [_VP, _F, _F, C.c_int, C.c_int]),
    "mappg_mlp_train": (C.c_int, [_VP, C.c_int, C.c_int, C.c_double, C.c_double, _D]),
    "mappg_mlp_grad": (C.c_int, [_VP, _F, _F, C.c_int, _F, _D]),
    "mappg_mlp_predict": (C.c_int, [_VP, _F, C.c_int, _F]),
    "mappg_mlp_get_params": (C.c_int, [_VP, _F, _F]),
    "mappg_mlp_set_params": (C.c_int, [_VP, _F, _F]),
    "mappg_sys_descriptors": (C.c_int, [_VP, _F]),
    "mappg_sys_hessian_diag": (C.c_int, [_VP, _I, C.c_double, _D]),
    "mappg_lbfgs_run_precond": (C.c_int, [_VP, _VP, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                          C.c_double, C.c_double, C.c_int, _D]),
    "mappg_batch_create": (C.c_int, [_VP, C.c_int, _I, _D, _D, _U8, _D, C.c_double, C.c_int, C.POINTER(_VP)]),
    "mappg_batch_ncell": (C.c_int, [_VP]),
    "mappg_batch_force": (C.c_int, [_VP, _D, _D]),
    "mappg_batch_energy": (C.c_int, [_VP, _D]),
    "mappg_batch_nvt_begin": (C.c_int, [_VP, _D, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int,
                                        C.c_longlong, _D, C.c_int]),
    "mappg_batch_nvt_end": (C.c_int, [_VP, _D, _D]),
    "mappg_batch_nvt_run": (C.c_int, [_VP, _D, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int, C.c_int,
                                      _D, _D]),
}

_lib = None


class LineSearch(C.Structure):
    """mappg_ls: kind (LS_BT, LS_GOLDEN, LS_BRENT) and the parameters."""
    _fields_ = [("kind", C.c_int), ("c", C.c_double), ("rho", C.c_double), ("min_alpha", C.c_double),
                ("tol", C.c_double), ("max_iter", C.c_int), ("bracket", C.c_int), ("zeps", C.c_double)]


LS_BT, LS_GOLDEN, LS_BRENT = 0, 1, 2


def line_search(kind=LS_BT, c=0.4, rho=0.5, min_alpha=0.0, tol=(2.0 * np.finfo(float).eps) ** 0.5, max_iter=5,
                bracket=True, zeps=np.finfo(float).eps * 1e-3):
    return LineSearch(int(kind), float(c), float(rho), float(min_alpha), float(tol), int(max_iter),
                      int(bool(bracket)), float(zeps))


class MappgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("libmappg error %d: %s" % (code, msg))
        self.code = code


def load(path=None):
    """Load libmappg.so (raises if it has not been built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise ImportError("libmappg.so is not built (run mapp4py_gb300.build.build()); "
                          "the EAM path has no CPU fallback")
    L = C.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = L
    return L


def check(rc):
    if rc != 0:
        raise MappgError(rc, load().mappg_last_error().decode(errors="replace"))
    return rc


def dptr(a):
    return a.ctypes.data_as(_D)


def f64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if shape is not None:
        a = a.reshape(shape)
    return a


def cstrings(items):
    arr = (C.c_char_p * max(1, len(items)))()
    for i, s in enumerate(items):
        arr[i] = os.fsencode(s) if not isinstance(s, bytes) else s
    return arr


class ForceField:
    """EAM tables on the device (one mappg_ff handle)."""

    def __init__(self, handle, kind):
        self.h = handle
        self.kind = kind
        L = load()
        ne, nr, nrho = C.c_int(), C.c_int(), C.c_int()
        dr, drho = C.c_double(), C.c_double()
        check(L.mappg_ff_info(self.h, C.byref(ne), C.byref(nr), C.byref(nrho), C.byref(dr), C.byref(drho)))
        self.nelem, self.nr, self.nrho, self.dr, self.drho = ne.value, nr.value, nrho.value, dr.value, drho.value
        names = []
        buf = C.create_string_buffer(256)
        for i in range(self.nelem):
            check(L.mappg_ff_element_name(self.h, i, buf, 256))
            names.append(buf.value.decode())
        self.names = names

    @classmethod
    def setfl(cls, path, elems=None):
        out = _VP()
        elems = list(elems or [])
        check(load().mappg_ff_setfl(os.fsencode(path), len(elems), cstrings(elems), C.byref(out)))
        return cls(out, "setfl")

    @classmethod
    def fs(cls, path, elems=None):
        out = _VP()
        elems = list(elems or [])
        check(load().mappg_ff_fs(os.fsencode(path), len(elems), cstrings(elems), C.byref(out)))
        return cls(out, "fs")

    @classmethod
    def funcfl(cls, paths):
        out = _VP()
        paths = list(paths)
        check(load().mappg_ff_funcfl(len(paths), cstrings(paths), C.byref(out)))
        return cls(out, "funcfl")

    @classmethod
    def knots(cls, nr, nrho, dr, drho, F, rho, rphi):
        F, rho, rphi = f64(F), f64(rho), f64(rphi)
        out = _VP()
        check(load().mappg_ff_from_knots(F.shape[0], nr, nrho, dr, drho, dptr(F), dptr(rho), dptr(rphi),
                                         C.byref(out)))
        return cls(out, "knots")

    def tables(self):
        ne, nr, nrho = self.nelem, self.nr, self.nrho
        F = np.zeros((ne, nrho, 4))
        rho = np.zeros((ne, ne, nr, 4))
        rphi = np.zeros((ne, ne, nr, 4))
        cut = np.zeros((ne, ne))
        check(load().mappg_ff_tables(self.h, dptr(F), dptr(rho), dptr(rphi), dptr(cut)))
        return F, rho, rphi, cut

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.mappg_ff_destroy(self.h)
            self.h = None


class System:
    """One periodic cell resident on the GPU (one mappg_sys handle)."""

    def __init__(self, ff, H, x, elem, masses, skin=0.5, precision=FP64):
        self.ff = ff
        H = f64(H, (3, 3))
        x = f64(x, (-1, 3))
        self.elem = np.ascontiguousarray(elem, dtype=np.uint8)
        masses = f64(masses)
        self.n = x.shape[0]
        out = _VP()
        check(load().mappg_sys_create(ff.h, self.n, dptr(H), dptr(x), self.elem.ctypes.data_as(_U8),
                                      dptr(masses), float(skin), int(precision), C.byref(out)))
        self.h = out
        self.precision = precision

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.mappg_sys_destroy(self.h)
            self.h = None

    def _get(self, fn, out=None):
        if out is not None and not (isinstance(out, np.ndarray) and out.dtype == np.float64 and out.flags.c_contiguous
                                    and out.flags.writeable and out.size == 3 * self.n):
            raise ValueError("out must be a writable C-contiguous float64 array of shape (n, 3)")
        a = np.empty((self.n, 3)) if out is None else out
        check(fn(self.h, dptr(a)))
        return a

    def set_x(self, x):
        check(load().mappg_sys_set_x(self.h, dptr(f64(x, (-1, 3)))))

    def get_x(self, out=None):
        return self._get(load().mappg_sys_get_x, out)

    def set_v(self, v):
        check(load().mappg_sys_set_v(self.h, dptr(f64(v, (-1, 3)))))

    def get_v(self, out=None):
        return self._get(load().mappg_sys_get_v, out)

    def get_f(self, out=None):
        return self._get(load().mappg_sys_get_f, out)

    def set_box(self, H):
        check(load().mappg_sys_set_box(self.h, dptr(f64(H, (3, 3)))))

    def build(self):
        check(load().mappg_sys_build(self.h))

    def update(self):
        r = C.c_int(0)
        check(load().mappg_sys_update(self.h, C.byref(r)))
        return bool(r.value)

    def force(self):
        pe = C.c_double()
        vir = np.zeros(6)
        check(load().mappg_sys_force(self.h, C.byref(pe), dptr(vir)))
        return pe.value, vir

    def energy(self):
        pe = C.c_double()
        check(load().mappg_sys_energy(self.h, C.byref(pe)))
        return pe.value

    def energy_delta(self, h, alpha):
        """E(x + alpha h) - E(x) as the mixed minimizers' line searches take it."""
        h = f64(h, (self.n, 3))
        de = C.c_double()
        self._checked(load().mappg_sys_energy_delta(self.h, dptr(h), float(alpha), C.byref(de)))
        return de.value

    def rho_dF(self):
        rho = np.zeros(self.n)
        dF = np.zeros(self.n)
        check(load().mappg_sys_get_rho(self.h, dptr(rho), dptr(dF)))
        return rho, dF

    def neighbors(self):
        cnt = np.zeros(self.n, dtype=np.int32)
        tot = C.c_longlong()
        check(load().mappg_sys_neighbors(self.h, cnt.ctypes.data_as(_I), None, C.byref(tot)))
        ent = np.zeros((tot.value, 4), dtype=np.int32)
        check(load().mappg_sys_neighbors(self.h, cnt.ctypes.data_as(_I), ent.ctypes.data_as(_I), C.byref(tot)))
        return cnt, ent

    def stats(self):
        out = np.zeros(6, dtype=np.int64)
        check(load().mappg_sys_stats(self.h, out.ctypes.data_as(_LL)))
        keys = ("rebuilds", "capacity", "max_row", "mean_row_x1000", "bins", "precision")
        return dict(zip(keys, (int(v) for v in out)))

    def nvt_run(self, T, dt, kB, nsteps, t_relax=None, L=3, niters=1, eta=None, thermo=False):
        if t_relax is None:
            t_relax = 100.0 * dt
        eta_a = np.zeros(max(L, 1)) if eta is None else f64(eta).copy()
        th = np.zeros((nsteps + 1, 14)) if thermo else None
        check(load().mappg_nvt_run(self.h, float(T), float(dt), float(kB), float(t_relax), int(L), int(niters),
                                   int(nsteps), dptr(eta_a), dptr(th) if th is not None else None))
        return th, eta_a

    def nvt_run_host(self, x, v, T, dt, kB, nsteps, t_relax=None, L=3, niters=1, eta=None, thermo=False,
                     x_out=None, v_out=None, f_out=None):
        """nvt_run with host arrays in and out in one call (mappg_nvt_run_host):
        x, v (n, 3) in; x_out, v_out, f_out (n, 3) C-contiguous float64 arrays
        written in place (None: not returned).  Returns (thermo rows, eta)."""
        if t_relax is None:
            t_relax = 100.0 * dt
        eta_a = np.zeros(max(L, 1)) if eta is None else f64(eta).copy()
        th = np.zeros((nsteps + 1, 14)) if thermo else None
        for o in (x_out, v_out, f_out):
            if o is not None and not (isinstance(o, np.ndarray) and o.dtype == np.float64 and o.flags.c_contiguous
                                      and o.flags.writeable and o.size == 3 * self.n):
                raise ValueError("outputs must be writable C-contiguous float64 arrays of shape (n, 3)")
        check(load().mappg_nvt_run_host(self.h, dptr(f64(x, (-1, 3))), dptr(f64(v, (-1, 3))), float(T), float(dt),
                                        float(kB), float(t_relax), int(L), int(niters), int(nsteps), dptr(eta_a),
                                        dptr(th) if th is not None else None,
                                        None if x_out is None else dptr(x_out),
                                        None if v_out is None else dptr(v_out),
                                        None if f_out is None else dptr(f_out)))
        return th, eta_a

    def nvt_begin(self, T, dt, kB, nsteps, t_relax=None, L=3, niters=1, eta=None, thermo=False):
        if t_relax is None:
            t_relax = 100.0 * dt
        eta_a = np.zeros(max(L, 1)) if eta is None else f64(eta).copy()
        self._run = (L, nsteps, thermo)
        check(load().mappg_nvt_begin(self.h, float(T), float(dt), float(kB), float(t_relax), int(L), int(niters),
                                     int(nsteps), dptr(eta_a), 1 if thermo else 0))

    def nvt_steps(self, nsteps):
        check(load().mappg_nvt_steps(self.h, int(nsteps)))

    def nvt_end(self, steps_done=None):
        L, nsteps, thermo = self._run
        n = nsteps if steps_done is None else steps_done
        eta = np.zeros(max(L, 1))
        th = np.zeros((n + 1, 14)) if thermo else None
        check(load().mappg_nvt_end(self.h, dptr(eta), dptr(th) if th is not None else None))
        return th, eta

    def nvt_snapshot(self):
        """(x, x_d) of the begun run after the steps enqueued so far."""
        x = np.empty((self.n, 3))
        v = np.empty((self.n, 3))
        check(load().mappg_nvt_snapshot(self.h, dptr(x), dptr(v)))
        return x, v

    def set_hook(self, fn, nevery):
        """Call fn(iteration) after every nevery-th minimizer iteration
        (None removes it); an exception in fn stops the run and is raised."""
        if fn is None or nevery <= 0:
            self._hook = None
            check(load().mappg_sys_set_hook(self.h, None, None, 0))
            return
        box = {"error": None}

        def call(_user, it):
            try:
                fn(int(it))
                return 0
            except BaseException as e:  # carried across the C frames
                box["error"] = e
                return 1

        cb = _HOOK(call)
        self._hook = (cb, box)
        check(load().mappg_sys_set_hook(self.h, C.cast(cb, _VP), None, int(nevery)))

    def _hook_error(self):
        h = getattr(self, "_hook", None)
        if h is not None and h[1]["error"] is not None:
            e, h[1]["error"] = h[1]["error"], None
            return e
        return None

    def stream(self):
        p = _VP()
        check(load().mappg_sys_stream(self.h, C.byref(p)))
        return p.value or 0

    def sync(self):
        check(load().mappg_sys_sync(self.h))

    def autotune(self):
        """(lanes per atom, entries per step, {(lanes, entries): ms})"""
        tpa, unroll = C.c_int(), C.c_int()
        ms = np.zeros(7)
        check(load().mappg_sys_autotune(self.h, C.byref(tpa), C.byref(unroll), dptr(ms)))
        keys = ((4, 1), (8, 1), (16, 1), (4, 2), (8, 2), (16, 2), (32, 1))
        return tpa.value, unroll.value, {k: v for k, v in zip(keys, ms) if v > 0}

    def tuning(self):
        """The kernel shape in use: lanes per atom, the density and force
        passes' entries per loop step, the force records' shared-memory
        budget (KB) and a batch's atoms per chunk."""
        out = (C.c_int * 5)()
        check(load().mappg_sys_tuning(self.h, out))
        return dict(zip(("lanes_per_atom", "density_entries_per_step", "force_entries_per_step",
                         "force_smem_kb", "atoms_per_chunk"), list(out)))

    def force_tables(self, mode=None):
        """The mixed force pass's record source: 0 through L1, k > 0 the
        records of one element group at a time in k KB of shared memory
        (clamped to the largest budget); None only queries.  Returns the mode
        in use."""
        act = C.c_int()
        check(load().mappg_sys_force_tables(self.h, -1 if mode is None else int(mode), C.byref(act)))
        return act.value

    def enqueue(self, what):
        check(load().mappg_sys_enqueue(self.h, int(what)))

    def cg_run(self, e_tol=0.0, max_dx=1.0, f_tol=1e-4, c=0.4, rho=0.5, min_alpha=0.0, nsteps=100000):
        st = np.zeros(6)
        self._checked(load().mappg_cg_run(self.h, float(e_tol), float(max_dx), float(f_tol), float(c), float(rho),
                                          float(min_alpha), int(nsteps), dptr(st)))
        return {"niter": int(st[0]), "pe": st[1], "fmax": st[2], "err": int(st[3]),
                "n_energy": int(st[4]), "n_force": int(st[5])}

    def lbfgs_run(self, m=10, e_tol=0.0, max_dx=1.0, f_tol=1e-4, c=0.4, rho=0.5, min_alpha=0.0, nsteps=100000):
        st = np.zeros(6)
        self._checked(load().mappg_lbfgs_run(self.h, int(m), float(e_tol), float(max_dx), float(f_tol), float(c),
                                             float(rho), float(min_alpha), int(nsteps), dptr(st)))
        return {"niter": int(st[0]), "pe": st[1], "fmax": st[2], "err": int(st[3]),
                "n_energy": int(st[4]), "n_force": int(st[5])}

    def lbfgs_run_ls(self, ls, m=10, e_tol=0.0, max_dx=1.0, f_tol=1e-4, nsteps=100000):
        """L-BFGS with a given line search (line_search(...))."""
        st = np.zeros(6)
        self._checked(load().mappg_lbfgs_run_ls(self.h, int(m), float(e_tol), float(max_dx), float(f_tol),
                                                C.cast(C.pointer(ls), _VP), int(nsteps), dptr(st)))
        return {"niter": int(st[0]), "pe": st[1], "fmax": st[2], "err": int(st[3]),
                "n_energy": int(st[4]), "n_force": int(st[5])}

    def cg_run_ls(self, ls, e_tol=0.0, max_dx=1.0, f_tol=1e-4, nsteps=100000):
        st = np.zeros(6)
        self._checked(load().mappg_cg_run_ls(self.h, float(e_tol), float(max_dx), float(f_tol),
                                             C.cast(C.pointer(ls), _VP), int(nsteps), dptr(st)))
        return {"niter": int(st[0]), "pe": st[1], "fmax": st[2], "err": int(st[3]),
                "n_energy": int(st[4]), "n_force": int(st[5])}

    def min_box_run(self, ls, H_dof, affine=False, method="lbfgs", m=10, e_tol=0.0, max_dx=1.0, nsteps=100000):
        """L-BFGS ("lbfgs") or CG ("cg") with box degrees of freedom: H_dof
        is a 3x3 mask (its lower triangle is read); affine moves the atoms
        only with the box."""
        st = np.zeros(6)
        mask = np.ascontiguousarray(np.asarray(H_dof, dtype=bool).reshape(3, 3), dtype=np.int32)
        self._checked(load().mappg_min_box_run(self.h, 0 if method == "lbfgs" else 1, int(m), float(e_tol),
                                               float(max_dx), mask.ctypes.data_as(_I), int(bool(affine)),
                                               C.cast(C.pointer(ls), _VP), int(nsteps), dptr(st)))
        return {"niter": int(st[0]), "pe": st[1], "fmax": st[2], "err": int(st[3]),
                "n_energy": int(st[4]), "n_force": int(st[5])}

    def nst_run(self, S, T, dt, kB, nsteps, tau=None, t_relax=None, L=3, niters=1, t_relax_S=None, L_S=3,
                niters_S=1, nreset=0, V_H=None, eta=None, eta_S=None, thermo=True):
        """Constant-stress MD (mappg_nst_run).  S: 3x3, NaN where the box
        entry has no degree of freedom.  Returns (thermo rows or None, V_H,
        eta, eta_S)."""
        S = f64(S, (3, 3))
        tau = np.full((3, 3), 1000.0 * dt) if tau is None else f64(tau, (3, 3))
        t_relax = 100.0 * dt if t_relax is None else t_relax
        t_relax_S = 1000.0 * dt if t_relax_S is None else t_relax_S
        V_H = np.zeros((3, 3)) if V_H is None else f64(V_H, (3, 3)).copy()
        eta = np.zeros(L) if eta is None else f64(eta).copy()
        eta_S = np.zeros(L_S) if eta_S is None else f64(eta_S).copy()
        th = np.zeros((nsteps + 1, 23)) if thermo else None
        self._checked(load().mappg_nst_run(self.h, dptr(S), dptr(tau), float(T), float(dt), float(kB),
                                           float(t_relax), int(L), int(niters), float(t_relax_S), int(L_S),
                                           int(niters_S), int(nreset), int(nsteps), dptr(V_H), dptr(eta),
                                           dptr(eta_S), dptr(th) if th is not None else None))
        return th, V_H, eta, eta_S

    def set_dof(self, dof):
        """atoms.x_dof: (n, 3) bool, True where the component is free; None clears."""
        if dof is None:
            check(load().mappg_sys_set_dof(self.h, None))
            return
        d = np.ascontiguousarray(np.asarray(dof, dtype=bool).reshape(self.n, 3), dtype=np.uint8)
        check(load().mappg_sys_set_dof(self.h, d.ctypes.data_as(_U8)))

    def get_box(self):
        H = np.zeros((3, 3))
        check(load().mappg_sys_get_box(self.h, dptr(H)))
        return H

    def _checked(self, rc):
        # an exception raised by the iteration hook comes first
        e = self._hook_error()
        if e is not None:
            raise e
        return check(rc)


class Batch(System):
    """Independent periodic cells in one device system (one mappg_sys handle
    made by mappg_batch_create); per-atom arrays are the cells' atoms one cell
    after the other, energies and MD state are per cell."""

    def __init__(self, ff, cells, masses, skin=0.5, precision=MIXED):
        """cells: sequence of (H, x, elem)."""
        self.ff = ff
        Hs = np.ascontiguousarray(np.stack([f64(c[0], (3, 3)) for c in cells]))
        xs = [f64(c[1], (-1, 3)) for c in cells]
        self.natoms = np.array([x.shape[0] for x in xs], dtype=np.int32)
        x = np.ascontiguousarray(np.concatenate(xs))
        self.elem = np.ascontiguousarray(np.concatenate([np.asarray(c[2], dtype=np.uint8) for c in cells]))
        self.n = x.shape[0]
        self.ncell = len(cells)
        self.offsets = np.concatenate([[0], np.cumsum(self.natoms)])
        masses = f64(masses)
        out = _VP()
        check(load().mappg_batch_create(ff.h, self.ncell, self.natoms.ctypes.data_as(_I), dptr(Hs), dptr(x),
                                        self.elem.ctypes.data_as(_U8), dptr(masses), float(skin), int(precision),
                                        C.byref(out)))
        self.h = out
        self.precision = precision

    def split(self, a):
        """Per-cell views of a concatenated per-atom array."""
        return [a[self.offsets[c]:self.offsets[c + 1]] for c in range(self.ncell)]


    def autotune(self):
        """(lanes per atom, entries per step, {(chunk atoms, lanes, entries): ms})
        over atoms per chunk 128/256/512 and the lanes/entries candidates;
        the chosen chunk size is in self.chunk_atoms."""
        tpa, unroll, chunk = C.c_int(), C.c_int(), C.c_int()
        ms = np.zeros(21)
        check(load().mappg_batch_autotune(self.h, C.byref(tpa), C.byref(unroll), C.byref(chunk), dptr(ms)))
        keys = ((4, 1), (8, 1), (16, 1), (4, 2), (8, 2), (16, 2), (32, 1))
        self.chunk_atoms = chunk.value
        out = {}
        for q, ch in enumerate((128, 256, 512)):
            for k, v in zip(keys, ms[7 * q:7 * q + 7]):
                if v > 0:
                    out[(ch,) + k] = v
        return tpa.value, unroll.value, out
    def force(self):
        pe = np.zeros(self.ncell)
        vir = np.zeros((self.ncell, 6))
        check(load().mappg_batch_force(self.h, dptr(pe), dptr(vir)))
        return pe, vir

    def energy(self):
        pe = np.zeros(self.ncell)
        check(load().mappg_batch_energy(self.h, dptr(pe)))
        return pe

    def nvt_run(self, T, dt, kB, nsteps, t_relax=None, L=3, niters=1, eta=None, thermo=False):
        if t_relax is None:
            t_relax = 100.0 * dt
        Tc = f64(np.broadcast_to(np.asarray(T, dtype=np.float64), (self.ncell,)).copy())
        eta_a = np.zeros((self.ncell, max(L, 1))) if eta is None else f64(eta).copy()
        th = np.zeros((nsteps + 1, self.ncell, 2)) if thermo else None
        check(load().mappg_batch_nvt_run(self.h, dptr(Tc), float(dt), float(kB), float(t_relax), int(L),
                                         int(niters), int(nsteps), dptr(eta_a), dptr(th) if th is not None else None))
        return th, eta_a

    def nvt_begin(self, T, dt, kB, nsteps, t_relax=None, L=3, niters=1, eta=None, thermo=False):
        if t_relax is None:
            t_relax = 100.0 * dt
        Tc = f64(np.broadcast_to(np.asarray(T, dtype=np.float64), (self.ncell,)).copy())
        eta_a = np.zeros((self.ncell, max(L, 1))) if eta is None else f64(eta).copy()
        self._run = (L, nsteps, thermo)
        check(load().mappg_batch_nvt_begin(self.h, dptr(Tc), float(dt), float(kB), float(t_relax), int(L),
                                           int(niters), int(nsteps), dptr(eta_a), 1 if thermo else 0))

    def lbfgs_run(self, m=10, e_tol=0.0, max_dx=1.0, f_tol=1e-4, c=0.4, rho=0.5, min_alpha=0.0, nsteps=100000,
                  net=None):
        st = np.zeros((self.ncell, 7))
        args = (int(m), float(e_tol), float(max_dx), float(f_tol), float(c), float(rho), float(min_alpha),
                int(nsteps), dptr(st))
        if net is None:
            check(load().mappg_batch_lbfgs_run(self.h, *args))
        else:
            check(load().mappg_batch_lbfgs_run_precond(self.h, net.h, *args))
        keys = ("niter", "pe", "fmax", "err", "n_energy", "n_force", "fallbacks")
        return [{k: (st[c][i] if k in ("pe", "fmax") else int(st[c][i])) for i, k in enumerate(keys)}
                for c in range(self.ncell)]

    def nvt_end(self, steps_done=None):
        L, nsteps, thermo = self._run
        n = nsteps if steps_done is None else steps_done
        eta = np.zeros((self.ncell, max(L, 1)))
        th = np.zeros((n + 1, self.ncell, 2)) if thermo else None
        check(load().mappg_batch_nvt_end(self.h, dptr(eta), dptr(th) if th is not None else None))
        return th, eta


def fptr(a):
    return a.ctypes.data_as(_F)


def f32(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a.reshape(shape) if shape is not None else a


class Mlp:
    """The learned L-BFGS preconditioner network (one mappg_mlp handle)."""

    def __init__(self, seed=0):
        out = _VP()
        check(load().mappg_mlp_create(int(seed), C.byref(out)))
        self.h = out
        self.nparams = load().mappg_mlp_nparams()

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.mappg_mlp_destroy(self.h)
            self.h = None

    def set_data(self, feat, target, seed=0):
        feat = f32(feat, (-1, 33))
        target = f32(target, (-1, 3))
        check(load().mappg_mlp_set_data(self.h, fptr(feat), fptr(target), feat.shape[0], int(seed)))

    def train(self, epochs, batch=4096, lr=2e-3, wd=1e-4):
        losses = np.zeros(max(epochs, 1))
        check(load().mappg_mlp_train(self.h, int(epochs), int(batch), float(lr), float(wd), dptr(losses)))
        return losses[:epochs]

    def grad(self, feat, target):
        feat = f32(feat, (-1, 33))
        target = f32(target, (-1, 3))
        g = np.zeros(self.nparams, dtype=np.float32)
        loss = C.c_double()
        check(load().mappg_mlp_grad(self.h, fptr(feat), fptr(target), feat.shape[0], fptr(g), C.byref(loss)))
        return loss.value, g

    def set_refresh(self, every):
        """L-BFGS runs with this network recompute the diagonal every `every`
        iterations (0: once, at the start)."""
        check(load().mappg_mlp_set_refresh(self.h, int(every)))

    def predict(self, feat):
        feat = f32(feat, (-1, 33))
        out = np.zeros((feat.shape[0], 3), dtype=np.float32)
        check(load().mappg_mlp_predict(self.h, fptr(feat), feat.shape[0], fptr(out)))
        return out

    def params(self):
        w = np.zeros(self.nparams, dtype=np.float32)
        norm = np.zeros(66, dtype=np.float32)
        check(load().mappg_mlp_get_params(self.h, fptr(w), fptr(norm)))
        return w, norm[:33].copy(), norm[33:].copy()

    def set_params(self, w=None, mean=None, sdev=None):
        wp = fptr(f32(w)) if w is not None else None
        norm = None
        if mean is not None:
            norm = f32(np.concatenate([mean, sdev]))
        check(load().mappg_mlp_set_params(self.h, wp, fptr(norm) if norm is not None else None))


def descriptors(system):
    out = np.zeros((system.n, 33), dtype=np.float32)
    check(load().mappg_sys_descriptors(system.h, fptr(out)))
    return out


def hessian_diag(system, color, h=1e-4):
    color = np.ascontiguousarray(color, dtype=np.int32)
    out = np.zeros((system.n, 3))
    check(load().mappg_sys_hessian_diag(system.h, color.ctypes.data_as(_I), float(h), dptr(out)))
    return out


def lbfgs_run_precond(system, net, m=10, e_tol=0.0, max_dx=1.0, f_tol=1e-4, c=0.4, rho=0.5, min_alpha=0.0,
                      nsteps=100000):
    st = np.zeros(7)
    system._checked(load().mappg_lbfgs_run_precond(system.h, net.h, int(m), float(e_tol), float(max_dx),
                                                   float(f_tol), float(c), float(rho), float(min_alpha), int(nsteps),
                                                   dptr(st)))
    return {"niter": int(st[0]), "pe": st[1], "fmax": st[2], "err": int(st[3]), "n_energy": int(st[4]),
            "n_force": int(st[5]), "fallbacks": int(st[6])}


def lbfgs_run_diag(system, hdiag, m=10, e_tol=0.0, max_dx=1.0, f_tol=1e-4, c=0.4, rho=0.5, min_alpha=0.0,
                   nsteps=100000):
    """L-BFGS with H0 = diag(1/hdiag), hdiag the (n, 3) Hessian diagonal in the
    caller's atom order; a Batch relaxes every cell (a list of stats)."""
    hd = f64(hdiag).reshape(-1, 3)
    if hd.shape[0] != system.n:
        raise ValueError("hdiag must be (n, 3)")
    batch = getattr(system, "ncell", 1) > 1
    st = np.zeros((system.ncell, 7)) if batch else np.zeros(7)
    system._checked(load().mappg_lbfgs_run_diag(system.h, dptr(hd), int(m), float(e_tol), float(max_dx),
                                                float(f_tol), float(c), float(rho), float(min_alpha), int(nsteps),
                                                dptr(st)))
    keys = ("niter", "pe", "fmax", "err", "n_energy", "n_force", "fallbacks")
    conv = lambda r: {k: (r[i] if k in ("pe", "fmax") else int(r[i])) for i, k in enumerate(keys)}
    return [conv(r) for r in st] if batch else conv(st)


def create_temp_dof(elem, masses, dof, T, kB, seed, v):
    """create_temp for the free components of dof only; v holds the others."""
    elem = np.ascontiguousarray(elem, dtype=np.uint8)
    out = np.array(v, dtype=np.float64).reshape(-1, 3)
    d = np.ascontiguousarray(np.asarray(dof, dtype=bool).reshape(-1, 3), dtype=np.uint8)
    check(load().mappg_create_temp_dof(elem.shape[0], elem.ctypes.data_as(_U8), dptr(f64(masses)),
                                       d.ctypes.data_as(_U8), float(T), float(kB), int(seed), dptr(out)))
    return out


def create_temp(elem, masses, T, kB, seed):
    elem = np.ascontiguousarray(elem, dtype=np.uint8)
    v = np.zeros((elem.shape[0], 3))
    check(load().mappg_create_temp(elem.shape[0], elem.ctypes.data_as(_U8), dptr(f64(masses)), float(T),
                                   float(kB), int(seed), dptr(v)))
    return v


def fp64_fma_rate(iters=4096, reps=5):
    """FP64 FMA throughput of the current GPU in TFLOP/s (measured)."""
    t = C.c_double()
    check(load().mappg_fp64_fma_rate(int(iters), int(reps), C.byref(t)))
    return t.value


def device_info():
    buf = C.create_string_buffer(256)
    sm = C.c_int()
    check(load().mappg_device_info(buf, 256, C.byref(sm)))
    return buf.value.decode(), sm.value


def read_cfg(path):
    """An AtomEye CFG file as a dict: H (lower triangular), x, x_d (None
    without velocities), elem, names, masses."""
    L = load()
    h = _VP()
    check(L.mappg_cfg_read(os.fsencode(path), C.byref(h)))
    try:
        n, ne, hv = C.c_int(), C.c_int(), C.c_int()
        H = np.zeros((3, 3))
        check(L.mappg_cfg_info(h, C.byref(n), C.byref(ne), C.byref(hv), dptr(H)))
        x = np.zeros((n.value, 3))
        v = np.zeros((n.value, 3)) if hv.value else None
        elem = np.zeros(n.value, dtype=np.uint8)
        check(L.mappg_cfg_atoms(h, dptr(x), dptr(v) if v is not None else None, elem.ctypes.data_as(_U8)))
        names, masses = [], []
        buf = C.create_string_buffer(4096)
        m = C.c_double()
        for i in range(ne.value):
            check(L.mappg_cfg_element(h, i, C.byref(m), buf, 4096))
            names.append(buf.value.decode())
            masses.append(m.value)
        return {"H": H, "x": x, "x_d": v, "elem": elem, "names": names, "masses": np.array(masses)}
    finally:
        L.mappg_cfg_destroy(h)


def write_cfg(path, H, x, elem, masses, names, vecs=()):
    """Write an extended CFG file; vecs is a sequence of (name, [n][dim])
    extra per-atom vectors, "x_d" being written as reduced velocities."""
    H = f64(H, (3, 3))
    x = f64(x, (-1, 3))
    n = x.shape[0]
    elem = np.ascontiguousarray(elem, dtype=np.uint8)
    masses = f64(masses)
    arrs = [f64(a).reshape(n, -1) for _, a in vecs]
    vnames = cstrings([nm for nm, _ in vecs])
    dims = np.array([a.shape[1] for a in arrs] or [0], dtype=np.int32)
    ptrs = (_D * max(1, len(arrs)))(*[dptr(a) for a in arrs])
    check(load().mappg_cfg_write(os.fsencode(path), n, dptr(H), dptr(x), elem.ctypes.data_as(_U8), len(names),
                                 dptr(masses), cstrings(names), len(arrs), vnames,
                                 dims.ctypes.data_as(_I), ptrs))
