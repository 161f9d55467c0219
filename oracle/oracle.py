"""ctypes front end of the CPU oracle (oracle.c).

Test infrastructure only: imported by tests/, by the smoke check and by the
CPU-baseline leg of bench.py, never by the product package.
"""
import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int)
_U8 = C.POINTER(C.c_ubyte)


def build(force=False):
    """Compile the oracle with its Makefile (gcc, a second or two)."""
    if force or not os.path.exists(_LIB_PATH) or (
        os.path.getmtime(_LIB_PATH) < os.path.getmtime(os.path.join(_HERE, "oracle.c"))
    ):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        L.orc_last_error.restype = C.c_char_p
        L.orc_eam_from_knots.restype = C.c_void_p
        L.orc_eam_from_knots.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, _D, _D, _D]
        L.orc_eam_read_setfl.restype = C.c_void_p
        L.orc_eam_read_setfl.argtypes = [C.c_char_p]
        L.orc_eam_free.argtypes = [C.c_void_p]
        L.orc_eam_info.argtypes = [C.c_void_p, _I, _I, _I, _D, _D]
        L.orc_eam_tables.argtypes = [C.c_void_p, _D, _D, _D, _D]
        L.orc_sys_new.restype = C.c_void_p
        L.orc_sys_new.argtypes = [C.c_int, _D, _D, _U8, _D, C.c_double, C.c_void_p]
        L.orc_sys_free.argtypes = [C.c_void_p]
        for nm in ("orc_sys_set_x", "orc_sys_get_x", "orc_sys_set_v", "orc_sys_get_v", "orc_sys_get_f"):
            getattr(L, nm).argtypes = [C.c_void_p, _D]
        L.orc_sys_set_pair_wise.argtypes = [C.c_void_p, C.c_int]
        L.orc_sys_nghost.argtypes = [C.c_void_p]
        L.orc_sys_nrebuild.argtypes = [C.c_void_p]
        L.orc_sys_init_dynamic.argtypes = [C.c_void_p]
        L.orc_sys_update.argtypes = [C.c_void_p]
        L.orc_sys_neighbors.restype = C.c_long
        L.orc_sys_neighbors.argtypes = [C.c_void_p, _I, _I]
        L.orc_sys_force.restype = C.c_double
        L.orc_sys_force.argtypes = [C.c_void_p, _D]
        L.orc_sys_force_full.restype = C.c_double
        L.orc_sys_force_full.argtypes = [C.c_void_p, _D, C.c_int]
        L.orc_sys_energy.restype = C.c_double
        L.orc_sys_energy.argtypes = [C.c_void_p]
        L.orc_sys_get_rho.argtypes = [C.c_void_p, _D, _D]
        L.orc_md_nvt_run.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_double,
                                     C.c_int, C.c_int, C.c_int, _D, _D, C.c_int, _D]
        L.orc_lbfgs_run.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_double,
                                    C.c_double, C.c_double, C.c_double, C.c_int, _D]
        L.orc_cg_run.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                                 C.c_double, C.c_int, C.POINTER(C.c_double)]
        L.orc_lbfgs_run_ls.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_double,
                                       C.POINTER(OrcLs), C.c_int, _D]
        L.orc_cg_run_ls.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_double, C.POINTER(OrcLs), C.c_int, _D]
        L.orc_lbfgs_run_diag.argtypes = [C.c_void_p, _D, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                         C.c_double, C.c_double, C.c_int, _D]
        L.orc_min_box_run.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_double, C.POINTER(C.c_int),
                                      C.c_int, C.POINTER(OrcLs), C.c_int, _D]
        L.orc_sys_get_box.argtypes = [C.c_void_p, _D]
        L.orc_md_nst_run.argtypes = [C.c_void_p, _D, _D, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int,
                                     C.c_int, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int, _D, _D, _D, _D]
        L.orc_create_temp.argtypes = [C.c_int, _U8, _D, C.c_double, C.c_double, C.c_int, _D]
        L.orc_create_temp_dof.argtypes = [C.c_int, _U8, _D, _U8, C.c_double, C.c_double, C.c_int, _D]
        L.orc_sys_set_dof.argtypes = [C.c_void_p, _U8]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(_D)


class OrcLs(C.Structure):
    """orc_ls: the line search of a minimizer (0 back-tracking, 1 golden
    section, 2 Brent) and its parameters."""
    _fields_ = [("kind", C.c_int), ("c", C.c_double), ("rho", C.c_double), ("min_alpha", C.c_double),
                ("tol", C.c_double), ("max_iter", C.c_int), ("bracket", C.c_int), ("zeps", C.c_double)]


LS_KINDS = {"bt": 0, "golden": 1, "brent": 2}


def line_search(kind="bt", c=0.4, rho=0.5, min_alpha=0.0, tol=(2.0 * np.finfo(float).eps) ** 0.5, max_iter=5,
                bracket=True, zeps=np.finfo(float).eps * 1e-3):
    return OrcLs(LS_KINDS[kind], c, rho, min_alpha, tol, max_iter, int(bool(bracket)), zeps)


def _err():
    return lib().orc_last_error().decode()


class Eam:
    """Spline tables built exactly as ImportEAM does (import_eam.h:348-613)."""

    def __init__(self, handle):
        if not handle:
            raise RuntimeError("oracle: " + _err())
        self.h = handle
        ne, nr, nrho = C.c_int(), C.c_int(), C.c_int()
        dr, drho = C.c_double(), C.c_double()
        lib().orc_eam_info(self.h, C.byref(ne), C.byref(nr), C.byref(nrho), C.byref(dr), C.byref(drho))
        self.nelem, self.nr, self.nrho = ne.value, nr.value, nrho.value
        self.dr, self.drho = dr.value, drho.value

    @classmethod
    def setfl(cls, path):
        return cls(lib().orc_eam_read_setfl(os.fsencode(path)))

    @classmethod
    def knots(cls, nr, nrho, dr, drho, F, rho, rphi):
        F = np.ascontiguousarray(F, dtype=np.float64)
        rho = np.ascontiguousarray(rho, dtype=np.float64)
        rphi = np.ascontiguousarray(rphi, dtype=np.float64)
        ne = F.shape[0]
        return cls(lib().orc_eam_from_knots(ne, nr, nrho, dr, drho, _dp(F), _dp(rho), _dp(rphi)))

    def tables(self):
        ne, nr, nrho = self.nelem, self.nr, self.nrho
        F = np.zeros((ne, nrho, 4))
        rho = np.zeros((ne, ne, nr, 4))
        rphi = np.zeros((ne, ne, nr, 4))
        cut = np.zeros((ne, ne))
        lib().orc_eam_tables(self.h, _dp(F), _dp(rho), _dp(rphi), _dp(cut))
        return F, rho, rphi, cut

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_eam_free(self.h)
            self.h = None


class System:
    """One periodic cell on one rank (AtomsMD + ForceFieldEAM + DynamicMD)."""

    def __init__(self, eam, H, x, elem, masses, skin=0.5, pair_wise=True):
        self.eam = eam
        H = np.ascontiguousarray(H, dtype=np.float64).reshape(3, 3)
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 3)
        self.elem = np.ascontiguousarray(elem, dtype=np.uint8)
        self.masses = np.ascontiguousarray(masses, dtype=np.float64)
        self.n = x.shape[0]
        self.h = lib().orc_sys_new(self.n, _dp(H), _dp(x), self.elem.ctypes.data_as(_U8),
                                   _dp(self.masses), skin, eam.h)
        lib().orc_sys_set_pair_wise(self.h, 1 if pair_wise else 0)
        self.initialized = False

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_sys_free(self.h)
            self.h = None

    def _get(self, fn):
        a = np.zeros((self.n, 3))
        fn(self.h, _dp(a))
        return a

    @property
    def x(self):
        return self._get(lib().orc_sys_get_x)

    @x.setter
    def x(self, v):
        v = np.ascontiguousarray(v, dtype=np.float64).reshape(-1, 3)
        lib().orc_sys_set_x(self.h, _dp(v))

    @property
    def v(self):
        return self._get(lib().orc_sys_get_v)

    @v.setter
    def v(self, val):
        val = np.ascontiguousarray(val, dtype=np.float64).reshape(-1, 3)
        lib().orc_sys_set_v(self.h, _dp(val))

    @property
    def f(self):
        return self._get(lib().orc_sys_get_f)

    def init_dynamic(self):
        if lib().orc_sys_init_dynamic(self.h) != 0:
            raise RuntimeError("oracle: " + _err())
        self.initialized = True

    def force(self):
        """ForceFieldMD::force_calc: returns (pe, virial F_H voigt[6]); forces in .f"""
        if not self.initialized:
            self.init_dynamic()
        out = np.zeros(7)
        lib().orc_sys_force(self.h, _dp(out))
        return out[0], out[1:].copy()

    def force_full(self, nthreads=1):
        if not self.initialized:
            self.init_dynamic()
        out = np.zeros(7)
        lib().orc_sys_force_full(self.h, _dp(out), int(nthreads))
        return out[0], out[1:].copy()

    def energy(self):
        if not self.initialized:
            self.init_dynamic()
        return lib().orc_sys_energy(self.h)

    def rho_dF(self):
        rho = np.zeros(self.n)
        dF = np.zeros(self.n)
        lib().orc_sys_get_rho(self.h, _dp(rho), _dp(dF))
        return rho, dF

    def neighbors(self):
        """Full/half list as a list (per local atom) of sorted (owner, n0, n1, n2) tuples."""
        cnt = np.zeros(self.n, dtype=np.int32)
        tot = lib().orc_sys_neighbors(self.h, cnt.ctypes.data_as(_I), None)
        ent = np.zeros((tot, 4), dtype=np.int32)
        lib().orc_sys_neighbors(self.h, cnt.ctypes.data_as(_I), ent.ctypes.data_as(_I))
        return cnt, ent

    def nvt_run(self, T, dt, kB, nsteps, t_relax=None, L=3, niters=1, eta=None, threads=0):
        """MDNVT::run.  threads > 0 switches to the full-list multi-threaded
        restatement (timing baseline); the loop time is in self.loop_seconds."""
        if t_relax is None:
            t_relax = 100.0 * dt
        eta_a = np.zeros(max(L, 1)) if eta is None else np.ascontiguousarray(eta, dtype=np.float64)
        thermo = np.zeros((nsteps + 1, 14))
        secs = np.zeros(1)
        r = lib().orc_md_nvt_run(self.h, T, dt, kB, t_relax, L, niters, nsteps, _dp(eta_a), _dp(thermo),
                                 int(threads), _dp(secs))
        if r < 0:
            raise RuntimeError("oracle: " + _err())
        self.initialized = True
        self.loop_seconds = float(secs[0])
        return thermo, eta_a, r

    def lbfgs_run(self, m=10, e_tol=0.0, max_dx=1.0, f_tol=1e-4, c=0.4, rho=0.5, min_alpha=0.0, nsteps=10000):
        st = np.zeros(6)
        r = lib().orc_lbfgs_run(self.h, m, e_tol, max_dx, f_tol, c, rho, min_alpha, nsteps, _dp(st))
        if r != 0:
            raise RuntimeError("oracle: " + _err())
        self.initialized = True
        return {"niter": int(st[0]), "pe": st[1], "fmax": st[2], "err": int(st[3]),
                "n_energy": int(st[4]), "n_force": int(st[5])}

    def lbfgs_run_ls(self, ls, m=10, e_tol=0.0, max_dx=1.0, f_tol=1e-4, nsteps=10000):
        """L-BFGS with any line search (ls = line_search(...))."""
        st = np.zeros(6)
        r = lib().orc_lbfgs_run_ls(self.h, m, e_tol, max_dx, f_tol, C.byref(ls), nsteps, _dp(st))
        if r != 0:
            raise RuntimeError("oracle: " + _err())
        self.initialized = True
        return {"niter": int(st[0]), "pe": st[1], "fmax": st[2], "err": int(st[3]),
                "n_energy": int(st[4]), "n_force": int(st[5])}

    def lbfgs_run_diag(self, hdiag, m=10, e_tol=0.0, max_dx=1.0, f_tol=1e-4, c=0.4, rho=0.5, min_alpha=0.0,
                       nsteps=10000):
        """L-BFGS with H0 = tau diag(1/hdiag) (hdiag: (n, 3) Hessian diagonal),
        as the library's mappg_lbfgs_run_diag."""
        hd = np.ascontiguousarray(hdiag, dtype=np.float64).reshape(-1, 3)
        st = np.zeros(7)
        r = lib().orc_lbfgs_run_diag(self.h, _dp(hd), m, e_tol, max_dx, f_tol, c, rho, min_alpha, nsteps, _dp(st))
        if r != 0:
            raise RuntimeError("oracle: " + _err())
        self.initialized = True
        return {"niter": int(st[0]), "pe": st[1], "fmax": st[2], "err": int(st[3]),
                "n_energy": int(st[4]), "n_force": int(st[5]), "fallbacks": int(st[6])}

    def min_box_run(self, ls, H_dof, affine=False, method="lbfgs", m=10, e_tol=0.0, max_dx=1.0, nsteps=10000):
        """L-BFGS or CG with box degrees of freedom (H_dof: 3x3 mask, lower
        triangle read)."""
        st = np.zeros(6)
        mask = np.ascontiguousarray(np.asarray(H_dof, dtype=bool).reshape(3, 3), dtype=np.int32)
        r = lib().orc_min_box_run(self.h, 0 if method == "lbfgs" else 1, m, e_tol, max_dx,
                                  mask.ctypes.data_as(C.POINTER(C.c_int)), int(bool(affine)), C.byref(ls), nsteps,
                                  _dp(st))
        if r != 0:
            raise RuntimeError("oracle: " + _err())
        self.initialized = True
        return {"niter": int(st[0]), "pe": st[1], "fmax": st[2], "err": int(st[3]),
                "n_energy": int(st[4]), "n_force": int(st[5])}

    def nst_run(self, S, T, dt, kB, nsteps, tau=None, t_relax=None, L=3, niters=1, t_relax_S=None, L_S=3,
                niters_S=1, nreset=0, V_H=None, eta=None, eta_S=None):
        """MDNST::run restated; S: 3x3 with NaN for components without a
        degree of freedom.  Returns thermo rows [pe, T, mvv6, F_H6, H9] and
        the carried state (V_H, eta, eta_S)."""
        S = np.ascontiguousarray(S, dtype=np.float64).reshape(3, 3)
        tau = np.full((3, 3), 1000.0 * dt) if tau is None else np.ascontiguousarray(tau, dtype=np.float64)
        t_relax = 100.0 * dt if t_relax is None else t_relax
        t_relax_S = 1000.0 * dt if t_relax_S is None else t_relax_S
        V_H = np.zeros((3, 3)) if V_H is None else np.array(V_H, dtype=np.float64)
        eta = np.zeros(L) if eta is None else np.array(eta, dtype=np.float64)
        eta_S = np.zeros(L_S) if eta_S is None else np.array(eta_S, dtype=np.float64)
        th = np.zeros((nsteps + 1, 23))
        r = lib().orc_md_nst_run(self.h, _dp(S), _dp(tau), T, dt, kB, t_relax, L, niters, t_relax_S, L_S, niters_S,
                                 nreset, nsteps, _dp(V_H), _dp(eta), _dp(eta_S), _dp(th))
        if r != 0:
            raise RuntimeError("oracle: " + _err())
        self.initialized = True
        return th, V_H, eta, eta_S

    def set_dof(self, dof):
        """atoms.x_dof: (n, 3) bool, True where the component is free; None
        clears it."""
        if dof is None:
            lib().orc_sys_set_dof(self.h, None)
            return
        d = np.ascontiguousarray(np.asarray(dof, dtype=bool).reshape(-1, 3), dtype=np.uint8)
        lib().orc_sys_set_dof(self.h, d.ctypes.data_as(_U8))

    def box(self):
        H = np.zeros((3, 3))
        lib().orc_sys_get_box(self.h, _dp(H))
        return H

    def cg_run_ls(self, ls, e_tol=0.0, max_dx=1.0, f_tol=1e-4, nsteps=10000):
        st = np.zeros(6)
        r = lib().orc_cg_run_ls(self.h, e_tol, max_dx, f_tol, C.byref(ls), nsteps, _dp(st))
        if r != 0:
            raise RuntimeError("oracle: " + _err())
        self.initialized = True
        return {"niter": int(st[0]), "pe": st[1], "fmax": st[2], "err": int(st[3]),
                "n_energy": int(st[4]), "n_force": int(st[5])}

    def cg_run(self, e_tol=0.0, max_dx=1.0, f_tol=1e-4, c=0.4, rho=0.5, min_alpha=0.0, nsteps=10000):
        st = np.zeros(6)
        r = lib().orc_cg_run(self.h, e_tol, max_dx, f_tol, c, rho, min_alpha, nsteps, _dp(st))
        if r != 0:
            raise RuntimeError("oracle: " + _err())
        self.initialized = True
        return {"niter": int(st[0]), "pe": st[1], "fmax": st[2], "err": int(st[3]),
                "n_energy": int(st[4]), "n_force": int(st[5])}


def create_temp_dof(elem, masses, dof, T, kB, seed, v):
    """AtomsMD::create_T with x_dof: free components drawn, the others kept."""
    elem = np.ascontiguousarray(elem, dtype=np.uint8)
    out = np.array(v, dtype=np.float64).reshape(-1, 3)
    d = np.ascontiguousarray(np.asarray(dof, dtype=bool).reshape(-1, 3), dtype=np.uint8)
    masses = np.ascontiguousarray(masses, dtype=np.float64)
    r = lib().orc_create_temp_dof(elem.shape[0], elem.ctypes.data_as(_U8), _dp(masses), d.ctypes.data_as(_U8),
                                  float(T), float(kB), int(seed), _dp(out))
    if r != 0:
        raise RuntimeError("oracle: " + _err())
    return out


def create_temp(elem, masses, T, kB, seed):
    """AtomsMD::create_T restated (Park-Miller); seed 0 is rejected."""
    elem = np.ascontiguousarray(elem, dtype=np.uint8)
    masses = np.ascontiguousarray(masses, dtype=np.float64)
    v = np.zeros((elem.shape[0], 3))
    if lib().orc_create_temp(elem.shape[0], elem.ctypes.data_as(_U8), _dp(masses), T, kB, seed, _dp(v)):
        raise ValueError("oracle: " + _err())
    return v
