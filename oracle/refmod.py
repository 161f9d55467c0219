"""Front end of the MAPP reference built from its own sources (oracle/_ref,
recipe oracle/ref.mk).

Test infrastructure only: the fixture script under tests/golden/ and the CPU
tests use it to pin oracle.c against the reference itself.  The product
package never imports it, and it exists only where the reference tree does
(the reference is not available on every machine the tests run on).

The reference tree is found from the MAPPG_REFERENCE_ROOT environment
variable (the directory holding the reference's src/ and examples/).

A RefSystem drives the reference through its public Python API (md.atoms,
md.nvt, md.min_lbfgs, mapp4py.ls_bt) plus the probe entry points of
refshim/ref_probe.cpp, which set exact box/positions/velocities and read the
forces of ForceFieldMD::force_calc.
"""
import ctypes as C
import glob
import importlib.util
import os
import subprocess
import sys
import tempfile

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_OUT = os.path.join(_HERE, "_ref")
_mod = None
_probe = None
_D = C.POINTER(C.c_double)


def ref_root():
    """The reference tree named by MAPPG_REFERENCE_ROOT, or None."""
    r = os.environ.get("MAPPG_REFERENCE_ROOT")
    if r and os.path.isdir(os.path.join(r, "src")):
        return r
    return None


def module_path():
    hits = sorted(glob.glob(os.path.join(_OUT, "mapp4py*.so")))
    return hits[0] if hits else None


def build(root=None, jobs=None):
    """Compile the reference into oracle/_ref with ref.mk (about 30 s on 16
    cores).  Returns the module path, or None when no reference tree."""
    root = root or ref_root()
    if root is None:
        return None
    jobs = jobs or max(1, os.cpu_count() or 1)
    subprocess.run(["make", "-s", "-f", os.path.join(_HERE, "ref.mk"), "-j%d" % jobs, "REF=" + root,
                    "PY=" + sys.executable], check=True)
    return module_path()


def available():
    return module_path() is not None


def module():
    """The reference's `mapp4py` module (imported from oracle/_ref)."""
    global _mod, _probe
    if _mod is None:
        path = module_path()
        if path is None:
            raise RuntimeError("reference module not built (oracle/ref.mk)")
        spec = importlib.util.spec_from_file_location("mapp4py", path)
        m = importlib.util.module_from_spec(spec)
        sys.modules["mapp4py"] = m
        spec.loader.exec_module(m)
        L = C.CDLL(path)
        L.mappg_ref_natms.argtypes = [C.py_object]
        L.mappg_ref_set_state.argtypes = [C.py_object, _D, _D, _D]
        L.mappg_ref_get_state.argtypes = [C.py_object, _D, _D, _D]
        L.mappg_ref_force.argtypes = [C.py_object, _D, _D]
        _mod, _probe = m, L
    return _mod


def _dp(a):
    return a.ctypes.data_as(_D) if a is not None else None


def _cfg_text(H, elem, masses, names):
    """An extended CFG whose element blocks come in element order, so the
    reference numbers the elements as the caller does; positions are set
    exactly afterwards (reduced coordinates here are placeholders)."""
    n = elem.shape[0]
    lines = ["Number of particles = %d" % n, "A = 1.0 Angstrom (basic length-scale)"]
    for i in range(3):
        for j in range(3):
            lines.append("H0(%d,%d) = %.17g A" % (i + 1, j + 1, H[i, j]))
    lines += [".NO_VELOCITY.", "entry_count = 3"]
    for e in range(len(names)):
        idx = np.nonzero(elem == e)[0]
        if idx.size == 0:
            continue
        lines += ["%.17g" % masses[e], names[e]]
        lines += ["0.5 0.5 0.5"] * idx.size
    return "\n".join(lines) + "\n"


class RefSystem:
    """md.atoms of the reference holding the caller's cell, with a force
    field from a potential file: kind 'setfl', 'fs' or 'funcfl'."""

    def __init__(self, H, x, elem, masses, names, pot_path, kind="setfl", v=None, skin=0.5, kB=8.617330350e-5):
        md = module().md
        self.H = np.ascontiguousarray(H, dtype=np.float64).reshape(3, 3)
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 3)
        self.elem = np.ascontiguousarray(elem, dtype=np.uint8)
        self.n = x.shape[0]
        if sorted(set(self.elem.tolist())) != list(range(len(set(self.elem.tolist())))):
            raise ValueError("every element 0..k-1 must occur")
        # ids follow the CFG rows: atoms grouped by element, stable order
        self.order = np.argsort(self.elem, kind="stable")
        with tempfile.TemporaryDirectory() as d:
            p = os.path.join(d, "cell.cfg")
            with open(p, "w") as f:
                f.write(_cfg_text(self.H, self.elem, np.asarray(masses, dtype=np.float64), names))
            self.sim = md.atoms.import_cfg(p)
        self.sim.kB = kB
        self.sim.skin = skin
        self.set_state(x, v)
        if kind == "setfl":
            self.sim.ff_eam_setfl(pot_path)
        elif kind == "fs":
            self.sim.ff_eam_fs(pot_path)
        elif kind == "funcfl":
            self.sim.ff_eam_funcfl(pot_path if isinstance(pot_path, (list, tuple)) else [pot_path])
        else:
            raise ValueError(kind)

    def set_state(self, x, v=None, H=None):
        if H is not None:
            self.H = np.ascontiguousarray(H, dtype=np.float64).reshape(3, 3)
        xs = np.ascontiguousarray(np.asarray(x, dtype=np.float64).reshape(-1, 3)[self.order])
        vs = None if v is None else np.ascontiguousarray(np.asarray(v, dtype=np.float64).reshape(-1, 3)[self.order])
        if _probe.mappg_ref_set_state(self.sim, _dp(self.H), _dp(xs), _dp(vs)) != 0:
            raise RuntimeError("reference probe: set_state failed")

    def state(self):
        H = np.zeros((3, 3))
        xs = np.zeros((self.n, 3))
        vs = np.zeros((self.n, 3))
        _probe.mappg_ref_get_state(self.sim, _dp(H), _dp(xs), _dp(vs))
        x = np.empty_like(xs)
        v = np.empty_like(vs)
        x[self.order] = xs
        v[self.order] = vs
        return H, x, v

    def force(self):
        """ForceFieldMD::force_calc: (pe, S_pe 3x3, value(), f in caller order)."""
        fs = np.zeros((self.n, 3))
        res = np.zeros(11)
        if _probe.mappg_ref_force(self.sim, _dp(fs), _dp(res)) != 0:
            raise RuntimeError("reference probe: force failed (no force field?)")
        f = np.empty_like(fs)
        f[self.order] = fs
        return res[0], res[1:10].reshape(3, 3).copy(), res[10], f

    def nvt(self, T, dt, nsteps, t_relax=None, L=3, niters=1):
        """md.nvt(T, dt).run(atoms, nsteps) as a user calls it."""
        nvt = module().md.nvt(T, dt)
        if t_relax is not None:
            nvt.t_relax = t_relax
        nvt.L = L
        nvt.niters = niters
        nvt.ntally = 0
        nvt.run(self.sim, nsteps)
        return self.state()

    def lbfgs(self, nsteps, m=10, e_tol=0.0, max_dx=1.0, c=0.4, rho=0.5, min_alpha=0.0):
        """md.min_lbfgs(m, e_tol, max_dx) with mapp4py.ls_bt(): nsteps
        iterations (e_tol 0 stops only at the cap or a failed search)."""
        M = module()
        mn = M.md.min_lbfgs(m=m, e_tol=e_tol, max_dx=max_dx)
        ls = M.ls_bt()
        ls.c = c
        ls.rho = rho
        ls.min_alpha = min_alpha
        mn.ls = ls
        mn.ntally = 0
        mn.run(self.sim, nsteps)
        return self.state()

    def set_dof(self, dof):
        """atoms.x_dof through atoms.do, as the reference's examples set it:
        dof (n, 3) bool in caller order, True where the component is free."""
        dof = np.asarray(dof, dtype=bool).reshape(-1, 3)
        by_id = dof[self.order]  # ids follow the CFG rows

        def put(id, x_dof):
            x_dof[:] = by_id[int(id[0])]

        self.sim.do(put)

    def nst(self, S, T, dt, nsteps, L=3, niters=1):
        """md.nst(S, T, dt).run(atoms, nsteps) (MDNST::run) as a user calls
        it; S: 3x3 with NaN where the box entry has no degree of freedom
        (passed to the reference in its triangular form, None for NaN)."""
        S = np.asarray(S, dtype=np.float64).reshape(3, 3)
        tri = [[None if np.isnan(S[i][j]) else float(S[i][j]) for j in range(i + 1)] for i in range(3)]
        nst = module().md.nst(tri, T, dt)
        nst.L = L
        nst.niters = niters
        nst.ntally = 0
        nst.run(self.sim, nsteps)
        return self.state()

    def minimize(self, method, nsteps, ls="bt", m=10, e_tol=0.0, max_dx=1.0, bracket=True, H_dof=None,
                 affine=False):
        """md.min_lbfgs(m, e_tol, max_dx) or md.min_cg_new(e_tol, max_dx)
        (MinCG, min_cg.h:454-536) with mapp4py.ls_bt(), ls_golden() or
        ls_brent() at their defaults (bracket set as given): nsteps
        iterations."""
        M = module()
        if method == "lbfgs":
            mn = M.md.min_lbfgs(m=m, e_tol=e_tol, max_dx=max_dx)
        elif method == "cg":
            mn = M.md.min_cg_new(e_tol=e_tol, max_dx=max_dx)
        else:
            raise ValueError(method)
        if H_dof is not None:
            mn.H_dof = [[bool(H_dof[i][j]) for j in range(3)] for i in range(3)]
            mn.affine = bool(affine)
        search = {"bt": M.ls_bt, "golden": M.ls_golden, "brent": M.ls_brent}[ls]()
        if ls != "bt":
            search.bracket = bool(bracket)
        mn.ls = search
        mn.ntally = 0
        mn.run(self.sim, nsteps)
        return self.state()

    def create_temp(self, T, seed):
        """atoms.create_temp(T, seed): the velocities it draws, caller order."""
        self.sim.create_temp(T, seed)
        return self.state()[2]
