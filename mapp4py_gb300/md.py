"""The `mapp4py.md` surface for the EAM path, backed by libmappg on the GPU.

Names, arguments and defaults follow the reference's Python types:
  md.atoms             AtomsMD (atoms_md.cpp); here built from arrays, with
                       ff_eam_setfl / ff_eam_funcfl / ff_eam_fs (ff_eam.cpp:594-801),
                       create_temp (atoms_md.cpp:490-531), kB, skin, H, x, x_d,
                       x_dof (frozen components: zero force, no kick)
  md.nvt(T, dt)        MDNVT (md_nvt.cpp:14-26,493-881): t_relax=100*dt, L=3,
                       niters=1, ntally=10000, run(atoms, nsteps)
  md.nst(S, T, dt)     MDNST (md_nst.cpp:10-38,374-450): as md.nvt plus S, tau,
                       t_relax_s, nreset; moves the box
  md.min_lbfgs(...)    MinLBFGS (min_l-bfgs.cpp:69-127): m=2, e_tol=sqrt(eps),
                       affine=False, max_dx=1.0, ls=ls_bt(); run(atoms, max_nsteps)
  ls_bt()              LineSearchBackTrack (ls.cpp:456-461): c=0.4, rho=0.5,
                       min_alpha=0.0
  ls_golden()          LineSearchGoldenSection (ls.cpp:95-100): tol=sqrt(2 eps),
                       max_iter=5, bracket=True
  ls_brent()           LineSearchBrent (ls.cpp:262-268): as ls_golden plus
                       zeps=1e-3 eps
  md.atoms.import_cfg  ImportCFGMD (import_cfg.cpp:496-652): an AtomEye CFG file
                       (standard or extended) as an atoms object
  md.export_cfg(...)   ExportCFGMD (export_cfg_md.cpp:9-16,167-226):
                       file_pattern, nevery=10000, extra_vecs=[], sort=False;
                       called as (atoms, file_name), or set as the .export of
                       nvt / min_lbfgs / min_cg to write every nevery steps
Additive: atoms.precision ('fp64' | 'mixed') selects the GPU arithmetic, and
min_lbfgs.f_tol adds the max|F| stop.

Each run keeps the reference's semantics: positions and velocities are read
from the atoms object, the neighbour list is rebuilt at the start, and the
results are written back when the run returns.
"""
import math
import sys

import numpy as np

from . import _lib

_PREC = {"fp64": _lib.FP64, "mixed": _lib.MIXED}


class ls_bt:
    """Back-tracking (Armijo) line search parameters."""

    def __init__(self, c=0.4, rho=0.5, min_alpha=0.0):
        if not (0.0 < c < 1.0):
            raise TypeError("c must be in (0,1)")
        if not (0.0 < rho < 1.0):
            raise TypeError("rho must be in (0,1)")
        if min_alpha < 0.0:
            raise TypeError("min_alpha must be >= 0")
        self.c, self.rho, self.min_alpha = float(c), float(rho), float(min_alpha)


class _bounded:
    """A validated attribute of a line search (the reference's VarAPI logics)."""

    def __init__(self, name, check, message, cast=float):
        self.name, self.check, self.message, self.cast = "_" + name, check, message, cast

    def __get__(self, obj, owner=None):
        return self if obj is None else getattr(obj, self.name)

    def __set__(self, obj, value):
        value = self.cast(value)
        if not self.check(value):
            raise TypeError(self.message)
        setattr(obj, self.name, value)


class ls_golden:
    """Golden-section line search (LineSearchGoldenSection, ls.h:340-515;
    defaults ls.cpp:95-100), bracketed first unless bracket is False."""

    tol = _bounded("tol", lambda v: v > 0.0, "tol should be greater than 0.0")
    max_iter = _bounded("max_iter", lambda v: v > 0, "max_iter should be greater than 0", int)

    def __init__(self, tol=math.sqrt(2.0 * sys.float_info.epsilon), max_iter=5, bracket=True):
        self.tol, self.max_iter, self.bracket = tol, max_iter, bool(bracket)

    def _struct(self):
        return _lib.line_search(_lib.LS_GOLDEN, tol=self.tol, max_iter=self.max_iter, bracket=self.bracket)


class ls_brent(ls_golden):
    """Brent's line search (LineSearchBrent, ls.h:524-706; defaults
    ls.cpp:262-268)."""

    zeps = _bounded("zeps", lambda v: v > 0.0, "zeps should be greater than 0.0")

    def __init__(self, tol=math.sqrt(2.0 * sys.float_info.epsilon), max_iter=5, bracket=True,
                 zeps=sys.float_info.epsilon * 1.0e-3):
        super().__init__(tol, max_iter, bracket)
        self.zeps = zeps

    def _struct(self):
        return _lib.line_search(_lib.LS_BRENT, tol=self.tol, max_iter=self.max_iter, bracket=self.bracket,
                                zeps=self.zeps)


def _ls_struct(ls):
    if isinstance(ls, ls_bt):
        return _lib.line_search(_lib.LS_BT, c=ls.c, rho=ls.rho, min_alpha=ls.min_alpha)
    if isinstance(ls, ls_golden):
        return ls._struct()
    raise TypeError("ls must be ls_bt, ls_golden or ls_brent")


class atoms:
    """A periodic cell: H (lower-triangular rows), x [N][3], elem [N] indices
    into elems, masses per element."""

    def __init__(self, H, x, elem, elems=("A",), masses=(63.5,), x_d=None):
        self.H = np.ascontiguousarray(H, dtype=np.float64).reshape(3, 3)
        self.x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 3).copy()
        self.elem = np.ascontiguousarray(elem, dtype=np.uint8).copy()
        if self.elem.shape[0] != self.x.shape[0]:
            raise TypeError("elem and x sizes differ")
        self.elems = tuple(elems)
        self.masses = np.ascontiguousarray(masses, dtype=np.float64)
        self.x_d = None if x_d is None else np.ascontiguousarray(x_d, dtype=np.float64).reshape(-1, 3).copy()
        self.f = None
        self.kB = float("nan")
        self.skin = 0.5
        self.precision = "fp64"
        self.step = 0
        self.pe = float("nan")
        self.S_pe = np.full((3, 3), np.nan)
        self.ff = None
        self.x_dof = None  # None, or [N][3] bool: True where a component is free
        self._sys = None
        self._sys_key = None
        self._sys_elem = None
        self._dof_set = None

    @property
    def natms(self):
        return self.x.shape[0]

    @property
    def vol(self):
        return float(self.H[0, 0] * self.H[1, 1] * self.H[2, 2])

    @classmethod
    def import_cfg(cls, cfg_file):
        """The configuration of an AtomEye CFG file: elements in order of
        first appearance with their masses, velocities when the file has
        them (libmappg's mappg_cfg_read)."""
        try:
            d = _lib.read_cfg(cfg_file)
        except _lib.MappgError as e:
            raise TypeError(str(e)) from None
        a = cls(d["H"], d["x"], d["elem"], elems=tuple(d["names"]), masses=d["masses"], x_d=d["x_d"])
        return a

    # ---------------------------------------------------------- force fields
    def _remap(self, ff):
        # the file's elements become the system's; an existing element list
        # selects and orders them, as the reference's element mapping does
        self.ff = ff
        if ff.names and all(ff.names):
            self.elems = tuple(ff.names)
        if self.masses.shape[0] != ff.nelem:
            m = np.full(ff.nelem, self.masses[0] if self.masses.size else 1.0)
            m[: min(ff.nelem, self.masses.shape[0])] = self.masses[: ff.nelem]
            self.masses = m
        self._sys = None

    def ff_eam_setfl(self, setfl_file):
        elems = list(self.elems) if all(self.elems) else None
        try:
            self._remap(_lib.ForceField.setfl(setfl_file, elems))
        except _lib.MappgError as e:
            raise TypeError(str(e)) from None

    def ff_eam_fs(self, fs_file):
        elems = list(self.elems) if all(self.elems) else None
        try:
            self._remap(_lib.ForceField.fs(fs_file, elems))
        except _lib.MappgError as e:
            raise TypeError(str(e)) from None

    def ff_eam_funcfl(self, funcfl_files, elems=None):
        if isinstance(funcfl_files, str):
            funcfl_files = [funcfl_files]
        try:
            self._remap(_lib.ForceField.funcfl(funcfl_files))
        except _lib.MappgError as e:
            raise TypeError(str(e)) from None
        if elems is not None:
            self.elems = tuple(elems)

    def create_temp(self, temp, seed):
        if math.isnan(self.kB):
            raise TypeError("boltzmann constant should be set prior to create_temp")
        dof = self._dof()
        if dof is None:
            self.x_d = _lib.create_temp(self.elem, self.masses, temp, self.kB, seed)
        else:
            # only the free components draw (AtomsMD::create_T, atoms_md.cpp:138-149)
            v = self.x_d if self.x_d is not None else np.zeros_like(self.x)
            self.x_d = _lib.create_temp_dof(self.elem, self.masses, dof, temp, self.kB, seed, v)

    # ---------------------------------------------------------- device state
    def _f_out(self):
        # the force array is refilled in place when it has the right shape
        # (a caller may have given pinned memory)
        f = self.f
        if isinstance(f, np.ndarray) and f.shape == self.x.shape and f.dtype == np.float64 and f.flags.c_contiguous:
            return f
        return None

    def _download(self, s):
        """x, x_d and f from the system, into the atoms' arrays when they can
        take them in place (C-contiguous float64 (n, 3)), else new arrays"""
        self.x = s.get_x(_inplace(self.x))
        self.x_d = s.get_v(_inplace(self.x_d) if self.x_d is not None else None)
        self.f = s.get_f(self._f_out())

    def _dof(self):
        if self.x_dof is None:
            return None
        d = np.asarray(self.x_dof, dtype=bool)
        if d.shape != self.x.shape:
            raise TypeError("x_dof should be an array of shape (natms, 3)")
        return None if d.all() else np.ascontiguousarray(d)

    def _key(self):
        # elem by content (compared against the copy kept with the key)
        return (id(self.ff), self.natms, self.precision, self.skin, self.H.tobytes())

    def _same_system(self):
        return self._sys is not None and self._sys_key == self._key() and self._sys_elem is not None \
            and self._sys_elem.shape == self.elem.shape and np.array_equal(self._sys_elem, self.elem)

    def _system(self):
        if self.ff is None:
            raise TypeError("cannot start without governing equations (force field)")
        key = self._key()
        if not self._same_system():
            self._sys = None
            self._sys = _lib.System(self.ff, self.H, self.x, self.elem, self.masses, self.skin,
                                    _PREC[self.precision])
            if self.precision == "mixed" and self.natms >= _AUTOTUNE_ATOMS:
                # lanes per atom and entries per step of the density and force
                # passes, timed once on this system's own list (~20 passes)
                self._sys.autotune()
            self._sys_key = key
            self._sys_elem = self.elem.copy()
            self._dof_set = None
        dof = self._dof()
        dkey = None if dof is None else dof.tobytes()
        if dkey != self._dof_set:
            self._sys.set_dof(dof)
            self._dof_set = dkey
        return self._sys


class export_cfg:
    """Writer of extended AtomEye CFG files.  Called as (atoms, file_name) it
    writes one file; as the .export of a run it writes
    file_pattern.%09d.cfg (the step number) at the start, every nevery
    steps and at the end.  extra_vecs lists per-atom vectors to add after
    the positions: "x_d" (velocities, written in reduced units) and "f"."""

    _VECS = ("x_d", "f")

    def __init__(self, file_pattern, nevery=10000, extra_vecs=None, sort=False):
        if not (int(nevery) > 0):
            raise TypeError("nevery should be greater than 0")
        self.file_pattern = str(file_pattern)
        self.nevery = int(nevery)
        self.extra_vecs = list(extra_vecs or [])
        self.sort = bool(sort)

    @property
    def default_vecs(self):
        # atoms keep the caller's order, which is already the id order that
        # sort=True asks for
        return ["elem", "x"] + (["id"] if self.sort else [])

    def __call__(self, atoms, file_name):
        self._write(atoms, file_name, atoms.x, atoms.x_d, atoms.f)

    def _write_step(self, atoms, step, x, x_d, f, H=None):
        self._write(atoms, "%s.%09d.cfg" % (self.file_pattern, step), x, x_d, f, H)

    def _write(self, atoms, path, x, x_d, f, H=None):
        vecs = []
        for name in self.extra_vecs:
            if name not in self._VECS:
                raise TypeError("cannot export vector '%s' to file, it does not exist" % name)
            arr = x_d if name == "x_d" else f
            if arr is None:
                raise TypeError("cannot export vector '%s' to file, it is empty" % name)
            vecs.append((name, arr))
        try:
            _lib.write_cfg(path, atoms.H if H is None else H, x, atoms.elem, atoms.masses, list(atoms.elems), vecs)
        except _lib.MappgError as e:
            raise TypeError(str(e)) from None

    def _wants_f(self):
        return "f" in self.extra_vecs


_ROWS_FOR_PE = 4096
_AUTOTUNE_ATOMS = 50000  # mixed systems from this size are autotuned when created


def _inplace(a):
    """a, when a run can write its result into it directly."""
    if isinstance(a, np.ndarray) and a.dtype == np.float64 and a.flags.c_contiguous and a.flags.writeable \
            and a.ndim == 2 and a.shape[1] == 3:
        return a
    return None


def _print_thermo(th, step0, ntally, vol):
    hdr = "%8s %14s %16s %12s %12s %12s" % ("step", "T", "PE", "S[0][0]", "S[1][1]", "S[2][2]")
    print(hdr)
    n = th.shape[0] - 1
    for k in range(n + 1):
        if k == 0 or k == n or (ntally and k % ntally == 0):
            r = th[k]
            # S_part = S_pe - mvv/V with S_pe = -F_H/V
            s = [-(r[8 + q] + r[2 + q]) / vol for q in (0, 3, 5)]
            print("%8d %14.6f %16.8f %12.6e %12.6e %12.6e" % (step0 + k, r[1], r[0], s[0], s[1], s[2]))
    sys.stdout.flush()


class nvt:
    """Canonical MD with a Nose-Hoover chain (NVE: t_relax = inf)."""

    def __init__(self, T, dt):
        if not (T > 0.0):
            raise TypeError("T should be greater than 0.0")
        if not (dt > 0.0):
            raise TypeError("dt should be greater than 0.0")
        self.T = float(T)
        self.dt = float(dt)
        self.t_relax = 100.0 * self.dt
        self.L = 3
        self.niters = 1
        self.ntally = 10000
        self.export = None
        self._eta = np.zeros(3)

    def run(self, atoms, nsteps):
        if nsteps < 0:
            raise TypeError("nsteps should be greater than or equal to 0")
        if atoms.ff is None:
            raise TypeError("cannot start md without governing equations (force field)")
        if math.isnan(atoms.kB):
            raise TypeError("boltzmann constant should be set prior to MD")
        if self._eta.shape[0] != self.L:
            self._eta = np.zeros(self.L)
        s = atoms._system()
        v_in = atoms.x_d if atoms.x_d is not None else np.zeros_like(atoms.x)
        # the per-step rows (14 doubles) also carry the last step's energy and
        # virial, which atoms.pe / S_pe take; short runs keep them even
        # without a tally instead of paying for one more force call
        rows = bool(self.ntally) or nsteps <= _ROWS_FOR_PE
        xprt = self.export
        if xprt is None:
            # one call: x, v in, the run, x, v, f out (the arrays refilled in
            # place when they have the right form)
            x_out = _inplace(atoms.x)
            v_out = _inplace(atoms.x_d) if atoms.x_d is not None else None
            x_out = x_out if x_out is not None else np.empty((atoms.natms, 3))
            v_out = v_out if v_out is not None else np.empty((atoms.natms, 3))
            f_out = atoms._f_out()
            f_out = f_out if f_out is not None else np.empty((atoms.natms, 3))
            th, self._eta = s.nvt_run_host(atoms.x, v_in, self.T, self.dt, atoms.kB, nsteps, t_relax=self.t_relax,
                                           L=self.L, niters=self.niters, eta=self._eta, thermo=rows, x_out=x_out,
                                           v_out=v_out, f_out=f_out)
            atoms.x, atoms.x_d, atoms.f = x_out, v_out, f_out
        else:
            s.set_x(atoms.x)
            s.set_v(v_in)
            # MDNVT::run's exports (md_nvt.cpp:390,436,470): the run goes on
            # the device in nevery-step pieces, each export is a snapshot
            s.nvt_begin(self.T, self.dt, atoms.kB, nsteps, t_relax=self.t_relax, L=self.L, niters=self.niters,
                        eta=self._eta, thermo=rows)
            try:
                def snap(step):
                    x, v = s.nvt_snapshot()
                    xprt._write_step(atoms, step, x, v, s.get_f() if xprt._wants_f() else None)

                snap(atoms.step)
                done = 0
                while done < nsteps:
                    k = min(xprt.nevery - done % xprt.nevery, nsteps - done)
                    s.nvt_steps(k)
                    done += k
                    if done % xprt.nevery == 0 or done == nsteps:
                        snap(atoms.step + done)
            finally:
                th, self._eta = s.nvt_end()
            atoms._download(s)
        if th is not None:
            if self.ntally:
                _print_thermo(th, atoms.step, self.ntally, atoms.vol)
            atoms.pe = float(th[-1, 0])
            F_H = th[-1, 8:14]
        else:
            atoms.pe, F_H = s.force()
        atoms.S_pe = _voigt_to_matrix(-np.asarray(F_H) / atoms.vol)
        atoms.step += nsteps


def _stress_arg(S):
    """The reference's symmetric S (rows of lengths 1, 2, 3, or a full 3x3;
    None or NaN where the box entry has no degree of freedom) as 3x3."""
    rows = [list(r) for r in S]
    if len(rows) != 3 or any(len(r) not in (i + 1, 3) for i, r in enumerate(rows)):
        raise TypeError("S should be [[Sxx],[Syx,Syy],[Szx,Szy,Szz]] or a 3x3 array")
    out = np.full((3, 3), np.nan)
    for i in range(3):
        for j in range(i + 1):
            v = rows[i][j]
            out[i, j] = out[j, i] = np.nan if v is None else float(v)
    return out


class nst(nvt):
    """Constant-stress (NST) MD: MDNST (md_nst.cpp) with the particle chain
    of md.nvt and a box chain (t_relax_s, default 1000 dt); S is the applied
    stress, NaN (or None) where the box entry stays fixed; tau the box
    relaxation times (default 1000 dt); nreset renews the reference box every
    nreset steps (0: never)."""

    def __init__(self, S, T, dt):
        super().__init__(T, dt)
        self.S = _stress_arg(S)
        if np.all(np.isnan(self.S)):
            raise TypeError("at least one component of S must be set")
        self.tau = np.full((3, 3), 1000.0 * self.dt)
        self.t_relax_s = 1000.0 * self.dt
        self.nreset = 0
        self._V_H = np.zeros((3, 3))
        self._eta_s = np.zeros(3)

    def run(self, atoms, nsteps):
        if nsteps < 0:
            raise TypeError("nsteps should be greater than or equal to 0")
        if atoms.ff is None:
            raise TypeError("cannot start md without governing equations (force field)")
        if math.isnan(atoms.kB):
            raise TypeError("boltzmann constant should be set prior to MD")
        if self._eta.shape[0] != self.L:
            self._eta = np.zeros(self.L)
        s = atoms._system()
        s.set_x(atoms.x)
        s.set_v(atoms.x_d if atoms.x_d is not None else np.zeros_like(atoms.x))
        xprt = self.export
        step0 = atoms.step
        if xprt is not None:
            # MDNST::run's exports: the start, every nevery steps and the last
            # step (the library calls the hook after those steps)
            f0 = None
            if xprt._wants_f():
                s.force()
                f0 = s.get_f()
            xprt._write_step(atoms, step0, atoms.x, atoms.x_d, f0)

            def at(it):
                xprt._write_step(atoms, step0 + it, s.get_x(), s.get_v(),
                                 s.get_f() if xprt._wants_f() else None, s.get_box())

            s.set_hook(at, xprt.nevery)
        try:
            th, self._V_H, self._eta, self._eta_s = s.nst_run(
                self.S, self.T, self.dt, atoms.kB, nsteps, tau=self.tau, t_relax=self.t_relax, L=self.L,
                niters=self.niters, t_relax_S=self.t_relax_s, nreset=self.nreset, V_H=self._V_H, eta=self._eta,
                eta_S=self._eta_s, thermo=True)
        finally:
            if xprt is not None:
                s.set_hook(None, 0)
        atoms._download(s)
        atoms.H = s.get_box()
        atoms._sys_key = atoms._key()
        if self.ntally:
            vol = float(atoms.H[0, 0] * atoms.H[1, 1] * atoms.H[2, 2])
            _print_thermo(th[:, :14], atoms.step, self.ntally, vol)
        atoms.pe = float(th[-1, 0])
        atoms.S_pe = _voigt_to_matrix(-th[-1, 8:14] / atoms.vol)
        atoms.step += nsteps
        self.last_thermo = th


def _voigt_to_matrix(v):
    v = np.asarray(v)
    return np.array([[v[0], v[1], v[2]], [v[1], v[3], v[4]], [v[2], v[4], v[5]]])


def _min_run(atoms, xprt, run):
    """A minimizer run with the reference's exports (MinHelper::ExportHandler,
    min.h:207-227): at the start, after every nevery-th iteration and at
    the end when that step was not already written."""
    s = atoms._system()
    s.set_x(atoms.x)
    if xprt is None:
        return s, run(s)
    step0 = atoms.step
    f0 = None
    if xprt._wants_f():
        s.force()
        f0 = s.get_f()
    xprt._write_step(atoms, step0, atoms.x, atoms.x_d, f0)

    def at(it):
        xprt._write_step(atoms, step0 + it, s.get_x(), atoms.x_d, s.get_f() if xprt._wants_f() else None,
                         s.get_box())

    s.set_hook(at, xprt.nevery)
    try:
        r = run(s)
    finally:
        s.set_hook(None, 0)
    if r["niter"] % xprt.nevery:
        xprt._write_step(atoms, step0 + r["niter"], s.get_x(), atoms.x_d,
                         s.get_f() if xprt._wants_f() else None, s.get_box())
    return s, r


def _h_dof_mask(H_dof):
    """The reference's symmetric bool[3][3] (rows of lengths 1, 2, 3 for the
    lower triangle, or a full 3x3) as a 3x3 mask of its lower triangle."""
    mask = np.zeros((3, 3), dtype=bool)
    if H_dof is None:
        return mask
    rows = [list(r) for r in H_dof]
    if len(rows) != 3 or any(len(r) not in (i + 1, 3) for i, r in enumerate(rows)):
        raise TypeError("H_dof should be [[bool],[bool,bool],[bool,bool,bool]] or a 3x3 array of bool")
    for i in range(3):
        for j in range(i + 1):
            mask[i, j] = bool(rows[i][j])
    return mask


class _min:
    """What md.min_lbfgs and md.min_cg share (Min, min.cpp:30-60): e_tol,
    H_dof (box entries that relax), affine, max_dx, ls, plus f_tol."""

    def __init__(self, e_tol, H_dof, affine, max_dx, ls, f_tol):
        if e_tol < 0.0:
            raise TypeError("e_tol should be greater than or equal to 0.0")
        if not (max_dx > 0.0):
            raise TypeError("max_dx should be greater than 0.0")
        self.H_dof = _h_dof_mask(H_dof)
        self.affine = bool(affine)
        self.e_tol = float(e_tol)
        self.max_dx = float(max_dx)
        self.ls = ls if ls is not None else ls_bt()
        self.f_tol = float(f_tol)
        self.ntally = 1000
        self.export = None
        self.last = None

    def _box(self):
        return bool(self.H_dof.any()) or self.affine

    def _run(self, atoms, max_nsteps, method, atoms_only):
        if max_nsteps < 0:
            raise TypeError("max_nsteps should be greater than or equal to 0")
        ls = _ls_struct(self.ls)
        if self._box():
            if self.f_tol > 0.0:
                raise TypeError("f_tol is not available with box degrees of freedom (use e_tol)")
            run = lambda s: s.min_box_run(ls, self.H_dof, self.affine, method, getattr(self, "m", 0),  # noqa: E731
                                          self.e_tol, self.max_dx, max_nsteps)
        else:
            run = atoms_only(ls)
        s, r = _min_run(atoms, self.export, run)
        atoms.x = s.get_x(_inplace(atoms.x))
        if self._box():
            atoms.H = s.get_box()
            atoms._sys_key = atoms._key()
        atoms.f = s.get_f(atoms._f_out())
        atoms.pe = r["pe"]
        atoms.step += r["niter"]
        self.last = r
        return r


class min_lbfgs(_min):
    """L-BFGS minimization (MinLBFGS, min_l-bfgs.cpp; min_l-bfgs.h:113-219) of
    the positions and, with H_dof or affine, of the box."""

    def __init__(self, m=2, e_tol=math.sqrt(sys.float_info.epsilon), H_dof=None, affine=False, max_dx=1.0,
                 ls=None, f_tol=0.0):
        if m < 0:
            raise TypeError("m should be greater than or equal to 0")
        super().__init__(e_tol, H_dof, affine, max_dx, ls, f_tol)
        self.m = int(m)

    def run(self, atoms, max_nsteps):
        return self._run(atoms, max_nsteps, "lbfgs", lambda ls: lambda s: s.lbfgs_run_ls(
            ls, m=self.m, e_tol=self.e_tol, max_dx=self.max_dx, f_tol=self.f_tol, nsteps=max_nsteps))


class min_cg(_min):
    """Polak-Ribiere conjugate-gradient minimization (MinCG::__run,
    min_cg.h:454-536) with any of the three line searches, of the positions
    and, with H_dof or affine, of the box."""

    def __init__(self, e_tol=math.sqrt(sys.float_info.epsilon), H_dof=None, affine=False, max_dx=1.0, ls=None,
                 f_tol=0.0):
        super().__init__(e_tol, H_dof, affine, max_dx, ls, f_tol)

    def run(self, atoms, max_nsteps):
        return self._run(atoms, max_nsteps, "cg", lambda ls: lambda s: s.cg_run_ls(
            ls, e_tol=self.e_tol, max_dx=self.max_dx, f_tol=self.f_tol, nsteps=max_nsteps))


min_cg_new = min_cg  # the name the reference registers for this minimizer
