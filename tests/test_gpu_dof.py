"""atoms.x_dof on the GPU against the oracle: forces on frozen components are
zero (ForceFieldMD::force_calc, ff_md.cpp:138-144), the minimizers leave
them in place, FP64 NVT runs take the reference's _w_dof steps
(md_nvt.cpp:144-215), and the paths that do not take x_dof refuse it.
Tolerances as in the other parity tests: forces 1e-10 relative, energies
1e-11 relative, trajectories 1e-8 A."""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from mapp4py_gb300 import _lib, md, synth

pytestmark = pytest.mark.gpu


def dof_mask(n, seed=5):
    rng = np.random.default_rng(seed)
    d = np.ones((n, 3), dtype=bool)
    r = rng.random(n)
    d[r < 0.2] = False
    d[(r >= 0.2) & (r < 0.3), 2] = False
    d[(r >= 0.3) & (r < 0.35), 0] = False
    return d


@pytest.fixture(scope="module")
def cell():
    return synth.alloy((5, 5, 5), xB=0.3, sigma=0.1, T=600.0, seed=2)


def pair(potentials, c, d, precision=_lib.FP64):
    path = potentials[("A", "B")][0]
    s = _lib.System(_lib.ForceField.setfl(path), c.H, c.x, c.elem, c.masses, precision=precision)
    o = O.System(O.Eam.setfl(path), c.H, c.x, c.elem, c.masses)
    s.set_dof(d)
    o.set_dof(d)
    return s, o


@pytest.mark.parametrize("precision", [_lib.FP64, _lib.MIXED])
def test_forces_zero_on_frozen_components(potentials, cell, precision):
    d = dof_mask(cell.natoms)
    s, o = pair(potentials, cell, d, precision)
    pe, vir = s.force()
    f = s.get_f()
    pe_o, vir_o = o.force()
    assert np.all(f[~d] == 0.0)
    tol = 1e-10 if precision == _lib.FP64 else 1e-4
    assert np.max(np.abs(f - o.f)) <= tol * max(1.0, np.max(np.abs(o.f)))
    assert abs(pe - pe_o) <= (1e-11 if precision == _lib.FP64 else 1e-6) * abs(pe_o)
    # clearing the mask restores the full forces
    s.set_dof(None)
    s.force()
    assert np.any(s.get_f()[~d] != 0.0)


def test_noalloc_forces_zero_on_frozen_components(potentials, cell):
    torch = pytest.importorskip("torch")
    d = dof_mask(cell.natoms)
    s, o = pair(potentials, cell, d)
    s.build()
    f = torch.full((s.n, 3), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    _lib.check(_lib.load().mappg_sys_force_noalloc(s.h, C.c_void_p(f.data_ptr()), None))
    s.sync()
    fn = f.cpu().numpy()
    o.force()
    assert np.all(fn[~d] == 0.0)
    assert np.max(np.abs(fn - o.f)) <= 1e-10 * max(1.0, np.max(np.abs(o.f)))


@pytest.mark.parametrize("kind", ["lbfgs", "cg"])
def test_minimizer_keeps_frozen_components(potentials, cell, kind):
    d = dof_mask(cell.natoms)
    s, o = pair(potentials, cell, d)
    if kind == "lbfgs":
        r = s.lbfgs_run(m=10, e_tol=0.0, f_tol=1e-4, nsteps=3000)
        ro = o.lbfgs_run(m=10, e_tol=0.0, f_tol=1e-4, nsteps=3000)
    else:
        r = s.cg_run(e_tol=0.0, f_tol=1e-4, nsteps=3000)
        ro = o.cg_run(e_tol=0.0, f_tol=1e-4, nsteps=3000)
    assert r["err"] == ro["err"] == 100
    assert r["niter"] == ro["niter"] and r["n_energy"] == ro["n_energy"]
    assert abs(r["pe"] - ro["pe"]) <= 1e-11 * abs(ro["pe"])
    x = s.get_x()
    dx = x - o.x
    dx -= np.round(dx @ np.linalg.inv(cell.H)) @ cell.H
    assert np.max(np.abs(dx)) < 1e-8
    d0 = x - cell.x
    d0 -= np.round(d0 @ np.linalg.inv(cell.H)) @ cell.H
    assert np.max(np.abs(d0[~d])) < 1e-12


def test_fp64_nvt_with_frozen_components(potentials, cell):
    d = dof_mask(cell.natoms)
    s, o = pair(potentials, cell, d)
    v = O.create_temp_dof(cell.elem, cell.masses, d, 600.0, synth.KB, 77, np.full((cell.natoms, 3), 1e-3))
    s.set_v(v)
    o.v = v
    nsteps = 60
    th_o, eta_o, nreb_o = o.nvt_run(600.0, synth.FS, synth.KB, nsteps, t_relax=20 * synth.FS)
    th, eta = s.nvt_run(600.0, synth.FS, synth.KB, nsteps, t_relax=20 * synth.FS, thermo=True)
    assert np.max(np.abs(th[:, 0] - th_o[:, 0])) <= 1e-10 * np.max(np.abs(th_o[:, 0]))
    assert np.max(np.abs(th[:, 1] - th_o[:, 1])) <= 1e-9 * np.max(np.abs(th_o[:, 1]))
    dx = s.get_x() - o.x
    dx -= np.round(dx @ np.linalg.inv(cell.H)) @ cell.H
    assert np.max(np.abs(dx)) < 1e-8
    vg = s.get_v()
    assert np.max(np.abs(vg - o.v)) < 1e-8
    assert np.all(vg[~d] == 1e-3)
    assert np.max(np.abs(eta - eta_o)) <= 1e-9 * max(1.0, np.max(np.abs(eta_o)))


def test_md_api_x_dof(potentials, cell):
    """md.atoms.x_dof through md.nvt and md.min_lbfgs, and create_temp."""
    d = dof_mask(cell.natoms)
    a = md.atoms(cell.H, cell.x, cell.elem, elems=("A", "B"), masses=cell.masses, x_d=np.zeros_like(cell.x))
    a.ff_eam_setfl(potentials[("A", "B")][0])
    a.kB = synth.KB
    a.x_dof = d
    a.create_temp(600.0, 77)
    assert np.all(a.x_d[~d] == 0.0)
    x0 = a.x.copy()
    integ = md.nvt(600.0, synth.FS)
    integ.ntally = 0
    integ.run(a, 20)
    dx = a.x - x0
    dx -= np.round(dx @ np.linalg.inv(a.H)) @ a.H
    assert np.max(np.abs(dx[~d])) < 1e-12 and np.all(a.x_d[~d] == 0.0)
    m = md.min_lbfgs(m=5, e_tol=0.0)
    m.run(a, 30)
    assert np.all(a.f[~d] == 0.0)
    dx = a.x - x0
    dx -= np.round(dx @ np.linalg.inv(a.H)) @ a.H
    assert np.max(np.abs(dx[~d])) < 1e-12
    # clearing x_dof brings the full forces back
    a.x_dof = None
    md.min_lbfgs(m=5, e_tol=0.0).run(a, 1)
    assert np.any(a.f[~d] != 0.0)


def test_mixed_nvt_with_frozen_components(potentials, cell):
    """The mixed-precision step kernels take the same dof branches: the run
    follows the FP64 one within the mixed-precision budget, and frozen
    components keep their velocity exactly."""
    d = dof_mask(cell.natoms)
    v = O.create_temp_dof(cell.elem, cell.masses, d, 600.0, synth.KB, 77, np.full((cell.natoms, 3), 1e-3))
    runs = {}
    for prec in (_lib.FP64, _lib.MIXED):
        s, _ = pair(potentials, cell, d, prec)
        s.set_v(v)
        th, eta = s.nvt_run(600.0, synth.FS, synth.KB, 60, t_relax=20 * synth.FS, thermo=True)
        runs[prec] = (s.get_x(), s.get_v(), th)
    x64, v64, th64 = runs[_lib.FP64]
    x32, v32, th32 = runs[_lib.MIXED]
    assert np.all(v32[~d] == 1e-3)
    dx = x32 - x64
    dx -= np.round(dx @ np.linalg.inv(cell.H)) @ cell.H
    assert np.max(np.abs(dx)) < 1e-5
    assert np.max(np.abs(v32 - v64)) < 1e-5
    assert np.max(np.abs(th32[:, 1] - th64[:, 1])) < 1e-4 * np.max(th64[:, 1])
    assert np.max(np.abs(th32[:, 0] - th64[:, 0])) / cell.natoms < 1e-6


def test_paths_without_x_dof_refuse_it(potentials, cell):
    d = dof_mask(cell.natoms)
    t, _ = pair(potentials, cell, d)
    t.set_v(cell.v)
    with pytest.raises(ValueError):
        t.set_dof(np.ones((cell.natoms + 1, 3), bool))


@pytest.mark.parametrize("precision", [_lib.FP64, _lib.MIXED])
def test_nst_with_frozen_components(potentials, precision):
    """md.nst with x_dof against the oracle (FP64) or the FP64 GPU run
    (mixed): frozen components leave ndof and carry no force; a stress along
    a frozen direction is refused with the reference's message."""
    path = potentials[("A", "B")][0]
    c = synth.alloy((5, 5, 5), a=2.9, xB=0.3, sigma=0.02, T=300.0, seed=4)
    d = np.ones((c.natoms, 3), bool)
    d[::5, 2] = False
    nan = np.nan
    S = np.array([[0.0, nan, nan], [nan, 0.0, nan], [nan, nan, nan]])
    tau = np.full((3, 3), 50 * synth.FS)
    o = O.System(O.Eam.setfl(path), c.H, c.x, c.elem, c.masses)
    o.set_dof(d)
    o.v = c.v
    tho, VHo, _, _ = o.nst_run(S, 300.0, synth.FS, synth.KB, 30, tau=tau)
    s = _lib.System(_lib.ForceField.setfl(path), c.H, c.x, c.elem, c.masses, precision=precision)
    s.set_dof(d)
    s.set_v(c.v)
    th, VH, _, _ = s.nst_run(S, 300.0, synth.FS, synth.KB, 30, tau=tau)
    assert np.all(s.get_f()[~d] == 0.0)
    if precision == _lib.FP64:
        assert np.max(np.abs(th[:, 0] - tho[:, 0])) <= 1e-9 * np.max(np.abs(tho[:, 0]))
        assert np.max(np.abs(th[:, 1] - tho[:, 1])) <= 1e-8 * np.max(tho[:, 1])
        assert np.max(np.abs(th[:, 14:] - tho[:, 14:])) < 1e-10
        d_x = s.get_x() - o.x
        H = s.get_box()
        d_x -= np.round(d_x @ np.linalg.inv(H)) @ H
        assert np.max(np.abs(d_x)) < 1e-9 and np.max(np.abs(s.get_v() - o.v)) < 1e-10
    else:
        assert np.max(np.abs(th[:, 0] - tho[:, 0])) / c.natoms < 1e-6
        assert np.max(np.abs(th[:, 14:] - tho[:, 14:])) < 2e-6 * np.max(np.abs(c.H))
    S[2, 2] = 0.0
    t = _lib.System(_lib.ForceField.setfl(path), c.H, c.x, c.elem, c.masses, precision=precision)
    t.set_dof(d)
    t.set_v(c.v)
    with pytest.raises(_lib.MappgError, match=r"cannot impose stress component \[2\]\[2\]"):
        t.nst_run(S, 300.0, synth.FS, synth.KB, 1)
