"""The mapp4py-style surface (mapp4py_gb300.md) on the GPU: md.atoms with a
setfl force field, md.nvt / md.min_lbfgs / md.min_cg runs against the same
runs through the system-level binding, CFG exports during runs
(md.export_cfg as a run's .export: files at the start, every nevery steps
and at the end, as MDNVT::run and MinHelper::ExportHandler write them), and
md.atoms.import_cfg feeding a run."""
import os

import numpy as np
import pytest

from mapp4py_gb300 import _lib, md, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setfl(potentials):
    return potentials[("A", "B")][0]


def make_atoms(setfl, precision="fp64", n=(5, 5, 5), T=600.0, seed=3, sigma=0.05):
    c = synth.alloy(n, xB=0.5, sigma=sigma, T=T, seed=seed)
    a = md.atoms(c.H, c.x, c.elem, elems=("A", "B"), masses=c.masses, x_d=c.v)
    a.ff_eam_setfl(setfl)
    a.kB = synth.KB
    a.precision = precision
    return a


def files(pattern):
    d, base = os.path.split(pattern)
    out = {}
    for f in os.listdir(d):
        if f.startswith(base + ".") and f.endswith(".cfg"):
            out[int(f[len(base) + 1:-4])] = os.path.join(d, f)
    return out


def test_nvt_run_matches_system_binding(setfl):
    a = make_atoms(setfl)
    x0, v0 = a.x.copy(), a.x_d.copy()
    integ = md.nvt(600.0, synth.FS)
    integ.ntally = 0
    integ.run(a, 40)
    s = _lib.System(_lib.ForceField.setfl(setfl, ["A", "B"]), a.H, x0, a.elem, a.masses)
    s.set_v(v0)
    s.nvt_run(600.0, synth.FS, synth.KB, 40, t_relax=100 * synth.FS)
    assert np.array_equal(a.x, s.get_x()) and np.array_equal(a.x_d, s.get_v())
    assert a.step == 40 and np.isfinite(a.pe) and a.S_pe.shape == (3, 3)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_nvt_export_every_nevery(setfl, tmp_path, precision):
    a = make_atoms(setfl, precision)
    b = make_atoms(setfl, precision)
    pattern = str(tmp_path / "run")
    integ = md.nvt(600.0, synth.FS)
    integ.ntally = 0
    integ.export = md.export_cfg(pattern, nevery=10, extra_vecs=["x_d"])
    integ.run(a, 25)
    plain = md.nvt(600.0, synth.FS)
    plain.ntally = 0
    plain.run(b, 25)
    # the pieces and the snapshots leave the trajectory as it is
    assert np.array_equal(a.x, b.x) and np.array_equal(a.x_d, b.x_d)
    got = files(pattern)
    assert sorted(got) == [0, 10, 20, 25]
    first = md.atoms.import_cfg(got[0])
    d0 = first.x - make_atoms(setfl, precision).x
    assert np.max(np.abs(d0 - np.round(d0 @ np.linalg.inv(a.H)) @ a.H)) < 1e-12
    last = md.atoms.import_cfg(got[25])
    d = last.x - a.x
    d -= np.round(d @ np.linalg.inv(a.H)) @ a.H
    assert np.max(np.abs(d)) < 1e-12
    # the file holds the velocities before the run's final thermostat
    # scale: one common factor close to 1 separates them
    r = a.x_d / last.x_d
    fac = np.median(r)
    assert abs(fac - 1.0) < 1e-2 and np.max(np.abs(a.x_d - fac * last.x_d)) < 1e-12
    # a second run continues the step numbering
    integ.run(a, 10)
    assert sorted(files(pattern)) == [0, 10, 20, 25, 35]  # steps counted within each run


@pytest.mark.parametrize("kind", ["lbfgs", "cg"])
def test_minimizer_export(setfl, tmp_path, kind):
    def minimizer():
        return md.min_lbfgs(m=5, e_tol=0.0) if kind == "lbfgs" else md.min_cg(e_tol=0.0)

    a = make_atoms(setfl, T=0.0, sigma=0.1)
    ref = make_atoms(setfl, T=0.0, sigma=0.1)
    pattern = str(tmp_path / kind)
    m = minimizer()
    m.export = md.export_cfg(pattern, nevery=4, extra_vecs=["f"])
    r = m.run(a, 10)
    r_ref = minimizer().run(ref, 10)
    assert r["niter"] == r_ref["niter"] == 10
    assert np.array_equal(a.x, ref.x) and r["pe"] == r_ref["pe"]
    got = files(pattern)
    assert sorted(got) == [0, 4, 8, 10]
    # the file of iteration 4 holds the positions after four iterations
    four = make_atoms(setfl, T=0.0, sigma=0.1)
    minimizer().run(four, 4)
    snap = md.atoms.import_cfg(got[4])
    d = snap.x - four.x
    d -= np.round(d @ np.linalg.inv(a.H)) @ a.H
    assert np.max(np.abs(d)) < 1e-12
    # the forces column of the last file is the run's final force
    with open(got[10]) as fh:
        lines = fh.read().splitlines()
    body = lines[lines.index("auxiliary[2] = f_2 [reduced unit]") + 1:]
    rows = [ln.split() for ln in body if len(ln.split()) == 6]
    f_file = np.array(rows, dtype=float)[:, 3:]
    assert np.max(np.abs(f_file - a.f)) < 1e-12


def test_export_failure_stops_the_run(setfl, tmp_path):
    class Failing(md.export_cfg):
        def _write_step(self, atoms, step, x, x_d, f, H=None):
            if step == 4:
                raise RuntimeError("disk full")
            super()._write_step(atoms, step, x, x_d, f, H)

    a = make_atoms(setfl, T=0.0, sigma=0.1)
    m = md.min_lbfgs(m=5, e_tol=0.0)
    m.export = Failing(str(tmp_path / "x"), nevery=2)
    # the exception raised inside the iteration hook ends the device run
    with pytest.raises(RuntimeError, match="disk full"):
        m.run(a, 10)
    assert sorted(files(str(tmp_path / "x"))) == [0, 2]
    m.export = None
    assert m.run(a, 3)["niter"] == 3  # the system is usable afterwards


def test_import_cfg_runs(setfl, tmp_path):
    a = make_atoms(setfl, T=300.0)
    p = str(tmp_path / "start.cfg")
    md.export_cfg("unused", extra_vecs=["x_d"])(a, p)
    b = md.atoms.import_cfg(p)
    b.ff_eam_setfl(setfl)
    b.kB = synth.KB
    assert b.elems == ("A", "B") or b.elems == ("B", "A")
    integ = md.nvt(300.0, synth.FS)
    integ.ntally = 0
    integ.run(b, 20)
    assert np.all(np.isfinite(b.x)) and np.isfinite(b.pe)
    # same start, same elements: the run follows the original to the file's
    # printed precision
    c = make_atoms(setfl, T=300.0)
    integ2 = md.nvt(300.0, synth.FS)
    integ2.ntally = 0
    integ2.run(c, 20)
    order = np.array([b.elems.index(e) for e in c.elems])
    assert np.array_equal(order[c.elem], b.elem)
    d = b.x - c.x
    d -= np.round(d @ np.linalg.inv(c.H)) @ c.H
    assert np.max(np.abs(d)) < 1e-8


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_short_runs_without_step_graph(setfl, precision):
    """Runs of fewer than eight steps launch their kernels directly instead
    of through the captured step graph; atoms.pe and S_pe of a run come from
    its last step.  One 5-step run against the oracle (FP64) or the FP64 GPU
    run (mixed, the mixed-precision budget), and run(atoms, 1) repeated
    against one run of the same total length."""
    import oracle as O

    a = make_atoms(setfl, precision)
    x0, v0 = a.x.copy(), a.x_d.copy()
    integ = md.nvt(600.0, synth.FS)
    integ.ntally = 0
    integ.run(a, 5)
    if precision == "fp64":
        o = O.System(O.Eam.setfl(setfl), a.H, x0, a.elem, a.masses)
        o.v = v0
        th_o, _, _ = o.nvt_run(600.0, synth.FS, synth.KB, 5, t_relax=100 * synth.FS)
        d = a.x - o.x
        d -= np.round(d @ np.linalg.inv(a.H)) @ a.H
        assert np.max(np.abs(d)) < 1e-9 and np.max(np.abs(a.x_d - o.v)) < 1e-9
        assert abs(a.pe - th_o[-1, 0]) <= 1e-11 * abs(th_o[-1, 0])
        F_H = th_o[-1, 8:14]
        S = -np.array([[F_H[0], F_H[1], F_H[2]], [F_H[1], F_H[3], F_H[4]], [F_H[2], F_H[4], F_H[5]]]) / a.vol
        assert np.max(np.abs(a.S_pe - S)) <= 1e-10 * np.max(np.abs(S))
    else:
        b = make_atoms(setfl, "fp64")
        integ64 = md.nvt(600.0, synth.FS)
        integ64.ntally = 0
        integ64.run(b, 5)
        assert np.max(np.abs(a.x - b.x)) < 1e-5
        assert abs(a.pe - b.pe) / a.natms < 1e-6
    # the energy the run reports is the energy of its final positions
    s = a._system()
    s.set_x(a.x)
    pe, _ = s.force()
    assert abs(pe - a.pe) <= (1e-11 * abs(pe) if precision == "fp64" else 1e-7 * a.natms)
    c = make_atoms(setfl, precision)
    one = md.nvt(600.0, synth.FS)
    one.ntally = 0
    for _ in range(3):
        one.run(c, 1)
    assert c.step == 3 and np.all(np.isfinite(c.x)) and np.isfinite(c.pe)


@pytest.mark.parametrize("precision", [_lib.FP64, _lib.MIXED])
def test_nvt_run_host_matches_separate_calls(setfl, precision):
    """mappg_nvt_run_host (x, v in; run; x, v, f out in one call, the
    velocity upload on a second stream) gives the bits of set_x, set_v,
    nvt_run, get_x, get_v, get_f; outputs may alias the inputs."""
    c = synth.alloy((5, 5, 5), xB=0.5, sigma=0.05, T=600.0, seed=8)
    ff = _lib.ForceField.setfl(setfl, ["A", "B"])
    runs = []
    for one_call in (False, True):
        s = _lib.System(ff, c.H, c.x, c.elem, c.masses, precision=precision)
        for _ in range(2):  # a second run reuses the list and the side stream
            x = c.x.copy()
            v = c.v.copy()
            if one_call:
                f = np.empty_like(x)
                th, eta = s.nvt_run_host(x, v, 600.0, synth.FS, synth.KB, 12, thermo=True, x_out=x, v_out=v,
                                         f_out=f)
            else:
                s.set_x(x)
                s.set_v(v)
                th, eta = s.nvt_run(600.0, synth.FS, synth.KB, 12, thermo=True)
                x, v, f = s.get_x(), s.get_v(), s.get_f()
        runs.append((x, v, f, th, eta))
    for a, b in zip(runs[0], runs[1]):
        assert np.array_equal(a, b)
    with pytest.raises(ValueError):
        s.nvt_run_host(c.x, c.v, 600.0, synth.FS, synth.KB, 1, x_out=np.empty((3, 3)))
    with pytest.raises(_lib.MappgError):
        s.nvt_run_host(c.x, c.v, -1.0, synth.FS, synth.KB, 1)
    # the system stays usable after the refused run
    th, _ = s.nvt_run_host(c.x, c.v, 600.0, synth.FS, synth.KB, 2, thermo=True)
    assert np.all(np.isfinite(th))


def test_mixed_md_in_a_triclinic_box(setfl):
    """Mixed-precision NVT in a sheared (triclinic) box: the non-orthogonal
    frame of the integrator and of the list builder, over enough steps for
    list rebuilds, against the FP64 run of the same cell."""
    strain = [[0.0, 0.0, 0.0], [0.06, 0.0, 0.0], [-0.04, 0.05, 0.0]]
    c = synth.alloy((6, 6, 6), xB=0.4, sigma=0.05, T=1200.0, seed=12, strain=strain)
    assert c.H[1, 0] != 0.0 and c.H[2, 1] != 0.0
    ff = _lib.ForceField.setfl(setfl, ["A", "B"])
    out = {}
    for prec in (_lib.FP64, _lib.MIXED):
        s = _lib.System(ff, c.H, c.x, c.elem, c.masses, precision=prec)
        s.set_v(c.v)
        th, _ = s.nvt_run(1200.0, synth.FS, synth.KB, 300, thermo=True)
        out[prec] = (th, s.get_x(), s.get_v(), s.stats()["rebuilds"])
    th64, x64, v64, nreb64 = out[_lib.FP64]
    th32, x32, v32, nreb32 = out[_lib.MIXED]
    assert nreb64 >= 2 and nreb32 >= 2  # the run crossed list rebuilds
    d = x32 - x64
    d -= np.round(d @ np.linalg.inv(c.H)) @ c.H
    assert np.max(np.abs(d)) < 1e-4 and np.max(np.abs(v32 - v64)) < 1e-4
    assert np.max(np.abs(th32[:, 0] - th64[:, 0])) / c.natoms < 1e-6
    assert np.max(np.abs(th32[:, 1] - th64[:, 1])) < 1e-3 * np.max(th64[:, 1])
