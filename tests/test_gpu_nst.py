"""Constant-stress MD (md.nst; MDNST::run, md_nst.cpp) on the device against
the oracle's restatement: energies, temperatures, boxes, positions and
velocities over the first steps, for a diagonal and a sheared stress
target; the md-level run updates atoms.H and carries the box velocity."""
import numpy as np
import pytest

import oracle as O
from mapp4py_gb300 import _lib, md, synth

pytestmark = pytest.mark.gpu

nan = np.nan


def cell():
    return synth.alloy((5, 5, 5), a=2.9, xB=0.3, sigma=0.02, T=300.0, seed=4)


@pytest.mark.parametrize("shear", [False, True])
def test_nst_follows_oracle(potentials, shear):
    path, _ = potentials[("A", "B")]
    c = cell()
    S = np.array([[0.0, nan, nan], [nan, 0.0, nan], [nan, nan, 0.0]])
    if shear:
        S[1, 0] = S[0, 1] = 0.0
        S[2, 1] = S[1, 2] = 0.0
    tau = np.full((3, 3), 50 * synth.FS)
    o = O.System(O.Eam.setfl(path), c.H, c.x, c.elem, c.masses, skin=0.5)
    o.v = c.v
    tho, VHo, eo, eSo = o.nst_run(S, 300.0, synth.FS, synth.KB, 30, tau=tau)
    s = _lib.System(_lib.ForceField.setfl(path), c.H, c.x, c.elem, c.masses, skin=0.5, precision=_lib.FP64)
    s.set_v(c.v)
    th, VH, e, eS = s.nst_run(S, 300.0, synth.FS, synth.KB, 30, tau=tau)
    # pe and T per step, boxes
    assert np.max(np.abs(th[:, 0] - tho[:, 0])) <= 1e-9 * np.max(np.abs(tho[:, 0]))
    assert np.max(np.abs(th[:, 1] - tho[:, 1])) <= 1e-8 * np.max(tho[:, 1])
    assert np.max(np.abs(th[:, 14:] - tho[:, 14:])) < 1e-10
    assert np.max(np.abs(VH - VHo)) <= 1e-9 * max(1e-30, np.max(np.abs(VHo)))
    H = s.get_box()
    d = s.get_x() - o.x
    d -= np.round(d @ np.linalg.inv(H)) @ H
    assert np.max(np.abs(d)) < 1e-9
    assert np.max(np.abs(s.get_v() - o.v)) < 1e-10
    assert np.max(np.abs(e - eo)) < 1e-9 and np.max(np.abs(eS - eSo)) < 1e-9


def test_md_nst_updates_the_box(potentials):
    path, _ = potentials[("A", "B")]
    c = cell()
    a = md.atoms(c.H, c.x, c.elem, elems=("A", "B"), masses=c.masses, x_d=c.v)
    a.ff_eam_setfl(path)
    a.kB = synth.KB
    integ = md.nst([[0.0], [None, 0.0], [None, None, 0.0]], 300.0, synth.FS)
    integ.tau = np.full((3, 3), 50 * synth.FS)
    integ.ntally = 0
    integ.run(a, 100)
    assert np.max(np.abs(np.diag(a.H) - np.diag(c.H))) > 0.1 and a.step == 100
    vh = integ._V_H.copy()
    integ.run(a, 10)  # the box velocity carries over
    assert np.any(vh != 0.0)
    # a mixed-precision system runs md.nst with the FP32 force passes
    a.precision = "mixed"
    H0 = a.H.copy()
    integ.run(a, 20)
    assert a.step == 130 and np.all(np.isfinite(a.x)) and np.max(np.abs(a.H - H0)) > 0.0


def test_mixed_nst_follows_fp64(potentials):
    """md.nst on a mixed-precision system: FP32 force passes under the same
    FP64 box algebra and chains; the run stays within the mixed-precision
    budget of the FP64 one over 60 steps."""
    path, _ = potentials[("A", "B")]
    c = cell()
    S = np.array([[0.0, nan, nan], [nan, 0.0, nan], [nan, nan, 0.0]])
    tau = np.full((3, 3), 50 * synth.FS)
    out = {}
    for prec in (_lib.FP64, _lib.MIXED):
        s = _lib.System(_lib.ForceField.setfl(path), c.H, c.x, c.elem, c.masses, skin=0.5, precision=prec)
        s.set_v(c.v)
        th, VH, e, eS = s.nst_run(S, 300.0, synth.FS, synth.KB, 60, tau=tau)
        out[prec] = (th, VH, s.get_box(), s.get_x(), s.get_v())
    th64, VH64, H64, x64, v64 = out[_lib.FP64]
    th32, VH32, H32, x32, v32 = out[_lib.MIXED]
    assert np.max(np.abs(th32[:, 0] - th64[:, 0])) / c.natoms < 1e-6
    assert np.max(np.abs(th32[:, 1] - th64[:, 1])) < 1e-4 * np.max(th64[:, 1])
    # the barostat integrates the virial, whose FP32 pair terms differ from
    # FP64 by ~1e-7 relative: the boxes agree to ~1e-6 of their size
    assert np.max(np.abs(H32 - H64)) < 2e-6 * np.max(np.abs(H64))
    assert np.max(np.abs(VH32 - VH64)) <= 1e-2 * np.max(np.abs(VH64))
    d = x32 - x64
    d -= np.round(d @ np.linalg.inv(H64)) @ H64
    assert np.max(np.abs(d)) < 5e-5 and np.max(np.abs(v32 - v64)) < 5e-5
    # the box moved: the test compares a live relaxation, not a fixed box
    assert np.max(np.abs(H64 - c.H)) > 1e-3


def test_md_nst_exports(potentials, tmp_path):
    """md.nst with an export: files at the start, every nevery steps and at
    the last step, each with that step's box; the run is unchanged by them."""
    import os

    path, _ = potentials[("A", "B")]
    c = cell()

    def atoms():
        a = md.atoms(c.H, c.x, c.elem, elems=("A", "B"), masses=c.masses, x_d=c.v)
        a.ff_eam_setfl(path)
        a.kB = synth.KB
        return a

    def integ():
        i = md.nst([[0.0], [None, 0.0], [None, None, 0.0]], 300.0, synth.FS)
        i.tau = np.full((3, 3), 50 * synth.FS)
        i.ntally = 0
        return i

    a, b = atoms(), atoms()
    ia = integ()
    pattern = str(tmp_path / "nst")
    ia.export = md.export_cfg(pattern, nevery=10, extra_vecs=["x_d", "f"])
    ia.run(a, 25)
    integ().run(b, 25)
    assert np.array_equal(a.x, b.x) and np.array_equal(a.H, b.H)
    got = sorted(int(f.split(".")[-2]) for f in os.listdir(tmp_path) if f.startswith("nst."))
    assert got == [0, 10, 20, 25]
    last = md.atoms.import_cfg(pattern + ".%09d.cfg" % 25)
    assert np.max(np.abs(last.H - a.H)) < 1e-9
    d = last.x - a.x
    d -= np.round(d @ np.linalg.inv(a.H)) @ a.H
    assert np.max(np.abs(d)) < 1e-9
    mid = md.atoms.import_cfg(pattern + ".%09d.cfg" % 10)
    assert np.max(np.abs(mid.H - c.H)) > 0.0 and np.max(np.abs(mid.H - a.H)) > 0.0

    class Failing(md.export_cfg):
        def _write_step(self, atoms, step, x, x_d, f, H=None):
            if step == 10:
                raise RuntimeError("disk full")
            super()._write_step(atoms, step, x, x_d, f, H)

    ia.export = Failing(str(tmp_path / "fail"), nevery=5)
    with pytest.raises(RuntimeError, match="disk full"):
        ia.run(atoms(), 20)
