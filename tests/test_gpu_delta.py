"""Line-search energy differences of mixed-precision systems
(mappg_sys_energy_delta, the pass behind the mixed minimizers' trials)
against differences of FP64 energies, over steps from 1e-6 A to 0.05 A.

The bar is 2e-5 of the difference itself plus 1e-9 eV per atom: the mixed
model's own force error (~2e-6 eV/A RMS) already moves E(x + alpha h) -
E(x) by ~1e-6 of its size.  The plain difference of two FP32 energies is
shown to miss that bar at the small steps (its rounding, ~1e-4 eV here, is
larger than the differences), which is why the pass exists."""
import numpy as np
import pytest

from mapp4py_gb300 import _lib, synth

pytestmark = pytest.mark.gpu


def test_energy_delta_matches_fp64_differences(potentials):
    path, _ = potentials[("A", "B")]
    c = synth.alloy((20, 20, 20), xB=0.5, sigma=0.05, seed=5)
    ff = _lib.ForceField.setfl(path)
    s64 = _lib.System(ff, c.H, c.x, c.elem, c.masses)
    e0 = s64.energy()
    s64.force()
    f = s64.get_f()
    m = _lib.System(ff, c.H, c.x, c.elem, c.masses, precision=_lib.MIXED)
    m32 = _lib.System(ff, c.H, c.x, c.elem, c.masses, precision=_lib.MIXED)
    e0_32 = m32.energy()
    rng = np.random.default_rng(9)
    dirs = {"force": f / np.max(np.abs(f)), "random": rng.normal(size=c.x.shape)}
    worst_plain = 0.0
    for name, h in dirs.items():
        h = h / np.max(np.abs(h))
        for step in (1e-6, 1e-5, 1e-4, 1e-3, 1e-2, 5e-2):
            xa = c.x + step * h
            s64.set_x(xa)
            ref = s64.energy() - e0
            de = m.energy_delta(h, step)
            tol = 2e-5 * abs(ref) + 1e-9 * c.natoms
            assert abs(de - ref) <= tol, (name, step, de, ref)
            m32.set_x(xa)
            worst_plain = max(worst_plain, abs((m32.energy() - e0_32) - ref) / tol)
            m32.set_x(c.x)
    assert worst_plain > 1.0  # the plain FP32 difference would not meet the bar


def test_energy_delta_refuses_steps_beyond_the_skin(potentials):
    path, _ = potentials[("A", "B")]
    c = synth.alloy((6, 6, 6), xB=0.5, sigma=0.05, seed=6)
    m = _lib.System(_lib.ForceField.setfl(path), c.H, c.x, c.elem, c.masses, precision=_lib.MIXED)
    h = np.random.default_rng(7).uniform(-1.0, 1.0, c.x.shape)
    assert abs(m.energy_delta(h, 1e-3)) > 0.0
    # a rigid translation changes nothing
    assert abs(m.energy_delta(np.ones_like(c.x), 1e-3)) < 1e-9 * c.natoms
    with pytest.raises(_lib.MappgError, match="skin"):
        m.energy_delta(h, 0.2)
    f64 = _lib.System(_lib.ForceField.setfl(path), c.H, c.x, c.elem, c.masses)
    with pytest.raises(_lib.MappgError, match="mixed"):
        f64.energy_delta(h, 1e-3)
