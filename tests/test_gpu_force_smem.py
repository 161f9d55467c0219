"""The mixed force pass with its records in shared memory (k_force32s,
mappg_sys_force_tables with a budget in KB) against the pass that reads them
through L1 (mode 0): the same records, the same arithmetic and the same lane order, so
forces agree bit for bit; energies and virials are sums over other orders
of atoms (one element group after the other) and agree to rounding.

Cases: the analytic A/B alloy (every pair's knots in shared memory), one
element, and the potential files shipped with the reference (Cu_mishin, whose
table reaches beyond its cutoff; NiAl and FeH-sina, whose 10,000-knot tables
leave the short pairs to the global-memory records; Fe-H.eam.fs with its
per-pair densities and five records per knot)."""
import numpy as np
import pytest

import potfile
from conftest import golden
from mapp4py_gb300 import _lib, synth

pytestmark = pytest.mark.gpu


MODES = (0, 1, 64, 1 << 20)  # L1; 1 KB (nearly every pair from global memory); 64 KB; the largest budget


def both_modes(ff, H, x, elem, masses):
    out = []
    for mode in MODES:
        s = _lib.System(ff, H, x, elem, masses, precision=_lib.MIXED)
        got = s.force_tables(mode)
        assert got == mode if mode < (1 << 20) else 64 < got < mode
        pe, vir = s.force()
        out.append((pe, vir, s.get_f()))
    return out


def check(out, natoms):
    pe0, vir0, f0 = out[0]
    for pe1, vir1, f1 in out[1:]:
        assert np.array_equal(f0, f1)
        # compensated FP32 sums per thread over other atoms: equal to ~1e-11
        # eV/atom, far inside the mixed path's 1e-7 eV/atom budget
        assert abs(pe1 - pe0) <= 1e-9 * natoms
        assert np.max(np.abs(vir1 - vir0)) <= 1e-6 * np.max(np.abs(vir0))


@pytest.mark.parametrize("elems", [("A",), ("A", "B")])
def test_shared_records_match_global_records(potentials, elems):
    path, _ = potentials[elems]
    ff = _lib.ForceField.setfl(path)
    c = synth.alloy((12, 12, 12), xB=0.5 if len(elems) == 2 else 0.0, sigma=0.1, seed=11)
    elem = c.elem if len(elems) == 2 else np.zeros_like(c.elem)
    check(both_modes(ff, c.H, c.x, elem, c.masses[:len(elems)]), c.natoms)


@pytest.mark.parametrize("pot", ["cu", "nial", "feh", "feh_fs"])
def test_shared_records_on_reference_potentials(tmp_path, pot):
    g = golden("ref_pot_" + pot)
    d = potfile.from_fixture(g)
    path = potfile.write(str(tmp_path / (pot + ".pot")), d)
    ff = _lib.ForceField.setfl(path) if d["kind"] == "setfl" else _lib.ForceField.fs(path)
    for cell in [str(c) for c in g["cells"]]:
        H, x, elem = g[cell + "/H"], g[cell + "/x"], g[cell + "/elem"]
        out = both_modes(ff, H, x, elem, d["masses"])
        check(out, x.shape[0])
        # and still the reference's forces within the mixed-precision budget
        rms = np.sqrt(np.mean(np.sum((out[-1][2] - g[cell + "/f"]) ** 2, axis=1)))
        frms = np.sqrt(np.mean(np.sum(g[cell + "/f"] ** 2, axis=1)))
        assert rms <= max(1e-5, 3e-6 * frms), (cell, rms)


def test_shared_records_md_trajectory_is_the_same(potentials):
    """20 NVT steps: forces equal bit for bit, so positions and velocities
    are too."""
    path, _ = potentials[("A", "B")]
    ff = _lib.ForceField.setfl(path)
    c = synth.alloy((10, 10, 10), xB=0.5, sigma=0.05, T=600.0, seed=12)
    res = []
    for mode in (0, 1 << 20):
        s = _lib.System(ff, c.H, c.x, c.elem, c.masses, precision=_lib.MIXED)
        s.force_tables(mode)
        s.set_v(c.v)
        s.nvt_run(600.0, synth.FS, synth.KB, 20)
        res.append((s.get_x(), s.get_v()))
    assert np.array_equal(res[0][0], res[1][0]) and np.array_equal(res[0][1], res[1][1])


def test_shared_records_refused_where_unsupported(potentials):
    path, _ = potentials[("A", "B")]
    ff = _lib.ForceField.setfl(path)
    c = synth.alloy((4, 4, 4), xB=0.5, sigma=0.05, seed=13)
    s = _lib.System(ff, c.H, c.x, c.elem, c.masses)
    with pytest.raises(_lib.MappgError, match="single mixed-precision cell"):
        s.force_tables(1)
    assert s.force_tables() == 0
    b = _lib.Batch(ff, [(c.H, c.x, c.elem), (c.H, c.x, c.elem)], c.masses)
    with pytest.raises(_lib.MappgError, match="single mixed-precision cell"):
        b.force_tables(1)
