"""GPU parity: libmappg through its C ABI against the CPU oracle and the
golden fixtures.  Tolerances: FP64 forces 1e-10 relative to the largest force
component, energies 1e-12 relative, neighbour sets bit-exact; mixed precision
force RMS <= 1e-5 eV/A and energy <= 1e-7 eV/atom against the FP64 GPU path.
"""
import numpy as np
import pytest

import oracle as O
from conftest import golden, golden_potential
from mapp4py_gb300 import _lib, synth

pytestmark = pytest.mark.gpu

STATIC = ["fcc_a_256", "alloy_ab_475", "thin_a_32", "tric_ab_240"]


def keys(cnt, ent):
    atom = np.repeat(np.arange(cnt.shape[0]), cnt)
    rows = np.column_stack([atom, ent]).astype(np.int64)
    return rows[np.lexsort(rows.T[::-1])]


def make(path, c, precision=_lib.FP64, skin=0.5):
    ff = _lib.ForceField.setfl(path)
    return _lib.System(ff, c["H"], c["x"], c["elem"], c["masses"], skin=skin, precision=precision)


def assert_forces(fg, fr, rel=1e-10):
    scale = max(1.0, np.max(np.abs(fr)))
    err = np.max(np.abs(fg - fr))
    assert err <= rel * scale, "max force error %.3e > %.1e x %.3e" % (err, rel, scale)


@pytest.mark.parametrize("name", STATIC)
def test_fp64_force_energy_virial_match_golden(potentials, name):
    g = golden(name)
    s = make(golden_potential(potentials, g), g)
    pe, vir = s.force()
    assert abs(pe - g["pe"]) <= 1e-12 * abs(g["pe"])
    assert np.max(np.abs(vir - g["virial"])) <= 1e-11 * np.max(np.abs(g["virial"]))
    assert_forces(s.get_f(), g["f"])
    rho, dF = s.rho_dF()
    assert np.max(np.abs(rho - g["rho"])) <= 1e-12 * np.max(g["rho"])
    assert np.max(np.abs(dF - g["dF"])) <= 1e-12 * np.max(np.abs(g["dF"]))
    assert abs(s.energy() - g["energy"]) <= 1e-12 * abs(g["energy"])
    # wrapped positions after the build are the reference's x = S2X(wrap(X2S(x)))
    assert np.array_equal(s.get_x(), g["x_wrapped"])


@pytest.mark.parametrize("name", STATIC)
@pytest.mark.parametrize("precision", [_lib.FP64, _lib.MIXED])
def test_neighbor_sets_bit_exact(potentials, name, precision):
    g = golden(name)
    s = make(golden_potential(potentials, g), g, precision)
    s.build()
    got = keys(*s.neighbors())
    assert got.shape == g["nbr"].shape
    assert np.array_equal(got, g["nbr"])


def test_fp64_c1_cell_against_live_oracle(potentials):
    """4,000-atom FCC 10x10x10 cell with thermal-size noise, live oracle."""
    path, _ = potentials[("A",)]
    c = synth.alloy((10, 10, 10), xB=0.0, sigma=0.07, seed=5)
    c.elem[:] = 0
    e = O.Eam.setfl(path)
    o = O.System(e, c.H, c.x, c.elem, [synth.MASS], skin=0.5)
    pe_o, vir_o = o.force()
    ff = _lib.ForceField.setfl(path)
    s = _lib.System(ff, c.H, c.x, c.elem, [synth.MASS], skin=0.5)
    pe, vir = s.force()
    assert abs(pe - pe_o) <= 1e-12 * abs(pe_o)
    assert np.max(np.abs(vir - vir_o)) <= 1e-11 * np.max(np.abs(vir_o))
    assert_forces(s.get_f(), o.f)


def test_newton_third_law_translation_and_determinism(potentials):
    g = golden("alloy_ab_475")
    path = golden_potential(potentials, g)
    s = make(path, g)
    s.force()
    f1 = s.get_f()
    assert np.max(np.abs(f1.sum(axis=0))) < 1e-10
    s.force()
    assert np.array_equal(f1, s.get_f()), "repeated force calls must be bit-identical"
    g2 = dict(g)
    g2["x"] = g["x"] + np.array([0.31, -0.77, 1.9])
    t = make(path, g2)
    t.force()
    assert np.max(np.abs(t.get_f() - f1)) < 1e-9


def test_mixed_precision_error_budget(potentials):
    """FP32 pair math with FP64 totals against the FP64 GPU path on a
    32,000-atom random A/B alloy with 0.05 A noise (the 2.048M-atom cell's
    composition and disorder at a smaller size)."""
    path, _ = potentials[("A", "B")]
    c = synth.alloy((20, 20, 20), xB=0.5, sigma=0.05, seed=1)
    ff = _lib.ForceField.setfl(path)
    s64 = _lib.System(ff, c.H, c.x, c.elem, c.masses)
    s32 = _lib.System(ff, c.H, c.x, c.elem, c.masses, precision=_lib.MIXED)
    pe64, vir64 = s64.force()
    pe32, vir32 = s32.force()
    f64, f32 = s64.get_f(), s32.get_f()
    rms = np.sqrt(np.mean(np.sum((f64 - f32) ** 2, axis=1)))
    assert rms <= 1e-5, "force RMS error %.3e" % rms
    assert abs(pe32 - pe64) / c.natoms <= 1e-7
    assert np.max(np.abs(vir32 - vir64)) <= 1e-6 * np.max(np.abs(vir64))
    assert abs(s32.energy() - pe64) / c.natoms <= 1e-7


def test_mixed_precision_error_budget_full_workload_cell(potentials):
    """The bar on the MD workload cell itself: 2,048,000-atom 50/50 A/B alloy
    (FCC 80^3, a = 3.615 A, seed 1, 0.05 A noise), mixed precision against
    the FP64 GPU path on the same configuration."""
    path, _ = potentials[("A", "B")]
    c = synth.alloy((80, 80, 80), xB=0.5, sigma=0.05, seed=1)
    ff = _lib.ForceField.setfl(path)
    s64 = _lib.System(ff, c.H, c.x, c.elem, c.masses)
    pe64, vir64 = s64.force()
    f64 = s64.get_f()
    del s64
    s32 = _lib.System(ff, c.H, c.x, c.elem, c.masses, precision=_lib.MIXED)
    pe32, vir32 = s32.force()
    f32 = s32.get_f()
    rms = np.sqrt(np.mean(np.sum((f64 - f32) ** 2, axis=1)))
    assert rms <= 1e-5, "force RMS error %.3e" % rms
    assert abs(pe32 - pe64) / c.natoms <= 1e-7, (pe32 - pe64) / c.natoms
    assert np.max(np.abs(vir32 - vir64)) <= 1e-6 * np.max(np.abs(vir64))


def test_nvt_trajectory_matches_golden(potentials):
    g = golden("nvt_a_256")
    path, digest = potentials[("A",)]
    assert str(g["sha256"]) == digest
    s = make(path, g)
    s.set_v(g["v"])
    th, eta = s.nvt_run(float(g["T"]), float(g["dt"]), float(g["kB"]), int(g["nsteps"]), thermo=True)
    ref = g["thermo"]
    assert np.max(np.abs(th[:, 0] - ref[:, 0])) <= 1e-10 * np.max(np.abs(ref[:, 0]))
    assert np.max(np.abs(th[:, 1] - ref[:, 1])) <= 1e-9 * np.max(np.abs(ref[:, 1]))
    assert np.max(np.abs(s.get_x() - g["x_end"])) <= 1e-9
    assert np.max(np.abs(s.get_v() - g["v_end"])) <= 1e-9
    assert np.max(np.abs(eta - g["eta"])) <= 1e-9 * max(1.0, np.max(np.abs(g["eta"])))


def test_nve_c1_against_live_oracle(potentials):
    """4,000 atoms, 300 K, NVE (t_relax = inf), dt = 1 fs, 100 steps."""
    path, _ = potentials[("A",)]
    c = synth.md_single((10, 10, 10), T=300.0, seed=0)
    e = O.Eam.setfl(path)
    o = O.System(e, c.H, c.x, c.elem, c.masses, skin=0.5)
    o.v = c.v
    th_o, _, nreb_o = o.nvt_run(300.0, synth.FS, synth.KB, 100, t_relax=float("inf"))
    ff = _lib.ForceField.setfl(path)
    s = _lib.System(ff, c.H, c.x, c.elem, c.masses)
    s.set_v(c.v)
    th, _ = s.nvt_run(300.0, synth.FS, synth.KB, 100, t_relax=float("inf"), thermo=True)
    assert np.max(np.abs(th[:, 0] - th_o[:, 0])) <= 1e-10 * np.max(np.abs(th_o[:, 0]))
    assert np.max(np.abs(s.get_x() - o.x)) <= 1e-8
    assert s.stats()["rebuilds"] == nreb_o
    # NVE: total energy drift over 100 fs stays small
    etot = th[:, 0] + 0.5 * (th[:, 2] + th[:, 5] + th[:, 7])
    assert np.max(np.abs(etot - etot[0])) / c.natoms < 2e-5


def test_lbfgs_follows_oracle_on_a_rough_landscape(potentials):
    """A 5 %-vacancy alloy with 0.15 A noise: its relaxation is chaotic, so
    the oracle itself, started 1e-11 A away, ends in different minima (pe
    -4808 ... -4819 eV) and sometimes in a failed line search.  The GPU run
    must follow the oracle to rounding over the first iterations, then descend
    as far as the oracle's runs do and stop for one of the same reasons."""
    g = golden("lbfgs_ab_475")
    path = golden_potential(potentials, dict(g, elems=np.array(["A", "B"])))
    s = make(path, g)
    r5 = s.lbfgs_run(m=10, e_tol=0.0, f_tol=1e-4, nsteps=5)
    o = O.System(O.Eam.setfl(path), g["H"], g["x"], g["elem"], g["masses"], skin=0.5)
    ro5 = o.lbfgs_run(m=10, e_tol=0.0, f_tol=1e-4, nsteps=5)
    assert r5["niter"] == ro5["niter"] and r5["n_energy"] == ro5["n_energy"]
    assert abs(r5["pe"] - ro5["pe"]) <= 1e-11 * abs(ro5["pe"])
    s = make(path, g)
    r = s.lbfgs_run(m=10, e_tol=0.0, f_tol=1e-4, nsteps=5000)
    assert r["err"] in (100, 3)  # f_tol reached, or the line search ran out of step
    assert r["fmax"] < 1e-3 and r["pe"] < -4805.0


def test_lbfgs_converges_like_oracle(potentials):
    """A well-conditioned relaxation (1 % vacancies, 0.1 A noise) whose
    minimum does not move under 1e-11 A perturbations: same iteration count,
    energy and relaxed positions as the oracle."""
    path, _ = potentials[("A", "B")]
    c = synth.alloy((4, 4, 4), xB=0.3, sigma=0.1, seed=2, vac=0.01)
    o = O.System(O.Eam.setfl(path), c.H, c.x, c.elem, c.masses, skin=0.5)
    ro = o.lbfgs_run(m=10, e_tol=0.0, f_tol=1e-4, nsteps=5000)
    assert ro["err"] == 100
    s = make(path, dict(H=c.H, x=c.x, elem=c.elem, masses=c.masses))
    r = s.lbfgs_run(m=10, e_tol=0.0, f_tol=1e-4, nsteps=5000)
    assert r["err"] == 100 and r["fmax"] < 1e-4
    assert r["niter"] == ro["niter"] and r["n_energy"] == ro["n_energy"]
    assert abs(r["pe"] - ro["pe"]) <= 1e-11 * abs(ro["pe"])
    d = s.get_x() - o.x
    d -= np.round(d @ np.linalg.inv(c.H)) @ c.H
    assert np.max(np.abs(d)) < 1e-8


def test_per_pair_density_tables():
    """Finnis-Sinclair-style tables, where the density of j at i depends on
    both elements (rho_arr[e_j][e_i] differs across e_i, as ff_eam_fs
    reads): FP64 forces, energy and virial match the oracle built from the
    same knots, and the mixed path stays inside its error budget."""
    dr, drho, F, rho1, rphi = synth.analytic_knots(("A", "B"))
    nr = rho1.shape[1]
    rho = np.zeros((2, 2, nr))
    scale = np.array([[1.0, 0.8], [1.3, 1.1]])  # rho[i][j]: density of an i atom seen by a j atom
    for i in range(2):
        for j in range(2):
            rho[i, j] = scale[i, j] * rho1[i]
    nrho = F.shape[1]
    ff = _lib.ForceField.knots(nr, nrho, dr, drho, F, rho, rphi)
    e = O.Eam.knots(nr, nrho, dr, drho, F, rho, rphi)
    c = synth.alloy((5, 5, 5), xB=0.4, sigma=0.08, seed=21, vac=0.02)
    o = O.System(e, c.H, c.x, c.elem, c.masses)
    pe_o, vir_o = o.force()
    s = _lib.System(ff, c.H, c.x, c.elem, c.masses)
    pe, vir = s.force()
    assert abs(pe - pe_o) <= 1e-12 * abs(pe_o)
    assert np.max(np.abs(vir - vir_o)) <= 1e-11 * np.max(np.abs(vir_o))
    assert_forces(s.get_f(), o.f)
    m = _lib.System(ff, c.H, c.x, c.elem, c.masses, precision=_lib.MIXED)
    pe_m, _ = m.force()
    rms = np.sqrt(np.mean(np.sum((m.get_f() - o.f) ** 2, axis=1)))
    assert rms < 1e-5 and abs(pe_m - pe_o) / c.natoms < 1e-7


def test_cg_converges_like_oracle(potentials):
    """MinCG: the first iterations follow the oracle to rounding; the full
    run reaches the same minimum with the same iteration count."""
    path, _ = potentials[("A", "B")]
    c = synth.alloy((4, 4, 4), xB=0.3, sigma=0.1, seed=2, vac=0.01)
    o = O.System(O.Eam.setfl(path), c.H, c.x, c.elem, c.masses, skin=0.5)
    ro = o.cg_run(e_tol=0.0, f_tol=1e-4, nsteps=5000)
    assert ro["err"] == 100
    g = dict(H=c.H, x=c.x, elem=c.elem, masses=c.masses)
    s = make(path, g)
    r = s.cg_run(e_tol=0.0, f_tol=1e-4, nsteps=5000)
    assert r["err"] == 100 and r["fmax"] < 1e-4
    assert r["niter"] == ro["niter"] and r["n_energy"] == ro["n_energy"]
    assert abs(r["pe"] - ro["pe"]) <= 1e-11 * abs(ro["pe"])
    d = s.get_x() - o.x
    d -= np.round(d @ np.linalg.inv(c.H)) @ c.H
    assert np.max(np.abs(d)) < 1e-8


def test_errors_are_reported(potentials):
    path, _ = potentials[("A",)]
    ff = _lib.ForceField.setfl(path)
    H, x = synth.fcc((1, 4, 4))  # 3.6 A thick: thinner than cutoff + skin
    with pytest.raises(_lib.MappgError) as ei:
        _lib.System(ff, H, x, np.zeros(len(x), np.uint8), [synth.MASS])
    assert ei.value.code == -4
    H, x = synth.fcc((4, 4, 4))
    x[3, 1] = np.nan
    with pytest.raises(_lib.MappgError):
        _lib.System(ff, H, x, np.zeros(len(x), np.uint8), [synth.MASS])
    H, x = synth.fcc((4, 4, 4))
    s = _lib.System(ff, H, x, np.zeros(len(x), np.uint8), [synth.MASS])
    with pytest.raises(_lib.MappgError):
        s.nvt_run(300.0, synth.FS, float("nan"), 1)


def test_neighbor_capacity_grows(potentials):
    """A compressed cell overflows the density-based row estimate; the build
    grows the rows and the list still matches the oracle."""
    path, _ = potentials[("A",)]
    _, x = synth.fcc((4, 4, 4), a=3.0)  # a dense slab in a box 4x longer
    H = np.diag([48.0, 12.0, 12.0])
    elem = np.zeros(len(x), np.uint8)
    ff = _lib.ForceField.setfl(path)
    s = _lib.System(ff, H, x, elem, [synth.MASS], skin=0.5)
    cap0 = s.stats()["capacity"]
    s.build()
    assert s.stats()["capacity"] > cap0
    o = O.System(O.Eam.setfl(path), H, x, elem, [synth.MASS], skin=0.5, pair_wise=False)
    o.init_dynamic()
    assert np.array_equal(keys(*s.neighbors()), keys(*o.neighbors()))


@pytest.mark.parametrize("precision", [_lib.FP64, _lib.MIXED])
def test_autotune_keeps_the_forces(potentials, precision):
    """mappg_sys_autotune only picks lanes per atom and entries per step:
    the forces after it agree with those before it (FP64 to rounding, mixed
    within its summation-order budget)."""
    path, _ = potentials[("A", "B")]
    c = synth.alloy((5, 5, 5), xB=0.4, sigma=0.08, seed=4)
    s = _lib.System(_lib.ForceField.setfl(path), c.H, c.x, c.elem, c.masses, precision=precision)
    pe0, _ = s.force()
    f0 = s.get_f()
    tpa, unroll, ms = s.autotune()
    assert tpa in (4, 8, 16, 32) and unroll in (1, 2)
    assert (32, 1) in ms and all(v > 0 for v in ms.values())
    if precision == _lib.FP64:
        assert set(ms) == {(4, 1), (8, 1), (16, 1), (32, 1)}
    pe1, _ = s.force()
    f1 = s.get_f()
    tol = 1e-10 if precision == _lib.FP64 else 1e-5
    assert np.max(np.abs(f1 - f0)) <= tol * max(1.0, np.max(np.abs(f0)))
    assert abs(pe1 - pe0) <= (1e-12 if precision == _lib.FP64 else 1e-7) * abs(pe0)


@pytest.mark.parametrize("precision", [_lib.FP64, _lib.MIXED])
def test_set_box_then_forces_match_oracle(potentials, precision):
    """mappg_sys_set_box: the same system carried through three boxes (a
    small strain, a tilt, and a 25 % expansion that changes the number of
    bins), with the atoms mapped affinely each time.  Forces, energy and
    virial match the oracle built in that box (FP64 to the parity bars,
    mixed within its error budget).  A batch's boxes are fixed."""
    path, _ = potentials[("A", "B")]
    c = synth.alloy((6, 6, 6), xB=0.4, sigma=0.05, seed=9)
    s = make(path, dict(H=c.H, x=c.x, elem=c.elem, masses=c.masses), precision=precision)
    s.force()  # a list in the first box
    tilt = c.H.copy()
    tilt[1, 0] += 0.3 * c.H[1, 1]
    tilt[2, 1] -= 0.2 * c.H[2, 2]
    for H1 in (c.H @ np.diag([1.02, 0.99, 1.0]), tilt, 1.25 * c.H):
        x1 = c.x @ np.linalg.inv(c.H) @ H1
        s.set_box(H1)
        s.set_x(x1)
        pe, vir = s.force()
        o = O.System(O.Eam.setfl(path), H1, x1, c.elem, c.masses, skin=0.5)
        pe_o, vir_o = o.force()
        f = s.get_f()
        if precision == _lib.FP64:
            assert abs(pe - pe_o) <= 1e-12 * abs(pe_o)
            assert np.max(np.abs(vir - vir_o)) <= 1e-11 * np.max(np.abs(vir_o))
            assert_forces(f, o.f)
        else:
            assert np.sqrt(np.mean(np.sum((f - o.f) ** 2, axis=1))) <= 1e-5
            assert abs(pe - pe_o) / c.natoms <= 1e-7
    b = _lib.Batch(_lib.ForceField.setfl(path), [(c.H, c.x, c.elem)] * 2, c.masses)
    assert _lib.load().mappg_sys_set_box(b.h, _lib.dptr(np.ascontiguousarray(c.H))) == -8  # MAPPG_ERR_UNSUPP
