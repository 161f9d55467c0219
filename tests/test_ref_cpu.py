"""The CPU oracle pinned to MAPP itself.

The fixtures tests/golden/ref_*.npz hold results of the reference compiled
from its own sources (oracle/ref.mk) and driven through its Python API
(tests/golden/make_ref_golden.py): forces, energy and stress through
ForceFieldMD::force_calc on the analytic potential and on the four
potential files shipped with the reference's examples (setfl with one and
two elements, per-pair cutoffs, Finnis-Sinclair), host densities beyond
rho_max, md.nvt trajectories, md.nst states, md.min_lbfgs and md.min_cg_new
iterates (with the back-tracking, golden-section and Brent line searches, and
with box degrees of freedom), runs with frozen components (atoms.x_dof) and
create_temp draws.
The oracle must reproduce them to rounding.  Where the compiled reference
module is present (oracle/_ref), further seeded cases run live against it.
"""
import os

import numpy as np
import pytest

import oracle as O
import potfile
import refmod
from conftest import golden
from mapp4py_gb300 import _lib, synth

STATIC = ["fcc_a_256", "alloy_ab_475", "thin_a_32", "tric_ab_240"]
POTS = ["cu", "nial", "feh", "feh_fs"]


@pytest.fixture(scope="module")
def built():
    """libmappg.so, built here if it is not yet (its host code only is used)."""
    from mapp4py_gb300 import build

    build.build()
    return _lib.load()


def voigt_to_stress(vir, H):
    """F_H (Voigt xx, xy, xz, yy, yz, zz) -> S_pe = -F_H / V (ff_md.cpp:129-134)."""
    F = np.array([[vir[0], vir[1], vir[2]], [vir[1], vir[3], vir[4]], [vir[2], vir[4], vir[5]]])
    return -F / np.linalg.det(H)


def rel(a, b):
    return np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300)


def oracle_eam(d, path):
    """Tables of a fixture potential: setfl through the oracle's file reader,
    Finnis-Sinclair from its knots (per-pair densities rho[i][j])."""
    if d["kind"] == "setfl":
        return O.Eam.setfl(path)
    ne = len(d["names"])
    rphi = np.zeros((ne, ne, int(d["nr"])))
    k = 0
    for i in range(ne):
        for j in range(i + 1):
            rphi[i, j] = d["rphi"][k]
            k += 1
    return O.Eam.knots(int(d["nr"]), int(d["nrho"]), float(d["dr"]), float(d["drho"]), d["F"],
                       np.ascontiguousarray(d["rho"]), rphi)


@pytest.fixture(scope="module")
def ref():
    return golden("ref_synth")


@pytest.mark.parametrize("name", STATIC)
def test_oracle_forces_match_reference(potentials, ref, name):
    g = golden(name)
    elems = tuple(str(e) for e in g["elems"])
    path, digest = potentials[elems]
    assert str(ref[name + "/sha256"]) == digest
    s = O.System(O.Eam.setfl(path), g["H"], g["x"], g["elem"], g["masses"])
    pe, vir = s.force()
    assert abs(pe - ref[name + "/pe"]) <= 1e-13 * abs(pe)
    assert abs(s.energy() - ref[name + "/energy"]) <= 1e-13 * abs(pe)
    assert rel(s.f, ref[name + "/f"]) <= 1e-12
    assert rel(voigt_to_stress(vir, g["H"]), ref[name + "/S_pe"]) <= 1e-12


def test_oracle_nvt_matches_reference(potentials, ref):
    """md.nvt(300, 1 fs), NHC with t_relax = 100 dt, 40 steps on 256 atoms."""
    path, digest = potentials[("A",)]
    assert str(ref["sha256_A"]) == digest
    c = synth.md_single((4, 4, 4), T=300.0, seed=21)
    s = O.System(O.Eam.setfl(path), c.H, c.x, c.elem, c.masses)
    s.v = c.v
    s.nvt_run(300.0, synth.FS, synth.KB, 40)
    assert np.max(np.abs(s.x - ref["nvt_a_256/x_end"])) <= 1e-12
    assert rel(s.v, ref["nvt_a_256/v_end"]) <= 1e-12


def test_oracle_nve_4000_matches_reference(potentials, ref):
    """The plain FP64 MD workload: 4,000-atom FCC, 100 NVE steps of 1 fs."""
    path, _ = potentials[("A",)]
    c = synth.md_single((10, 10, 10), T=300.0, seed=0)
    s = O.System(O.Eam.setfl(path), c.H, c.x, c.elem, c.masses)
    s.v = c.v
    th, _, _ = s.nvt_run(300.0, synth.FS, synth.KB, 100, t_relax=float("inf"))
    assert np.max(np.abs(s.x - ref["nve_a_4000/x_end"])) <= 1e-12
    assert rel(s.v, ref["nve_a_4000/v_end"]) <= 1e-12
    assert abs(th[-1, 0] - ref["nve_a_4000/pe_end"]) <= 1e-12 * abs(th[-1, 0])


@pytest.mark.parametrize("name", ["lbfgs_ab_256", "lbfgs_ab_475"])
def test_oracle_lbfgs_iterates_match_reference(potentials, ref, name):
    """md.min_lbfgs(m=10, e_tol=0) with ls_bt: positions after k iterations."""
    path, digest = potentials[("A", "B")]
    assert str(ref["sha256_AB"]) == digest
    e = O.Eam.setfl(path)
    H = ref[name + "/H"]
    for it in ref[name + "/iters"]:
        s = O.System(e, H, ref[name + "/x"], ref[name + "/elem"], ref[name + "/masses"])
        r = s.lbfgs_run(m=10, e_tol=0.0, f_tol=0.0, nsteps=int(it))
        d = s.x - ref["%s/x_%d" % (name, it)]
        ds = d @ np.linalg.inv(H)
        d = (ds - np.round(ds)) @ H  # the reference leaves x unwrapped
        # iterates to rounding; once at the minimum (the oracle's line search
        # ends the run there) the last digits of x are free
        tol = 1e-12 if r["niter"] == it else 1e-6
        assert np.max(np.abs(d)) <= tol, (it, np.max(np.abs(d)))
        assert abs(r["pe"] - ref["%s/pe_%d" % (name, it)]) <= 1e-12 * abs(r["pe"])


@pytest.mark.parametrize("name", ["cg_bt", "lbfgs_golden", "lbfgs_brent", "cg_golden", "cg_brent_nobracket"])
def test_oracle_minimizer_iterates_match_reference(potentials, name):
    """md.min_cg_new (MinCG) with ls_bt, and md.min_lbfgs / md.min_cg_new
    with ls_golden and ls_brent (bracketing on and off), e_tol = 0:
    positions and energy after k iterations of each.  Back-tracking follows
    the reference to rounding.  Golden section and Brent refine the step
    until the bracket is tol |alpha| wide (tol = sqrt(2 eps)), where the
    energies they compare differ by less than their rounding; the oracle's
    energies agree with the reference's to ~1e-14, so it may settle
    elsewhere inside that last bracket (at most tol * max_dx = 2e-8 A after
    one step), and L-BFGS carries the difference on.  Measured: golden 1e-11
    A after five iterations, Brent 2e-9 A after one and 2e-7 A after five;
    the energies stay within 1e-12."""
    tol_x = {"bt": 1e-11, "golden": 1e-9, "brent": 1e-6}
    g = golden("ref_min")
    path, digest = potentials[("A", "B")]
    assert str(g["sha256_AB"]) == digest
    e = O.Eam.setfl(path)
    H = g["H"]
    method, ls, bracket = (str(v) for v in g[name + "/spec"])
    search = O.line_search(ls, bracket=bracket == "True")
    for it in g[name + "/iters"]:
        s = O.System(e, H, g["x"], g["elem"], g["masses"])
        if method == "lbfgs":
            r = s.lbfgs_run_ls(search, m=10, e_tol=0.0, f_tol=0.0, nsteps=int(it))
        else:
            r = s.cg_run_ls(search, e_tol=0.0, f_tol=0.0, nsteps=int(it))
        d = s.x - g["%s/x_%d" % (name, it)]
        ds = d @ np.linalg.inv(H)
        d = (ds - np.round(ds)) @ H  # the reference leaves x unwrapped
        assert r["niter"] == it
        assert np.max(np.abs(d)) <= tol_x[ls], (it, np.max(np.abs(d)))
        assert abs(r["pe"] - g["%s/pe_%d" % (name, it)]) <= 1e-12 * abs(r["pe"])


def _wrapped(d, H):
    ds = d @ np.linalg.inv(H)
    return (ds - np.round(ds)) @ H


def test_oracle_nst_matches_reference(potentials):
    """md.nst (MDNST::run) at zero stress on the diagonal, from an expanded
    alloy cell at 300 K: after 5 and 30 steps the box and the velocities
    follow the reference to rounding, and the positions up to one rigid
    translation.  The translation comes from the mean displacement that each
    step removes (md_nst.cpp:120-127): it includes the affine part x.V_H,
    which depends on the periodic image an atom is stored as, and the
    reference re-wraps atoms only at its skin-triggered rebuilds while the
    oracle (and libmappg) rebuild, and so wrap, at every step.  Forces and
    the dynamics do not depend on it."""
    g = golden("ref_box")
    path, digest = potentials[("A", "B")]
    assert str(g["sha256_AB"]) == digest
    e = O.Eam.setfl(path)
    for it in g["nst/iters"]:
        o = O.System(e, g["H"], g["x"], g["elem"], g["masses"], skin=0.5)
        o.v = g["nst/v"]
        o.nst_run(g["nst/S"], 300.0, synth.FS, synth.KB, int(it))
        H = o.box()
        assert np.max(np.abs(H - g["nst/H_%d" % it])) <= 1e-12 * np.max(np.abs(H))
        assert np.max(np.abs(o.v - g["nst/v_%d" % it])) <= 1e-12 * np.max(np.abs(o.v))
        d = _wrapped(o.x - g["nst/x_%d" % it], H)
        assert np.max(np.abs(d - d.mean(axis=0))) <= 1e-11


@pytest.mark.parametrize("name", ["box_lbfgs", "box_cg_affine"])
def test_oracle_box_minimizers_match_reference(potentials, name):
    """md.min_lbfgs and md.min_cg_new with H_dof on the diagonal (atoms free,
    or affine), ls_bt, e_tol = 0: box, positions and energy after k
    iterations."""
    g = golden("ref_box")
    path, _ = potentials[("A", "B")]
    e = O.Eam.setfl(path)
    method, affine = (str(v) for v in g[name + "/spec"])
    for it in g[name + "/iters"]:
        o = O.System(e, g["H"], g["x"], g["elem"], g["masses"], skin=0.5)
        r = o.min_box_run(O.line_search("bt"), np.eye(3, dtype=bool), affine == "True", method, m=10, e_tol=0.0,
                          nsteps=int(it))
        H = o.box()
        assert r["niter"] == it
        assert np.max(np.abs(H - g["%s/H_%d" % (name, it)])) <= 1e-10
        assert np.max(np.abs(_wrapped(o.x - g["%s/x_%d" % (name, it)], H))) <= 1e-10
        assert abs(r["pe"] - g["%s/pe_%d" % (name, it)]) <= 1e-12 * abs(r["pe"])


def test_oracle_frozen_components_match_reference(potentials):
    """atoms.x_dof set through atoms.do on some components and some whole
    atoms: md.nvt positions and velocities after 10 and 40 steps, and
    md.min_lbfgs positions and energy after 1, 5 and 20 iterations, to
    rounding."""
    g = golden("ref_dof")
    path, digest = potentials[("A", "B")]
    assert str(g["sha256_AB"]) == digest
    e = O.Eam.setfl(path)
    H = g["H"]
    for it in g["nvt/iters"]:
        o = O.System(e, H, g["x"], g["elem"], g["masses"])
        o.set_dof(g["dof"])
        o.v = g["v"]
        o.nvt_run(600.0, synth.FS, synth.KB, int(it), t_relax=20.0 * synth.FS)
        assert np.max(np.abs(_wrapped(o.x - g["nvt/x_%d" % it], H))) <= 1e-12
        assert np.max(np.abs(o.v - g["nvt/v_%d" % it])) <= 1e-12 * np.max(np.abs(o.v))
    for it in g["lbfgs/iters"]:
        o = O.System(e, H, g["x"], g["elem"], g["masses"])
        o.set_dof(g["dof"])
        r = o.lbfgs_run(m=10, e_tol=0.0, f_tol=0.0, nsteps=int(it))
        assert r["niter"] == it
        assert np.max(np.abs(_wrapped(o.x - g["lbfgs/x_%d" % it], H))) <= 1e-12
        assert abs(r["pe"] - g["lbfgs/pe_%d" % it]) <= 1e-12 * abs(r["pe"])


def test_library_funcfl_tables_match_reference(built, tmp_path):
    """ff_eam_funcfl (import_eam.h:68-346) on two funcfl files with
    different grids: libmappg's host table builder (mappg_ff_funcfl, no GPU
    involved) resamples them onto the common grid; the oracle, given those
    knots, reproduces the reference's forces and energy on a 256-atom A/B
    alloy to rounding."""
    import hashlib

    g = golden("ref_funcfl")
    paths = potfile.write_funcfl_pair(str(tmp_path))
    for k, p in enumerate(paths):
        with open(p, "rb") as fh:
            assert hashlib.sha256(fh.read()).hexdigest() == str(g["sha256_%d" % k])
    _lib.load()
    ff = _lib.ForceField.funcfl(paths)
    F, rho, rphi, _ = ff.tables()
    ne, nrho, nr = F.shape[0], F.shape[1], rho.shape[2]
    R = np.ascontiguousarray(rho[:, :, :, 0])
    P = np.zeros((ne, ne, nr))
    for i in range(ne):
        for j in range(ne):
            P[i, j] = rphi[max(i, j), min(i, j), :, 0]
    e = O.Eam.knots(nr, nrho, ff.dr, ff.drho, np.ascontiguousarray(F[:, :, 0]), R, P)
    o = O.System(e, g["H"], g["x"], g["elem"], g["masses"])
    pe, _ = o.force()
    assert abs(pe - g["pe"]) <= 1e-12 * abs(g["pe"])
    assert rel(o.f, g["f"]) <= 1e-12


def test_create_temp_matches_reference(ref):
    """atoms.create_temp(T, seed): the oracle and libmappg's host code draw
    the reference's velocities bit for bit."""
    elem, masses = ref["create_temp/elem"], ref["create_temp/masses"]
    T, seed = float(ref["create_temp/T"]), int(ref["create_temp/seed"])
    assert np.array_equal(O.create_temp(elem, masses, T, synth.KB, seed), ref["create_temp/v"])
    _lib.load()
    assert np.array_equal(_lib.create_temp(elem, masses, T, synth.KB, seed), ref["create_temp/v"])


def test_oracle_extrapolation_matches_reference(tmp_path):
    """Host densities above rho_max = nrho * drho: F extrapolated linearly
    (ff_eam.cpp:188-189)."""
    g = golden("ref_extrap")
    path = str(tmp_path / "extrap.setfl")
    synth.write_setfl(path, ("A",), drho=float(g["drho"]))
    s = O.System(O.Eam.setfl(path), g["H"], g["x"], g["elem"], g["masses"])
    pe, vir = s.force()
    rho, _ = s.rho_dF()
    assert rho.min() > 5000 * float(g["drho"])
    assert abs(pe - g["pe"]) <= 1e-13 * abs(pe)
    assert rel(s.f, g["f"]) <= 1e-12


@pytest.mark.parametrize("pot", POTS)
def test_oracle_matches_reference_on_its_potential_files(tmp_path, pot):
    """The potential files of the reference's examples (Cu_mishin setfl with
    nr = 10,001; NiAl and FeH-sina setfl with per-pair cutoffs; Fe-H
    Finnis-Sinclair), written back from their knots."""
    g = golden("ref_pot_" + pot)
    d = potfile.from_fixture(g)
    path = potfile.write(str(tmp_path / (pot + ".pot")), d)
    e = oracle_eam(d, path)
    for cell in [str(c) for c in g["cells"]]:
        H = g[cell + "/H"]
        s = O.System(e, H, g[cell + "/x"], g[cell + "/elem"], d["masses"])
        pe, vir = s.force()
        assert abs(pe - g[cell + "/pe"]) <= 1e-13 * abs(pe), cell
        assert rel(s.f, g[cell + "/f"]) <= 1e-12, cell
        assert rel(voigt_to_stress(vir, H), g[cell + "/S_pe"]) <= 1e-12, cell
    if "nvt/v0" in g:
        H = g["c0/H"]
        s = O.System(e, H, g["c0/x"], g["c0/elem"], d["masses"])
        s.v = g["nvt/v0"]
        s.nvt_run(float(g["nvt/T"]), synth.FS, synth.KB, int(g["nvt/nsteps"]))
        assert np.max(np.abs(s.x - g["nvt/x_end"])) <= 1e-11
        assert rel(s.v, g["nvt/v_end"]) <= 1e-11


def test_potential_fixtures_cover_the_branches(tmp_path):
    """The fixtures reach the code paths they are kept for: unequal per-pair
    cutoffs (NiAl, FeH), host densities beyond rho_max (dense Cu), a box
    thinner than two cutoffs (thin Cu), nr = 10,001 (Cu)."""
    for pot in ("nial", "feh", "feh_fs"):
        d = potfile.from_fixture(golden("ref_pot_" + pot))
        e = oracle_eam(d, potfile.write(str(tmp_path / pot), d))
        assert np.ptp(e.tables()[3]) > 0.1, pot
    cu = golden("ref_pot_cu")
    d = potfile.from_fixture(cu)
    e = oracle_eam(d, potfile.write(str(tmp_path / "cu"), d))
    s = O.System(e, cu["dense/H"], cu["dense/x"], cu["dense/elem"], d["masses"])
    s.force()
    assert s.rho_dF()[0].max() > int(d["nrho"]) * float(d["drho"])
    assert int(d["nr"]) == 10001
    assert np.min(np.diag(cu["thin/H"])) < 2 * float(d["rc"])


needs_ref = pytest.mark.skipif(not refmod.available(), reason="compiled reference (oracle/_ref) not built here")


@needs_ref
@pytest.mark.parametrize("seed", [101, 102])
def test_oracle_matches_live_reference(potentials, seed):
    """Fresh seeded alloys (strained, with vacancies) through the reference
    module: force call, then 30 NVT steps and 8 L-BFGS iterations."""
    path, _ = potentials[("A", "B")]
    rng = np.random.default_rng(seed)
    strain = np.tril(rng.uniform(-0.02, 0.02, (3, 3)))
    c = synth.alloy((4, 4, 3), xB=rng.uniform(0.2, 0.8), sigma=0.1, T=900.0, vac=0.02, strain=strain, seed=seed)
    r = refmod.RefSystem(c.H, c.x, c.elem, c.masses, ["A", "B"], path, v=c.v, kB=synth.KB)
    pe_r, S_r, val_r, f_r = r.force()
    e = O.Eam.setfl(path)
    s = O.System(e, c.H, c.x, c.elem, c.masses)
    pe, vir = s.force()
    assert abs(pe - pe_r) <= 1e-13 * abs(pe) and abs(s.energy() - val_r) <= 1e-13 * abs(pe)
    assert rel(s.f, f_r) <= 1e-12 and rel(voigt_to_stress(vir, c.H), S_r) <= 1e-12
    H, x_r, v_r = r.nvt(900.0, synth.FS, 30, t_relax=100.0 * synth.FS)
    s.v = c.v
    s.nvt_run(900.0, synth.FS, synth.KB, 30)
    assert np.max(np.abs(s.x - x_r)) <= 1e-11 and rel(s.v, v_r) <= 1e-11
    r2 = refmod.RefSystem(c.H, c.x, c.elem, c.masses, ["A", "B"], path)
    _, x_r, _ = r2.lbfgs(8, m=10, e_tol=0.0)
    s2 = O.System(e, c.H, c.x, c.elem, c.masses)
    s2.lbfgs_run(m=10, e_tol=0.0, f_tol=0.0, nsteps=8)
    d = (s2.x - x_r) @ np.linalg.inv(c.H)
    assert np.max(np.abs((d - np.round(d)) @ c.H)) <= 1e-10


@pytest.mark.parametrize("pot", POTS)
def test_library_tables_equal_oracle_on_reference_files(tmp_path, pot):
    """libmappg's host parser and spline builder (setfl and fs) give the
    oracle's tables bit for bit on the reference's potential files."""
    from mapp4py_gb300 import build

    build.build()
    _lib.load()
    d = potfile.from_fixture(golden("ref_pot_" + pot))
    path = potfile.write(str(tmp_path / (pot + ".pot")), d)
    ff = _lib.ForceField.setfl(path) if d["kind"] == "setfl" else _lib.ForceField.fs(path)
    for a, b in zip(ff.tables(), oracle_eam(d, path).tables()):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("name", ["alloy_v", "tric"])
def test_library_cfg_writer_matches_reference(built, tmp_path, name):
    """The CFG files md.export_cfg of the reference wrote (ExportCFGMD,
    export_cfg_md.cpp): libmappg's writer (mappg_cfg_write, host code) gives
    the same bytes for the same box, atoms, masses and velocities, in an
    orthorhombic alloy cell with velocities and in a triclinic cell."""
    g = golden("ref_cfg")
    _lib.load()
    p = str(tmp_path / (name + ".cfg"))
    vecs = (("x_d", g[name + "/v"]),) if bool(g[name + "/with_v"]) else ()
    _lib.write_cfg(p, g[name + "/H"], g[name + "/x"], g[name + "/elem"], g[name + "/masses"], ["A", "B"], vecs=vecs)
    with open(p) as fh:
        assert fh.read() == str(g[name + "/text"])
