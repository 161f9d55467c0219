"""The CPU oracle against its committed golden fixtures and against physics
it must satisfy: finite-difference forces, perfect-lattice symmetry,
Newton's third law, half-list vs full-list agreement, NVE energy
conservation, the thermostat reaching its temperature, and (when the
reference tree is present) the published cohesive energy of the Cu setfl
file shipped with the reference."""
import os

import numpy as np
import pytest

import mlp_ref as R
import oracle as O
from conftest import REF_ROOT, golden, golden_potential
from mapp4py_gb300 import synth

STATIC = ["fcc_a_256", "alloy_ab_475", "thin_a_32", "tric_ab_240"]


def keys(cnt, ent):
    atom = np.repeat(np.arange(cnt.shape[0]), cnt)
    rows = np.column_stack([atom, ent]).astype(np.int64)
    return rows[np.lexsort(rows.T[::-1])]


@pytest.mark.parametrize("name", STATIC)
def test_oracle_reproduces_golden(potentials, name):
    g = golden(name)
    path = golden_potential(potentials, g)
    e = O.Eam.setfl(path)
    s = O.System(e, g["H"], g["x"], g["elem"], g["masses"])
    pe, vir = s.force()
    assert pe == float(g["pe"]) and np.array_equal(vir, g["virial"])
    assert np.array_equal(s.f, g["f"])
    full = O.System(e, g["H"], g["x"], g["elem"], g["masses"], pair_wise=False)
    full.init_dynamic()
    assert np.array_equal(keys(*full.neighbors()), g["nbr"])


@pytest.mark.parametrize("name", ["alloy_ab_475", "tric_ab_240"])
def test_full_list_restatement_matches_half_list(potentials, name):
    g = golden(name)
    e = O.Eam.setfl(golden_potential(potentials, g))
    full = O.System(e, g["H"], g["x"], g["elem"], g["masses"], pair_wise=False)
    pe, vir = full.force_full(nthreads=2)
    assert abs(pe - g["pe"]) <= 1e-12 * abs(g["pe"])
    assert np.max(np.abs(vir - g["virial"])) <= 1e-11 * np.max(np.abs(g["virial"]))
    assert np.max(np.abs(full.f - g["f"])) <= 1e-11 * np.max(np.abs(g["f"]))


def test_finite_difference_forces(potentials):
    """Central differences of the energy (h = 1e-5 A) against the forces:
    the check MinCGOld::ff_test (min_cg_old.cpp:168-240) makes."""
    path, _ = potentials[("A", "B")]
    c = synth.alloy((3, 3, 3), xB=0.5, sigma=0.1, seed=4)
    e = O.Eam.setfl(path)
    s = O.System(e, c.H, c.x, c.elem, c.masses)
    s.force()
    f = s.f
    rng = np.random.default_rng(0)
    h = 1e-5
    for a in rng.choice(c.natoms, 6, replace=False):
        for k in range(3):
            xp = c.x.copy()
            xp[a, k] += h
            xm = c.x.copy()
            xm[a, k] -= h
            ep = O.System(e, c.H, xp, c.elem, c.masses).energy()
            em = O.System(e, c.H, xm, c.elem, c.masses).energy()
            fd = -(ep - em) / (2 * h)
            assert abs(fd - f[a, k]) < 2e-6 * max(1.0, abs(f[a, k])), (a, k, fd, f[a, k])


def test_perfect_lattice_symmetry(potentials):
    path, _ = potentials[("A",)]
    H, x = synth.fcc((5, 5, 5))
    e = O.Eam.setfl(path)
    s = O.System(e, H, x, np.zeros(len(x), np.uint8), [synth.MASS])
    pe, vir = s.force()
    assert np.max(np.abs(s.f)) < 1e-12
    assert abs(vir[1]) + abs(vir[2]) + abs(vir[4]) < 1e-9 * abs(vir[0])
    assert abs(vir[0] - vir[3]) < 1e-9 * abs(vir[0]) and abs(vir[0] - vir[5]) < 1e-9 * abs(vir[0])
    # energy per atom from the analytic functions on the FCC shells
    shells = [(12, 2.5561), (6, 3.615), (24, 4.4275), (12, 5.1124)]
    a = 3.615
    shells = [(12, a / np.sqrt(2)), (6, a), (24, a * np.sqrt(1.5)), (12, a * np.sqrt(2)), (24, a * np.sqrt(2.5))]
    D, r0, pref = synth.ELEMENTS["A"]
    rho = sum(n * synth.rho_fn(np.array([r]), r0)[0] for n, r in shells)
    ep = 0.5 * sum(n * synth.phi(np.array([r]), D, r0)[0] for n, r in shells)
    assert abs(pe / len(x) - (-pref * np.sqrt(rho) + ep)) < 1e-6


def test_newton_third_law_and_translation(potentials):
    g = golden("alloy_ab_475")
    e = O.Eam.setfl(golden_potential(potentials, g))
    s = O.System(e, g["H"], g["x"], g["elem"], g["masses"])
    s.force()
    assert np.max(np.abs(s.f.sum(axis=0))) < 1e-10
    t = O.System(e, g["H"], g["x"] + np.array([1.3, -0.4, 2.2]), g["elem"], g["masses"])
    t.force()
    assert np.max(np.abs(t.f - s.f)) < 1e-10


def test_nve_conservation_and_nhc_temperature(potentials):
    path, _ = potentials[("A",)]
    e = O.Eam.setfl(path)
    c = synth.md_single((4, 4, 4), T=300.0, seed=3)
    dev = []
    for dt_fs, n in ((1.0, 200), (0.5, 400)):
        s = O.System(e, c.H, c.x, c.elem, c.masses)
        s.v = c.v
        th, _, _ = s.nvt_run(300.0, dt_fs * synth.FS, synth.KB, n, t_relax=float("inf"))
        etot = th[:, 0] + 0.5 * (th[:, 2] + th[:, 5] + th[:, 7])
        dev.append(np.max(np.abs(etot - etot[0])) / c.natoms)
    # velocity Verlet: the total-energy offset is O(dt^2) and small
    assert dev[0] < 2e-5 and dev[1] < 0.35 * dev[0]
    # the chain drives a cold start towards its set temperature
    s = O.System(e, c.H, c.x, c.elem, c.masses)
    s.v = 0.2 * c.v
    th, eta, _ = s.nvt_run(600.0, 2 * synth.FS, synth.KB, 1500, t_relax=20 * synth.FS)
    assert abs(np.mean(th[-500:, 1]) - 600.0) < 60.0
    assert np.all(np.isfinite(eta))


def test_create_temp_statistics():
    elem = np.zeros(30000, np.uint8)
    v = O.create_temp(elem, [63.5], 300.0, synth.KB, 12345)
    assert abs(np.std(v) - np.sqrt(synth.KB * 300.0 / 63.5)) < 0.01 * np.sqrt(synth.KB * 300.0 / 63.5)
    with pytest.raises(ValueError):
        O.create_temp(elem[:4], [63.5], 300.0, synth.KB, 0)


def test_lbfgs_reaches_force_tolerance(potentials):
    g = golden("lbfgs_ab_475")
    path = golden_potential(potentials, dict(g, elems=np.array(["A", "B"])))
    s = O.System(O.Eam.setfl(path), g["H"], g["x"], g["elem"], g["masses"])
    r = s.lbfgs_run(m=10, e_tol=0.0, f_tol=1e-4, nsteps=5000)
    assert r["err"] == 100 and r["fmax"] < 1e-4
    assert r["pe"] == float(g["pe"]) and r["niter"] == int(g["niter"])


def test_lbfgs_with_a_unit_diagonal_is_plain_lbfgs(potentials):
    """The diagonal-H0 restatement (the library's mappg_lbfgs_run_diag): a unit
    Hessian diagonal makes tau*diag(1/h) equal gamma*I, so the run retraces
    plain L-BFGS step for step; a diagonal that is not positive is refused."""
    c = synth.alloy((4, 4, 4), xB=0.3, sigma=0.1, seed=2, vac=0.01)
    path = potentials[("A", "B")][0]
    a = O.System(O.Eam.setfl(path), c.H, c.x, c.elem, c.masses)
    b = O.System(O.Eam.setfl(path), c.H, c.x, c.elem, c.masses)
    r0 = a.lbfgs_run(m=10, e_tol=0.0, f_tol=1e-4, nsteps=400)
    r1 = b.lbfgs_run_diag(np.ones((c.natoms, 3)), m=10, e_tol=0.0, f_tol=1e-4, nsteps=400)
    keys = ("niter", "err", "n_energy", "n_force", "pe")
    assert [r1[k] for k in keys] == [r0[k] for k in keys]
    assert r1["fallbacks"] == 0 and np.array_equal(a.x, b.x)
    bad = np.ones((c.natoms, 3))
    bad[3, 1] = 0.0
    with pytest.raises(RuntimeError, match="positive"):
        O.System(O.Eam.setfl(path), c.H, c.x, c.elem, c.masses).lbfgs_run_diag(bad)


def test_cg_reaches_force_tolerance(potentials):
    path, _ = potentials[("A", "B")]
    c = synth.alloy((4, 4, 4), xB=0.3, sigma=0.1, seed=2, vac=0.01)
    s = O.System(O.Eam.setfl(path), c.H, c.x, c.elem, c.masses, skin=0.5)
    r = s.cg_run(e_tol=0.0, f_tol=1e-4, nsteps=5000)
    assert r["err"] == 100 and r["fmax"] < 1e-4
    # the same minimum as L-BFGS from the same start
    t = O.System(O.Eam.setfl(path), c.H, c.x, c.elem, c.masses, skin=0.5)
    rl = t.lbfgs_run(m=10, e_tol=0.0, f_tol=1e-4, nsteps=5000)
    assert abs(r["pe"] - rl["pe"]) < 1e-6 * abs(rl["pe"])


@pytest.mark.parametrize("kind", ["golden", "brent"])
def test_golden_and_brent_line_searches(potentials, kind):
    """ls_golden / ls_brent (ls.h:214-706) in both minimizers: bracketed,
    they reach the force tolerance at the same minimum as back-tracking;
    the back-tracking entry with a line-search record is the plain one."""
    path, _ = potentials[("A", "B")]
    c = synth.alloy((4, 4, 4), xB=0.3, sigma=0.1, seed=2, vac=0.01)

    def fresh():
        return O.System(O.Eam.setfl(path), c.H, c.x, c.elem, c.masses, skin=0.5)

    ref = fresh().lbfgs_run(m=10, e_tol=0.0, f_tol=1e-4, nsteps=5000)
    assert fresh().lbfgs_run_ls(O.line_search("bt"), m=10, e_tol=0.0, f_tol=1e-4, nsteps=5000) == ref
    for run in ("lbfgs", "cg"):
        s = fresh()
        ls = O.line_search(kind)
        r = (s.lbfgs_run_ls(ls, m=10, e_tol=0.0, f_tol=1e-4, nsteps=5000) if run == "lbfgs"
             else s.cg_run_ls(ls, e_tol=0.0, f_tol=1e-4, nsteps=5000))
        assert r["err"] == 100 and r["fmax"] < 1e-4, r
        assert abs(r["pe"] - ref["pe"]) < 1e-6 * abs(ref["pe"])
        # a line minimization costs several energies per iteration
        assert r["n_energy"] > 3 * r["niter"]
        # without bracketing the search spans [0, max_dx/max|h|] in max_iter
        # steps; the run stops on a failed search or descends
        s = fresh()
        r = s.lbfgs_run_ls(O.line_search(kind, bracket=False), m=10, e_tol=0.0, f_tol=1e-4, nsteps=50)
        assert r["err"] in (3, 100, 5) and r["pe"] < ref["pe"] + 2.0


@pytest.mark.parametrize("method", ["lbfgs", "cg"])
def test_box_degrees_of_freedom(potentials, method):
    """MinLBFGS / MinCG with H_dof (min_cg.h:89-331, new_min_vec.h): with
    affine atoms the box relaxes until F_H on the free entries vanishes;
    with atoms and box free the energy ends below the fixed-box relaxation;
    entries outside H_dof keep their value."""
    path, _ = potentials[("A", "B")]
    c = synth.alloy((4, 4, 4), a=3.7, xB=0.3, sigma=0.05, seed=2)

    def fresh():
        return O.System(O.Eam.setfl(path), c.H, c.x, c.elem, c.masses, skin=0.5)

    s = fresh()
    pe0, vir0 = s.force()
    r = s.min_box_run(O.line_search("bt"), np.eye(3, dtype=bool), True, method, m=10, e_tol=1e-10, nsteps=300)
    assert r["err"] == 4 and r["pe"] < pe0
    pe, vir = s.force()
    assert np.max(np.abs(vir[[0, 3, 5]])) < 1e-2 * np.max(np.abs(vir0[[0, 3, 5]]))
    H = s.box()
    assert H[1, 0] == H[2, 0] == H[2, 1] == 0.0  # off-diagonal entries were not free
    # only H[0][0] free: the others stay
    s = fresh()
    mask = np.zeros((3, 3), dtype=bool)
    mask[0, 0] = True
    s.min_box_run(O.line_search("bt"), mask, True, method, m=10, e_tol=1e-10, nsteps=100)
    H = s.box()
    assert H[0, 0] != c.H[0, 0] and H[1, 1] == c.H[1, 1] and H[2, 2] == c.H[2, 2]
    # atoms and box together go below the fixed-box minimum
    fixed = fresh().lbfgs_run(m=10, e_tol=1e-10, f_tol=0.0, nsteps=300)
    s = fresh()
    r = s.min_box_run(O.line_search("brent"), np.eye(3, dtype=bool), False, method, m=10, e_tol=1e-10, nsteps=300)
    assert r["pe"] < fixed["pe"]


def test_nst_relaxes_toward_the_applied_stress(potentials):
    """MDNST restated (md_nst.cpp): a cell far from zero stress changes its
    box until the pressure drops; the box entries without a degree of
    freedom stay; the box velocity and both chains are carried out."""
    path, _ = potentials[("A", "B")]
    c = synth.alloy((5, 5, 5), a=2.9, xB=0.3, sigma=0.02, T=300.0, seed=4)
    o = O.System(O.Eam.setfl(path), c.H, c.x, c.elem, c.masses, skin=0.5)
    o.v = c.v
    nan = np.nan
    S = np.array([[0.0, nan, nan], [nan, 0.0, nan], [nan, nan, 0.0]])
    th, VH, eta, eta_S = o.nst_run(S, 300.0, synth.FS, synth.KB, 1000, tau=np.full((3, 3), 50 * synth.FS))
    H0, H = th[0, 14:].reshape(3, 3), th[-1, 14:].reshape(3, 3)
    assert np.max(np.abs(np.diag(H) - np.diag(H0))) > 0.1  # the cell transforms (FCC -> BCT for this alloy)
    assert H[1, 0] == H[2, 0] == H[2, 1] == 0.0  # shear entries have no degree of freedom
    # the virial pressure oscillates about the target and settles near it
    vol = np.prod(th[:, [14, 18, 22]], axis=1)
    p = -(th[:, 8] + th[:, 11] + th[:, 13]) / 3.0 / vol * 160.2  # GPa
    assert abs(np.mean(p[500:])) < 1.5 and np.max(np.abs(p[:100])) > 5.0
    assert np.all(np.isfinite(th)) and np.any(VH != 0.0) and np.any(eta_S != 0.0)
    with pytest.raises(RuntimeError, match="stress"):
        o.nst_run(np.full((3, 3), nan), 300.0, synth.FS, synth.KB, 1)


REF_CU = os.path.join(REF_ROOT, "examples/diff/potentials/Cu_mishin.eam.alloy") if REF_ROOT else None


@pytest.mark.skipif(not (REF_CU and os.path.exists(REF_CU)), reason="MAPPG_REFERENCE_ROOT unset or without the example")
def test_cu_mishin_cohesive_energy():
    """Mishin et al. (2001) Cu: FCC a0 = 3.615 A, E_coh = -3.54 eV/atom; the
    setfl file shipped with the reference, read by the oracle."""
    e = O.Eam.setfl(REF_CU)
    H, x = synth.fcc((5, 5, 5), a=3.615)
    s = O.System(e, H, x, np.zeros(len(x), np.uint8), [63.546])
    pe, vir = s.force()
    assert abs(pe / len(x) - (-3.54)) < 0.005
    # a0 is the energy minimum: the pressure (virial) nearly vanishes
    assert abs(vir[0]) / len(x) < 0.01


def _dof_mask(n, seed=5):
    """About a fifth of the atoms fully frozen, a few more frozen along one
    component (z only for some, x only for others)."""
    rng = np.random.default_rng(seed)
    d = np.ones((n, 3), dtype=bool)
    r = rng.random(n)
    d[r < 0.2] = False
    d[(r >= 0.2) & (r < 0.3), 2] = False
    d[(r >= 0.3) & (r < 0.35), 0] = False
    return d


def test_x_dof_forces_minimizer_and_nvt(potentials):
    """atoms.x_dof (ff_md.cpp:138-144, md_nvt.cpp:144-215): forces on frozen
    components are zero, the minimizer leaves them in place, an NVT run
    drifts them with their velocity without kicking or thermostatting them,
    counts only the free components in the temperature, and draws only the
    free components in create_temp."""
    path, _ = potentials[("A", "B")]
    e = O.Eam.setfl(path)
    c = synth.alloy((4, 4, 4), xB=0.3, sigma=0.1, T=600.0, seed=2)
    d = _dof_mask(c.natoms)
    free = O.System(e, c.H, c.x, c.elem, c.masses)
    pe0, vir0 = free.force()
    s = O.System(e, c.H, c.x, c.elem, c.masses)
    s.set_dof(d)
    pe, vir = s.force()
    assert pe == pe0 and np.array_equal(vir, vir0)
    assert np.array_equal(s.f, np.where(d, free.f, 0.0))
    # an all-free mask is the plain path, bit for bit
    t = O.System(e, c.H, c.x, c.elem, c.masses)
    t.set_dof(np.ones((c.natoms, 3), bool))
    t.v = c.v
    th_t, eta_t, _ = t.nvt_run(600.0, synth.FS, synth.KB, 30)
    u = O.System(e, c.H, c.x, c.elem, c.masses)
    u.v = c.v
    th_u, eta_u, _ = u.nvt_run(600.0, synth.FS, synth.KB, 30)
    assert np.array_equal(th_t, th_u) and np.array_equal(t.x, u.x)
    # the minimizer: frozen components stay where they are, up to the
    # rounding of the fractional-coordinate round trip at each rebuild
    m = O.System(e, c.H, c.x, c.elem, c.masses)
    m.set_dof(d)
    r = m.lbfgs_run(m=10, e_tol=0.0, f_tol=1e-4, nsteps=3000)
    assert r["err"] == 100
    assert np.max(np.abs(m.x[~d] - c.x[~d])) < 1e-13
    assert np.max(np.abs(m.f[d])) < 1e-4 and np.all(m.f[~d] == 0.0)
    # NVT: frozen components keep their velocity and drift with it
    v = O.create_temp_dof(c.elem, c.masses, d, 600.0, synth.KB, 77, np.full((c.natoms, 3), 1e-3))
    assert np.all(v[~d] == 1e-3) and np.all(v[d] != 1e-3)
    n = O.System(e, c.H, c.x, c.elem, c.masses)
    n.set_dof(d)
    n.v = v
    nsteps = 40
    th, eta, _ = n.nvt_run(600.0, synth.FS, synth.KB, nsteps, t_relax=20 * synth.FS)
    assert np.all(n.v[~d] == 1e-3)
    dx = n.x - c.x
    dx -= np.round(dx @ np.linalg.inv(c.H)) @ c.H
    assert np.max(np.abs(dx[~d] - nsteps * synth.FS * 1e-3)) < 1e-12
    # the temperature column counts the free components only
    vf = np.where(d, n.v, 0.0)
    mvv = np.sum(c.masses[c.elem][:, None] * vf * vf)
    assert abs(th[-1, 1] - mvv / (d.sum() * synth.KB)) < 1e-9 * th[-1, 1]
    assert np.all(np.isfinite(eta))


def test_x_dof_with_nst(potentials):
    """MDNST with x_dof (md_nst.cpp:259-279, md_nvt.cpp:265-330): frozen
    components leave the degrees of freedom, carry no force, and no stress
    may act along a direction in which an atom is frozen."""
    path, _ = potentials[("A", "B")]
    e = O.Eam.setfl(path)
    c = synth.alloy((4, 4, 4), a=2.9, xB=0.3, sigma=0.02, T=300.0, seed=4)
    d = np.ones((c.natoms, 3), bool)
    d[::5, 2] = False
    nan = np.nan
    s = O.System(e, c.H, c.x, c.elem, c.masses)
    s.set_dof(d)
    s.v = c.v
    S = np.array([[0.0, nan, nan], [nan, 0.0, nan], [nan, nan, nan]])
    th, VH, _, _ = s.nst_run(S, 300.0, synth.FS, synth.KB, 20, tau=np.full((3, 3), 50 * synth.FS))
    assert np.all(np.isfinite(th)) and np.all(s.f[~d] == 0.0)
    assert th[-1, 14 + 8] == c.H[2, 2]  # no stress along z: that box entry stays
    S[2, 2] = 0.0
    t = O.System(e, c.H, c.x, c.elem, c.masses)
    t.set_dof(d)
    t.v = c.v
    with pytest.raises(RuntimeError, match="degree freedom"):
        t.nst_run(S, 300.0, synth.FS, synth.KB, 1)


def test_descriptor_restatement_on_a_perfect_lattice():
    """The network inputs' restatement (mlp_ref.descriptors) on a perfect
    single-element FCC crystal: every atom's 16 radial functions equal the
    shell sum of the four neighbour shells inside 5.5 A (12 at a/sqrt2, 6 at
    a, 24 at a sqrt(3/2), 12 at a sqrt2); no element-1 neighbours."""
    a = 3.615
    H, x = synth.fcc((3, 3, 3), a=a)
    f = R.descriptors(H, x, np.zeros(len(x), np.uint8), np.full(len(x), 7.0))
    want = np.zeros(16)
    for count, r in ((12, a / np.sqrt(2.0)), (6, a), (24, a * np.sqrt(1.5)), (12, a * np.sqrt(2.0))):
        fc = 0.5 * (1.0 + np.cos(np.pi * r / 5.5))
        want += count * np.exp(-((r - R.DESC_CENTRES) ** 2) / (2.0 * 0.3 ** 2)) * fc
    assert np.max(np.abs(f[:, :16] - want)) < 1e-12
    assert np.all(f[:, 16:32] == 0.0) and np.all(f[:, 32] == 7.0)
