"""Regenerate the reference-pinned fixtures (ref_*.npz) from MAPP itself.

    MAPPG_REFERENCE_ROOT=/path/to/mapp4py python tests/golden/make_ref_golden.py

The reference is compiled from its own sources into oracle/_ref (recipe
oracle/ref.mk) and driven through its Python API (md.atoms, md.nvt,
md.min_lbfgs, atoms.create_temp) plus the probe of oracle/refshim, which
sets exact states and reads ForceFieldMD::force_calc's forces.  Nothing here
runs where the reference tree is absent; the fixtures it writes are what the
tests compare the oracle and the GPU against there.

Fixtures:
  ref_synth.npz      the analytic-potential cases of make_golden.py (forces,
                     energy, stress), the 256-atom NVT run's end state, the
                     first L-BFGS iterates of two cells, create_temp draws
  ref_min.npz        iterates of md.min_cg_new (back-tracking) and of
                     md.min_lbfgs / md.min_cg_new with ls_golden and ls_brent
                     on a 256-atom alloy cell
  ref_box.npz        md.nst states of an expanded alloy cell at zero stress,
                     and md.min_lbfgs / md.min_cg_new iterates with box
                     degrees of freedom (H_dof), atoms free or affine
  ref_dof.npz        md.nvt and md.min_lbfgs with frozen components
                     (atoms.x_dof)
  ref_funcfl.npz     forces, energy and stress through ff_eam_funcfl on two
                     seeded funcfl files with different grids
  ref_cfg.npz        files written by md.export_cfg (an alloy with its
                     velocities, a triclinic cell)
  ref_extrap.npz     an FCC cell whose host densities exceed rho_max
                     (linear extrapolation of F, ff_eam.cpp:188-189)
  ref_pot_<name>.npz the knot values of a potential file shipped with the
                     reference's examples, seeded cells on it and the
                     reference's forces, energy, stress (and a short NVT run
                     on Cu)
"""
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from mapp4py_gb300 import synth  # noqa: E402
import potfile  # noqa: E402
import refmod  # noqa: E402
import make_golden  # noqa: E402

EXTRAP_DRHO = 0.002  # rho_max = 5000 * 0.002 = 10 < the FCC host density (~17)

POTENTIALS = {
    # name: (path under the reference tree, kind)
    "cu": ("examples/diff/potentials/Cu_mishin.eam.alloy", "setfl"),
    "nial": ("examples/dmd/potentials/NiAl.eam.alloy", "setfl"),
    "feh": ("examples/beginner-tutorial/potentials/FeH-sina.eam.alloy", "setfl"),
    "feh_fs": ("examples/diff/potentials/Fe-H.eam.fs", "fs"),
}


def bcc_fe_h(n, a, nh, sigma, seed):
    """BCC Fe (n^3 cells) with nh H atoms at octahedral sites, noise sigma."""
    rng = np.random.default_rng(seed)
    g = np.stack(np.meshgrid(*[np.arange(n)] * 3, indexing="ij"), -1).reshape(-1, 3)
    s = (g[:, None, :] + np.array([[0, 0, 0], [0.5, 0.5, 0.5]])[None]).reshape(-1, 3)
    cells = rng.choice(g.shape[0], nh, replace=False)
    sh = g[cells] + np.array([0.5, 0.5, 0.0])
    x = np.concatenate([s, sh]) * a
    elem = np.concatenate([np.zeros(s.shape[0], np.uint8), np.ones(nh, np.uint8)])
    H = np.diag([n * a] * 3).astype(np.float64)
    x = synth.wrap(H, x + rng.normal(0.0, sigma, x.shape))
    return H, x, elem


def fcc_cell(n, a, xB, sigma, seed, strain=None):
    c = synth.alloy(n, a=a, xB=xB, sigma=sigma, strain=strain, seed=seed)
    return c.H, c.x, c.elem


def ref_force(H, x, elem, masses, names, path, kind, v=None):
    r = refmod.RefSystem(H, x, elem, masses, names, path, kind=kind, v=v)
    pe, S, val, f = r.force()
    return r, {"pe": pe, "S_pe": S, "energy": val, "f": f}


def synth_cases(tmp):
    out = {}
    pots = {}
    for elems in (("A",), ("A", "B")):
        pots[elems] = make_golden.potential(tmp, elems)
    for name, (elems, c) in make_golden.cases().items():
        path, digest = pots[elems]
        names = list(elems)
        _, res = ref_force(c.H, c.x, c.elem, c.masses, names, path, "setfl")
        for k, v in res.items():
            out[name + "/" + k] = v
        out[name + "/sha256"] = np.array(digest)
        print(name, res["pe"])
    # NVT: the nvt_a_256 case (NHC at 300 K, t_relax = 100 dt, 40 steps)
    path, digest = pots[("A",)]
    c = synth.md_single((4, 4, 4), T=300.0, seed=21)
    r = refmod.RefSystem(c.H, c.x, c.elem, c.masses, ["A"], path, v=c.v, kB=synth.KB)
    H, x, v = r.nvt(300.0, synth.FS, 40, t_relax=100.0 * synth.FS, L=3, niters=1)
    out.update({"nvt_a_256/x_end": x, "nvt_a_256/v_end": v, "nvt_a_256/pe_end": r.force()[0]})
    # NVE: 4,000-atom single-element FCC (the plain FP64 MD workload), 100 steps of
    # 1 fs at a 300 K start, thermostat off (t_relax = inf)
    c = synth.md_single((10, 10, 10), T=300.0, seed=0)
    r = refmod.RefSystem(c.H, c.x, c.elem, c.masses, ["A"], path, v=c.v, kB=synth.KB)
    H, x, v = r.nvt(300.0, synth.FS, 100, t_relax=float("inf"), L=3, niters=1)
    out.update({"nve_a_4000/x_end": x, "nve_a_4000/v_end": v, "nve_a_4000/pe_end": r.force()[0]})
    print("nve_a_4000 pe", out["nve_a_4000/pe_end"])
    # L-BFGS: iterates of the plain minimizer with back-tracking (m = 10)
    pathAB, digestAB = pots[("A", "B")]
    for name, (cell, iters) in {
        "lbfgs_ab_256": (synth.alloy((4, 4, 4), xB=0.3, sigma=0.1, seed=51), (1, 5, 20, 60)),
        "lbfgs_ab_475": (synth.alloy((5, 5, 5), xB=0.4, sigma=0.15, vac=0.05, seed=31), (1, 3, 8)),
    }.items():
        for it in iters:
            r = refmod.RefSystem(cell.H, cell.x, cell.elem, cell.masses, ["A", "B"], pathAB)
            H, x, v = r.lbfgs(it, m=10, e_tol=0.0)
            out["%s/x_%d" % (name, it)] = x
            out["%s/pe_%d" % (name, it)] = r.force()[0]
        out[name + "/iters"] = np.array(iters)
        out[name + "/H"] = cell.H
        out[name + "/x"] = cell.x
        out[name + "/elem"] = cell.elem
        out[name + "/masses"] = cell.masses
        print(name, [out["%s/pe_%d" % (name, it)] for it in iters])
    # create_temp: the Park-Miller / Box-Muller draw (two masses); the atoms are
    # in element order so the reference's local order is the caller's
    c = synth.alloy((3, 3, 3), xB=0.5, seed=61)
    elem = np.sort(c.elem)
    masses = np.array([63.5, 27.0])
    r = refmod.RefSystem(c.H, c.x, elem, masses, ["A", "B"], pathAB, kB=synth.KB)
    out.update({"create_temp/elem": elem, "create_temp/masses": masses, "create_temp/T": 450.0,
                "create_temp/seed": 987654, "create_temp/v": r.create_temp(450.0, 987654)})
    out["sha256_A"] = np.array(pots[("A",)][1])
    out["sha256_AB"] = np.array(digestAB)
    return out


def minimizer_cases(tmp):
    """Iterates of md.min_cg_new with back-tracking and of md.min_lbfgs and
    md.min_cg_new with the golden-section and Brent line searches (bracketing
    on and off), on the 256-atom alloy cell of the L-BFGS case."""
    out = {}
    path, digest = make_golden.potential(tmp, ("A", "B"))
    cell = synth.alloy((4, 4, 4), xB=0.3, sigma=0.1, seed=51)
    runs = {
        "cg_bt": ("cg", "bt", True, (1, 5, 20)),
        "lbfgs_golden": ("lbfgs", "golden", True, (1, 5)),
        "lbfgs_brent": ("lbfgs", "brent", True, (1, 5)),
        "cg_golden": ("cg", "golden", True, (1, 5)),
        "cg_brent_nobracket": ("cg", "brent", False, (1, 3)),
    }
    for name, (method, ls, bracket, iters) in runs.items():
        for it in iters:
            r = refmod.RefSystem(cell.H, cell.x, cell.elem, cell.masses, ["A", "B"], path)
            H, x, v = r.minimize(method, it, ls=ls, m=10, e_tol=0.0, bracket=bracket)
            out["%s/x_%d" % (name, it)] = x
            out["%s/pe_%d" % (name, it)] = r.force()[0]
        out[name + "/iters"] = np.array(iters)
        out[name + "/spec"] = np.array([method, ls, str(bool(bracket))])
        print(name, [out["%s/pe_%d" % (name, it)] for it in iters])
    out.update({"H": cell.H, "x": cell.x, "elem": cell.elem, "masses": cell.masses, "sha256_AB": np.array(digest)})
    return out


def box_cases(tmp):
    """md.nst (MDNST::run) at zero stress on the diagonal from an expanded
    256-atom alloy at 300 K, states after 5 and 30 steps; md.min_lbfgs and
    md.min_cg_new with box degrees of freedom (H_dof on the diagonal, atoms
    free or affine), states after a few iterations."""
    out = {}
    path, digest = make_golden.potential(tmp, ("A", "B"))
    c = synth.alloy((4, 4, 4), a=3.7, xB=0.3, sigma=0.02, T=300.0, seed=4)
    nan = float("nan")
    S = np.array([[0.0, nan, nan], [nan, 0.0, nan], [nan, nan, 0.0]])
    for it in (5, 30):
        r = refmod.RefSystem(c.H, c.x, c.elem, c.masses, ["A", "B"], path, v=c.v, kB=synth.KB)
        H, x, v = r.nst(S, 300.0, synth.FS, it)
        out.update({"nst/H_%d" % it: H, "nst/x_%d" % it: x, "nst/v_%d" % it: v})
        print("nst", it, np.diag(H))
    out.update({"nst/iters": np.array([5, 30]), "nst/S": S, "nst/v": c.v})
    H_dof = np.eye(3, dtype=bool)
    runs = {"box_lbfgs": ("lbfgs", False, (1, 5, 20)), "box_cg_affine": ("cg", True, (1, 5))}
    for name, (method, affine, iters) in runs.items():
        for it in iters:
            r = refmod.RefSystem(c.H, c.x, c.elem, c.masses, ["A", "B"], path)
            H, x, _ = r.minimize(method, it, ls="bt", m=10, e_tol=0.0, H_dof=H_dof, affine=affine)
            out.update({"%s/H_%d" % (name, it): H, "%s/x_%d" % (name, it): x, "%s/pe_%d" % (name, it): r.force()[0]})
        out[name + "/iters"] = np.array(iters)
        out[name + "/spec"] = np.array([method, str(affine)])
        print(name, [out["%s/pe_%d" % (name, it)] for it in iters])
    out.update({"H": c.H, "x": c.x, "elem": c.elem, "masses": c.masses, "sha256_AB": np.array(digest)})
    return out


def dof_cases(tmp):
    """atoms.x_dof (set through atoms.do): an NVT run (md_nvt.cpp:144-215)
    and md.min_lbfgs iterates of a 256-atom alloy with some components and
    some whole atoms frozen."""
    out = {}
    path, digest = make_golden.potential(tmp, ("A", "B"))
    c = synth.alloy((4, 4, 4), xB=0.3, sigma=0.1, T=600.0, seed=2)
    k = np.arange(c.natoms)
    dof = np.ones((c.natoms, 3), dtype=bool)
    dof[k % 5 == 0, 0] = False
    dof[k % 7 == 0, 2] = False
    dof[k % 11 == 0] = False
    v = c.v.copy()
    for it in (10, 40):
        r = refmod.RefSystem(c.H, c.x, c.elem, c.masses, ["A", "B"], path, v=v, kB=synth.KB)
        r.set_dof(dof)
        H, x, vv = r.nvt(600.0, synth.FS, it, t_relax=20.0 * synth.FS)
        out.update({"nvt/x_%d" % it: x, "nvt/v_%d" % it: vv})
    out["nvt/iters"] = np.array([10, 40])
    for it in (1, 5, 20):
        r = refmod.RefSystem(c.H, c.x, c.elem, c.masses, ["A", "B"], path)
        r.set_dof(dof)
        H, x, _ = r.minimize("lbfgs", it, ls="bt", m=10, e_tol=0.0)
        out.update({"lbfgs/x_%d" % it: x, "lbfgs/pe_%d" % it: r.force()[0]})
    out["lbfgs/iters"] = np.array([1, 5, 20])
    out.update({"H": c.H, "x": c.x, "v": v, "elem": c.elem, "masses": c.masses, "dof": dof,
                "sha256_AB": np.array(digest)})
    print("dof", out["lbfgs/pe_20"])
    return out


def funcfl_case(tmp):
    """ff_eam_funcfl on two seeded funcfl files with different grids
    (potfile.write_funcfl_pair): the reference's forces, energy and stress on
    a 256-atom A/B alloy."""
    paths = potfile.write_funcfl_pair(tmp)
    c = synth.alloy((4, 4, 4), xB=0.4, sigma=0.1, seed=81)
    _, res = ref_force(c.H, c.x, c.elem, c.masses, ["A", "B"], paths, "funcfl")
    out = {"H": c.H, "x": c.x, "elem": c.elem, "masses": c.masses}
    out.update(res)
    import hashlib
    for k, p in enumerate(paths):
        with open(p, "rb") as fh:
            out["sha256_%d" % k] = np.array(hashlib.sha256(fh.read()).hexdigest())
    print("funcfl pe", res["pe"])
    return out


def cfg_cases(tmp):
    """Files written by the reference's md.export_cfg (ExportCFGMD,
    export_cfg_md.cpp) called as (atoms, file): an alloy with its
    velocities as an extra vector, and a triclinic cell with the default
    vectors.  The atoms are stored in the file's (id) order."""
    out = {}
    path, _ = make_golden.potential(tmp, ("A", "B"))
    M = refmod.module()
    tric = synth.alloy((3, 3, 3), xB=0.4, sigma=0.05, T=300.0, seed=3)
    Ht = tric.H.copy()
    Ht[1, 0] += 2.1
    Ht[2, 0] -= 1.3
    Ht[2, 1] += 0.8
    cases = {"alloy_v": (synth.alloy((3, 3, 3), xB=0.4, sigma=0.05, T=300.0, seed=2), None, ["x_d"]),
             "tric": (tric, Ht, [])}
    for name, (c, H, extra) in cases.items():
        H = c.H if H is None else H
        x = c.x @ np.linalg.inv(c.H) @ H
        r = refmod.RefSystem(H, x, c.elem, c.masses, ["A", "B"], path, v=c.v)
        e = M.md.export_cfg("", 1, extra_vecs=extra) if extra else M.md.export_cfg("", 1)
        f = os.path.join(tmp, name + ".cfg")
        e(r.sim, f)
        Hs, xs, vs = r.state()
        o = r.order
        with open(f, "rb") as fh:
            out[name + "/text"] = np.array(fh.read().decode())
        out.update({name + "/H": Hs, name + "/x": xs[o], name + "/v": vs[o], name + "/elem": c.elem[o],
                    name + "/masses": c.masses, name + "/with_v": np.array(bool(extra))})
    return out


def extrap_case(tmp):
    path = os.path.join(tmp, "A_extrap.setfl")
    synth.write_setfl(path, ("A",), drho=EXTRAP_DRHO)
    H, x, elem = fcc_cell((4, 4, 4), 3.615, 0.0, 0.1, 71)
    elem = np.zeros_like(elem)
    masses = np.array([synth.MASS])
    _, res = ref_force(H, x, elem, masses, ["A"], path, "setfl")
    print("extrap pe", res["pe"])
    return dict(H=H, x=x, elem=elem, masses=masses, drho=EXTRAP_DRHO, **res)


def potential_case(tmp, name, root):
    rel, kind = POTENTIALS[name]
    src = os.path.join(root, rel)
    d = potfile.parse(src, kind)
    path = os.path.join(tmp, os.path.basename(src))
    potfile.write(path, d)  # the tests run on this rewrite of the file
    out = potfile.to_fixture(d)
    masses = d["masses"]
    names = d["names"]
    cells = {}
    if name == "cu":
        cells["c0"] = fcc_cell((4, 4, 4), 3.615, 0.0, 0.1, 81)
        cells["thin"] = fcc_cell((2, 2, 3), 3.615, 0.0, 0.08, 82)
        cells["dense"] = fcc_cell((5, 5, 5), 2.9, 0.0, 0.05, 83)  # host densities beyond rho_max
    elif name == "nial":
        cells["c0"] = fcc_cell((5, 5, 5), 3.52, 0.25, 0.08, 84)
        cells["tric"] = fcc_cell((5, 5, 6), 3.52, 0.5, 0.08, 85,
                                 strain=[[0.01, 0, 0], [0.02, -0.01, 0], [-0.015, 0.01, 0.004]])
    else:
        cells["c0"] = bcc_fe_h(5, 2.8553, 12, 0.05, 86)
    for cname, (H, x, elem) in cells.items():
        elem = np.asarray(elem, np.uint8)
        if name == "cu":
            elem = np.zeros_like(elem)
        r, res = ref_force(H, x, elem, masses, names, path, kind)
        out.update({cname + "/H": H, cname + "/x": x, cname + "/elem": elem})
        for k, v in res.items():
            out[cname + "/" + k] = v
        print(name, cname, x.shape[0], res["pe"] / x.shape[0])
        if name == "cu" and cname == "c0":
            rng = np.random.default_rng(87)
            v0 = synth.maxwell(rng, masses[elem], 600.0)
            r.set_state(x, v0)
            H1, x1, v1 = r.nvt(600.0, synth.FS, 40, t_relax=100.0 * synth.FS)
            out.update({"nvt/v0": v0, "nvt/x_end": x1, "nvt/v_end": v1, "nvt/T": 600.0, "nvt/nsteps": 40})
    out["cells"] = np.array(list(cells))
    return out


def main():
    root = refmod.ref_root()
    if root is None:
        raise SystemExit("set MAPPG_REFERENCE_ROOT to the reference tree")
    refmod.build(root)
    with tempfile.TemporaryDirectory() as tmp:
        np.savez_compressed(os.path.join(HERE, "ref_synth.npz"), **synth_cases(tmp))
        np.savez_compressed(os.path.join(HERE, "ref_extrap.npz"), **extrap_case(tmp))
        np.savez_compressed(os.path.join(HERE, "ref_min.npz"), **minimizer_cases(tmp))
        np.savez_compressed(os.path.join(HERE, "ref_box.npz"), **box_cases(tmp))
        np.savez_compressed(os.path.join(HERE, "ref_dof.npz"), **dof_cases(tmp))
        np.savez_compressed(os.path.join(HERE, "ref_funcfl.npz"), **funcfl_case(tmp))
        np.savez_compressed(os.path.join(HERE, "ref_cfg.npz"), **cfg_cases(tmp))
        for name in POTENTIALS:
            np.savez_compressed(os.path.join(HERE, "ref_pot_%s.npz" % name), **potential_case(tmp, name, root))


if __name__ == "__main__":
    main()
