"""The golden-section and Brent line searches (ls_golden, ls_brent;
ls.h:214-706) in the device L-BFGS and CG minimizers against the oracle's
restatement: the same trial sequence (energy-call counts), energies and
positions over the first iterations, and the same outcome of full runs; the
md-level minimizers accept all three line searches."""
import numpy as np
import pytest

import oracle as O
from mapp4py_gb300 import _lib, ls_brent, ls_bt, ls_golden, md, synth

pytestmark = pytest.mark.gpu

KINDS = {"golden": _lib.LS_GOLDEN, "brent": _lib.LS_BRENT}


def cell():
    return synth.alloy((4, 4, 4), xB=0.3, sigma=0.1, seed=2, vac=0.01)


def run_pair(path, kind, bracket, minimizer, nsteps):
    c = cell()
    o = O.System(O.Eam.setfl(path), c.H, c.x, c.elem, c.masses, skin=0.5)
    s = _lib.System(_lib.ForceField.setfl(path), c.H, c.x, c.elem, c.masses, skin=0.5, precision=_lib.FP64)
    ols = O.line_search(kind, bracket=bracket)
    gls = _lib.line_search(KINDS[kind], bracket=bracket)
    if minimizer == "lbfgs":
        ro = o.lbfgs_run_ls(ols, m=10, e_tol=0.0, f_tol=1e-4, nsteps=nsteps)
        r = s.lbfgs_run_ls(gls, m=10, e_tol=0.0, f_tol=1e-4, nsteps=nsteps)
    else:
        ro = o.cg_run_ls(ols, e_tol=0.0, f_tol=1e-4, nsteps=nsteps)
        r = s.cg_run_ls(gls, e_tol=0.0, f_tol=1e-4, nsteps=nsteps)
    d = s.get_x() - o.x
    d -= np.round(d @ np.linalg.inv(c.H)) @ c.H
    return r, ro, np.max(np.abs(d))


def same(r, ro):
    return (r["niter"], r["err"], r["n_energy"], r["n_force"]) == (ro["niter"], ro["err"], ro["n_energy"],
                                                                   ro["n_force"])


@pytest.mark.parametrize("minimizer", ["lbfgs", "cg"])
@pytest.mark.parametrize("bracket", [True, False])
@pytest.mark.parametrize("kind", ["golden", "brent"])
def test_line_search_follows_oracle(potentials, kind, bracket, minimizer):
    path, _ = potentials[("A", "B")]
    if kind == "brent" and bracket:
        # Brent refines the step to tol*|x| (tol = sqrt(2 eps)), where energy
        # differences sink below rounding: the oracle's own energy-call count
        # over six iterations moves by a few calls when the start moves by
        # 1e-13 A.  The first iteration is exact; six agree to that spread.
        r, ro, dx = run_pair(path, kind, bracket, minimizer, 1)
        assert same(r, ro) and abs(r["pe"] - ro["pe"]) <= 1e-12 * abs(ro["pe"]) and dx < 1e-8
        r, ro, dx = run_pair(path, kind, bracket, minimizer, 6)
        assert (r["niter"], r["err"], r["n_force"]) == (ro["niter"], ro["err"], ro["n_force"])
        assert abs(r["n_energy"] - ro["n_energy"]) <= 6
        assert abs(r["pe"] - ro["pe"]) <= 1e-10 * abs(ro["pe"])
    else:
        r, ro, dx = run_pair(path, kind, bracket, minimizer, 6)
        assert same(r, ro)
        assert abs(r["pe"] - ro["pe"]) <= 1e-11 * abs(ro["pe"]) and dx < 1e-9
    r, ro, dx = run_pair(path, kind, bracket, minimizer, 5000)
    assert r["err"] == ro["err"]
    if bracket:
        # with bracketing this cell relaxes to max|F| < 1e-4 (stop code 100)
        assert ro["err"] == 100
        assert r["fmax"] < 1e-4 and abs(r["pe"] - ro["pe"]) <= 1e-9 * abs(ro["pe"])
    else:
        # without it the search on this cell fails a few iterations in (line-search
        # stop LS_MIN_ALPHA, code 3): the same stop at the same iteration and energy
        assert ro["err"] == 3 and ro["niter"] < 10
        assert r["niter"] == ro["niter"] and abs(r["pe"] - ro["pe"]) <= 1e-10 * abs(ro["pe"])


def test_md_minimizers_take_every_line_search(potentials):
    path, _ = potentials[("A", "B")]
    pes = []
    for ls in (ls_bt(), ls_golden(), ls_brent()):
        for cls in (md.min_lbfgs, md.min_cg):
            c = cell()
            a = md.atoms(c.H, c.x, c.elem, elems=("A", "B"), masses=c.masses)
            a.ff_eam_setfl(path)
            m = cls(e_tol=0.0, ls=ls, f_tol=1e-4) if cls is md.min_cg else cls(m=10, e_tol=0.0, ls=ls, f_tol=1e-4)
            r = m.run(a, 5000)
            assert r["err"] == 100, (type(ls).__name__, cls.__name__, r)
            pes.append(a.pe)
    assert max(pes) - min(pes) < 1e-6 * abs(pes[0])
    with pytest.raises(TypeError):
        md.min_lbfgs(ls=object()).run(a, 1)


@pytest.mark.parametrize("kind,minimizer", [("brent", "lbfgs"), ("golden", "cg")])
def test_mixed_precision_line_searches(potentials, kind, minimizer):
    """Golden-section and Brent searches on a mixed-precision system (FP64
    trial energies, FP32-computed forces): the run reaches max|F| < 1e-4 at
    the FP64 run's energy."""
    path, _ = potentials[("A", "B")]
    c = cell()
    out = {}
    for prec in (_lib.FP64, _lib.MIXED):
        s = _lib.System(_lib.ForceField.setfl(path), c.H, c.x, c.elem, c.masses, skin=0.5, precision=prec)
        ls = _lib.line_search(KINDS[kind])
        if minimizer == "lbfgs":
            out[prec] = s.lbfgs_run_ls(ls, m=10, e_tol=0.0, f_tol=1e-4, nsteps=5000)
        else:
            out[prec] = s.cg_run_ls(ls, e_tol=0.0, f_tol=1e-4, nsteps=5000)
    r64, r32 = out[_lib.FP64], out[_lib.MIXED]
    assert r64["err"] == 100 and r32["err"] == 100
    assert r32["fmax"] < 1e-4
    # the mixed-precision energy budget (1e-7 eV/atom against FP64)
    assert abs(r32["pe"] - r64["pe"]) / c.natoms < 1e-7
