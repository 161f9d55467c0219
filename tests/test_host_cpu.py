"""Host-side checks that need no GPU: the product's potential readers and
spline tables against the oracle, file errors, create_temp, and that the
C-ABI library exports every entry point its header declares."""
import os
import re
import subprocess

import numpy as np
import pytest

import oracle as O
from conftest import ROOT
from mapp4py_gb300 import _lib, md, synth


@pytest.fixture(scope="module")
def built():
    from mapp4py_gb300 import build

    build.build()
    return _lib.load()


@pytest.mark.parametrize("elems", [("A",), ("A", "B")])
def test_setfl_tables_bitwise_equal_oracle(built, potentials, elems):
    path, _ = potentials[elems]
    ff = _lib.ForceField.setfl(path)
    ref = O.Eam.setfl(path).tables()
    for a, b in zip(ff.tables(), ref):
        assert np.array_equal(a, b)
    F, rho, rphi, cut = ff.tables()
    # cutoff = last knot where any table is nonzero (5.5 A switch, dr = 5.5/5000)
    assert np.allclose(cut, 4999 * 5.5 / 5000, rtol=0, atol=1e-15)


def test_knot_tables_match_setfl(built, potentials):
    path, _ = potentials[("A", "B")]
    dr, drho, F, rho, rphi = synth.analytic_knots(("A", "B"))
    rho2 = np.stack([rho, rho], axis=1)  # setfl: rho[i][j] = rho_i for every j
    ff = _lib.ForceField.knots(5000, 5000, dr, drho, F, rho2, rphi)
    ref = _lib.ForceField.setfl(path).tables()
    for a, b in zip(ff.tables(), ref):
        assert np.allclose(a, b, rtol=1e-13, atol=1e-15)


def test_element_selection_and_order(built, potentials):
    path, _ = potentials[("A", "B")]
    ff = _lib.ForceField.setfl(path, ["B", "A"])
    assert ff.names == ["B", "A"]
    F, rho, rphi, cut = ff.tables()
    F0, rho0, rphi0, cut0 = _lib.ForceField.setfl(path).tables()
    assert np.array_equal(F[0], F0[1]) and np.array_equal(rphi[0, 0], rphi0[1, 1])
    assert np.array_equal(rphi[0, 1], rphi0[1, 0])
    with pytest.raises(_lib.MappgError) as ei:
        _lib.ForceField.setfl(path, ["C"])
    assert "element C" in str(ei.value)


def test_malformed_setfl_is_rejected(built, potentials, tmp_path):
    path, _ = potentials[("A",)]
    lines = open(path).read().splitlines(True)
    bad = tmp_path / "trunc.setfl"
    bad.write_text("".join(lines[: len(lines) // 2]))
    with pytest.raises(_lib.MappgError) as ei:
        _lib.ForceField.setfl(str(bad))
    assert ei.value.code == -3 and "immaturely" in str(ei.value)
    extra = tmp_path / "extra.setfl"
    k = 7
    extra.write_text("".join(lines[:k]) + lines[k].rstrip("\n") + " 1.0\n" + "".join(lines[k + 1:]))
    with pytest.raises(_lib.MappgError) as ei:
        _lib.ForceField.setfl(str(extra))
    assert "extra arguments" in str(ei.value)
    with pytest.raises(_lib.MappgError):
        _lib.ForceField.setfl(str(tmp_path / "missing.setfl"))


def test_create_temp_matches_oracle(built):
    elem = (np.arange(1000) % 2).astype(np.uint8)
    masses = [63.5, 40.0]
    v = _lib.create_temp(elem, masses, 300.0, synth.KB, 846244)
    vo = O.create_temp(elem, masses, 300.0, synth.KB, 846244)
    assert np.array_equal(v, vo)
    with pytest.raises(_lib.MappgError):
        _lib.create_temp(elem, masses, 300.0, synth.KB, 0)


def test_library_exports_every_declared_symbol(built):
    hdr = open(os.path.join(ROOT, "include", "mappg.h")).read()
    declared = set(re.findall(r"\b(mappg_[a-z0-9_]+)\s*\(", hdr))
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(l.split()[-1] for l in out.splitlines() if " T mappg_" in l)
    assert declared and declared <= exported, sorted(declared - exported)
    assert declared == set(_lib.SIGNATURES), sorted(declared ^ set(_lib.SIGNATURES))
    L = _lib.load()
    for name in declared:
        assert hasattr(L, name)


def test_gcmc_hooks_report_unsupported(built):
    L = built
    for name, args in (("mappg_sys_init_xchng", (None,)), ("mappg_sys_fin_xchng", (None,)),
                       ("mappg_sys_pre_xchng_energy", (None, None)),
                       ("mappg_sys_xchng_energy", (None, None, None)),
                       ("mappg_sys_post_xchng_energy", (None, None))):
        assert getattr(L, name)(*args) == -8  # MAPPG_ERR_UNSUPP
        assert b"GCMC" in L.mappg_last_error()


def test_h_dof_forms():
    from mapp4py_gb300 import md

    m = md.min_lbfgs(H_dof=[[True], [False, True], [False, False, True]])
    assert m.H_dof.tolist() == np.eye(3, dtype=bool).tolist() and m._box()
    full = np.ones((3, 3), dtype=bool)
    assert md.min_cg(H_dof=full).H_dof.tolist() == np.tril(full).tolist()
    assert not md.min_lbfgs()._box() and md.min_cg(affine=True)._box()
    with pytest.raises(TypeError):
        md.min_lbfgs(H_dof=[[True, False]])


def test_api_surface_mirrors_reference(built):
    from mapp4py_gb300 import md, ls_bt

    n = md.nvt(300.0, 0.1)
    assert (n.t_relax, n.L, n.niters, n.ntally) == (10.0, 3, 1, 10000)
    m = md.min_lbfgs()
    assert m.m == 2 and m.max_dx == 1.0 and abs(m.e_tol - 2 ** -26) < 1e-20
    ls = ls_bt()
    assert (ls.c, ls.rho, ls.min_alpha) == (0.4, 0.5, 0.0)
    with pytest.raises(TypeError):
        md.nvt(-1.0, 0.1)
    H, x = synth.fcc((4, 4, 4))
    a = md.atoms(H, x, np.zeros(len(x), np.uint8))
    with pytest.raises(TypeError):
        a.create_temp(300.0, 1)  # kB not set


def test_create_temp_dof_matches_oracle(built):
    """create_temp with x_dof: free components drawn in order, the others
    keep their value (atoms_md.cpp:138-149)."""
    elem = (np.arange(600) % 2).astype(np.uint8)
    masses = [63.5, 40.0]
    rng = np.random.default_rng(1)
    dof = rng.random((600, 3)) > 0.25
    v0 = rng.normal(size=(600, 3))
    v = _lib.create_temp_dof(elem, masses, dof, 300.0, synth.KB, 846244, v0)
    vo = O.create_temp_dof(elem, masses, dof, 300.0, synth.KB, 846244, v0)
    assert np.array_equal(v, vo) and np.array_equal(v[~dof], v0[~dof])
    # all free: the plain draw
    assert np.array_equal(_lib.create_temp_dof(elem, masses, np.ones((600, 3), bool), 300.0, synth.KB, 9, v0),
                          _lib.create_temp(elem, masses, 300.0, synth.KB, 9))
    a = md.atoms(np.eye(3) * 10.0, rng.random((600, 3)) * 10.0, elem, elems=("A", "B"), masses=masses)
    a.kB = synth.KB
    a.x_d = v0.copy()
    a.x_dof = dof
    a.create_temp(300.0, 846244)
    assert np.array_equal(a.x_d, vo)
    a.x_dof = np.ones((5, 3), bool)
    with pytest.raises(TypeError):
        a.create_temp(300.0, 1)


class _FakeSystem:
    """Stands in for _lib.System in md.nvt.run's host logic: records the
    call and writes recognisable outputs."""

    def __init__(self, n):
        self.n = n
        self.calls = []

    def nvt_run_host(self, x, v, T, dt, kB, nsteps, t_relax=None, L=3, niters=1, eta=None, thermo=False,
                     x_out=None, v_out=None, f_out=None):
        self.calls.append(dict(x=np.array(x), v=np.array(v), nsteps=nsteps, thermo=thermo, L=L, eta=np.array(eta)))
        x_out[:] = x + 1.0
        v_out[:] = v * 2.0
        f_out[:] = 3.0
        th = np.zeros((nsteps + 1, 14))
        th[-1, 0] = -7.5
        th[-1, 8:14] = [1.0, 0.1, 0.2, 2.0, 0.3, 3.0]
        return th, np.full(L, 0.25)


def test_md_nvt_run_host_logic(monkeypatch):
    """md.nvt.run without an export: one nvt_run_host call; the atoms'
    arrays are refilled in place when they are C-contiguous float64 (n, 3),
    replaced otherwise; pe and S_pe come from the last thermo row; the chain
    state is carried; step advances."""
    n = 6
    H = np.diag([10.0, 11.0, 12.0])
    x = np.arange(3 * n, dtype=np.float64).reshape(n, 3)
    a = md.atoms(H, x, np.zeros(n, np.uint8), masses=(50.0,), x_d=np.ones((n, 3)))
    a.kB = synth.KB
    a.ff = object()
    fake = _FakeSystem(n)
    monkeypatch.setattr(a, "_system", lambda: fake)
    x_obj, v_obj = a.x, a.x_d
    a.f = np.zeros((n, 3))
    f_obj = a.f
    integ = md.nvt(300.0, synth.FS)
    integ.ntally = 0
    integ.run(a, 3)
    assert len(fake.calls) == 1 and fake.calls[0]["nsteps"] == 3 and fake.calls[0]["thermo"]
    assert a.x is x_obj and a.x_d is v_obj and a.f is f_obj  # refilled in place
    assert np.array_equal(a.x, x + 1.0) and np.all(a.x_d == 2.0) and np.all(a.f == 3.0)
    assert a.pe == -7.5 and a.step == 3
    vol = 10.0 * 11.0 * 12.0
    assert np.allclose(a.S_pe, -np.array([[1.0, 0.1, 0.2], [0.1, 2.0, 0.3], [0.2, 0.3, 3.0]]) / vol)
    assert np.all(integ._eta == 0.25)
    integ.run(a, 2)
    assert np.all(fake.calls[1]["eta"] == 0.25) and a.step == 5  # the chain state carries over
    # arrays that cannot take the result in place are replaced
    a.x = np.asfortranarray(a.x)
    a.x_d = a.x_d.astype(np.float32)
    xf = a.x.copy()
    integ.run(a, 1)
    assert a.x.flags.c_contiguous and a.x.dtype == np.float64 and np.array_equal(a.x, xf + 1.0)
    assert a.x_d.dtype == np.float64


def test_system_download_targets_are_checked():
    """System._get refuses an output array it would fill in the wrong layout
    (no device work is reached: the check comes first)."""
    s = _lib.System.__new__(_lib.System)
    s.n = 4
    s.h = None
    for bad in (np.zeros((4, 3), np.float32), np.asfortranarray(np.zeros((4, 3))), np.zeros((5, 3)),
                np.zeros((4, 3))[:, :2]):
        with pytest.raises(ValueError):
            s._get(None, bad)
