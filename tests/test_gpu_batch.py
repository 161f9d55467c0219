"""Batches of independent cells (mappg_batch_*) against the same cells run
one at a time: neighbour sets, forces, energies, virials and NVT
trajectories, plus the mixed-precision error budget against the oracle."""
import numpy as np
import pytest

import oracle as O
from mapp4py_gb300 import _lib, synth

pytestmark = pytest.mark.gpu


def _cells():
    # orthorhombic cells of uneven size and composition, and strained
    # (triclinic) ones, some small enough for 1-2 bins per axis
    a, Ta = synth.batch_cells(4, seed=5, nmin=300, nmax=4000)
    b, Tb = synth.batch_cells(3, seed=6, nmin=300, nmax=2500, strain=0.02)
    return a + b, np.concatenate([Ta, Tb])


def _keys(cnt, ent):
    atom = np.repeat(np.arange(cnt.shape[0]), cnt)
    rows = np.column_stack([atom, ent]).astype(np.int64)
    return rows[np.lexsort(rows.T[::-1])]


@pytest.fixture(scope="module")
def ff(potentials):
    return _lib.ForceField.setfl(potentials[("A", "B")][0])


def test_batch_forces_match_single_cells(ff):
    cells, _ = _cells()
    b = _lib.Batch(ff, [(c.H, c.x, c.elem) for c in cells], cells[0].masses)
    pe, vir = b.force()
    f = b.split(b.get_f())
    cnt, ent = b.neighbors()
    off = b.offsets
    for k, c in enumerate(cells):
        s = _lib.System(ff, c.H, c.x, c.elem, c.masses, precision=_lib.MIXED)
        pe1, vir1 = s.force()
        # same rows, same order, same arithmetic: forces agree bit for bit
        assert np.array_equal(f[k], s.get_f())
        # energies and virials are FP32 sums per thread over other sets of
        # atoms (chunks instead of a grid stride): equal well inside the
        # mixed-precision budget, not bit for bit
        assert abs(pe[k] - pe1) / c.natoms < 1e-8
        assert np.max(np.abs(vir[k] - vir1)) <= 1e-6 * np.max(np.abs(vir1))
        # the cell's neighbour set, in its own atom numbering
        sel = slice(off[k], off[k + 1])
        first = int(cnt[:off[k]].sum())
        ek = ent[first:first + int(cnt[sel].sum())].copy()
        ek[:, 0] -= off[k]
        assert np.array_equal(_keys(cnt[sel], ek), _keys(*s.neighbors()))


def test_batch_mixed_error_against_oracle(ff, potentials):
    cells, _ = _cells()
    b = _lib.Batch(ff, [(c.H, c.x, c.elem) for c in cells], cells[0].masses)
    pe, _ = b.force()
    f = b.split(b.get_f())
    e = O.Eam.setfl(potentials[("A", "B")][0])
    for k, c in enumerate(cells):
        o = O.System(e, c.H, c.x, c.elem, c.masses)
        pe_o, _ = o.force()
        rms = np.sqrt(np.mean(np.sum((f[k] - o.f) ** 2, axis=1)))
        assert rms < 1e-5, rms
        assert abs(pe[k] - pe_o) / c.natoms < 1e-7


def test_batch_nvt_follows_single_cell_runs(ff):
    cells, T = _cells()
    b = _lib.Batch(ff, [(c.H, c.x, c.elem) for c in cells], cells[0].masses)
    b.set_v(np.concatenate([c.v for c in cells]))
    dt = synth.FS
    th, eta = b.nvt_run(T, dt, synth.KB, 20, thermo=True)
    xb = b.split(b.get_x())
    vb = b.split(b.get_v())
    assert th.shape == (21, len(cells), 2) and np.all(np.isfinite(th))
    for k, c in enumerate(cells):
        s = _lib.System(ff, c.H, c.x, c.elem, c.masses, precision=_lib.MIXED)
        s.set_v(c.v)
        th1, eta1 = s.nvt_run(T[k], dt, synth.KB, 20, thermo=True)
        # the per-cell totals are summed in another order than the single
        # cell's, and FP32 forces carry the last-bit differences along: the
        # runs agree within the mixed-precision budget, not bit for bit
        assert np.max(np.abs(th[:, k, 0] - th1[:, 0])) / c.natoms < 1e-7
        assert np.max(np.abs(th[:, k, 1] - th1[:, 1])) <= 1e-5 * np.max(th1[:, 1])
        assert np.max(np.abs(eta[k] - eta1)) <= 1e-6 * max(1.0, np.max(np.abs(eta1)))
        d = xb[k] - s.get_x()
        d -= np.round(d @ np.linalg.inv(c.H)) @ c.H
        assert np.max(np.abs(d)) < 1e-5
        v1 = s.get_v()
        assert np.max(np.abs(vb[k] - v1)) < 1e-5 * np.max(np.abs(v1))


def _cell_keys(b, k):
    """cell k's neighbour set in its own atom numbering"""
    cnt, ent = b.neighbors()
    off = b.offsets
    sel = slice(off[k], off[k + 1])
    first = int(cnt[:off[k]].sum())
    ek = ent[first:first + int(cnt[sel].sum())].copy()
    ek[:, 0] -= off[k]
    return _keys(cnt[sel], ek)


def test_batch_rebuilds_only_cells_that_moved(ff):
    """A hot cell that needs list rebuilds does not rebuild a cold cell of
    the same batch: the cold cell keeps the list of its start positions
    (still valid: no atom moved skin/2), although a list built at its final
    positions differs.  The single-cell runs rebuild the same way."""
    hot = synth.alloy((5, 5, 5), xB=0.5, sigma=0.05, T=2500.0, seed=41)
    # the cold cell's fifth neighbour shell sits at the list radius (a sqrt(5/2)
    # = 6.0 A = cutoff + skin), so any motion changes which pairs a fresh list
    # holds, while at 20 K no atom moves skin/2 in 40 steps
    cold = synth.alloy((6, 5, 5), a=6.0 / np.sqrt(2.5), xB=0.5, sigma=0.02, T=20.0, seed=42)
    b = _lib.Batch(ff, [(c.H, c.x, c.elem) for c in (hot, cold)], hot.masses)
    b.build()
    k_hot0, k_cold0 = _cell_keys(b, 0), _cell_keys(b, 1)
    b.set_v(np.concatenate([hot.v, cold.v]))
    b.nvt_run(np.array([2500.0, 20.0]), synth.FS, synth.KB, 40)
    assert not np.array_equal(_cell_keys(b, 0), k_hot0)  # the hot cell was rebuilt
    assert np.array_equal(_cell_keys(b, 1), k_cold0)  # the cold one kept its list
    xc = b.split(b.get_x())[1]
    fresh = _lib.System(ff, cold.H, xc, cold.elem, cold.masses, precision=_lib.MIXED)
    assert not np.array_equal(_keys(*fresh.neighbors()), k_cold0)  # the test has teeth
    s = _lib.System(ff, cold.H, cold.x, cold.elem, cold.masses, precision=_lib.MIXED)
    s.set_v(cold.v)
    s.nvt_run(20.0, synth.FS, synth.KB, 40)
    assert np.array_equal(_keys(*s.neighbors()), k_cold0)
    d = xc - s.get_x()
    d -= np.round(d @ np.linalg.inv(cold.H)) @ cold.H
    assert np.max(np.abs(d)) < 1e-5


def test_batch_capacity_grows_and_cells_keep_their_lists(ff):
    """A dense slab in one cell overflows the rows sized from the batch's
    mean density: the build regrows them for every cell, and each cell's
    neighbour set and forces equal the cell's own run alone."""
    masses = np.array([synth.MASS, synth.MASS])
    normal = synth.alloy((4, 4, 4), xB=0.5, sigma=0.05, seed=51)
    _, xs = synth.fcc((4, 4, 4), a=3.0)  # a dense slab in a box 4x longer
    Hs = np.diag([48.0, 12.0, 12.0])
    es = np.zeros(len(xs), np.uint8)
    cells = [(normal.H, normal.x, normal.elem), (Hs, xs, es)]
    b = _lib.Batch(ff, cells, masses)
    cap0 = b.stats()["capacity"]
    b.force()
    assert b.stats()["capacity"] > cap0
    f = b.split(b.get_f())
    for k, (H, x, elem) in enumerate(cells):
        s = _lib.System(ff, H, x, elem, masses, precision=_lib.MIXED)
        s.force()
        assert np.array_equal(_cell_keys(b, k), _keys(*s.neighbors()))
        assert np.array_equal(f[k], s.get_f())


def test_batch_autotune_keeps_forces_and_runs(ff):
    """The batch autotuner (atoms per chunk x lanes per atom x entries per
    step) changes how the work is cut, not the result: forces agree to FP32
    rounding (another lanes-per-atom choice sums each row in other lane
    partials), totals to rounding; an NVT run of more than 8 steps (its steps
    captured as one graph) equals the same steps run one by one, bit for
    bit."""
    cells, T = _cells()
    b = _lib.Batch(ff, [(c.H, c.x, c.elem) for c in cells], cells[0].masses)
    pe0, vir0 = b.force()
    f0 = b.get_f()
    tpa, unroll, tune = b.autotune()
    assert b.chunk_atoms in (128, 256, 512) and len(tune) == 21
    pe1, vir1 = b.force()
    assert np.max(np.abs(b.get_f() - f0)) <= 1e-5 * max(1.0, np.max(np.abs(f0)))
    assert np.max(np.abs(pe1 - pe0) / np.abs(pe0)) < 1e-9
    v = np.concatenate([c.v for c in cells])
    runs = []
    for k in (12, None):
        c = _lib.Batch(ff, [(q.H, q.x, q.elem) for q in cells], cells[0].masses)
        c.set_v(v)
        if k is None:
            c.nvt_begin(T, synth.FS, synth.KB, 12)
            for _ in range(12):
                c.nvt_steps(1)
            c.nvt_end(12)
        else:
            c.nvt_run(T, synth.FS, synth.KB, k)
        runs.append((c.get_x(), c.get_v()))
    assert np.array_equal(runs[0][0], runs[1][0]) and np.array_equal(runs[0][1], runs[1][1])


def test_batch_refuses_single_cell_calls(ff):
    cells, _ = _cells()
    b = _lib.Batch(ff, [(c.H, c.x, c.elem) for c in cells[:2]], cells[0].masses)
    with pytest.raises(_lib.MappgError):
        _lib.System.force(b)
    with pytest.raises(_lib.MappgError):
        _lib.System.nvt_run(b, 300.0, synth.FS, synth.KB, 1)
    with pytest.raises(_lib.MappgError):
        _lib.Batch(ff, [(c.H, c.x, c.elem) for c in cells[:2]], cells[0].masses, precision=_lib.FP64)


def test_batch_lbfgs_follows_single_cells(ff):
    """Each cell of a batched relaxation runs the single-cell iteration: the
    first iterations agree with mappg_lbfgs_run on the cell alone to
    rounding, and well-conditioned cells all reach the force tolerance."""
    cells = [synth.alloy((4, 4, 4), xB=0.3, sigma=0.1, seed=2 + k, vac=0.01) for k in range(3)]
    cells += [synth.alloy((3, 4, 5), xB=0.6, sigma=0.08, seed=9, vac=0.0)]
    b = _lib.Batch(ff, [(c.H, c.x, c.elem) for c in cells], cells[0].masses)
    r5 = b.lbfgs_run(m=10, f_tol=1e-4, nsteps=5)
    for k, c in enumerate(cells):
        s = _lib.System(ff, c.H, c.x, c.elem, c.masses, precision=_lib.MIXED)
        s5 = s.lbfgs_run(m=10, f_tol=1e-4, nsteps=5)
        assert r5[k]["niter"] == s5["niter"] and r5[k]["n_energy"] == s5["n_energy"]
        assert abs(r5[k]["pe"] - s5["pe"]) / c.natoms < 1e-7
    b = _lib.Batch(ff, [(c.H, c.x, c.elem) for c in cells], cells[0].masses)
    r = b.lbfgs_run(m=10, f_tol=1e-4, nsteps=3000)
    for k, c in enumerate(cells):
        assert r[k]["err"] == 100 and r[k]["fmax"] < 1e-4, r[k]
