"""The learned L-BFGS preconditioner: the tensor-core network's loss and
gradient against the CPU restatement (oracle/mlp_ref.py), the
finite-difference Hessian diagonals against the oracle's forces, training,
and what the trained network does against plain L-BFGS on held-out cells."""
import numpy as np
import pytest

import mlp_ref as R
import oracle as O
from mapp4py_gb300 import _lib, precond, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ff(potentials):
    return _lib.ForceField.setfl(potentials[("A", "B")][0])


def test_network_gradient_matches_oracle():
    rng = np.random.default_rng(1)
    net = _lib.Mlp(seed=3)
    n = 300  # two full tiles of 128 atoms and a partial one
    feat = rng.normal(size=(n, 33)).astype(np.float32) * 2.0 + 1.0
    target = np.exp(rng.normal(1.5, 0.5, size=(n, 3))).astype(np.float32)
    mean = feat.mean(axis=0).astype(np.float32)
    sdev = feat.std(axis=0).astype(np.float32)
    w, _, _ = net.params()
    w = w + rng.normal(0.0, 0.05, w.shape).astype(np.float32)  # not the initial zeros of the biases
    net.set_params(w, mean, sdev)
    loss, g = net.grad(feat, target)
    X = R.inputs(feat, mean, sdev)
    loss_ref, g_ref = R.loss_grad(w, X, target.astype(np.float64))
    assert abs(loss - loss_ref) <= 1e-4 * loss_ref
    scale = np.max(np.abs(g_ref))
    assert np.max(np.abs(g - g_ref)) <= 2e-2 * scale, np.max(np.abs(g - g_ref)) / scale
    assert np.corrcoef(g, g_ref)[0, 1] > 0.9999
    y = net.predict(feat)
    _, _, Z3 = R.forward(w, X)
    y_ref = R.softplus(Z3[:, :3])
    assert np.max(np.abs(y - y_ref) / y_ref) < 1e-2


def test_hessian_diagonal_matches_oracle_differences(ff, potentials):
    rng = np.random.default_rng(2)
    H, x, elem, col = precond.alloy_cell((4, 4, 4), rng, 0.5, 0.02, 0.05)
    s = _lib.System(ff, H, x, elem, [synth.MASS, synth.MASS])
    hd = _lib.hessian_diag(s, col, 1e-4)
    # the system is left where it was
    d = s.get_x() - x
    d -= np.round(d @ np.linalg.inv(H)) @ H
    assert np.max(np.abs(d)) < 1e-12
    e = O.Eam.setfl(potentials[("A", "B")][0])
    h = 1e-4
    for a in rng.choice(len(x), 5, replace=False):
        for ax in range(3):
            fs = []
            for sg in (1, -1):
                xp = x.copy()
                xp[a, ax] += sg * h
                o = O.System(e, H, xp, elem, [synth.MASS, synth.MASS])
                o.force()
                fs.append(o.f[a, ax])
            ref = -(fs[0] - fs[1]) / (2 * h)
            assert abs(hd[a, ax] - ref) <= 1e-6 * max(1.0, abs(ref)), (a, ax, hd[a, ax], ref)


def test_training_and_preconditioned_lbfgs(ff):
    net, losses = precond.train(ff, count=16, epochs=30, seed=5, batch=2048, n=(4, 4, 4))
    assert np.all(np.isfinite(losses)) and losses[-1] < 0.5 * losses[0]
    # held-out cells: the preconditioned run converges; its force + energy
    # evaluations are measured beside plain L-BFGS's.  On this potential a
    # diagonal H0 does not beat the scalar one (even the exact diagonal
    # needs more iterations on C5-like cells), so the bar is convergence and
    # no more than twice plain L-BFGS's evaluations, not a gain
    plain, learned = 0, 0
    for seed in range(4):
        c = synth.alloy((5, 5, 5), xB=0.4, sigma=0.1, vac=0.01, seed=100 + seed)
        s = _lib.System(ff, c.H, c.x, c.elem, c.masses)
        r0 = s.lbfgs_run(m=10, f_tol=1e-4, nsteps=5000)
        s = _lib.System(ff, c.H, c.x, c.elem, c.masses)
        r1 = _lib.lbfgs_run_precond(s, net, m=10, f_tol=1e-4, nsteps=5000)
        assert r1["err"] == 100 and r1["fmax"] < 1e-4
        plain += r0["n_force"] + r0["n_energy"]
        learned += r1["n_force"] + r1["n_energy"]
    print("force+energy evaluations, plain %d, learned %d" % (plain, learned))
    assert learned <= 2 * plain


def test_lbfgs_with_a_callers_hessian_diagonal(ff):
    """mappg_lbfgs_run_diag: H0 from a Hessian diagonal the caller supplies
    (here the exact finite-difference one), one cell and a batch; a diagonal
    that is not positive is refused."""
    rng = np.random.default_rng(17)
    masses = np.array([synth.MASS, synth.MASS])
    cells = [precond.alloy_cell((4, 4, 8), rng, 0.4, 0.01, 0.1), precond.alloy_cell((8, 4, 4), rng, 0.7, 0.02, 0.1)]
    hds = []
    for H, x, elem, col in cells:
        s = _lib.System(ff, H, x, elem, masses)
        s.build()
        hds.append(_lib.hessian_diag(s, col, 1e-4))
    H, x, elem, _ = cells[0]
    s = _lib.System(ff, H, x, elem, masses, precision=_lib.MIXED)
    r = _lib.lbfgs_run_diag(s, np.maximum(hds[0], 0.5), m=10, f_tol=1e-4, nsteps=5000)
    assert r["err"] == 100 and r["fmax"] < 1e-4
    b = _lib.Batch(ff, [(c[0], c[1], c[2]) for c in cells], masses)
    rb = _lib.lbfgs_run_diag(b, np.maximum(np.concatenate(hds), 0.5), m=10, f_tol=1e-4, nsteps=5000)
    assert len(rb) == 2 and all(q["err"] == 100 and q["fmax"] < 1e-4 for q in rb)
    bad = np.maximum(hds[0], 0.5)
    bad[3, 1] = 0.0
    with pytest.raises(_lib.MappgError, match="positive"):
        _lib.lbfgs_run_diag(s, bad)


@pytest.mark.parametrize("diag", ["mild", "wide"])
def test_diagonal_lbfgs_follows_oracle(ff, potentials, diag):
    """mappg_lbfgs_run_diag against the oracle's restatement of the same
    recursion (H0 = tau diag(1/h), tau = s.y / y.P.y of the newest pair): in
    FP64, over five iterations and over a full relaxation, the same
    iterations, energy and force calls, energies and relaxed positions.  The
    diagonals are synthetic: a mild one (3-9) and one spread over two
    decades (e^-2 - e^2); this cell's relaxation under either does not move
    when its start moves by 1e-11 A."""
    path = potentials[("A", "B")][0]
    c = synth.alloy((4, 4, 4), xB=0.3, sigma=0.1, seed=2, vac=0.01)
    k = np.arange(3 * c.natoms)
    hd = (6.0 + 3.0 * np.cos(0.7 * k) if diag == "mild" else np.exp(2.0 * np.sin(1.3 * k))).reshape(-1, 3)
    for nsteps in (5, 5000):
        o = O.System(O.Eam.setfl(path), c.H, c.x, c.elem, c.masses, skin=0.5)
        ro = o.lbfgs_run_diag(hd, m=10, e_tol=0.0, f_tol=1e-4, nsteps=nsteps)
        s = _lib.System(ff, c.H, c.x, c.elem, c.masses, skin=0.5, precision=_lib.FP64)
        r = _lib.lbfgs_run_diag(s, hd, m=10, e_tol=0.0, f_tol=1e-4, nsteps=nsteps)
        for key in ("niter", "err", "n_energy", "n_force", "fallbacks"):
            assert r[key] == ro[key], (nsteps, key, r, ro)
        assert abs(r["pe"] - ro["pe"]) <= 1e-11 * abs(ro["pe"])
        d = s.get_x() - o.x
        d -= np.round(d @ np.linalg.inv(c.H)) @ c.H
        assert np.max(np.abs(d)) < 1e-8
    assert ro["err"] == 100


@pytest.mark.parametrize("cells", [(4, 4, 4), (2, 2, 5)])
def test_descriptors_match_restatement(ff, potentials, cells):
    """k_descriptors (mappg_sys_descriptors), the network's inputs, against
    the numpy restatement (mlp_ref.descriptors): the 32 radial functions
    within FP32 rounding, the host density to the oracle's FP64 density.  The
    (2, 2, 5) cell is thinner than twice the 5.5 A range, so an atom sees
    several images of one neighbour."""
    rng = np.random.default_rng(4)
    H, x, elem, _ = precond.alloy_cell(cells, rng, 0.5, 0.0, 0.1)
    masses = [synth.MASS, synth.MASS]
    s = _lib.System(ff, H, x, elem, masses)
    s.build()
    feat = _lib.descriptors(s)
    o = O.System(O.Eam.setfl(potentials[("A", "B")][0]), H, x, elem, masses)
    o.force()
    rho, _ = o.rho_dF()
    ref = R.descriptors(H, x, elem, rho)
    scale = max(1.0, np.max(np.abs(ref[:, :32])))
    assert np.max(np.abs(feat[:, :32] - ref[:, :32])) <= 1e-5 * scale
    assert np.max(np.abs(feat[:, 32] - ref[:, 32])) <= 1e-6 * np.max(ref[:, 32])


def test_refresh_of_the_learned_diagonal(ff):
    """mappg_mlp_set_refresh: a refresh period longer than the run leaves the
    run exactly as without refresh; a period of five iterations recomputes
    the diagonal from the moved atoms, takes another path and still
    converges; a negative period is refused.  The network is untrained
    (seeded weights, inputs standardised on this cell): the refresh
    mechanics do not depend on what it predicts."""
    c = synth.alloy((4, 4, 4), xB=0.3, sigma=0.1, seed=2, vac=0.01)
    s = _lib.System(ff, c.H, c.x, c.elem, c.masses, precision=_lib.FP64)
    s.build()
    feat = _lib.descriptors(s)
    net = _lib.Mlp(seed=3)
    w, _, _ = net.params()
    net.set_params(w, feat.mean(axis=0), feat.std(axis=0) + 1e-3)

    def run(every):
        net.set_refresh(every)
        q = _lib.System(ff, c.H, c.x, c.elem, c.masses, precision=_lib.FP64)
        r = _lib.lbfgs_run_precond(q, net, m=10, f_tol=1e-4, nsteps=5000)
        return r, q.get_x()

    r0, x0 = run(0)
    rl, xl = run(100000)
    r5, x5 = run(5)
    assert r0["err"] == 100 and r5["err"] == 100
    assert rl == r0 and np.array_equal(xl, x0)
    assert (r5["niter"], r5["n_energy"], r5["pe"]) != (r0["niter"], r0["n_energy"], r0["pe"])
    with pytest.raises(_lib.MappgError):
        net.set_refresh(-1)
