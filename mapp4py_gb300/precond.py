"""Training data and training of the learned L-BFGS preconditioner.

The network (libmappg: mappg_mlp_*) maps 33 local features of an atom to its
three diagonal Hessian elements.  Its training set comes from the method's
own runs: configurations of random A/B alloy cells taken from NVT MD at
300-1500 K and from partial L-BFGS relaxations, each labelled with
finite-difference Hessian diagonals (central differences of the FP64
forces, step 1e-4 A) computed on the GPU.

Finite differences move many atoms at once: atoms of one colour are at
least four FCC repeats (14.5 A, more than twice the 5.5 A cutoff) apart, so
the force change on a moved atom comes from its own displacement only.
The colour of an atom is (i0 mod 4, i1 mod 4, i2 mod 4, basis) of its
lattice site, which needs cells with a multiple of 4 repeats per axis.
"""
import numpy as np

from . import _lib, synth


def fcc_sites(n):
    """Lattice indices (i0, i1, i2, basis) of synth.fcc(n)'s atoms, in its order."""
    n0, n1, n2 = n
    g = np.stack(np.meshgrid(np.arange(n0), np.arange(n1), np.arange(n2), indexing="ij"), -1).reshape(-1, 3)
    idx = np.repeat(g, 4, axis=0)
    basis = np.tile(np.arange(4), g.shape[0])
    return np.column_stack([idx, basis])


def site_colors(sites):
    """256 colours: same-coloured sites are 4 repeats apart on every axis."""
    i = sites
    return (((i[:, 0] % 4) * 16 + (i[:, 1] % 4) * 4 + (i[:, 2] % 4)) * 4 + i[:, 3]).astype(np.int32)


def alloy_cell(n, rng, xB, vac, sigma):
    """An A/B FCC alloy cell with vacancies and noise, and its atoms' colours."""
    H, x = synth.fcc(n)
    sites = fcc_sites(n)
    keep = rng.random(x.shape[0]) >= vac
    x, sites = x[keep], sites[keep]
    elem = (rng.random(x.shape[0]) < xB).astype(np.uint8)
    x = synth.wrap(H, x + rng.normal(0.0, sigma, x.shape))
    return H, x, elem, site_colors(sites)


def snapshots(ff, count, seed=0, n=(8, 8, 8), temps=(300.0, 1500.0), md_steps=(50, 300), relax_steps=(5, 200)):
    """Configurations for training: half from NVT MD at T in temps, half from
    partial L-BFGS relaxations of noisy cells.  Yields (H, x, elem, colour)."""
    rng = np.random.default_rng(seed)
    masses = np.array([synth.MASS, synth.MASS])
    for k in range(count):
        xB = rng.uniform(0.0, 1.0)
        vac = rng.uniform(0.0, 0.03)
        if k % 2 == 0:
            H, x, elem, col = alloy_cell(n, rng, xB, vac, 0.05)
            T = rng.uniform(*temps)
            s = _lib.System(ff, H, x, elem, masses, precision=_lib.MIXED)
            s.set_v(synth.maxwell(rng, masses[elem], T))
            s.nvt_run(T, synth.FS, synth.KB, int(rng.integers(*md_steps)))
        else:
            H, x, elem, col = alloy_cell(n, rng, xB, vac, rng.uniform(0.05, 0.2))
            s = _lib.System(ff, H, x, elem, masses)
            s.lbfgs_run(m=10, f_tol=0.0, nsteps=int(rng.integers(*relax_steps)))
        yield H, s.get_x(), elem, col


def label(ff, H, x, elem, col, h=1e-4):
    """Features and finite-difference Hessian diagonals of one configuration."""
    s = _lib.System(ff, H, x, elem, np.array([synth.MASS, synth.MASS]))
    s.build()
    return _lib.descriptors(s), _lib.hessian_diag(s, col, h)


def training_set(ff, count, seed=0, n=(8, 8, 8)):
    feats, targets = [], []
    for H, x, elem, col in snapshots(ff, count, seed, n):
        f, t = label(ff, H, x, elem, col)
        feats.append(f)
        targets.append(t)
    return np.concatenate(feats), np.concatenate(targets)


def train(ff, count=100, epochs=40, seed=0, batch=4096, lr=2e-3, wd=1e-4, n=(8, 8, 8)):
    """Generate a training set of `count` configurations and fit a network;
    returns (network, per-epoch losses)."""
    feat, target = training_set(ff, count, seed, n)
    net = _lib.Mlp(seed)
    net.set_data(feat, target, seed)
    losses = net.train(epochs, batch, lr, wd)
    return net, losses


WEIGHTS = __file__.replace("precond.py", "precond_net.npz")


def save(net, path=WEIGHTS, **meta):
    w, mean, sdev = net.params()
    np.savez(path, w=w, mean=mean, sdev=sdev, **meta)


def load(path=WEIGHTS, seed=0):
    """The network stored by `python -m mapp4py_gb300.precond` (trained on
    the GPU by this package's kernels)."""
    d = np.load(path)
    net = _lib.Mlp(seed)
    net.set_params(d["w"], d["mean"], d["sdev"])
    return net


if __name__ == "__main__":
    import argparse
    import os
    import tempfile
    import time

    ap = argparse.ArgumentParser(description="train the L-BFGS preconditioner network and store it")
    ap.add_argument("--configs", type=int, default=100, help="training configurations of 2048 atoms")
    ap.add_argument("--epochs", type=int, default=40)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--out", default=WEIGHTS)
    args = ap.parse_args()
    with tempfile.TemporaryDirectory() as d:
        path = synth.write_setfl(os.path.join(d, "AB.setfl"), ("A", "B"))
        ff = _lib.ForceField.setfl(path)
        t0 = time.time()
        feat, target = training_set(ff, args.configs, args.seed)
        t1 = time.time()
        net = _lib.Mlp(args.seed)
        net.set_data(feat, target, args.seed)
        losses = net.train(args.epochs)
        t2 = time.time()
        save(net, args.out, rows=feat.shape[0], losses=losses, label_seconds=t1 - t0, train_seconds=t2 - t1)
        print("rows %d, labels %.1f s, training %.1f s, loss %.4f -> %.4f" %
              (feat.shape[0], t1 - t0, t2 - t1, losses[0], losses[-1]))
