"""Regenerate the golden fixtures in this folder from the CPU oracle.

    python tests/golden/make_golden.py

Each case is a small seeded cell on the analytic EAM potential of
mapp4py_gb300.synth (setfl, nr = nrho = 5000); the potential file is written
afresh and its SHA-256 is stored so a test can tell that it rebuilt the same
tables.  Fixtures hold the oracle's forces, energy, virial, host densities,
full neighbour sets, a short NVT trajectory and an L-BFGS relaxation.
"""
import hashlib
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from mapp4py_gb300 import synth  # noqa: E402
import oracle as O  # noqa: E402


def potential(tmpdir, elems):
    path = os.path.join(tmpdir, "%s.setfl" % "".join(elems))
    synth.write_setfl(path, elems)
    with open(path, "rb") as fh:
        digest = hashlib.sha256(fh.read()).hexdigest()
    return path, digest


def cases():
    """name -> (elements, Cell) for the static force/neighbour cases."""
    out = {}
    c = synth.alloy((4, 4, 4), xB=0.0, sigma=0.1, seed=11)
    out["fcc_a_256"] = (("A",), synth.Cell(c.H, c.x, np.zeros(c.natoms, np.uint8), c.v, ("A",), [synth.MASS]))
    out["alloy_ab_475"] = (("A", "B"), synth.alloy((5, 5, 5), xB=0.4, sigma=0.12, vac=0.05, seed=12))
    c = synth.alloy((2, 2, 2), xB=0.0, sigma=0.08, seed=13)
    out["thin_a_32"] = (("A",), synth.Cell(c.H, c.x, np.zeros(c.natoms, np.uint8), c.v, ("A",), [synth.MASS]))
    c = synth.alloy((4, 3, 5), xB=0.5, sigma=0.1, strain=[[0.01, 0, 0], [0.015, -0.01, 0], [-0.02, 0.01, 0.005]],
                    seed=14)
    out["tric_ab_240"] = (("A", "B"), c)
    return out


def neighbor_keys(cnt, ent):
    """Sorted (atom, owner, n0, n1, n2) rows of a full list."""
    atom = np.repeat(np.arange(cnt.shape[0]), cnt)
    rows = np.column_stack([atom, ent]).astype(np.int64)
    order = np.lexsort(rows.T[::-1])
    return rows[order]


def main():
    with tempfile.TemporaryDirectory() as tmp:
        pots = {}
        for elems in (("A",), ("A", "B")):
            pots[elems] = potential(tmp, elems)
        for name, (elems, c) in cases().items():
            path, digest = pots[elems]
            e = O.Eam.setfl(path)
            s = O.System(e, c.H, c.x, c.elem, c.masses, skin=0.5, pair_wise=True)
            pe, vir = s.force()
            f = s.f
            rho, dF = s.rho_dF()
            ef = s.energy()
            full = O.System(e, c.H, c.x, c.elem, c.masses, skin=0.5, pair_wise=False)
            full.init_dynamic()
            keys = neighbor_keys(*full.neighbors())
            np.savez_compressed(os.path.join(HERE, name + ".npz"), H=c.H, x=c.x, elem=c.elem, masses=c.masses,
                                elems=np.array(elems), sha256=digest, pe=pe, virial=vir, f=f, rho=rho, dF=dF,
                                energy=ef, nbr=keys.astype(np.int32), x_wrapped=s.x)
            print(name, c.natoms, pe / c.natoms, keys.shape[0])
        # NVT trajectory: 256 atoms, 300 K start, NHC at 300 K, 40 steps
        path, digest = pots[("A",)]
        e = O.Eam.setfl(path)
        c = synth.md_single((4, 4, 4), T=300.0, seed=21)
        s = O.System(e, c.H, c.x, c.elem, c.masses, skin=0.5)
        s.v = c.v
        th, eta, nreb = s.nvt_run(300.0, synth.FS, synth.KB, 40)
        np.savez_compressed(os.path.join(HERE, "nvt_a_256.npz"), H=c.H, x=c.x, v=c.v, elem=c.elem, masses=c.masses,
                            sha256=digest, thermo=th, eta=eta, x_end=s.x, v_end=s.v, nrebuild=nreb, T=300.0,
                            dt=synth.FS, kB=synth.KB, nsteps=40)
        print("nvt_a_256 rebuilds", nreb, "pe", th[0, 0], th[-1, 0])
        # L-BFGS: 475-atom alloy with displacements, to max|F| < 1e-4
        path, digest = pots[("A", "B")]
        e = O.Eam.setfl(path)
        c = synth.alloy((5, 5, 5), xB=0.4, sigma=0.15, vac=0.05, seed=31)
        s = O.System(e, c.H, c.x, c.elem, c.masses, skin=0.5)
        r = s.lbfgs_run(m=10, e_tol=0.0, max_dx=1.0, f_tol=1e-4, nsteps=2000)
        np.savez_compressed(os.path.join(HERE, "lbfgs_ab_475.npz"), H=c.H, x=c.x, elem=c.elem, masses=c.masses,
                            sha256=digest, x_end=s.x, pe=r["pe"], fmax=r["fmax"], niter=r["niter"], err=r["err"],
                            n_energy=r["n_energy"], n_force=r["n_force"])
        print("lbfgs_ab_475", r)


if __name__ == "__main__":
    main()
