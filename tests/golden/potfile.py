"""DYNAMO setfl / Finnis-Sinclair potential files as knot arrays and back.

Test helper: the reference-pinned fixtures (make_ref_golden.py) keep the
knot values of the potential files shipped with the reference's examples,
and the tests write them back out as files that the library and the oracle
read through their own parsers.  Values are written with 17 significant
digits, so a file written here holds the same doubles as the original.

Layout (import_eam.h:348-613 setfl, 617-901 fs): three comment lines; the
element count and names; nrho drho nr dr rc; per element a line
"Z mass a lattice", F on the rho grid, then the density on the r grid (setfl:
one function; fs: one per source element j); finally r*phi for every pair
i >= j.  Values are read as a token stream, as the reference does.
"""
import numpy as np


def parse(path, kind="setfl"):
    with open(path) as fh:
        lines = fh.read().split("\n")
    head = lines[3].split()
    ne = int(head[0])
    names = head[1:1 + ne]
    toks = " ".join(lines[4:]).split()
    pos = 0

    def take(n):
        nonlocal pos
        out = np.array([float(t) for t in toks[pos:pos + n]], dtype=np.float64)
        pos += n
        return out

    nrho = int(toks[pos]); drho = float(toks[pos + 1]); nr = int(toks[pos + 2])
    dr = float(toks[pos + 3]); rc = float(toks[pos + 4])
    pos += 5
    Z, mass, a0, lat = [], [], [], []
    F = np.zeros((ne, nrho))
    rho = np.zeros((ne, nr)) if kind == "setfl" else np.zeros((ne, ne, nr))
    for i in range(ne):
        Z.append(int(float(toks[pos]))); mass.append(float(toks[pos + 1])); a0.append(float(toks[pos + 2]))
        lat.append(toks[pos + 3])
        pos += 4
        F[i] = take(nrho)
        if kind == "setfl":
            rho[i] = take(nr)
        else:
            for j in range(ne):
                rho[i, j] = take(nr)
    npair = ne * (ne + 1) // 2
    rphi = np.zeros((npair, nr))
    for k in range(npair):
        rphi[k] = take(nr)
    return {"kind": kind, "names": names, "Z": np.array(Z), "masses": np.array(mass), "a0": np.array(a0),
            "lattice": lat, "nrho": nrho, "drho": drho, "nr": nr, "dr": dr, "rc": rc, "F": F, "rho": rho,
            "rphi": rphi, "comments": lines[:3]}


def write(path, d):
    """Write the knot arrays of parse() (or of a fixture) as a potential file."""
    kind = str(d["kind"])
    names = [str(n) for n in d["names"]]
    ne = len(names)

    def block(fh, a):
        a = np.asarray(a).ravel()
        for k in range(0, a.size, 5):
            fh.write(" ".join("%.17e" % v for v in a[k:k + 5]) + "\n")

    with open(path, "w") as fh:
        for c in list(d.get("comments", ["", "", ""]))[:3]:
            fh.write(str(c).rstrip("\n") + "\n")
        fh.write("%d %s\n" % (ne, " ".join(names)))
        fh.write("%d %.17e %d %.17e %.17e\n" % (int(d["nrho"]), float(d["drho"]), int(d["nr"]), float(d["dr"]),
                                               float(d["rc"])))
        for i in range(ne):
            fh.write("%d %.17e %.17e %s\n" % (int(d["Z"][i]), float(d["masses"][i]), float(d["a0"][i]),
                                             str(d["lattice"][i])))
            block(fh, d["F"][i])
            if kind == "setfl":
                block(fh, d["rho"][i])
            else:
                for j in range(ne):
                    block(fh, d["rho"][i][j])
        for k in range(ne * (ne + 1) // 2):
            block(fh, d["rphi"][k])
    return path


def to_fixture(d, prefix="pot_"):
    """Flatten parse() output into npz-storable arrays."""
    return {prefix + "kind": np.array(d["kind"]), prefix + "names": np.array(d["names"]),
            prefix + "Z": d["Z"], prefix + "masses": d["masses"], prefix + "a0": d["a0"],
            prefix + "lattice": np.array(d["lattice"]), prefix + "nrho": d["nrho"], prefix + "drho": d["drho"],
            prefix + "nr": d["nr"], prefix + "dr": d["dr"], prefix + "rc": d["rc"], prefix + "F": d["F"],
            prefix + "rho": d["rho"], prefix + "rphi": d["rphi"],
            prefix + "comments": np.array([c if c else " " for c in d["comments"]])}


def from_fixture(g, prefix="pot_"):
    out = {}
    for k, v in g.items():
        if k.startswith(prefix):
            out[k[len(prefix):]] = v
    out["kind"] = str(out["kind"])
    out["names"] = [str(n) for n in out["names"]]
    out["lattice"] = [str(n) for n in out["lattice"]]
    return out


def write_funcfl_pair(dirname):
    """Two seeded single-element DYNAMO funcfl files on different grids
    (import_eam.h:68-346: a comment line; "Z mass a lattice"; "nrho drho nr
    dr rc"; F on the rho grid, the effective charge Z on the r grid, the
    density on the r grid), so that reading both resamples them onto the
    coarser grid.  Returns the two paths."""
    import os

    specs = (("A", 29, 63.5, 3.615, 500, 0.05, 600, 0.01, 1.0, 1.2),
             ("B", 28, 58.7, 3.52, 400, 0.06, 500, 0.012, 0.8, 1.5))
    paths = []
    for name, Z, mass, a, nrho, drho, nr, dr, z0, F0 in specs:
        r = np.arange(nr) * dr
        rc = 5.5
        sw = np.where(r < rc, (1.0 - r / rc) ** 3, 0.0)
        Zr = z0 * np.exp(-0.9 * r) * sw
        dens = np.exp(-3.0 * (r / 2.55 - 1.0)) * sw
        rh = np.arange(nrho) * drho
        F = -F0 * np.sqrt(rh)
        p = os.path.join(dirname, "%s.funcfl" % name)
        with open(p, "w") as fh:
            fh.write("seeded funcfl test potential %s\n" % name)
            fh.write("%d %.17g %.17g fcc\n" % (Z, mass, a))
            fh.write("%d %.17g %d %.17g %.17g\n" % (nrho, drho, nr, dr, rc))
            for arr in (F, Zr, dens):
                for k in range(0, len(arr), 5):
                    fh.write(" ".join("%.17g" % v for v in arr[k:k + 5]) + "\n")
        paths.append(p)
    return paths
