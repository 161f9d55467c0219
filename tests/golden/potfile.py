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
