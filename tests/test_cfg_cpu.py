"""AtomEye CFG snapshots on the host (no GPU): libmappg's reader and writer
against the oracle restatement (oracle/cfg_ref.py), bit for bit, on
generated files covering both layouts, the header keys, comments, wraps and
every error; known answers; the configuration files shipped with the
reference's examples when the reference tree is present; md-level round
trips through md.atoms.import_cfg and md.export_cfg."""
import glob
import math
import os

import numpy as np
import pytest

import cfg_ref as R
from conftest import REF_ROOT
from mapp4py_gb300 import _lib, md

REF_EXAMPLES = os.path.join(REF_ROOT, "examples") if REF_ROOT else None


@pytest.fixture(scope="module")
def built():
    from mapp4py_gb300 import build

    build.build()
    return _lib.load()


def ours(path):
    try:
        return _lib.read_cfg(path)
    except _lib.MappgError as e:
        return str(e).split(": ", 1)[1]


def oracle(path):
    try:
        return R.read(path)
    except R.CfgError as e:
        return str(e)


def assert_same(path):
    a, b = ours(path), oracle(path)
    if isinstance(b, str) or isinstance(a, str):
        assert a == b, (a, b)
        return a
    assert np.array_equal(a["H"], np.array(b["H"]))
    n = len(b["x"])
    assert a["x"].shape == (n, 3)
    assert np.array_equal(a["x"], np.array(b["x"]).reshape(n, 3))
    assert (a["x_d"] is None) == (b["x_d"] is None)
    if b["x_d"] is not None:
        assert np.array_equal(a["x_d"], np.array(b["x_d"]).reshape(n, 3))
    assert a["elem"].tolist() == b["elem"]
    assert a["names"] == b["names"]
    assert a["masses"].tolist() == b["masses"]
    return a


def write(tmp_path, name, text):
    p = str(tmp_path / name)
    with open(p, "w", newline="") as fh:
        fh.write(text)
    return p


def header(n, H0, extra=(), A=1.0):
    out = ["Number of particles = %d" % n, "A = %r Angstrom (basic length-scale)" % float(A)]
    for i in range(3):
        for j in range(3):
            out.append("H0(%d,%d) = %r A" % (i + 1, j + 1, float(H0[i][j])))
    out.extend(extra)
    return "\n".join(out) + "\n"


def test_known_answer_bcc_pair(built, tmp_path):
    # two atoms of a BCC cell, extended layout without velocities
    text = header(2, np.eye(3), [".NO_VELOCITY.", "entry_count = 3"], A=2.86016)
    text += "55.845\nFe\n0.0 0.0 0.0\n0.5 0.5 0.5\n"
    a = assert_same(write(tmp_path, "fe.cfg", text))
    assert np.array_equal(a["H"], 2.86016 * np.eye(3))
    assert np.array_equal(a["x"], [[0, 0, 0], [1.43008, 1.43008, 1.43008]])
    assert a["x_d"] is None and a["names"] == ["Fe"] and a["masses"].tolist() == [55.845]
    at = md.atoms.import_cfg(write(tmp_path, "fe2.cfg", text))
    assert at.natms == 2 and at.elems == ("Fe",) and at.x_d is None


def test_known_answer_triclinic_box(built, tmp_path):
    # rows of a sheared box: the box is rotated to lower-triangular form with
    # the same row lengths and angles
    H0 = [[3.0, 0.4, 0.0], [0.5, 2.0, 0.3], [0.2, -0.1, 4.0]]
    text = header(1, H0, [".NO_VELOCITY.", "entry_count = 3"]) + "1.0\nX\n0.25 0.5 0.75\n"
    a = assert_same(write(tmp_path, "tri.cfg", text))
    H = a["H"]
    M = np.array(H0)
    assert np.allclose(H @ H.T, M @ M.T, rtol=1e-14, atol=1e-14)
    assert H[0, 1] == H[0, 2] == H[1, 2] == 0.0 and np.all(np.diag(H) > 0)
    assert np.allclose(a["x"][0], np.array([0.25, 0.5, 0.75]) @ H, rtol=1e-15, atol=1e-15)


def random_body(rng, n, names, masses, ncol, std, vel_cols, extras=0):
    lines = []
    cur = None
    for i in range(n):
        e = int(rng.integers(len(names)))
        s = np.where(rng.random(3) < 0.7, rng.uniform(0, 1, 3), rng.uniform(-1.5, 2.5, 3)).tolist()
        v = rng.normal(0, 0.01, 3).tolist()
        aux = rng.normal(0, 1, extras).tolist()
        if std:
            cols = [repr(float(masses[e])), names[e]] + [repr(c) for c in s] + [repr(c) for c in v]
        else:
            if e != cur:
                lines.append(repr(masses[e]))
                lines.append(names[e])
                cur = e
            cols = [repr(c) for c in s] + ([repr(c) for c in v] if vel_cols else []) + [repr(c) for c in aux]
            assert len(cols) == ncol
        sep = rng.choice([" ", "  ", "\t", " \t "])
        lines.append(sep.join(cols) + ("  # atom %d" % i if rng.random() < 0.1 else ""))
        if rng.random() < 0.05:
            lines.append("   ")
    return "\n".join(lines) + "\n"


@pytest.mark.parametrize("seed", range(6))
def test_generated_files_match_oracle_bitwise(built, tmp_path, seed):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(1, 400))
    names = ["Cu", "Ni", "Al"][: int(rng.integers(1, 4))]
    masses = [63.546, 58.6934, 26.9815][: len(names)]
    H0 = np.diag(rng.uniform(5, 30, 3)) + np.tril(rng.uniform(-2, 2, (3, 3)), -1)
    if seed % 2:
        H0 += np.triu(rng.uniform(-1, 1, (3, 3)), 1)  # a general box, rotated by the reader
    extra = []
    if seed % 3 == 1:
        extra += ["Transform(%d,%d) = %r" % (i + 1, j + 1, (1.0 if i == j else 0.0) + float(rng.uniform(-0.05, 0.05)))
                  for i in range(3) for j in range(3)]
    if seed % 3 == 2:
        extra += ["eta(1,1) = 0.01", "eta(2,2) = -0.02", "eta(1,2) = 0.005", "eta(2,1) = 0.005"]
    layout = seed % 3  # 0 standard, 1 extended with velocities and auxiliaries, 2 extended without
    if layout == 0:
        ext, ncol, vel = [], 8, True
        body = random_body(rng, n, names, masses, 8, True, True)
    elif layout == 1:
        ext = ["R = 2.5 [ns^-1]", "entry_count = 8", "auxiliary[0] = c [reduced unit]",
               "auxiliary[1] = d [reduced unit]"]
        body = random_body(rng, n, names, masses, 8, False, True, extras=2)
    else:
        ext = ["# a comment line", ".NO_VELOCITY.", "entry_count = 4", "auxiliary[0] = q [x]"]
        body = random_body(rng, n, names, masses, 4, False, False, extras=1)
    text = header(n, H0, extra + ext, A=float(rng.uniform(0.5, 2.0))) + body
    if seed == 4:
        text = text.replace("\n", "\r\n")
    a = assert_same(write(tmp_path, "g%d.cfg" % seed, text))
    assert not isinstance(a, str), a
    assert a["x"].shape[0] == n


def test_edge_rules_match_oracle(built, tmp_path):
    base = header(2, np.eye(3) * 10, [".NO_VELOCITY.", "entry_count = 3"])
    cases = {
        # a last line without a newline is never read: one atom short
        "unterminated": base + "1.0\nA\n0.1 0.1 0.1\n0.2 0.2 0.2",
        # a repeated name keeps its first mass
        "repeat": base + "1.0\nA\n0.1 0.1 0.1\n2.0\nA\n0.2 0.2 0.2\n",
        # coordinates are wrapped; a tiny negative one rounds to 1.0 and is dropped
        "tiny_negative": base + "1.0\nA\n0.1 0.1 0.1\n-1e-20 0.2 0.2\n",
        "wrap": base + "1.0\nA\n3.25 -2.75 1.0\n-0.5 0.999999999 7\n",
        # .NO_VELOCITY. after entry_count does not remove the velocity columns
        "late_novel": header(1, np.eye(3), ["entry_count = 6", ".NO_VELOCITY."]) + "1\nA\n.1 .2 .3 1 2 3\n",
        "empty": "Number of particles = 0\nA = 1.0 Angstrom\n",
        "body_before_element": base + "0.1 0.2 0.3\n",
        "mass_then_row": base + "1.0\n0.1 0.2 0.3\n",
        "bad_mass": base + "-1.0\nA\n0.1 0.1 0.1\n0.2 0.2 0.2\n",
        "bad_columns": base + "1.0\nA\n0.1 0.1\n",
        "bad_header": "Number of particles = 1\nfoo = 3\n",
        "negative_count": "Number of particles = -1\n",
        "bad_A": "A = 0\n",
        "bad_entry_count": "entry_count = 5\n",
        "aux_first": "auxiliary[0] = c [x]\n",
        "aux_range": ".NO_VELOCITY.\nentry_count = 4\nauxiliary[1] = c [x]\n",
        "bad_index": "H0(4,1) = 2.0 A\n",
        "bad_eta": "eta(1,1) = -0.6\n" + base[base.index("\n") + 1:] + "1.0\nA\n.1 .1 .1\n.2 .2 .2\n",
        "ended": "Number of particles = 3\nA = 1.0\n",
        "count": base + "1.0\nA\n0.1 0.1 0.1\n",
        "std_bad": header(1, np.eye(3)) + "1.0 A 0.1 0.2 0.3 0 0\n",
        "std_ok": header(2, np.eye(3) * 4) + "1.0 A 0.1 0.2 0.3 0 0 0\n2.0 B 0.5 0.5 0.5 1e-3 0 -2e-3\n",
        "inf_coord": base + "1.0\nA\ninf 0.1 0.1\n0.2 0.2 0.2\n",
    }
    results = {}
    for name, text in cases.items():
        results[name] = assert_same(write(tmp_path, name + ".cfg", text))
    assert "but read 1" in results["unterminated"]
    assert results["repeat"]["masses"].tolist() == [1.0]
    assert "but read 1" in results["tiny_negative"]
    w = results["wrap"]["x"]
    assert np.allclose(w, [[2.5, 2.5, 0.0], [5.0, 9.99999999, 0.0]], rtol=0, atol=1e-12)
    assert results["late_novel"]["x_d"] is not None
    assert results["empty"]["x"].shape == (0, 3)
    for k in ("body_before_element", "mass_then_row", "bad_mass", "bad_columns", "bad_header", "negative_count",
              "bad_A", "bad_entry_count", "aux_first", "aux_range", "bad_index", "bad_eta", "ended", "count",
              "std_bad", "inf_coord"):
        assert isinstance(results[k], str), k
    assert results["std_ok"]["names"] == ["A", "B"]
    assert np.array_equal(results["std_ok"]["x_d"][1], [4e-3 * 1.0, 0.0, -8e-3])


@pytest.mark.skipif(not (REF_EXAMPLES and os.path.isdir(REF_EXAMPLES)), reason="MAPPG_REFERENCE_ROOT unset")
def test_reference_example_files(built):
    files = sorted(glob.glob(os.path.join(REF_EXAMPLES, "**", "*.cfg"), recursive=True))
    assert files
    for p in files:
        a = assert_same(p)
        assert not isinstance(a, str), (p, a)


def test_writer_text_matches_oracle(built, tmp_path):
    rng = np.random.default_rng(7)
    n = 300
    H = np.array([[12.0, 0, 0], [1.5, 11.0, 0], [-0.7, 2.2, 13.0]])
    s = rng.uniform(-0.5, 1.5, (n, 3))
    x = s @ H
    elem = np.sort(rng.integers(0, 2, n)).astype(np.uint8)
    elem[n // 2:] = rng.integers(0, 2, n - n // 2)  # element changes along the order
    v = rng.normal(0, 0.02, (n, 3))
    f = rng.normal(0, 1.0, (n, 3))
    for vecs in ([], [("x_d", v)], [("f", f), ("x_d", v)]):
        p = str(tmp_path / "w.cfg")
        _lib.write_cfg(p, H, x, elem, [63.546, 58.6934], ["Cu", "Ni"], vecs)
        with open(p) as fh:
            text = fh.read()
        assert text == R.write_text(H.tolist(), x.tolist(), elem.tolist(), [63.546, 58.6934], ["Cu", "Ni"],
                                    [(nm, a.tolist()) for nm, a in vecs])
        back = assert_same(p)
        # the reader factors H H^T again: the box comes back to rounding
        assert np.allclose(back["H"], H, rtol=0, atol=1e-14)
        # positions come back wrapped into the box, to the 16 printed decimals
        d = back["x"] - x
        d -= np.round(d @ np.linalg.inv(H)) @ H
        assert np.max(np.abs(d)) < 1e-13
        assert back["elem"].tolist() == elem.tolist()
        if vecs and vecs[0][0] == "x_d":
            assert np.allclose(back["x_d"], v, rtol=0, atol=1e-14)
        # the reader takes the three columns after s as the velocity, and the
        # writer keeps the caller's order (as the reference's does): with f
        # listed before x_d those columns are f, read as s_d
        if len(vecs) == 2:
            assert np.allclose(back["x_d"], f @ back["H"], rtol=0, atol=1e-12)


def test_writer_rejects_bad_input(built, tmp_path):
    p = str(tmp_path / "bad.cfg")
    with pytest.raises(_lib.MappgError, match="lower triangular"):
        _lib.write_cfg(p, [[1, 1, 0], [0, 1, 0], [0, 0, 1]], np.zeros((1, 3)), [0], [1.0], ["A"])
    with pytest.raises(_lib.MappgError, match="non-finite"):
        _lib.write_cfg(p, np.eye(3), [[math.nan, 0, 0]], [0], [1.0], ["A"])
    with pytest.raises(_lib.MappgError, match="element index"):
        _lib.write_cfg(p, np.eye(3), np.zeros((1, 3)), [1], [1.0], ["A"])


def test_md_round_trip(built, tmp_path):
    rng = np.random.default_rng(3)
    H = np.diag([20.0, 21.0, 22.0])
    x = rng.uniform(0, 1, (50, 3)) @ H
    at = md.atoms(H, x, rng.integers(0, 2, 50), elems=("A", "B"), masses=(63.5, 27.0),
                  x_d=rng.normal(0, 0.01, (50, 3)))
    xp = md.export_cfg("unused", extra_vecs=["x_d"])
    p = str(tmp_path / "rt.cfg")
    xp(at, p)
    b = md.atoms.import_cfg(p)
    assert b.elems == ("A", "B") or b.elems == ("B", "A")
    order = [b.elems.index(e) for e in at.elems]
    assert np.array_equal(np.array(order)[at.elem], b.elem)
    assert np.allclose(b.x, at.x, rtol=0, atol=1e-13) and np.allclose(b.x_d, at.x_d, rtol=0, atol=1e-14)
    with pytest.raises(TypeError, match="does not exist"):
        md.export_cfg("p", extra_vecs=["c"])(at, p)
    with pytest.raises(TypeError, match="is empty"):
        md.export_cfg("p", extra_vecs=["f"])(at, p)
    with pytest.raises(TypeError):
        md.export_cfg("p", nevery=0)
    with pytest.raises(TypeError, match="failed to open"):
        md.atoms.import_cfg(str(tmp_path / "missing.cfg"))
