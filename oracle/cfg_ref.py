"""CPU restatement of MAPP's AtomEye CFG reader and writer, in plain Python.

Test infrastructure only (the checker of libmappg's mappg_cfg_read /
mappg_cfg_write): imported by tests/, never by the product package.

It follows, rule by rule:
  read_header      import_cfg.cpp:32-191   (header keys, header end, box)
  read_body_ext    import_cfg.cpp:196-372  (mass line, name line, rows)
  read_body_std    import_cfg.cpp:377-478  (8-column rows)
  operator()       import_cfg.cpp:496-595  (x = s H, x_d = s_d R H)
  FileReader       import.cpp:92-120,156-196 (lines, '#' comments, words)
  write_header     export_cfg_md.cpp:26-47
  write_body       export_cfg_md.cpp:89-113
  box arithmetic   xmath.h:850-880 (right-nested dot), 1403-1450 (inverse
                   of a lower-triangular box), 1849-1884 (square box to
                   lower triangular), 2636-2722 (s <-> x), xmath.cpp:598-660
                   (square root of the strain, Franca 1989)
The reference's own tests hold no CFG fixtures; the checks pin this file
against the configuration files shipped with the reference's examples
(read in place when present) and against hand-computed values.
"""
import math
import re

_WS = re.compile(r"\s+")
_INT = r"([+-]?\d+)"
_FLT = r"([+-]?(?:\d+\.?\d*|\.\d+)(?:[eE][+-]?\d+)?|[+-]?(?:inf|infinity|nan)(?![a-z]))"


class CfgError(Exception):
    pass


def _key(words):
    """A header pattern as sscanf reads it: whitespace between the words is
    optional, a number converts its longest prefix, the rest of the line is
    not looked at (sscanf counts conversions, not the trailing text)."""
    conv = {"%d": _INT, "%lf": _FLT}
    return re.compile(r"^\s*" + r"\s*".join(conv.get(w, re.escape(w)) for w in words))


_P_NUM = _key(["Number", "of", "particles", "=", "%d"])
_P_A = _key(["A", "=", "%lf"])
_P_EC = _key(["entry_count", "=", "%d"])
_P_R = _key(["R", "=", "%lf"])
_P_AUX = _key(["auxiliary", "[", "%d"])
_P_TR = _key(["Transform", "(", "%d", ",", "%d", ")", "=", "%lf"])
_P_H0 = _key(["H0", "(", "%d", ",", "%d", ")", "=", "%lf"])
_P_ETA = _key(["eta", "(", "%d", ",", "%d", ")", "=", "%lf"])


def atof(w):
    """C atof: the longest numeric prefix, 0.0 when there is none."""
    m = re.match(r"\s*" + _FLT, w, re.I)
    if not m:
        return 0.0
    return float(m.group(1))


def _lines(path):
    with open(path, "rb") as fh:
        data = fh.read().decode("latin-1")
    parts = data.split("\n")
    return parts[:-1]  # a last line without a newline is never read


def _normalise(line):
    line = line.split("#", 1)[0]
    words = [w for w in _WS.split(line) if w]
    return " ".join(words), len(words)


def dotr(a, b):
    """a0 b0 + (a1 b1 + (...)), the right-nested order."""
    if not a:
        return 0.0
    t = a[-1] * b[-1]
    for k in range(len(a) - 2, -1, -1):
        t = a[k] * b[k] + t
    return t


def rows_to_lower(M):
    L = [[0.0] * 3 for _ in range(3)]
    for i in range(3):
        for j in range(i):
            L[i][j] = (dotr(M[j], M[i]) - dotr(L[j][:j], L[i][:j])) / L[j][j]
        L[i][i] = math.sqrt(dotr(M[i], M[i]) - dotr(L[i][:i], L[i][:i]))
    return L


def lower_inverse(H):
    B = [[0.0] * 3 for _ in range(3)]
    for i in range(3):
        B[i][i] = 1.0 / H[i][i]
        for d in range(1, i + 1):
            j = i - d
            B[i][j] = -B[i][i] * dotr([B[q][j] for q in range(j, i)], [H[i][q] for q in range(j, i)])
    return B


def s_to_x(H, s):
    return [H[0][0] * s[0] + (H[1][0] * s[1] + H[2][0] * s[2]), H[1][1] * s[1] + H[2][1] * s[2], H[2][2] * s[2]]


def x_to_s(B, x):
    return [B[0][0] * x[0] + (B[1][0] * x[1] + B[2][0] * x[2]), B[1][1] * x[1] + B[2][1] * x[2], B[2][2] * x[2]]


def spd_sqrt3(A):
    """Square root of a symmetric positive-definite 3x3 matrix from its
    invariants (Franca 1989); None when A is not positive definite."""
    I1 = A[0][0] + A[1][1] + A[2][2]
    tr2 = 0.0
    for i in range(3):
        for j in range(3):
            tr2 += A[i][j] * A[j][i]
    I2 = 0.5 * (I1 * I1 - tr2)
    I3 = (A[0][0] * (A[1][1] * A[2][2] - A[1][2] * A[2][1]) - A[0][1] * (A[1][0] * A[2][2] - A[1][2] * A[2][0]) +
          A[0][2] * (A[1][0] * A[2][1] - A[1][1] * A[2][0]))
    k = I1 * I1 - 3.0 * I2
    if k < 0.0 or I3 <= 0.0:  # the reference's test misses I3 <= 0 (it ends with NaN)
        return None
    if k < 1e-10:
        if I1 <= 0.0:
            return None
        r = math.sqrt(I1 / 3.0)
        return [[r if i == j else 0.0 for j in range(3)] for i in range(3)]
    l = I1 * (I1 * I1 - 4.5 * I2) + 13.5 * I3
    c = l / (k * math.sqrt(k))
    if c > 1.0 or c < -1.0:
        return None
    lam = math.sqrt((I1 + 2.0 * math.sqrt(k) * math.cos(math.acos(c) / 3.0)) / 3.0)
    J3 = math.sqrt(I3)
    y = I1 - lam * lam + 2.0 * J3 / lam
    if y < 0.0:
        return None
    J1 = lam + math.sqrt(y)
    J2 = 0.5 * (J1 * J1 - I1)
    den = J1 * J2 - J3
    if den == 0.0:
        return None
    inv = 1.0 / den
    R = [[0.0] * 3 for _ in range(3)]
    for i in range(3):
        for j in range(3):
            a2 = 0.0
            for q in range(3):
                a2 += A[i][q] * A[q][j]
            R[i][j] = inv * (-a2 + (J1 * J1 - J2) * A[i][j] + (J1 * J3 if i == j else 0.0))
    return R


def _wrap_read(s):
    while s >= 1.0:
        s -= 1.0
    while s < 0.0:
        s += 1.0
    return s


def _wrap_write(s):
    while s < 0.0:
        s += 1.0
    while s >= 1.0:
        s -= 1.0
    return s


def read(path):
    """dict(H, x, x_d or None, elem, names, masses), or CfgError with the
    reference's message."""
    lines = _lines(path)
    natoms, empty, A, R = 0, False, 1.0, 1.0
    entry_count, vel, ext = 6, True, False
    H0 = [[1.0 if i == j else 0.0 for j in range(3)] for i in range(3)]
    tr = [[1.0 if i == j else 0.0 for j in range(3)] for i in range(3)]
    eta = [[0.0] * 3 for _ in range(3)]
    li, body = 0, None
    while li < len(lines):
        line, nw = _normalise(lines[li])
        li += 1
        if nw == 0:
            continue
        m = _P_NUM.match(line)
        if m:
            k = int(m.group(1))
            if k < 0:
                raise CfgError("Number of particles in %s file should be greater than 0" % path)
            empty = empty or k == 0
            natoms = k
            continue
        m = _P_A.match(line)
        if m:
            t = float(m.group(1))
            if t <= 0.0:
                raise CfgError("A in %s file should be greater than 0.0" % path)
            A = t
            continue
        if line == ".NO_VELOCITY.":
            if not ext:
                vel, ext = False, True
            continue
        m = _P_EC.match(line)
        if m:
            k = int(m.group(1))
            minc = 3 + (3 if vel else 0)
            if k < minc:
                raise CfgError("entry_count in %s should at least be equal to %d" % (path, minc))
            entry_count, ext = k, True
            continue
        m = _P_R.match(line)
        if m:
            R = float(m.group(1))
            continue
        m = _P_AUX.match(line)
        if m:
            i = int(m.group(1))
            if not ext:
                raise CfgError("auxiliary [ ... ] = ... must come after entry_count = ... in %s" % path)
            if i + 3 + (3 if vel else 0) + 1 > entry_count:
                raise CfgError("wrong component in %s file for auxiliary[%d]" % (path, i))
            continue
        hit = False
        for pat, M, nm in ((_P_TR, tr, "Transform"), (_P_H0, H0, "H0"), (_P_ETA, eta, "eta")):
            m = pat.match(line)
            if m:
                i, j, t = int(m.group(1)), int(m.group(2)), float(m.group(3))
                if i < 1 or i > 3 or j < 1 or j > 3:
                    raise CfgError("wrong component in %s file for %s(%d,%d)" % (path, nm, i, j))
                M[i - 1][j - 1] = t
                hit = True
                break
        if hit:
            continue
        if (nw == 8 and not ext) or (nw == 1 and ext):
            body = li - 1
            break
        raise CfgError("invalid line in %s file: %s" % (path, line))
    if body is None and not empty:
        raise CfgError("file %s ended unexpectedly" % path)

    # box
    Hx = [[0.0] * 3 for _ in range(3)]
    for i in range(3):
        for j in range(3):
            t = 0.0
            for k in range(3):
                t += H0[i][k] * tr[k][j]
            Hx[i][j] = t
    if any(eta[i][j] != 0.0 for i in range(3) for j in range(3)):
        E = [[2.0 * eta[i][j] + (1.0 if i == j else 0.0) for j in range(3)] for i in range(3)]
        Es = spd_sqrt3(E)
        if Es is None:
            raise CfgError("eta in %s should be positive definite" % path)
        P = [[0.0] * 3 for _ in range(3)]
        for i in range(3):
            for j in range(3):
                t = 0.0
                for k in range(3):
                    t += Hx[i][k] * Es[k][j]
                P[i][j] = t
        Hx = P
    L = rows_to_lower(Hx)
    H = [[L[i][j] * A for j in range(3)] for i in range(3)]

    names, masses, elem, xs, vs = [], [], [], [], []
    if body is None:
        return {"H": H, "x": [], "x_d": None, "elem": [], "names": [], "masses": []}

    def add(mass, name):
        if name in names:
            return names.index(name)
        if len(names) == 255:
            raise CfgError("cannot have more than 256 elements")
        names.append(name)
        masses.append(mass)
        return len(names) - 1

    ncol = entry_count if ext else 8
    first = 0 if ext else 2
    mass_next_name, have_elem, mass, ie = False, False, 0.0, 0
    for raw in lines[body:]:
        line, nw = _normalise(raw)
        w = line.split(" ") if nw else []
        if nw == 0:
            continue
        if ext:
            if nw != 1 and nw != ncol:
                raise CfgError("invalid line in %s file: %s" % (path, line))
            if mass_next_name and nw != 1:
                raise CfgError("expected chemical symbol of element after mass in %s" % path)
            if nw == 1:
                if not mass_next_name:
                    mass = atof(w[0])
                    if mass <= 0.0:
                        raise CfgError("mass of %s in %s file should be greater than 0.0" % (w[0], path))
                    mass_next_name = True
                else:
                    ie = add(mass, w[0])
                    mass_next_name, have_elem = False, True
                continue
            if not have_elem:
                raise CfgError("line %s in file %s comes before any element was defined" % (line, path))
        else:
            if nw != 8:
                raise CfgError("invalid line in %s file: %s" % (path, line))
            mass = atof(w[0])
            if mass <= 0.0:
                raise CfgError("mass of %s in %s file should be greater than 0.0" % (w[0], path))
            ie = add(mass, w[1])
        s = []
        for d in range(3):
            v = atof(w[first + d])
            if not math.isfinite(v):
                raise CfgError("non-finite coordinate in %s file: %s" % (path, line))
            s.append(_wrap_read(v))
        if any(c < 0.0 or c >= 1.0 for c in s):
            continue
        xs.append(s_to_x(H, s))
        if vel:
            sd = [atof(w[first + 3 + d]) for d in range(3)]
            M = [[R * H[i][j] for j in range(3)] for i in range(3)]
            vs.append(s_to_x(M, sd))
        elem.append(ie)
    if len(xs) != natoms:
        raise CfgError("expected %d natms_lcl in %s but read %d" % (natoms, path, len(xs)))
    return {"H": H, "x": xs, "x_d": vs if vel else None, "elem": elem, "names": names, "masses": masses}


def write_text(H, x, elem, masses, names, vecs=()):
    """The text ExportCFGMD writes for these atoms (vecs: (name, rows))."""
    B = lower_inverse(H)
    vel = any(nm == "x_d" for nm, _ in vecs)
    ncol = 3 + sum(len(rows[0]) if len(rows) else 3 for _, rows in vecs)
    out = ["Number of particles = %d\n" % len(x), "A = %.16f Angstrom (basic length-scale)\n" % 1.0]
    for i in range(3):
        for j in range(3):
            out.append("H0(%d,%d) = %.16f A\n" % (i + 1, j + 1, H[i][j]))
    out.append("R = 1.0\n" if vel else ".NO_VELOCITY.\n")
    out.append("entry_count = %d\n" % ncol)
    aux = 0
    for nm, rows in vecs:
        if nm == "x_d":
            continue
        for d in range(len(rows[0]) if len(rows) else 0):
            out.append("auxiliary[%d] = %s_%d [reduced unit]\n" % (aux, nm, d))
            aux += 1
    cur = -1
    for i in range(len(x)):
        if elem[i] != cur:
            cur = elem[i]
            out.append("%f\n" % masses[cur])
            out.append("%s\n" % names[cur])
        s = x_to_s(B, list(x[i]))
        row = "".join("%.16f " % _wrap_write(c) for c in s)
        for nm, rows in vecs:
            if nm == "x_d":
                row += "".join("%.16f " % c for c in x_to_s(B, list(rows[i])))
            else:
                row += "".join("%.16f " % c for c in rows[i])
        out.append(row + "\n")
    return "".join(out)
