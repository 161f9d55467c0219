"""Seeded synthetic inputs for the EAM workloads: an analytic EAM potential
written as a DYNAMO setfl file, and FCC cells (single element or random
binary alloys, with vacancies, strain, position noise and Maxwell-Boltzmann
velocities).

Units are MAPP's: Angstrom, eV, amu; one time unit is A*sqrt(amu/eV)
(about 10.18 fs).
"""
import math
import os

import numpy as np

KB = 8.617330350e-5  # eV/K, the value MAPP's examples assign to atoms.kB
FS = 1.0 / 10.180505671156723  # 1 fs in MAPP time units
MASS = 63.5

# analytic potential parameters: (D [eV], r0 [A], F prefactor)
ELEMENTS = {"A": (0.35, 2.55, 1.2), "B": (0.42, 2.75, 1.5)}
ALPHA = 1.4  # 1/A, Morse stiffness of the pair term
R_SW0, R_SW1 = 5.0, 5.5  # cubic switch applied to phi and rho


_LN2_HI = 0.693147180369123816490  # ln 2 split so that k*_LN2_HI is exact for |k| < 2^11
_LN2_LO = 1.90821492927058770002e-10


def pexp(x):
    """exp(x) from IEEE +,-,*,/ only (range reduction by ln 2, then the
    Taylor series of exp(r) for |r| <= ln2/2 to 20 terms, then an exact
    scaling by 2^k), so generated tables are bit-identical on every host
    whatever its libm.  Accurate to about one unit in the last place."""
    x = np.asarray(x, dtype=np.float64)
    k = np.rint(x / 0.6931471805599453)
    r = (x - k * _LN2_HI) - k * _LN2_LO
    t = np.ones_like(r)
    for n in range(20, 0, -1):
        t = 1.0 + t * r / float(n)
    return np.ldexp(t, k.astype(np.int64))


def switch(r):
    """1 below 5.0 A, 1-3t^2+2t^3 on [5.0,5.5) with t=(r-5)/0.5, 0 beyond."""
    r = np.asarray(r, dtype=np.float64)
    t = np.clip((r - R_SW0) / (R_SW1 - R_SW0), 0.0, 1.0)
    return 1.0 - 3.0 * t * t + 2.0 * t * t * t


def phi(r, D, r0):
    e = pexp(-ALPHA * (r - r0))
    return D * (e * e - 2.0 * e) * switch(r)


def rho_fn(r, r0):
    return pexp(-3.0 * (r / r0 - 1.0)) * switch(r)


def analytic_knots(elems=("A",), nr=5000, nrho=5000, rc=5.5, drho=0.01):
    """Knot values of the analytic potential on the setfl grids.

    Returns (dr, drho, F[ne][nrho], rho[ne][nr], rphi[ne][ne][nr]); the cross
    pair is the arithmetic mean of the two pure pair functions.
    """
    dr = rc / nr
    r = np.arange(nr, dtype=np.float64) * dr
    rh = np.arange(nrho, dtype=np.float64) * drho
    ne = len(elems)
    F = np.zeros((ne, nrho))
    rho = np.zeros((ne, nr))
    ph = np.zeros((ne, nr))
    for i, e in enumerate(elems):
        D, r0, pref = ELEMENTS[e]
        F[i] = -pref * np.sqrt(rh)
        rho[i] = rho_fn(r, r0)
        ph[i] = phi(r, D, r0)
    rphi = np.zeros((ne, ne, nr))
    for i in range(ne):
        for j in range(ne):
            rphi[i, j] = r * 0.5 * (ph[i] + ph[j])
    return dr, drho, F, rho, rphi


def write_setfl(path, elems=("A",), nr=5000, nrho=5000, rc=5.5, drho=0.01, mass=MASS):
    """Write the analytic potential as a setfl file (5 values per line)."""
    dr, drho, F, rho, rphi = analytic_knots(elems, nr, nrho, rc, drho)
    ne = len(elems)

    def block(fh, a):
        a = np.asarray(a).ravel()
        for k in range(0, a.size, 5):
            fh.write(" ".join("%.17e" % v for v in a[k:k + 5]) + "\n")

    tmp = path + ".tmp%d" % os.getpid()
    with open(tmp, "w") as fh:
        fh.write("analytic EAM: Morse pair, exponential density, -c*sqrt(rho) embedding\n")
        fh.write("cubic switch on phi and rho over 5.0-5.5 A; cross pair = mean of pure pairs\n")
        fh.write("written by mapp4py_gb300.synth\n")
        fh.write("%d %s\n" % (ne, " ".join(elems)))
        fh.write("%d %.17e %d %.17e %.17e\n" % (nrho, drho, nr, dr, rc))
        for i in range(ne):
            fh.write("29 %.6f 3.615 fcc\n" % mass)
            block(fh, F[i])
            block(fh, rho[i])
        for i in range(ne):
            for j in range(i + 1):
                block(fh, rphi[i, j])
    os.replace(tmp, path)
    return path


def fcc(n, a=3.615):
    """FCC lattice of n=(n0,n1,n2) unit cells: H (lower triangular rows) and x."""
    n0, n1, n2 = n
    basis = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    g = np.stack(np.meshgrid(np.arange(n0), np.arange(n1), np.arange(n2), indexing="ij"), -1).reshape(-1, 3)
    s = (g[:, None, :] + basis[None, :, :]).reshape(-1, 3)
    x = s * a
    H = np.diag([n0 * a, n1 * a, n2 * a]).astype(np.float64)
    return H, np.ascontiguousarray(x, dtype=np.float64)


def maxwell(rng, masses_per_atom, T, kB=KB):
    """Gaussian velocities sqrt(kB T / m) per component (no drift removal,
    as AtomsMD::create_T)."""
    fac = np.sqrt(kB * T / np.asarray(masses_per_atom))
    return rng.standard_normal((fac.shape[0], 3)) * fac[:, None]


def wrap(H, x):
    """Wrap Cartesian rows into the periodic cell (s in [0,1))."""
    B = np.linalg.inv(H)
    s = x @ B
    s -= np.floor(s)
    return s @ H


class Cell:
    """A synthetic periodic cell: H, x, elem (uint8), v, element names, masses."""

    def __init__(self, H, x, elem, v, names, masses):
        self.H = np.ascontiguousarray(H, dtype=np.float64)
        self.x = np.ascontiguousarray(x, dtype=np.float64)
        self.elem = np.ascontiguousarray(elem, dtype=np.uint8)
        self.v = np.ascontiguousarray(v, dtype=np.float64)
        self.names = tuple(names)
        self.masses = np.ascontiguousarray(masses, dtype=np.float64)

    @property
    def natoms(self):
        return self.x.shape[0]


def md_single(n=(10, 10, 10), a=3.615, T=300.0, seed=0):
    """Plain FP64 MD cell: single element FCC, velocities at T from `seed`."""
    H, x = fcc(n, a)
    elem = np.zeros(x.shape[0], np.uint8)
    rng = np.random.default_rng(seed)
    v = maxwell(rng, np.full(x.shape[0], MASS), T)
    return Cell(H, x, elem, v, ("A",), [MASS])


def alloy(n, a=3.615, xB=0.5, sigma=0.0, T=0.0, vac=0.0, strain=None, seed=1):
    """Random binary A/B alloy on FCC with vacancies, strain and noise."""
    rng = np.random.default_rng(seed)
    H, x = fcc(n, a)
    N = x.shape[0]
    elem = (rng.random(N) < xB).astype(np.uint8)
    if vac > 0.0:
        keep = rng.random(N) >= vac
        x, elem = x[keep], elem[keep]
    if strain is not None:
        E = np.eye(3) + np.asarray(strain, dtype=np.float64)
        E = np.tril(E)
        H = H @ E
        x = x @ E
    if sigma > 0.0:
        x = x + rng.normal(0.0, sigma, size=x.shape)
    x = wrap(H, x)
    masses = np.array([MASS, MASS])
    v = maxwell(rng, masses[elem], T) if T > 0 else np.zeros_like(x)
    return Cell(H, x, elem, v, ("A", "B"), masses)


def fcc_repeats(natoms, rng, min_side=4):
    """FCC repeats (n0, n1, n2), each >= min_side, with a random aspect ratio
    and 4*n0*n1*n2 close to natoms."""
    cells = max(natoms / 4.0, float(min_side ** 3))
    logs = rng.normal(0.0, 0.25, 3)
    logs -= logs.mean()
    side = cells ** (1.0 / 3.0) * np.exp(logs)
    n = np.maximum(np.rint(side).astype(int), min_side)
    return tuple(int(v) for v in n)


def batch_cells(ncell, seed=7, nmin=500, nmax=32000, T=(100.0, 1200.0), vac=(0.0, 0.02), sigma=(0.05, 0.05),
                strain=0.0, min_side=4):
    """Independent A/B alloy cells: atom counts log-uniform in [nmin, nmax]
    rounded to whole FCC repeats (every side at least min_side repeats, 14.5 A
    for min_side 4), x_B ~ U(0,1), vacancy fraction ~ U(vac), temperature ~
    U(T) with Maxwell-Boltzmann velocities, position noise ~ U(sigma), and a
    random homogeneous strain up to +-strain per component (lower-triangular
    so the box stays in MAPP's form).  Returns (cells, temperatures)."""
    rng = np.random.default_rng(seed)
    out, temps = [], []
    for c in range(ncell):
        target = math.exp(rng.uniform(math.log(nmin), math.log(nmax)))
        n = fcc_repeats(target, rng, min_side)
        xb = rng.uniform(0.0, 1.0)
        vf = rng.uniform(*vac)
        tc = rng.uniform(*T)
        sg = rng.uniform(*sigma)
        st = None
        if strain > 0.0:
            st = np.tril(rng.uniform(-strain, strain, (3, 3)))
        cell = alloy(n, xB=xb, sigma=sg, T=tc, vac=vf, strain=st, seed=int(rng.integers(1 << 30)))
        out.append(cell)
        temps.append(tc)
    return out, np.array(temps)
