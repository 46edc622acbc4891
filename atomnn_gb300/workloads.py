"""Seeded synthetic workloads for the NNP energy/force path.

Every input is generated here from a seed: the potential file (written in AtomNN's text format,
``NNP::write`` in src/nnp/nnp.cpp:198-237) and the periodic structures.  No public dataset is
involved.  The five workloads are:

``small64``   64 atoms of one species, 4x4x4 simple-cubic site grid (spacing 2.025 A) in an
              8.1 A cube, Gaussian displacements sigma=0.1 A, COS cutoff 6.0 A, 16 G2 + 16 G4,
              network 32-32-32-1 tanh.
``cell1728``  two species A:B = 1:2 (A on sites with (ix+iy+iz) % 3 == 0 of a 12^3 grid), cubic
              cell at 0.07 atoms/A^3, sigma=0.15 A, rc 6.5 A; per centre species 24 G2 (12 per
              neighbour species: eta 4 log-spaced 0.001-4 A^-2 x rs {0,1.5,3} A) and 32 G4
              (AA 8, AB 12, BB 12); networks 56-64-64-1 tanh.
``mixed512``  512 triclinic structures, N log-uniform over [16, 2048], density U(0.05, 0.09),
              cell angles U(80, 100) degrees, basis and networks as ``cell1728``.
``cell65536`` one cubic 65536-atom cell at 0.07 atoms/A^3, 32 G2 + 64 G4 per species,
              networks 96-128-128-1 tanh.
``serve``     request sizes log-uniform over [16, 4096], structures as ``mixed512``.

Angular functions: the reference's GAUSS form is exp(-(r_ij^a + r_ik^a)/eta^a); a G4 width
eta' given in exp(-eta' r^2) form (A^-2) is written as eta = eta'^(-1/2) with alpha = 2.

Input scaling (``inpb``/``inpw`` of each network) is set from an analytic estimate of the
descriptor means at the workload's density (radial integrals of each function times the
neighbour density; <((1+lambda cos)/2)^zeta> = 1/(zeta+1) for isotropic angles):
inpb = -mean, inpw = 1/(0.2*mean).  The reference's trainers set the same layer from data
statistics (src/nnp/nnpte.cpp:437-500); the estimate keeps the networks out of saturation
without a descriptor evaluation at generation time.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np

# ----------------------------------------------------------------------------- potential model


@dataclass
class RadialBasis:
    rc: float
    rs: list
    eta: list
    cutname: str = "COS"
    cutnorm: str = "UNIT"
    phi: str = "GAUSSIAN"


@dataclass
class AngularBasis:
    rc: float
    eta: list
    zeta: list
    lam: list
    alpha: int = 2
    cutname: str = "COS"
    cutnorm: str = "UNIT"
    phi: str = "GAUSS"


@dataclass
class Network:
    nin: int
    nodes: list  # hidden layers then output (last is 1)
    neuron: str
    inpw: np.ndarray
    inpb: np.ndarray
    outw: np.ndarray
    outb: np.ndarray
    b: list
    w: list  # w[l] has shape (nodes[l], cols)


@dataclass
class Species:
    name: str
    mass: float
    energy: float


@dataclass
class Potential:
    rc: float
    species: list
    radial: dict = field(default_factory=dict)   # (I, J) -> RadialBasis
    angular: dict = field(default_factory=dict)  # (I, J, K) with J <= K -> AngularBasis
    nets: dict = field(default_factory=dict)     # I -> Network

    @property
    def ntypes(self):
        return len(self.species)

    def ninput(self, i):
        n = sum(len(self.radial[(i, j)].rs) for j in range(self.ntypes))
        for j in range(self.ntypes):
            for k in range(j, self.ntypes):
                n += len(self.angular[(i, j, k)].eta)
        return n


def _f6(x):
    """Round to what '%f' writes, so that the in-memory model equals the file."""
    return float("%f" % x)


def write_potential(pot: Potential, path: str) -> None:
    """Write ``pot`` in the reference text format (NNP::write, src/nnp/nnp.cpp:198-237)."""
    out = ["ann", "ntypes %i" % pot.ntypes]
    for s in pot.species:
        out.append("name %s mass %f energy %f " % (s.name, s.mass, s.energy))
    out.append("rc %f" % pot.rc)
    n = pot.ntypes
    for i in range(n):
        out.append("basis %s" % pot.species[i].name)
        for j in range(n):
            b = pot.radial[(i, j)]
            out.append("basis_radial %s" % pot.species[j].name)
            out.append("BasisR %s %s %f %s %i" % (b.cutnorm, b.cutname, b.rc, b.phi, len(b.rs)))
            for rs, eta in zip(b.rs, b.eta):
                out.append("\t%f %f" % (rs, eta))
        for j in range(n):
            for k in range(j, n):
                b = pot.angular[(i, j, k)]
                out.append("basis_angular %s %s" % (pot.species[j].name, pot.species[k].name))
                out.append("BasisA %s %s %f %s %i %i" % (b.cutnorm, b.cutname, b.rc, b.phi, len(b.eta), b.alpha))
                for eta, zeta, lam in zip(b.eta, b.zeta, b.lam):
                    out.append("\t%f %f %i" % (eta, zeta, lam))
    for i in range(n):
        net = pot.nets[i]
        out.append("nn %s" % pot.species[i].name)
        out.append("nn %i " % net.nin + "".join("%i " % x for x in net.nodes))
        out.append("neuron %s" % net.neuron)
        for tag, v in (("inpw", net.inpw), ("outw", net.outw), ("inpb", net.inpb), ("outb", net.outb)):
            out.append(tag + " " + "".join("%.15f " % x for x in v))
        for l, bl in enumerate(net.b):
            out.append("bias[%i] " % (l + 1) + "".join("%.15f " % x for x in bl))
        for l, wl in enumerate(net.w):
            out.append("weight[%i,%i] " % (l, l + 1) + "".join("%.15f " % x for x in np.asarray(wl).ravel()))
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")


# ----------------------------------------------------------------------------- analytic statistics


def _cut_cos(r, rc):
    return np.where(r > rc, 0.0, 0.5 * (np.cos(np.pi * r / rc) + 1.0))


def _shell_integral(fn, rc, npts=4001):
    r = np.linspace(0.0, rc, npts)
    return float(np.trapezoid(fn(r) * 4.0 * np.pi * r * r, r))


def _estimate_means(pot: Potential, i: int, rho: float, frac: list) -> np.ndarray:
    """Mean of each input of centre species i for a homogeneous system of density rho."""
    means = []
    n = pot.ntypes
    for j in range(n):
        b = pot.radial[(i, j)]
        for rs, eta in zip(b.rs, b.eta):
            means.append(rho * frac[j] * _shell_integral(
                lambda r: np.exp(-eta * (r - rs) ** 2) * _cut_cos(r, b.rc), b.rc))
    for j in range(n):
        for k in range(j, n):
            b = pot.angular[(i, j, k)]
            for eta, zeta, lam in zip(b.eta, b.zeta, b.lam):
                ietap = (1.0 / eta) ** b.alpha
                s = _shell_integral(lambda r: np.exp(-ietap * r ** b.alpha) * _cut_cos(r, b.rc), b.rc)
                sj, sk = rho * frac[j] * s, rho * frac[k] * s
                pairs = sj * sk if j != k else 0.5 * sj * sj
                means.append(pairs / (zeta + 1.0))
    return np.asarray(means)


def _make_network(rng, nin, hidden, means):
    nodes = list(hidden) + [1]
    b, w = [], []
    cols = nin
    for n in nodes:
        w.append(rng.normal(0.0, math.sqrt(1.0 / cols), size=(n, cols)))
        b.append(np.zeros(n))
        cols = n
    scale = 0.2 * np.maximum(means, 1e-6)
    return Network(nin=nin, nodes=nodes, neuron="TANH", inpw=1.0 / scale, inpb=-means,
                   outw=np.ones(1), outb=np.zeros(1), b=b, w=w)


def _logspace(lo, hi, n):
    if n == 1:
        return [lo]
    return [lo * (hi / lo) ** (k / (n - 1)) for k in range(n)]


def _angular(rc, etas_prime, zetas, lams):
    eta, zeta, lam = [], [], []
    for e in etas_prime:
        for z in zetas:
            for l in lams:
                eta.append(_f6(e ** -0.5))
                zeta.append(_f6(z))
                lam.append(int(l))
    return AngularBasis(rc=_f6(rc), eta=eta, zeta=zeta, lam=lam)


def make_potential(name: str, seed: int = 1234) -> Potential:
    """Seeded potential for workload ``name`` (see the module docstring)."""
    rng = np.random.default_rng(seed)
    if name == "small64":
        rc = 6.0
        pot = Potential(rc=_f6(rc), species=[Species("Al", 26.9815, -0.3)])
        etas = [_f6(x) for x in _logspace(0.001, 2.0, 16)]
        pot.radial[(0, 0)] = RadialBasis(rc=_f6(rc), rs=[0.0] * 16, eta=etas)
        pot.angular[(0, 0, 0)] = _angular(rc, [0.005, 0.05], [1, 2, 4, 16], [1, -1])
        means = _estimate_means(pot, 0, 64 / 8.1 ** 3, [1.0])
        pot.nets[0] = _make_network(rng, pot.ninput(0), [32, 32], means)
        return pot
    if name in ("cell1728", "mixed512", "serve", "cell65536"):
        rc = 6.5
        pot = Potential(rc=_f6(rc), species=[Species("A", 24.305, -0.5), Species("B", 15.999, -0.25)])
        big = name == "cell65536"
        for i in range(2):
            for j in range(2):
                if big:
                    etas = _logspace(0.001, 4.0, 8)
                    rss = [0.0, 3.0]
                else:
                    etas = _logspace(0.001, 4.0, 4)
                    rss = [0.0, 1.5, 3.0]
                rs_l, eta_l = [], []
                for rs in rss:
                    for e in etas:
                        rs_l.append(_f6(rs))
                        eta_l.append(_f6(e))
                pot.radial[(i, j)] = RadialBasis(rc=_f6(rc), rs=rs_l, eta=eta_l)
            if big:
                pot.angular[(i, 0, 0)] = _angular(rc, [0.005, 0.05], [1, 2, 4, 16], [1, -1])
                pot.angular[(i, 0, 1)] = _angular(rc, [0.005, 0.02, 0.05], [1, 2, 4, 16], [1, -1])
                pot.angular[(i, 1, 1)] = _angular(rc, [0.005, 0.02, 0.05], [1, 2, 4, 16], [1, -1])
            else:
                pot.angular[(i, 0, 0)] = _angular(rc, [0.005], [1, 2, 4, 16], [1, -1])
                pot.angular[(i, 0, 1)] = _angular(rc, [0.005, 0.05], [1, 2, 4], [1, -1])
                pot.angular[(i, 1, 1)] = _angular(rc, [0.005, 0.05], [1, 2, 4], [1, -1])
        hidden = [128, 128] if big else [64, 64]
        for i in range(2):
            means = _estimate_means(pot, i, 0.07, [1.0 / 3.0, 2.0 / 3.0])
            pot.nets[i] = _make_network(rng, pot.ninput(i), hidden, means)
        return pot
    raise ValueError("unknown workload " + name)


# ----------------------------------------------------------------------------- structures


@dataclass
class Structure:
    """One periodic structure: Cartesian positions (N,3) FP64, species index per atom, and the
    lattice as a 3x3 matrix whose COLUMNS are the lattice vectors (as Cell::R_ in the reference)."""
    posn: np.ndarray
    species: np.ndarray
    cell: np.ndarray

    @property
    def natoms(self):
        return int(self.posn.shape[0])

    def cell_colmajor(self):
        """9 doubles, column-major: the layout the C interface takes."""
        return np.ascontiguousarray(self.cell.T).ravel()


def lattice(a, b, c, alpha, beta, gamma):
    """Columns a1, a2, a3 of a triclinic cell from lengths and angles (degrees)."""
    al, be, ga = (math.radians(x) for x in (alpha, beta, gamma))
    a1 = [a, 0.0, 0.0]
    a2 = [b * math.cos(ga), b * math.sin(ga), 0.0]
    cx = c * math.cos(be)
    cy = c * (math.cos(al) - math.cos(be) * math.cos(ga)) / math.sin(ga)
    cz = math.sqrt(max(c * c - cx * cx - cy * cy, 0.0))
    return np.array([a1, a2, [cx, cy, cz]]).T


def _grid_structure(rng, n, cell, sigma, nA):
    m = int(math.ceil(n ** (1.0 / 3.0) - 1e-9))
    sites = np.array([(x, y, z) for x in range(m) for y in range(m) for z in range(m)], dtype=float)
    pick = rng.permutation(len(sites))[:n]
    frac = (sites[pick] + 0.5) / m
    posn = frac @ cell.T + rng.normal(0.0, sigma, size=(n, 3))
    species = np.ones(n, dtype=np.int32)
    species[rng.permutation(n)[:nA]] = 0
    return Structure(posn=posn, species=species, cell=cell)


def make_structures(name: str, seed: int = 4321, count: int | None = None, sizes=None):
    """Seeded structures of workload ``name``.  ``count`` overrides the number of structures of
    the multi-structure workloads; ``sizes`` (list of atom counts) overrides their sizes."""
    rng = np.random.default_rng(seed)
    if name == "small64":
        L, m = 8.1, 4
        sites = np.array([(x, y, z) for x in range(m) for y in range(m) for z in range(m)], dtype=float)
        posn = sites * (L / m) + rng.normal(0.0, 0.1, size=(64, 3))
        return [Structure(posn=posn, species=np.zeros(64, dtype=np.int32), cell=np.eye(3) * L)]
    if name == "cell1728":
        m = 12
        L = (1728 / 0.07) ** (1.0 / 3.0)
        idx = np.array([(x, y, z) for x in range(m) for y in range(m) for z in range(m)])
        posn = idx * (L / m) + rng.normal(0.0, 0.15, size=(1728, 3))
        species = np.where(idx.sum(axis=1) % 3 == 0, 0, 1).astype(np.int32)
        return [Structure(posn=posn, species=species, cell=np.eye(3) * L)]
    if name == "cell65536":
        n = 65536
        L = (n / 0.07) ** (1.0 / 3.0)
        return [_grid_structure(rng, n, np.eye(3) * L, 0.15, n // 3)]
    if name in ("mixed512", "serve"):
        hi = 2048 if name == "mixed512" else 4096
        nstruc = count if count is not None else 512
        out = []
        for s in range(nstruc):
            n = int(sizes[s]) if sizes is not None else int(round(math.exp(rng.uniform(math.log(16), math.log(hi)))))
            rho = rng.uniform(0.05, 0.09)
            ang = rng.uniform(80.0, 100.0, size=3)
            unit = lattice(1.0, 1.0, 1.0, *ang)
            vol1 = abs(np.linalg.det(unit))
            a = (n / rho / vol1) ** (1.0 / 3.0)
            out.append(_grid_structure(rng, n, unit * a, 0.15, max(1, int(round(n / 3)))))
        return out
    raise ValueError("unknown workload " + name)


def workload_files(name: str, directory: str, seed: int = 1234) -> str:
    """Write the potential of workload ``name`` into ``directory``; returns its path."""
    os.makedirs(directory, exist_ok=True)
    path = os.path.join(directory, "%s_seed%d.nnp" % (name, seed))
    if not os.path.exists(path):
        tmp = path + ".tmp%d" % os.getpid()
        write_potential(make_potential(name, seed), tmp)
        os.replace(tmp, path)
    return path


def write_poscar(struc: Structure, names, path: str, comment: str = "generated") -> None:
    """POSCAR with Cartesian coordinates, scale 1 (read by VASP::POSCAR::read,
    src/format/vasp_struc.cpp:51-160).  Atoms must be grouped by species."""
    order = np.argsort(struc.species, kind="stable")
    if not np.array_equal(order, np.arange(struc.natoms)):
        raise ValueError("POSCAR needs atoms grouped by species")
    counts = [int((struc.species == t).sum()) for t in range(len(names))]
    lines = [comment, "1.0"]
    for c in range(3):
        lines.append("%.16e %.16e %.16e" % tuple(struc.cell[:, c]))
    used = [i for i, c in enumerate(counts) if c > 0]
    lines.append(" ".join(names[i] for i in used))
    lines.append(" ".join(str(counts[i]) for i in used))
    lines.append("Cartesian")
    for p in struc.posn:
        lines.append("%.16e %.16e %.16e" % tuple(p))
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")
