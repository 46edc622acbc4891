"""Generates tests/golden/cell65536.npz: the FP64 oracle on the 65,536-atom two-species cell with
its own potential (32 G2 + 64 G4 per species, networks 96-128-128-1 tanh, rc 6.5 A).

The oracle evaluates one structure per call and its neighbour build scans all pairs (as
NeighborList::build does, src/struc/neighbor.cpp:59-171), so this takes several minutes of one
core; it runs once, offline, and the fixture is committed.  The structure and the potential are
not stored: they come from the seeded generator (atomnn_gb300/workloads.py), and the fixture
keeps SHA-256 digests of both so that a test on another machine fails loudly if the generator
produced different inputs there.  Stored: the total energy (with and without vacuum energies),
the forces of every 8th atom, the symmetry functions of 64 atoms, and the neighbour counts.

Run:  python tests/golden/make_cell65536.py
"""
import hashlib
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from atomnn_gb300 import workloads as W  # noqa: E402

NAME = "cell65536"
FORCE_STRIDE = 8
SYMM_ATOMS = 64


def inputs(workdir):
    """The potential file path and the structure of the workload, with their digests."""
    potfile = W.workload_files(NAME, workdir)
    s = W.make_structures(NAME)[0]
    with open(potfile, "rb") as f:
        pot_sha = hashlib.sha256(f.read()).hexdigest()
    h = hashlib.sha256()
    for a in (np.ascontiguousarray(s.posn, dtype=np.float64), np.ascontiguousarray(s.species, dtype=np.int32),
              np.ascontiguousarray(s.cell, dtype=np.float64)):
        h.update(a.tobytes())
    return potfile, s, pot_sha, h.hexdigest()


def symm_rows(natoms, seed=65536):
    return np.sort(np.random.default_rng(seed).choice(natoms, SYMM_ATOMS, replace=False)).astype(np.int64)


def main():
    from oracle import pyoracle as O
    workdir = os.path.join(REPO, "atomnn_gb300", "_build", "workloads")
    potfile, s, pot_sha, struc_sha = inputs(workdir)
    orc = O.OracleNNP(potfile)
    t0 = time.time()
    e, F, G = orc.compute(s.posn, s.species, s.cell, force=True, symm=True)
    t1 = time.time()
    # NNP::compute's energy leaves out the species' vacuum energies (src/nnp/nnp.cpp:496-566)
    vac = np.array([sp.energy for sp in W.make_potential(NAME).species])
    ec = e - float(vac[s.species].sum())
    nb = O.neighbors(orc.rc, s.posn, s.cell)
    counts = np.array([len(x["index"]) for x in nb], dtype=np.int32)
    rows = symm_rows(s.natoms)
    np.savez_compressed(os.path.join(HERE, NAME + ".npz"),
                        energy=np.array([e]), energy_compute=np.array([ec]),
                        force_atoms=np.arange(0, s.natoms, FORCE_STRIDE, dtype=np.int64),
                        force=F[::FORCE_STRIDE], symm_atoms=rows, symm=G[rows],
                        nb_count=counts, natoms=np.array([s.natoms]),
                        potential_sha256=np.array([pot_sha]), structure_sha256=np.array([struc_sha]),
                        oracle_seconds=np.array([t1 - t0]))
    print("wrote %s.npz: E=%.9f eV, %.1f s for E+F+G in the oracle" % (NAME, e, t1 - t0))


if __name__ == "__main__":
    main()
