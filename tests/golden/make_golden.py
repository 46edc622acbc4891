"""Generates the golden fixtures of tests/golden/ from the FP64 oracle.

The reference (markdellostritto/AtomNN) holds no golden vectors for this path and cannot be
built here, so these fixtures pin the oracle's own outputs: potentials and structures come
from the seeded generator, energies/forces/symmetry functions/neighbour lists from the oracle.
Run:  python tests/golden/make_golden.py
"""
import os
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from atomnn_gb300 import workloads as W  # noqa: E402
from oracle import pyoracle as O  # noqa: E402


def cluster(n, seed):
    rng = np.random.default_rng(seed)
    pts = []
    while len(pts) < n:
        p = rng.uniform(-4.5, 4.5, size=3)
        if all(np.linalg.norm(p - q) > 1.8 for q in pts):
            pts.append(p)
    sp = np.array([0 if k % 3 == 0 else 1 for k in range(n)], dtype=np.int32)
    return W.Structure(posn=np.array(pts), species=sp, cell=np.zeros((3, 3)))


def cases():
    yield "small64", "small64", W.make_structures("small64")
    yield "mixed3", "mixed512", W.make_structures("mixed512", seed=77, count=3, sizes=[16, 64, 200])
    yield "cluster20", "mixed512", [cluster(20, 5)]


def main():
    for name, potname, strucs in cases():
        potfile = os.path.join(HERE, "%s.nnp" % potname)
        if not os.path.exists(potfile):
            W.write_potential(W.make_potential(potname), potfile)
        orc = O.OracleNNP(potfile)
        data = {}
        for k, s in enumerate(strucs):
            e, F, G = orc.compute(s.posn, s.species, s.cell, force=True, symm=True)
            ec, Fc, _ = orc.compute(s.posn, s.species, s.cell, compute_semantics=True)
            nb = O.neighbors(orc.rc, s.posn, s.cell)
            data["s%d_posn" % k] = s.posn
            data["s%d_species" % k] = s.species
            data["s%d_cell" % k] = s.cell
            data["s%d_energy" % k] = np.array([e])
            data["s%d_energy_compute" % k] = np.array([ec])
            data["s%d_force" % k] = F
            data["s%d_symm" % k] = G
            data["s%d_nb_count" % k] = np.array([len(x["index"]) for x in nb], dtype=np.int32)
            data["s%d_nb_index" % k] = np.concatenate([x["index"] for x in nb]).astype(np.int32)
            data["s%d_nb_shift" % k] = np.concatenate([x["shift"] for x in nb]).astype(np.int8)
            data["s%d_nb_min" % k] = np.concatenate([x["min"] for x in nb]).astype(np.uint8)
        data["nstruc"] = np.array([len(strucs)])
        data["potential"] = np.array([potname])
        np.savez_compressed(os.path.join(HERE, "%s.npz" % name), **data)
        print("wrote", name)


if __name__ == "__main__":
    main()
