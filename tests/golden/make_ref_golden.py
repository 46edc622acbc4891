"""Generates tests/golden/reference.npz: outputs of the reference's own code (markdellostritto/
AtomNN's NeighborList::build, NNP::symm, NNP::energy, NNP::force and NNP::compute, compiled from
its sources by oracle/Makefile.ref against the Eigen-API shim and driven by oracle/ref_driver.cpp).

These are the golden vectors that pin the FP64 oracle (tests/test_reference_pin.py) and the GPU
path (tests/test_gpu_parity.py) to the reference.  Cases:

  golden      the structures of the other fixtures (small64, mixed3, cluster20)
  edge        a strongly sheared cell (6-shift fallback of Cell::diff), exact lattice sites (ties
              between equidistant images), one atom in a small cell (self images only), two atoms,
              an isolated non-periodic cluster with a far atom
  variants    every radial and angular basis family, the TANH and STEP cutoffs, VOL normalisation,
              real zeta and six distinct eta in one angular block (tests/golden/variants.py), on a
              40-atom cell (image shells) and a 150-atom cell

Positions, species and cells are stored with the outputs, so readers need no random generator.
Neighbour lists (index, type, minimum-image flag, vector) are stored for the golden and edge
structures of at most 64 atoms; descriptors of every atom there, of the first 12 atoms of each
variant structure.  Needs the reference sources (ATOMNN_REFERENCE, default /root/reference).

Run:  python tests/golden/make_ref_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, HERE)

from atomnn_gb300 import workloads as W  # noqa: E402
import variants as V  # noqa: E402


SYMM_ROWS = 12    # descriptor rows stored per structure of a variant case
LIST_ATOMS = 64   # neighbour lists stored for structures of at most this many atoms


def _golden(name):
    d = np.load(os.path.join(HERE, name + ".npz"))
    return [W.Structure(posn=d["s%d_posn" % k], species=d["s%d_species" % k], cell=d["s%d_cell" % k]) for k in range(int(d["nstruc"][0]))]


def edge_structures():
    rng = np.random.default_rng(4)
    cell = W.lattice(7.0, 7.5, 8.0, 60.0, 115.0, 65.0)
    sheared = W.Structure(posn=rng.uniform(0, 1, size=(24, 3)) @ cell.T, species=(np.arange(24) % 2).astype(np.int32), cell=cell)
    m, a = 3, 2.8
    idx = np.array([(x, y, z) for x in range(m) for y in range(m) for z in range(m)], dtype=float)
    perfect = W.Structure(posn=idx * a, species=(np.arange(27) % 3 == 0).astype(np.int32), cell=np.eye(3) * m * a)
    one = W.Structure(posn=np.array([[0.3, 0.2, 0.1]]), species=np.array([1], np.int32), cell=np.eye(3) * 4.0)
    two = W.Structure(posn=np.array([[0.0, 0.0, 0.0], [1.9, 0.4, 0.2]]), species=np.array([0, 1], np.int32),
                      cell=W.lattice(5.0, 5.5, 6.0, 90.0, 95.0, 85.0))
    iso = W.Structure(posn=np.array([[0, 0, 0], [2.0, 0, 0], [0, 2.1, 0], [30.0, 30.0, 30.0]], dtype=float),
                      species=np.array([0, 1, 1, 0], np.int32), cell=np.zeros((3, 3)))
    return [sheared, perfect, one, two, iso]


def variant_structures():
    return W.make_structures("mixed512", seed=29, count=2, sizes=[40, 150])


def cases():
    """(case name, potential variant, structures, store neighbour lists)"""
    yield "small64", "base_small64", _golden("small64"), True
    yield "mixed3", "base_mixed512", _golden("mixed3"), True
    yield "cluster20", "base_mixed512", _golden("cluster20"), True
    yield "edge", "base_mixed512", edge_structures(), True
    for v in V.NAMES[2:]:
        yield v, v, variant_structures(), False


def main():
    from oracle import refrun
    if not refrun.available():
        sys.exit("the reference sources are needed (set ATOMNN_REFERENCE)")
    refrun.build()
    workdir = os.path.join(REPO, "atomnn_gb300", "_build", "variants")
    data = {}
    names = []
    for case, variant, strucs, lists in cases():
        pot = V.write(variant, workdir)
        res = refrun.run(pot, strucs, lists=lists)
        names.append(case)
        data[case + "/variant"] = np.array([variant])
        data[case + "/nstruc"] = np.array([len(strucs)])
        for k, (s, r) in enumerate(zip(strucs, res)):
            p = "%s/%d/" % (case, k)
            data[p + "posn"] = np.asarray(s.posn, dtype=np.float64)
            data[p + "species"] = np.asarray(s.species, dtype=np.int32)
            data[p + "cell"] = np.zeros((3, 3)) if s.cell is None else np.asarray(s.cell, dtype=np.float64)
            data[p + "energy"] = np.array([r["energy"]])
            data[p + "energy_compute"] = np.array([r["energy_compute"]])
            data[p + "force"] = r["force"]
            data[p + "force_compute"] = r["force_compute"]
            # descriptors of every atom, or of the first SYMM_ROWS atoms of a variant case
            rows = np.arange(s.natoms) if lists else np.arange(min(s.natoms, SYMM_ROWS))
            width = max(len(r["symm"][i]) for i in rows) if len(rows) else 0
            G = np.zeros((len(rows), width))
            for q, i in enumerate(rows):
                G[q, :len(r["symm"][i])] = r["symm"][i]
            data[p + "symm"] = G
            data[p + "symm_atoms"] = rows.astype(np.int32)
            data[p + "ninput"] = np.array([len(g) for g in r["symm"]], dtype=np.int32)
            if lists and s.natoms <= LIST_ATOMS:
                nb = r["nb"]
                data[p + "nb_count"] = np.array([len(x["index"]) for x in nb], dtype=np.int32)
                cat = lambda key, dt: (np.concatenate([x[key] for x in nb]) if nb else np.zeros(0)).astype(dt)
                data[p + "nb_index"] = cat("index", np.int32)
                data[p + "nb_type"] = cat("type", np.int8)
                data[p + "nb_min"] = cat("min", np.uint8)
                data[p + "nb_r"] = (np.concatenate([x["r"] for x in nb]) if nb else np.zeros((0, 3))).astype(np.float64)
        print("case %-16s %-16s %d structures" % (case, variant, len(strucs)))
    data["cases"] = np.array(names)
    out = os.path.join(HERE, "reference.npz")
    np.savez_compressed(out, **data)
    print("wrote", out, os.path.getsize(out), "bytes")


if __name__ == "__main__":
    main()
