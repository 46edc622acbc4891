"""Runs the reference's own NNP path (oracle/_ref/ref_nnp, built by oracle/Makefile.ref from the
markdellostritto/AtomNN sources against the Eigen-API shim) on structures and parses its output.

TEST INFRASTRUCTURE ONLY: used by tests/golden/make_ref_golden.py to write golden vectors and by
the CPU tests that pin the oracle when the reference sources are present.  The reference sources
exist only where the reference is mounted; the committed fixtures carry its outputs elsewhere.
"""
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.environ.get("ATOMNN_REFERENCE", "/root/reference")
BIN = os.path.join(HERE, "_ref", "ref_nnp")
BIN_FMA = os.path.join(HERE, "_ref", "ref_nnp_fma")


def available():
    """True when the reference sources are present (the binary can be built)."""
    return os.path.isdir(os.path.join(REF_DIR, "src", "nnp"))


def build(fma=False):
    """Compile the reference's path against the shim (make -f oracle/Makefile.ref)."""
    target = "fma" if fma else "all"
    subprocess.run(["make", "-s", "-j8", "-f", os.path.join(HERE, "Makefile.ref"), "REF=" + REF_DIR, target], check=True)
    return BIN_FMA if fma else BIN


def species_names(potfile):
    """Species names of a potential file in type order (the 'name X' tokens of NNP::write)."""
    toks = open(potfile).read().split()
    return [toks[k + 1] for k in range(len(toks) - 1) if toks[k] == "name"]


def run(potfile, structures, lists=True, fma=False):
    """Energy (NNP::energy), energy without vacuum energies (NNP::compute), forces of NNP::force and
    NNP::compute, symmetry functions and (optionally) neighbour lists of each structure, computed by
    the reference.  Structures: objects with .posn (N,3), .species (N,) and .cell (3x3, columns =
    lattice vectors; zeros or None = not periodic)."""
    exe = BIN_FMA if fma else BIN
    if not os.path.exists(exe):
        build(fma)
    names = species_names(potfile)
    with tempfile.NamedTemporaryFile("w", suffix=".txt", delete=False) as f:
        path = f.name
        f.write(os.path.abspath(potfile) + "\n%d\n" % len(structures))
        for s in structures:
            periodic = s.cell is not None and float(np.abs(s.cell).sum()) > 0
            f.write("%d %d\n" % (s.natoms, 1 if periodic else 0))
            if periodic:
                f.write(" ".join("%.17g" % v for v in np.asarray(s.cell, dtype=np.float64).T.ravel()) + "\n")
            for i in range(s.natoms):
                p = s.posn[i]
                f.write("%s %.17g %.17g %.17g\n" % (names[int(s.species[i])], p[0], p[1], p[2]))
    try:
        r = subprocess.run([exe, path] + ([] if lists else ["nolist"]), capture_output=True, text=True)
    finally:
        os.unlink(path)
    if r.returncode != 0:
        raise RuntimeError("reference run failed: %s" % r.stderr.strip())
    return parse(r.stdout)


def parse(text):
    out = []
    lines = text.splitlines()
    k = 0
    cur = None
    while k < len(lines):
        t = lines[k].split()
        k += 1
        if not t:
            continue
        if t[0] == "struc":
            n = int(t[2])
            cur = dict(natoms=n, force=np.zeros((n, 3)), force_compute=np.zeros((n, 3)), symm=[None] * n, nb=[None] * n)
            out.append(cur)
        elif t[0] == "energy":
            cur["energy"] = float(t[1])
        elif t[0] == "energy_compute":
            cur["energy_compute"] = float(t[1])
        elif t[0] == "f":
            cur["force"][int(t[1])] = [float(x) for x in t[2:5]]
        elif t[0] == "fc":
            cur["force_compute"][int(t[1])] = [float(x) for x in t[2:5]]
        elif t[0] == "g":
            cur["symm"][int(t[1])] = np.array([float(x) for x in t[3:3 + int(t[2])]])
        elif t[0] == "nb":
            i, cnt = int(t[1]), int(t[2])
            rows = [lines[k + q].split() for q in range(cnt)]
            k += cnt
            cur["nb"][i] = dict(index=np.array([int(r[0]) for r in rows], dtype=np.int32),
                                type=np.array([int(r[1]) for r in rows], dtype=np.int32),
                                min=np.array([r[2] == "1" for r in rows], dtype=bool),
                                dr=np.array([float(r[3]) for r in rows]),
                                r=np.array([[float(x) for x in r[4:7]] for r in rows]).reshape(cnt, 3))
    return out
