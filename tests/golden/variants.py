"""Potential variants for the reference-pinned fixtures: text substitutions on the committed
potential files (mixed512.nnp, small64.nnp), so that every machine rebuilds the same files
without a random generator.  Each variant changes one option of the reference's option space and
keeps the input sizes (and so the networks):

  base_mixed512 / base_small64   the committed files
  radial_<F>     BasisR family F (GAUSSIAN, TANH, SOFTPLUS, LOGCOSH, SWISH, MISH; basis_radial.cpp:302-444)
  angular_<F>    BasisA family F (GAUSS, IPOWP, IPOWS, SECHP, SECHS; basis_angular.cpp:406-640)
  cut_<C>        cutoff function C of every basis (COS, TANH, STEP; basis.cpp:80-120)
  norm_VOL       VOL normalisation of every basis (basis.cpp:160-168)
  zeta_real      angular zeta values 1, 2, 4, 16 replaced by 1.5, 2.7, 3.3, 7.25 (pow with real zeta)
  eta_many       the A-B angular block as 6 distinct eta x zeta 2 x lambda +-1 (12 functions)
"""
import os

HERE = os.path.dirname(os.path.abspath(__file__))

RADIAL = ("GAUSSIAN", "TANH", "SOFTPLUS", "LOGCOSH", "SWISH", "MISH")
ANGULAR = ("GAUSS", "IPOWP", "IPOWS", "SECHP", "SECHS")
CUTOFFS = ("TANH", "STEP")
NAMES = (["base_mixed512", "base_small64"] + ["radial_" + f for f in RADIAL[1:]] + ["angular_" + f for f in ANGULAR[1:]] +
         ["cut_" + c for c in CUTOFFS] + ["norm_VOL", "zeta_real", "eta_many"])

ZETA_MAP = {"1.000000": "1.500000", "2.000000": "2.700000", "4.000000": "3.300000", "16.000000": "7.250000"}
ETA_MANY = ["14.142136", "8.000000", "4.472136", "3.000000", "2.236068", "1.414214"]


def _lines(base):
    with open(os.path.join(HERE, base + ".nnp")) as f:
        return f.read().split("\n")


def text(name):
    """The potential file text of variant ``name``."""
    if name == "base_small64":
        return "\n".join(_lines("small64"))
    lines = _lines("mixed512")
    if name == "base_mixed512":
        return "\n".join(lines)
    out = []
    block = None  # (i, j, k) of the current angular block
    for ln in lines:
        t = ln.split()
        if t[:1] == ["basis_angular"]:
            block = tuple(t[1:3])
        elif t[:1] in (["basis_radial"], ["nn"]):
            block = None
        if t[:1] == ["BasisR"] or t[:1] == ["BasisA"]:
            # BasisR|BasisA <norm> <cut> <rc> <family> <n> [alpha]
            if name.startswith("radial_") and t[0] == "BasisR":
                t[4] = name[len("radial_"):]
            if name.startswith("angular_") and t[0] == "BasisA":
                t[4] = name[len("angular_"):]
            if name.startswith("cut_"):
                t[2] = name[len("cut_"):]
            if name == "norm_VOL":
                t[1] = "VOL"
            out.append(" ".join(t))
            continue
        if block is not None and ln.startswith("\t") and len(t) == 3:
            eta, zeta, lam = t
            if name == "zeta_real":
                zeta = ZETA_MAP.get(zeta, zeta)
            out.append("\t%s %s %s" % (eta, zeta, lam))
            continue
        out.append(ln)
    if name == "eta_many":
        out = _eta_many(out)
    return "\n".join(out)


def _eta_many(lines):
    res, k = [], 0
    while k < len(lines):
        ln = lines[k]
        res.append(ln)
        if ln.split()[:3] == ["basis_angular", "A", "B"] or ln.split()[:3] == ["basis_angular", "B", "A"]:
            head = lines[k + 1].split()
            n = int(head[5])
            res.append(lines[k + 1])
            entries = []
            for e in ETA_MANY:
                for lam in (1, -1):
                    entries.append("\t%s 2.000000 %d" % (e, lam))
            assert len(entries) == n, "the A-B block keeps its 12 functions"
            res.extend(entries)
            k += 2 + n
            continue
        k += 1
    return res


def write(name, directory):
    """Write variant ``name`` into ``directory``; returns its path."""
    os.makedirs(directory, exist_ok=True)
    path = os.path.join(directory, name + ".nnp")
    with open(path, "w") as f:
        f.write(text(name))
    return path
