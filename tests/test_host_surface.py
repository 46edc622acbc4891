"""The C++ host surface (include/atomnn_gpu.hpp, libatomnn_gpu.so) and the compute tool
nnp_compute_gpu (the counterpart of the reference's src/nnp/nnpce.cpp).

CPU tests: the parameter file and the POSCAR/XYZ readers (the tool's --dry-run path, which never
touches the GPU).  GPU tests: the tool's energies and forces, and the NNP / Structure /
NeighborList calls driven from C++ (tests/cpp/api_check.cpp), against the FP64 oracle."""
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, REPO
from atomnn_gb300 import workloads as W

E_TOL = 1e-5   # eV/atom, FP32 path
F_TOL = 1e-4   # eV/A max abs
NAMES = ["A", "B"]
BOHR_PER_ANG = 1.0 / 0.529177210903


@pytest.fixture(scope="module")
def tool(native_lib):
    from atomnn_gb300 import build
    _, exe = build.build_host()
    return exe


def _grouped(s):
    """The structure with its atoms grouped by species (POSCAR order), stable within a species."""
    order = np.argsort(s.species, kind="stable")
    return W.Structure(posn=s.posn[order].copy(), species=s.species[order].copy(), cell=s.cell.copy())


def _write_poscar(path, s, direct=True, scale=1.0):
    counts = [int((s.species == t).sum()) for t in range(len(NAMES))]
    lines = ["generated", "%.16g" % scale]
    for c in range(3):
        lines.append("%.16f %.16f %.16f" % tuple(s.cell[:, c] / scale))
    lines.append(" ".join(NAMES))
    lines.append(" ".join(str(c) for c in counts))
    lines.append("Direct" if direct else "Cartesian")
    frac = np.linalg.solve(s.cell, s.posn.T).T
    for p in (frac if direct else s.posn):
        lines.append("%.16f %.16f %.16f" % tuple(p))
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def _write_xyz(path, s, energy):
    lines = [str(s.natoms), "struc %.6f %.16f %.16f %.16f" % (energy, s.cell[0, 0], s.cell[1, 1], s.cell[2, 2])]
    for t, p in zip(s.species, s.posn):
        lines.append("%s %.16f %.16f %.16f" % ((NAMES[t],) + tuple(p)))
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def _params(tmp, files, fmt="POSCAR", units="METAL", force=True, extra=""):
    lst = os.path.join(tmp, "data.txt")
    with open(lst, "w") as f:
        f.write("\n".join(files) + "\n\n")
    par = os.path.join(tmp, "param.txt")
    with open(par, "w") as f:
        f.write("# compute parameters\nDATA %s\nNNPOT %s\nFORMAT %s\nUNITS %s\nFORCE %s  # forces too\nNORM F\n%s\n" % (
            lst, os.path.join(GOLDEN, "mixed512.nnp"), fmt, units, "T" if force else "F", extra))
    return par


def _run(exe, *args):
    r = subprocess.run([exe, *args], capture_output=True, text=True, timeout=600)
    return r.returncode, r.stdout + r.stderr


def _structures():
    strucs = W.make_structures("mixed512", seed=77, count=3, sizes=[40, 230, 700])
    return [_grouped(s) for s in strucs]


def test_dry_run_reads_poscar(tool, tmp_path):
    strucs = _structures()
    files = []
    for k, s in enumerate(strucs):
        p = str(tmp_path / ("POSCAR_%d" % k))
        _write_poscar(p, s, direct=(k != 1), scale=(1.7 if k == 2 else 1.0))
        files.append(p)
    rc, out = _run(tool, _params(str(tmp_path), files), "--dry-run")
    assert rc == 0, out
    assert "structures = 3" in out and "atoms = %d" % sum(s.natoms for s in strucs) in out
    lines = [l for l in out.splitlines() if l.startswith("struc ")]
    for k, (l, s) in enumerate(zip(lines, strucs)):
        f = l.split()
        assert int(f[4]) == s.natoms and f[6] == "1" and f[10] == NAMES[s.species[0]]
        np.testing.assert_allclose([float(x) for x in f[11:14]], s.posn[0], rtol=0, atol=1e-9)


def test_dry_run_reads_xyz_in_au(tool, tmp_path):
    s = _grouped(W.make_structures("cell1728")[0])
    p = str(tmp_path / "s.xyz")
    _write_xyz(p, s, -12.5)
    rc, out = _run(tool, _params(str(tmp_path), [p], fmt="XYZ", units="AU"), "--dry-run")
    assert rc == 0, out
    f = [l for l in out.splitlines() if l.startswith("struc ")][0].split()
    assert int(f[4]) == s.natoms
    assert abs(float(f[8]) - (-12.5 / 27.211386245988)) < 1e-6
    np.testing.assert_allclose([float(x) for x in f[11:14]], s.posn[0] * BOHR_PER_ANG, rtol=0, atol=1e-6)


@pytest.mark.parametrize("bad,msg", [("UNITS LJX", "Invalid unit system"), ("FORMAT QE", "Invalid file format")])
def test_parameter_errors(tool, tmp_path, bad, msg):
    par = str(tmp_path / "param.txt")
    with open(par, "w") as f:
        f.write("DATA x\nNNPOT y\n%s\n" % bad)
    rc, out = _run(tool, par, "--dry-run")
    assert rc == 1 and msg in out


def test_missing_structure_file(tool, tmp_path):
    rc, out = _run(tool, _params(str(tmp_path), [str(tmp_path / "nope")]), "--dry-run")
    assert rc == 1 and "Could not open" in out


@pytest.fixture(scope="module")
def binary_check(native_lib, tmp_path_factory):
    from atomnn_gb300 import build
    build.build_host()
    exe = str(tmp_path_factory.mktemp("bin") / "binary_check")
    out_dir = os.path.join(REPO, "atomnn_gb300", "_build")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I" + os.path.join(REPO, "include"), os.path.join(REPO, "tests", "cpp", "binary_check.cpp"),
                    "-o", exe, "-L" + out_dir, "-latomnn_gpu", "-lnnpgpu", "-Wl,-rpath," + out_dir], check=True)
    return exe


def _binary_struc(rng, natoms, flags):
    from oracle import struc_binary as SB
    s = {"R": rng.normal(size=(3, 3)), "natoms": natoms, "t": int(rng.integers(0, 1000)),
         "flags": {f: (f in flags) for f in SB.FLAGS}}
    for k in SB.STATE:
        s[k] = float(rng.normal())
    s["name"] = [["Mg", "O", "Xx_long_name"][k % 3] for k in range(natoms)]
    for k in SB.INTS:
        s[k] = rng.integers(-5, 100, natoms)
    for k in SB.DOUBLES:
        s[k] = rng.normal(size=natoms)
    for k in SB.VEC3:
        s[k] = rng.normal(size=(natoms, 3))
    s["symm"] = [rng.normal(size=int(rng.integers(0, 9))) for _ in range(natoms)]
    return s


@pytest.mark.parametrize("flags", ["all", "default", "posn_only"])
def test_binary_structure_roundtrip(binary_check, tmp_path, flags):
    """Structure::read_binary of a file written by the layout's restatement (oracle/struc_binary.py)
    gives every flagged property; Structure::write_binary writes the same bytes back."""
    from oracle import struc_binary as SB
    sel = {"all": SB.FLAGS, "default": ["name", "type", "index", "posn", "force", "symm"], "posn_only": ["posn"]}[flags]
    rng = np.random.default_rng(len(flags))
    s = _binary_struc(rng, 7, sel)
    src, dst = tmp_path / "in.dat", tmp_path / "out.dat"
    src.write_bytes(SB.pack(s))
    rc, out = _run(binary_check, str(src), str(dst))
    assert rc == 0, out
    assert dst.read_bytes() == src.read_bytes()
    rows = [l.split() for l in out.splitlines()]
    assert rows[0] == ["natoms", "7"]
    assert rows[1][1] == "".join("1" if f in sel else "0" for f in SB.FLAGS)
    np.testing.assert_array_equal([float(x) for x in rows[2][1:]], s["R"].flatten(order="F"))
    np.testing.assert_array_equal([float(x) for x in rows[3][1:9]], [s[k] for k in SB.STATE])
    assert int(rows[3][9]) == s["t"]
    atoms = [r for r in rows if r[0] == "atom"]
    extra = [r for r in rows if r[0] == "extra"]
    for i in range(7):
        a, x = atoms[i], extra[i]
        assert a[2] == (s["name"][i] if "name" in sel else "-")
        assert int(a[3]) == (s["type"][i] if "type" in sel else -1)
        assert int(a[4]) == (s["index"][i] if "index" in sel else i)
        np.testing.assert_array_equal([float(v) for v in a[5:8]], s["posn"][i])
        np.testing.assert_array_equal([float(v) for v in a[8:11]], s["force"][i] if "force" in sel else np.zeros(3))
        g = s["symm"][i] if "symm" in sel else np.zeros(0)
        total = 0.0
        for v in g.tolist():  # summed in order, as the C++ side does (sum() compensates)
            total += v
        assert int(a[11]) == len(g) and float(a[12]) == total
        assert int(x[2]) == (s["an"][i] if "an" in sel else 0)
        for k, name in enumerate(SB.DOUBLES):
            assert float(x[3 + k]) == (s[name][i] if name in sel else 0.0)
        np.testing.assert_array_equal([float(v) for v in x[10:13]], s["vel"][i] if "vel" in sel else np.zeros(3))
        np.testing.assert_array_equal([float(v) for v in x[13:16]], s["spin"][i] if "spin" in sel else np.zeros(3))


def test_binary_structure_rejects_malformed(binary_check, tmp_path):
    from oracle import struc_binary as SB
    rng = np.random.default_rng(3)
    good = SB.pack(_binary_struc(rng, 5, SB.FLAGS))
    bad_files = {
        "truncated": good[:-9],
        "count_mismatch": good[:4] + good[4:4 + 72 + 64 + 4 + 16] + (6).to_bytes(4, "little") + good[4 + 72 + 64 + 4 + 16 + 4:],
        "trailing": (len(good) - 4 + 3).to_bytes(4, "little") + good[4:] + b"abc",
    }
    for name, data in bad_files.items():
        p = tmp_path / (name + ".dat")
        p.write_bytes(data)
        rc, out = _run(binary_check, str(p), str(tmp_path / "o.dat"))
        assert rc == 1 and "ERROR" in out and "read_binary" in out, (name, out)
    rc, out = _run(binary_check, str(tmp_path / "missing.dat"), str(tmp_path / "o.dat"))
    assert rc == 1 and "Could not open" in out


@pytest.mark.gpu
def test_tool_matches_oracle(tool, tmp_path, oracle_lib):
    strucs = _structures()
    files = []
    for k, s in enumerate(strucs):
        p = str(tmp_path / ("POSCAR_%d" % k))
        _write_poscar(p, s, direct=(k != 1))
        files.append(p)
    rc, out = _run(tool, _params(str(tmp_path), files, extra="BATCH 500"))
    assert rc == 0, out
    energies = [float(l.split()[3]) for l in out.splitlines() if l.startswith("energy ")]
    forces, cur = [], None
    for l in out.splitlines():
        if l.startswith("struc["):
            cur = []
            forces.append(cur)
        elif l.startswith("force["):
            cur.append([float(x) for x in l.split("=")[1].split()])
    orc = oracle_lib.OracleNNP(os.path.join(GOLDEN, "mixed512.nnp"))
    assert len(energies) == 3 and len(forces) == 3
    for s, e, F in zip(strucs, energies, forces):
        eo, Fo, _ = orc.compute(s.posn, s.species, s.cell, force=True)
        assert abs(e - eo) / s.natoms <= E_TOL
        assert np.abs(np.array(F) - Fo).max() <= F_TOL


@pytest.mark.gpu
def test_cpp_api_matches_oracle(native_lib, tmp_path, oracle_lib):
    from atomnn_gb300 import build
    build.build_host()
    exe = str(tmp_path / "api_check")
    out_dir = os.path.join(REPO, "atomnn_gb300", "_build")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I" + os.path.join(REPO, "include"), os.path.join(REPO, "tests", "cpp", "api_check.cpp"),
                    "-o", exe, "-L" + out_dir, "-latomnn_gpu", "-lnnpgpu", "-Wl,-rpath," + out_dir], check=True)
    s = _structures()[1]
    p = str(tmp_path / "POSCAR")
    _write_poscar(p, s)
    rc, out = _run(exe, os.path.join(GOLDEN, "mixed512.nnp"), p, str(tmp_path / "struc.dat"))
    assert rc == 0, out
    rows = [l.split() for l in out.splitlines()]
    pot = os.path.join(GOLDEN, "mixed512.nnp")
    orc = oracle_lib.OracleNNP(pot)
    eo, Fo, Go = orc.compute(s.posn, s.species, s.cell, force=True, symm=True)
    ec, _, _ = orc.compute(s.posn, s.species, s.cell, compute_semantics=True)
    nb = oracle_lib.neighbors(orc.rc, s.posn, s.cell)
    nl = [r for r in rows if r[0] == "nlist"][0]
    assert int(nl[1]) == s.natoms and int(nl[2]) == sum(len(x["index"]) for x in nb)
    assert int(nl[3]) == sum(int(np.sum(x["min"])) for x in nb)
    G0 = np.array([float(r[3]) for r in rows if r[0] == "symm"])
    scale = np.abs(Go).max()
    np.testing.assert_allclose(G0, Go[0, :len(G0)], rtol=0, atol=1e-5 * scale)
    e = float([r for r in rows if r[0] == "energy"][0][1])
    assert abs(e - eo) / s.natoms <= E_TOL
    # stored descriptors read back from the binary file give the same energy; so do the positions
    assert float([r for r in rows if r[0] == "cached"][0][1]) == e
    assert abs(float([r for r in rows if r[0] == "positions"][0][1]) - eo) / s.natoms <= E_TOL
    F = np.array([[float(x) for x in r[2:5]] for r in rows if r[0] == "force"])
    assert np.abs(F - Fo).max() <= F_TOL
    assert abs(float([r for r in rows if r[0] == "compute"][0][1]) - ec) / s.natoms <= E_TOL
    b = [r for r in rows if r[0] == "batched"][0]
    assert abs(float(b[1]) - eo) / s.natoms <= E_TOL and float(b[1]) == float(b[2])
    assert ["invalid_argument", "ok"] in rows
    # the reference's trainer loop (NeighborList(struc, rc), NNP::symm, NNP::energy) and compute-tool
    # loop (build, symm, energy, force) compiled unchanged against the surface
    assert abs(float([r for r in rows if r[0] == "trainer"][0][1]) - eo) / s.natoms <= E_TOL
    t = [r for r in rows if r[0] == "tool"][0]
    assert abs(float(t[1]) - eo) / s.natoms <= E_TOL and abs(float(t[2]) - Fo[0, 0]) <= F_TOL
    assert ["nbtype", "ok"] in rows and ["subset", "ok"] in rows
    # FP64 neighbour vectors and distances of atom 0 (the reference keeps Eigen::Vector3d)
    r64 = np.array([[float(x) for x in r[1:]] for r in rows if r[0] == "r64"])
    np.testing.assert_array_equal(r64[:, 0].astype(int), nb[0]["index"])
    np.testing.assert_array_equal(r64[:, 1].astype(bool), nb[0]["min"])
    np.testing.assert_allclose(r64[:, 2:5], nb[0]["r"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(r64[:, 5], nb[0]["dr"], rtol=0, atol=1e-12)
