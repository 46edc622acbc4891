"""The FP64 oracle against the reference's own code.

tests/golden/reference.npz holds outputs of markdellostritto/AtomNN's NeighborList::build,
NNP::symm, NNP::energy, NNP::force and NNP::compute, compiled from the reference's sources
(oracle/Makefile.ref, against the Eigen-API shim oracle/ref_shim/) and written by
tests/golden/make_ref_golden.py.  The oracle must reproduce them: neighbour lists exactly (order,
indices, species, minimum-image flags) with vectors to 1e-12 A, energies and symmetry functions to
1e-12 relative, forces to 1e-12 relative to the largest force (the force sums' order differs in the
last bits).  Where the reference sources are present, the same holds on freshly drawn structures,
and an FMA-contracting build of the reference yields the same neighbour sets.
"""
import os
import platform
import sys

import numpy as np
import pytest

from conftest import GOLDEN
from atomnn_gb300 import workloads as W

sys.path.insert(0, GOLDEN)
import variants as V  # noqa: E402

REF = np.load(os.path.join(GOLDEN, "reference.npz"))
CASES = [str(c) for c in REF["cases"]]
REL = 1e-12


def _strucs(case):
    out = []
    for k in range(int(REF[case + "/nstruc"][0])):
        p = "%s/%d/" % (case, k)
        out.append((W.Structure(posn=REF[p + "posn"], species=REF[p + "species"], cell=REF[p + "cell"]), p))
    return out


def _check(orc, s, p, e, F, G, ec, Fc, lists):
    assert abs(e - REF[p + "energy"][0]) <= REL * max(1.0, abs(e))
    assert abs(ec - REF[p + "energy_compute"][0]) <= REL * max(1.0, abs(ec))
    fs = max(1.0, float(np.abs(REF[p + "force"]).max())) if s.natoms else 1.0
    assert np.abs(F - REF[p + "force"]).max(initial=0) <= REL * fs
    assert np.abs(Fc - REF[p + "force_compute"]).max(initial=0) <= REL * fs
    rows, Gr = REF[p + "symm_atoms"], REF[p + "symm"]
    if len(rows):
        assert np.abs(G[rows, :Gr.shape[1]] - Gr).max() <= REL * max(np.abs(Gr).max(), 1e-300)
    np.testing.assert_array_equal([orc.ninput[t] for t in s.species], REF[p + "ninput"])
    if lists and (p + "nb_count") in REF.files:
        from oracle import pyoracle
        nb = pyoracle.neighbors(orc.rc, s.posn, s.cell)
        np.testing.assert_array_equal([len(x["index"]) for x in nb], REF[p + "nb_count"])
        if s.natoms and len(REF[p + "nb_index"]):
            np.testing.assert_array_equal(np.concatenate([x["index"] for x in nb]), REF[p + "nb_index"])
            np.testing.assert_array_equal(np.concatenate([x["min"] for x in nb]).astype(np.uint8), REF[p + "nb_min"])
            np.testing.assert_array_equal(s.species[np.concatenate([x["index"] for x in nb])], REF[p + "nb_type"])
            assert np.abs(np.concatenate([x["r"] for x in nb]) - REF[p + "nb_r"]).max() <= 1e-12


@pytest.mark.parametrize("case", CASES)
def test_oracle_matches_reference_fixture(oracle_lib, tmp_path, case):
    pot = V.write(str(REF[case + "/variant"][0]), str(tmp_path))
    orc = oracle_lib.OracleNNP(pot)
    for s, p in _strucs(case):
        e, F, G = orc.compute(s.posn, s.species, s.cell, force=True, symm=True)
        ec, Fc, _ = orc.compute(s.posn, s.species, s.cell, compute_semantics=True)
        _check(orc, s, p, e, F, G, ec, Fc, lists=True)


def test_fixture_covers_the_option_space():
    """Every basis family, cutoff and norm of the reference, real zeta and many eta are pinned."""
    want = {"radial_" + f for f in V.RADIAL[1:]} | {"angular_" + f for f in V.ANGULAR[1:]} | {"cut_TANH", "cut_STEP", "norm_VOL",
                                                                                            "zeta_real", "eta_many"}
    assert want <= set(CASES)
    assert {"small64", "mixed3", "cluster20", "edge"} <= set(CASES)


# ---------------------------------------------------------------- live, where the reference is present
def _live():
    from oracle import refrun
    if not refrun.available():
        pytest.skip("reference sources not present (the committed fixture covers this machine)")
    return refrun


@pytest.mark.parametrize("variant", ["base_mixed512", "zeta_real", "cut_TANH", "angular_SECHS"])
def test_oracle_matches_reference_live(oracle_lib, tmp_path, variant):
    """Fresh seeded structures (triclinic cells of 12-300 atoms, a sheared cell, a cluster): the
    oracle equals the reference's own code run now."""
    refrun = _live()
    pot = V.write(variant, str(tmp_path))
    rng = np.random.default_rng(20260)
    strucs = W.make_structures("mixed512", seed=int(rng.integers(1 << 30)), count=4, sizes=[12, 35, 120, 300])
    cell = W.lattice(6.5, 7.0, 9.0, 55.0, 120.0, 70.0)
    strucs.append(W.Structure(posn=rng.uniform(0, 1, size=(30, 3)) @ cell.T, species=(np.arange(30) % 2).astype(np.int32), cell=cell))
    strucs.append(W.Structure(posn=rng.uniform(-4, 4, size=(15, 3)), species=(np.arange(15) % 2).astype(np.int32), cell=np.zeros((3, 3))))
    res = refrun.run(pot, strucs)
    orc = oracle_lib.OracleNNP(pot)
    from oracle import pyoracle
    for s, r in zip(strucs, res):
        e, F, G = orc.compute(s.posn, s.species, s.cell, force=True, symm=True)
        ec, Fc, _ = orc.compute(s.posn, s.species, s.cell, compute_semantics=True)
        assert abs(e - r["energy"]) <= REL * max(1.0, abs(e)) and abs(ec - r["energy_compute"]) <= REL * max(1.0, abs(ec))
        fs = max(1.0, float(np.abs(r["force"]).max()))
        assert np.abs(F - r["force"]).max() <= REL * fs and np.abs(Fc - r["force_compute"]).max() <= REL * fs
        for i in range(s.natoms):
            g = r["symm"][i]
            assert np.abs(G[i, :len(g)] - g).max(initial=0) <= REL * max(np.abs(g).max(initial=0), 1e-300)
        nb = pyoracle.neighbors(orc.rc, s.posn, s.cell)
        for i in range(s.natoms):
            np.testing.assert_array_equal(nb[i]["index"], r["nb"][i]["index"])
            np.testing.assert_array_equal(nb[i]["min"], r["nb"][i]["min"])
            if len(nb[i]["r"]):
                assert np.abs(nb[i]["r"] - r["nb"][i]["r"]).max() <= 1e-12


@pytest.mark.skipif(platform.machine() not in ("x86_64", "AMD64"), reason="the FMA build uses x86 -mfma")
def test_fma_build_gives_the_same_neighbour_sets(tmp_path):
    """The reference builds with -O3 -march=native (src/Makefile.gnu), which lets GCC contract
    multiply-adds on an FMA host.  Such a build yields the same neighbour sets with the same
    minimum images; only the list order may differ where lattice vectors have equal norms and the
    contracted norms sort them differently."""
    refrun = _live()
    pot = V.write("base_mixed512", str(tmp_path))
    strucs = [s for case in ("mixed3", "edge") for s, _ in _strucs(case)]
    a = refrun.run(pot, strucs)
    b = refrun.run(pot, strucs, fma=True)
    for s, x, y in zip(strucs, a, b):
        assert abs(x["energy"] - y["energy"]) <= 1e-12 * max(1.0, abs(x["energy"]))
        for i in range(s.natoms):
            key = lambda L: sorted(zip(L["index"].tolist(), np.round(L["r"], 9).tolist(), L["min"].tolist()))
            assert key(x["nb"][i]) == key(y["nb"][i])
