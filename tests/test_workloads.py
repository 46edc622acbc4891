"""CPU tests of the seeded workload generator (the stand-in for the reference's example data)."""
import numpy as np

from atomnn_gb300 import workloads as W


def test_structures_are_deterministic():
    a = W.make_structures("mixed512", count=4)
    b = W.make_structures("mixed512", count=4)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x.posn, y.posn)
        np.testing.assert_array_equal(x.species, y.species)


def test_mixed_workload_shapes():
    strucs = W.make_structures("mixed512")
    n = np.array([s.natoms for s in strucs])
    assert len(strucs) == 512 and n.min() >= 16 and n.max() <= 2048
    for s in strucs[:64]:
        vol = abs(np.linalg.det(s.cell))
        assert 0.049 <= s.natoms / vol <= 0.091
        a = s.cell[:, 0], s.cell[:, 1], s.cell[:, 2]
        for u, v in ((1, 2), (0, 2), (0, 1)):
            ang = np.degrees(np.arccos(a[u] @ a[v] / np.linalg.norm(a[u]) / np.linalg.norm(a[v])))
            assert 79.9 <= ang <= 100.1
        assert abs((s.species == 0).sum() - round(s.natoms / 3)) <= 1


def test_fixed_cells():
    s = W.make_structures("small64")[0]
    assert s.natoms == 64 and np.allclose(s.cell, np.eye(3) * 8.1)
    c = W.make_structures("cell1728")[0]
    assert c.natoms == 1728 and (c.species == 0).sum() == 576
    assert abs(1728 / np.linalg.det(c.cell) - 0.07) < 1e-9


def test_potentials_parse_in_oracle(oracle_lib, tmp_path):
    for name, nin in (("small64", [32]), ("mixed512", [56, 56]), ("cell65536", [96, 96])):
        p = str(tmp_path / (name + ".nnp"))
        W.write_potential(W.make_potential(name), p)
        orc = oracle_lib.OracleNNP(p)
        assert orc.ninput == nin
