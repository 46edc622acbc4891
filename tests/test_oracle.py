"""CPU tests of the FP64 oracle: golden fixtures and the properties the reference's own test
programs check (they print rather than assert; here each becomes an assertion)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, load_golden
from atomnn_gb300 import workloads as W


@pytest.mark.parametrize("name", ["small64", "mixed3", "cluster20"])
def test_golden_fixtures_reproduced(oracle_lib, name):
    cases = load_golden(name)
    pot = os.path.join(GOLDEN, str(np.load(os.path.join(GOLDEN, name + ".npz"))["potential"][0]) + ".nnp")
    orc = oracle_lib.OracleNNP(pot)
    for s, ref in cases:
        e, F, G = orc.compute(s.posn, s.species, s.cell, force=True, symm=True)
        ec, _, _ = orc.compute(s.posn, s.species, s.cell, compute_semantics=True)
        assert abs(e - ref["energy"][0]) <= 1e-10 * max(1.0, abs(e))
        assert abs(ec - ref["energy_compute"][0]) <= 1e-10 * max(1.0, abs(ec))
        np.testing.assert_allclose(F, ref["force"], rtol=0, atol=1e-10)
        np.testing.assert_allclose(G, ref["symm"], rtol=1e-12, atol=1e-12)
        nb = oracle_lib.neighbors(orc.rc, s.posn, s.cell)
        np.testing.assert_array_equal([len(x["index"]) for x in nb], ref["nb_count"])
        np.testing.assert_array_equal(np.concatenate([x["index"] for x in nb]), ref["nb_index"])
        np.testing.assert_array_equal(np.concatenate([x["shift"] for x in nb]), ref["nb_shift"])
        np.testing.assert_array_equal(np.concatenate([x["min"] for x in nb]).astype(np.uint8), ref["nb_min"])


def _rocksalt(a, rng, sigma=0.05):
    """Conventional 8-atom rocksalt cell (A on 4a, B on 4b) with small displacements."""
    fcc = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    frac = np.concatenate([fcc, fcc + [0.5, 0, 0]]) % 1.0
    posn = frac * a + rng.normal(0, sigma, size=(8, 3))
    species = np.array([0] * 4 + [1] * 4, dtype=np.int32)
    return W.Structure(posn=posn, species=species, cell=np.eye(3) * a)


def _supercell(s, reps):
    cells = [(i, j, k) for i in range(reps[0]) for j in range(reps[1]) for k in range(reps[2])]
    posn = np.concatenate([s.posn + s.cell @ np.array(c, dtype=float) for c in cells])
    species = np.concatenate([s.species] * len(cells))
    return W.Structure(posn=posn, species=species, cell=s.cell * np.array(reps, dtype=float)[None, :])


@pytest.mark.parametrize("kind", ["rocksalt", "random8"])
def test_supercell_invariance(oracle_lib, pot_mixed, kind):
    """Symmetry functions and energy per atom of a cell equal those of its supercell
    (src/nnp/test_nnp_symm.cpp:292-501)."""
    rng = np.random.default_rng(11)
    if kind == "rocksalt":
        s = _rocksalt(5.64, rng)
        reps = (2, 2, 2)
    else:
        cell = W.lattice(4.6, 5.1, 4.9, 84.0, 95.0, 88.0)
        frac = rng.uniform(0, 1, size=(8, 3))
        s = W.Structure(posn=frac @ cell.T, species=np.array([0, 1] * 4, dtype=np.int32), cell=cell)
        reps = (3, 3, 3)
    sup = _supercell(s, reps)
    orc = oracle_lib.OracleNNP(pot_mixed)
    e1, _, G1 = orc.compute(s.posn, s.species, s.cell, force=False, symm=True)
    e2, _, G2 = orc.compute(sup.posn, sup.species, sup.cell, force=False, symm=True)
    n = s.natoms
    for r in range(int(np.prod(reps))):
        np.testing.assert_allclose(G2[r * n:(r + 1) * n], G1, rtol=1e-9, atol=1e-9)
    assert abs(e2 / sup.natoms - e1 / n) < 1e-9


def test_neighbors_contained_in_supercell(oracle_lib):
    """Every neighbour displacement of a skewed cell appears in the supercell's list, without
    duplicates (src/struc/test_neigh_unit.cpp:14-109)."""
    rng = np.random.default_rng(3)
    cell = W.lattice(5.0, 5.5, 6.0, 75.0, 100.0, 85.0)
    s = W.Structure(posn=rng.uniform(0, 1, size=(5, 3)) @ cell.T, species=np.zeros(5, np.int32), cell=cell)
    sup = _supercell(s, (3, 3, 3))
    rc = 7.0
    nb = oracle_lib.neighbors(rc, s.posn, s.cell)
    nbs = oracle_lib.neighbors(rc, sup.posn, sup.cell, cap=2048)
    for i in range(s.natoms):
        mine = np.round(nb[i]["r"], 8)
        theirs = {tuple(v) for v in np.round(nbs[i]["r"], 8)}
        assert len({tuple(v) for v in mine}) == len(mine), "duplicate neighbour vectors"
        for v in mine:
            assert tuple(v) in theirs


def _big_cell(n=192, L=14.2, seed=9):
    rng = np.random.default_rng(seed)
    return W._grid_structure(rng, n, np.eye(3) * L, 0.15, n // 3)


def test_forces_match_finite_differences(oracle_lib, pot_mixed):
    """With every in-cutoff image unique (cell widths > 2 rc) the reference's forces are the exact
    gradient of its energy (finite differences as in src/ml/test_nn_grad.cpp)."""
    s = _big_cell()
    orc = oracle_lib.OracleNNP(pot_mixed)
    assert 14.2 > 2 * orc.rc
    _, F, _ = orc.compute(s.posn, s.species, s.cell, force=True)
    h = 1e-5
    for atom, x in [(0, 0), (5, 1), (77, 2), (150, 0)]:
        p = s.posn.copy()
        p[atom, x] += h
        ep, _, _ = orc.compute(p, s.species, s.cell, force=False)
        p[atom, x] -= 2 * h
        em, _, _ = orc.compute(p, s.species, s.cell, force=False)
        fd = -(ep - em) / (2 * h)
        assert abs(fd - F[atom, x]) < 1e-6 * max(1.0, abs(F[atom, x]))


@pytest.mark.parametrize("kind,family", [("radial", f) for f in ("TANH", "SOFTPLUS", "LOGCOSH", "SWISH", "MISH")] +
                         [("angular", f) for f in ("IPOWP", "IPOWS", "SECHP", "SECHS")])
def test_basis_families_match_finite_differences(oracle_lib, tmp_path, kind, family):
    """The force expressions of every radial (basis_radial.cpp:371-444) and angular
    (basis_angular.cpp:456-640) family are the gradient of the energy they give, the property the
    reference's test_basis_radial.cpp and test_basis_angular.cpp check by finite differences."""
    pot = W.make_potential("mixed512")
    for b in (pot.radial if kind == "radial" else pot.angular).values():
        b.phi = family
    path = str(tmp_path / "family.nnp")
    W.write_potential(pot, path)
    s = _big_cell()
    orc = oracle_lib.OracleNNP(path)
    _, F, _ = orc.compute(s.posn, s.species, s.cell, force=True)
    assert np.abs(F).max() > 1e-3
    h = 1e-5
    for atom, x in [(5, 1), (150, 0)]:
        p = s.posn.copy()
        p[atom, x] += h
        ep, _, _ = orc.compute(p, s.species, s.cell, force=False)
        p[atom, x] -= 2 * h
        em, _, _ = orc.compute(p, s.species, s.cell, force=False)
        fd = -(ep - em) / (2 * h)
        assert abs(fd - F[atom, x]) < 1e-6 * max(1.0, abs(F[atom, x]))


def test_min_image_quirk(oracle_lib, pot_small64, pot_mixed):
    """NNP::force adds the neighbour-side term only for the minimum image
    (src/nnp/nnp.cpp:445,471,475): forces of a cell narrower than 2 rc do not sum to zero,
    those of a wide cell do."""
    s = W.make_structures("small64")[0]
    _, F, _ = oracle_lib.OracleNNP(pot_small64).compute(s.posn, s.species, s.cell, force=True)
    assert np.abs(F.sum(axis=0)).max() > 1e-4
    b = _big_cell()
    _, Fb, _ = oracle_lib.OracleNNP(pot_mixed).compute(b.posn, b.species, b.cell, force=True)
    assert np.abs(Fb.sum(axis=0)).max() < 1e-10


def test_compute_semantics(oracle_lib, pot_mixed):
    """NNP::compute's energy omits the species vacuum energy that NNP::energy adds (nnh.cpp:127-130)."""
    s = W.make_structures("mixed512", seed=5, count=1, sizes=[40])[0]
    orc = oracle_lib.OracleNNP(pot_mixed)
    e, F, _ = orc.compute(s.posn, s.species, s.cell, force=True)
    ec, Fc, _ = orc.compute(s.posn, s.species, s.cell, compute_semantics=True)
    pot = W.make_potential("mixed512")
    evac = sum(pot.species[t].energy for t in s.species)
    assert abs((e - ec) - evac) < 1e-9
    np.testing.assert_allclose(F, Fc, rtol=0, atol=1e-12)


def test_potential_file_roundtrip(oracle_lib, pot_mixed, tmp_path):
    """NNP::write then NNP::read gives the same potential (src/nnp/nnp.cpp:198-308)."""
    orc = oracle_lib.OracleNNP(pot_mixed)
    out = str(tmp_path / "rt.nnp")
    orc.write(out)
    orc2 = oracle_lib.OracleNNP(out)
    s = W.make_structures("mixed512", seed=5, count=1, sizes=[30])[0]
    e1, F1, _ = orc.compute(s.posn, s.species, s.cell, force=True)
    e2, F2, _ = orc2.compute(s.posn, s.species, s.cell, force=True)
    assert abs(e1 - e2) < 1e-12 * max(1, abs(e1))
    np.testing.assert_allclose(F1, F2, rtol=0, atol=1e-12)


def test_nonperiodic_min_flags(oracle_lib):
    """Non-periodic lists never set the minimum-image flag (src/struc/neighbor.cpp:149-169)."""
    rng = np.random.default_rng(2)
    nb = oracle_lib.neighbors(6.0, rng.uniform(0, 6, size=(10, 3)), None)
    assert all(not x["min"].any() for x in nb)
    assert sum(len(x["index"]) for x in nb) > 0


def _param_slot(pot, t, q):
    """(kind, layer, node, input) of parameter q of species t in the reference's order: every
    layer's biases, then every layer's weights with the input index outer (Cost::grad)."""
    net = pot.nets[t]
    dims = [net.nin] + list(net.nodes)
    nb = sum(net.nodes)
    if q < nb:
        for l, n in enumerate(net.nodes):
            if q < n:
                return "b", l, q, None
            q -= n
    q -= nb
    for l in range(len(net.nodes)):
        R, C = dims[l + 1], dims[l]
        if q < R * C:
            return "w", l, q % R, q // R
        q -= R * C
    raise IndexError


@pytest.mark.parametrize("loss,delta", [(0, 1.0), (2, 0.05), (3, 0.05), (1, 1.0)])
def test_train_gradient_matches_finite_differences(oracle_lib, tmp_path, loss, delta):
    """The trainer's batch gradient (Cost::grad summed as in nnpte.cpp:870-921) equals central
    differences of its batch loss in single network parameters, for each loss type."""
    pot = W.make_potential("cell1728")
    path = str(tmp_path / "p.nnp")
    W.write_potential(pot, path)
    strucs = W.make_structures("mixed512", seed=61, count=3, sizes=[12, 20, 16])
    orc = oracle_lib.OracleNNP(path)
    e0 = np.array([orc.compute(s.posn, s.species, s.cell, force=False)[0] for s in strucs])
    eref = e0 + np.array([0.7, -1.3, 2.1])  # the loss is away from its kinks
    L0, _, grad = orc.train_grad(strucs, eref, loss, delta)
    nA = pot.nets[0]
    rng = np.random.default_rng(3)
    h = 1e-5
    for t in (0, 1):
        off = 0 if t == 0 else sum(n * (1 + c) for n, c in zip(nA.nodes, [nA.nin] + list(nA.nodes[:-1])))
        for q in rng.choice(200, size=4, replace=False).tolist() + [5000 % 9000]:
            kind, l, n, m = _param_slot(pot, t, q)
            vals = []
            for sgn in (1, -1):
                p2 = W.make_potential("cell1728")
                if kind == "b":
                    p2.nets[t].b[l][n] += sgn * h
                else:
                    p2.nets[t].w[l][n, m] += sgn * h
                W.write_potential(p2, path)
                vals.append(oracle_lib.OracleNNP(path).train_grad(strucs, eref, loss, delta)[0])
            fd = (vals[0] - vals[1]) / (2 * h)
            assert abs(fd - grad[off + q]) <= 1e-6 + 1e-4 * abs(fd), (t, q, kind, fd, grad[off + q])


@pytest.mark.parametrize("loss", [0, 2])
def test_force_train_gradient_matches_finite_differences(oracle_lib, tmp_path, loss):
    """The force trainer's batch gradient (energy term plus the force term through the networks'
    mixed second derivative) equals central differences of its batch loss (nnptef.cpp:1043-1135)
    in single network parameters of every layer, on small periodic cells whose forces carry the
    minimum-image rule."""
    pot = W.make_potential("mixed512")
    path = str(tmp_path / "p.nnp")
    W.write_potential(pot, path)
    strucs = W.make_structures("mixed512", seed=63, count=3, sizes=[10, 18, 14])
    orc = oracle_lib.OracleNNP(path)
    ref = [orc.compute(s.posn, s.species, s.cell, force=True) for s in strucs]
    rng = np.random.default_rng(4)
    eref = np.array([r[0] for r in ref]) + np.array([0.4, -0.9, 1.3])
    fref = [r[1] + rng.normal(0.0, 0.3, r[1].shape) for r in ref]
    beta = 2.5
    L0, r2, f2, grad = orc.train_force_grad(strucs, eref, fref, beta, loss, 0.05)
    assert f2 > 0 and r2 > 0
    h = 1e-6
    off = 0
    for t in (0, 1):
        p0 = orc.params(t)
        net = pot.nets[t]
        nb = sum(net.nodes)
        w0 = nb                                  # first layer-0 weight
        w1 = nb + net.nin * net.nodes[0]         # first layer-1 weight
        wl = p0.size - 1                         # last output weight
        for q in [0, net.nodes[0] + 3, nb - 1, w0 + 7, w0 + 5 * net.nodes[0] + 2, w1 + 11, wl]:
            vals = []
            for sgn in (1, -1):
                p = p0.copy()
                p[q] += sgn * h
                orc.set_params(t, p)
                vals.append(orc.train_force_grad(strucs, eref, fref, beta, loss, 0.05)[0])
            orc.set_params(t, p0)
            fd = (vals[0] - vals[1]) / (2 * h)
            assert abs(fd - grad[off + q]) <= 1e-7 + 1e-5 * abs(fd), (t, q, fd, grad[off + q])
        off += p0.size


def test_compute_centres_partitions_the_energy(oracle_lib, pot_mixed):
    """oracle_compute_centres (the per-centre work used for CPU timing samples of large cells):
    disjoint centre sets add up to the full evaluation's energy."""
    orc = oracle_lib.OracleNNP(pot_mixed)
    s = W.make_structures("mixed512", seed=12, count=1, sizes=[150])[0]
    e, _, _ = orc.compute(s.posn, s.species, s.cell, force=True)
    half = np.arange(0, s.natoms, 2)
    rest = np.arange(1, s.natoms, 2)
    ea = orc.compute_centres(s.posn, s.species, s.cell, half)
    eb = orc.compute_centres(s.posn, s.species, s.cell, rest)
    assert abs(ea + eb - e) <= 1e-12 * max(1.0, abs(e))
    assert abs(orc.compute_centres(s.posn, s.species, s.cell, np.arange(s.natoms)) - e) <= 1e-12 * max(1.0, abs(e))
