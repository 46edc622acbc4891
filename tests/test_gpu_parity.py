"""GPU parity tests: the CUDA path (through the C ABI) against the FP64 oracle and the golden
fixtures.  Tolerances: neighbour lists exact (pair sets, list order, minimum-image flags,
lattice translations); FP32 path energy <= 1e-5 eV/atom and forces <= 1e-4 eV/A (max abs);
symmetry functions <= 1e-5 relative to the largest value of the structure."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, load_golden
from atomnn_gb300 import workloads as W

pytestmark = pytest.mark.gpu

E_TOL = 1e-5   # eV/atom, FP32 path
F_TOL = 1e-4   # eV/A max abs, FP32 path
G_TOL = 1e-5   # relative to max |G|


@pytest.fixture(scope="module")
def engines(native_lib):
    from atomnn_gb300 import engine
    e1 = engine.Engine(os.path.join(GOLDEN, "small64.nnp"))
    e2 = engine.Engine(os.path.join(GOLDEN, "mixed512.nnp"))
    yield {"small64": e1, "mixed512": e2}
    e1.close()
    e2.close()


@pytest.fixture(scope="module")
def oracles(oracle_lib):
    return {k: oracle_lib.OracleNNP(os.path.join(GOLDEN, k + ".nnp")) for k in ("small64", "mixed512")}


def _flags(*names):
    from atomnn_gb300 import engine
    f = 0
    for n in names:
        f |= getattr(engine, n)
    return f


def _assert_lists_equal(g, o):
    assert len(g) == len(o)
    for i in range(len(o)):
        np.testing.assert_array_equal(g[i]["index"], o[i]["index"])
        np.testing.assert_array_equal(g[i]["shift"], o[i]["shift"])
        np.testing.assert_array_equal(g[i]["min"], o[i]["min"])
        if len(o[i]["r"]):
            np.testing.assert_allclose(g[i]["r"], o[i]["r"], rtol=0, atol=2e-5)


def _assert_ef(e, F, eo, Fo, n):
    assert abs(e - eo) / n <= E_TOL, (e, eo)
    assert np.abs(F - Fo).max() <= F_TOL


@pytest.mark.parametrize("name", ["small64", "mixed3", "cluster20"])
def test_golden_neighbors(engines, name):
    pot = str(np.load(os.path.join(GOLDEN, name + ".npz"))["potential"][0])
    for s, ref in load_golden(name):
        g = engines[pot].neighbors(s.posn, s.cell)
        np.testing.assert_array_equal([len(x["index"]) for x in g], ref["nb_count"])
        np.testing.assert_array_equal(np.concatenate([x["index"] for x in g]), ref["nb_index"])
        np.testing.assert_array_equal(np.concatenate([x["shift"] for x in g]), ref["nb_shift"])
        np.testing.assert_array_equal(np.concatenate([x["min"] for x in g]).astype(np.uint8), ref["nb_min"])


@pytest.mark.parametrize("name", ["small64", "mixed3", "cluster20"])
@pytest.mark.parametrize("batched", [False, True])
def test_golden_energy_force_symm(engines, name, batched):
    pot = str(np.load(os.path.join(GOLDEN, name + ".npz"))["potential"][0])
    cases = load_golden(name)
    strucs = [s for s, _ in cases]
    flags = _flags("ENERGY", "FORCE", "SYMM") | (_flags("BATCHED") if batched else 0)
    e, F, G = engines[pot].compute(strucs, flags)
    off = 0
    for k, (s, ref) in enumerate(cases):
        _assert_ef(e[k], F[k], ref["energy"][0], ref["force"], s.natoms)
        Gs = G[off:off + s.natoms, :ref["symm"].shape[1]]
        off += s.natoms
        assert np.abs(Gs - ref["symm"]).max() <= G_TOL * max(np.abs(ref["symm"]).max(), 1.0)


def test_compute_semantics_no_vacuum(engines):
    cases = load_golden("mixed3")
    e, _, _ = engines["mixed512"].compute([s for s, _ in cases], _flags("ENERGY", "FORCE", "NO_VACUUM", "BATCHED"))
    for k, (s, ref) in enumerate(cases):
        assert abs(e[k] - ref["energy_compute"][0]) / s.natoms <= E_TOL


def test_batched_equals_plain(engines):
    strucs = W.make_structures("mixed512", seed=21, count=12)
    a = engines["mixed512"].compute(strucs, _flags("ENERGY", "FORCE"))
    b = engines["mixed512"].compute(strucs, _flags("ENERGY", "FORCE", "BATCHED"))
    np.testing.assert_array_equal(a[0], b[0])
    for x, y in zip(a[1], b[1]):
        np.testing.assert_array_equal(x, y)


def _sheared_cell(rng):
    # strongly sheared cell: exercises the 6-shift fallback of Cell::diff and many images
    cell = W.lattice(7.0, 7.5, 8.0, 60.0, 115.0, 65.0)
    return W.Structure(posn=rng.uniform(0, 1, size=(24, 3)) @ cell.T, species=(np.arange(24) % 2).astype(np.int32), cell=cell)


def _perfect_lattice():
    # exact lattice sites: equidistant images tie, the first image in list order is the minimum
    m, a = 3, 2.8
    idx = np.array([(x, y, z) for x in range(m) for y in range(m) for z in range(m)], dtype=float)
    return W.Structure(posn=idx * a, species=(np.arange(27) % 3 == 0).astype(np.int32), cell=np.eye(3) * m * a)


@pytest.mark.parametrize("case", ["sheared", "perfect", "one_atom", "two_atoms", "isolated", "big_cell", "thin_slab", "needle",
                                  "left_handed", "one_species"])
def test_edge_cases_against_oracle(engines, oracles, case):
    rng = np.random.default_rng(4)
    if case == "sheared":
        s = _sheared_cell(rng)
    elif case == "left_handed":
        # lattice vectors in left-handed order (negative determinant), 180 atoms: cell lists
        base = W.make_structures("mixed512", seed=31, count=1, sizes=[180])[0]
        cell = np.asarray(base.cell)[:, [1, 0, 2]]
        s = W.Structure(posn=base.posn, species=base.species, cell=cell)
    elif case == "one_species":
        # only the second species present: the first one's network tiles, moment sets and
        # triplet blocks are empty
        base = W.make_structures("mixed512", seed=32, count=1, sizes=[300])[0]
        s = W.Structure(posn=base.posn, species=np.ones(base.natoms, np.int32), cell=base.cell)
    elif case in ("thin_slab", "needle"):
        # one (slab) or two (needle) short lattice vectors: 6 or 9 image shells along those axes
        cell = W.lattice(2.2, 16.0, 15.0, 88.0, 93.0, 86.0) if case == "thin_slab" else W.lattice(1.6, 1.9, 60.0, 90.0, 90.0, 75.0)
        n = 14 if case == "thin_slab" else 8
        f = rng.uniform(0, 1, size=(n, 3))
        if case == "needle":  # atoms spread along the long axis, no pair closer than the short vectors
            f[:, 2] = (np.arange(n) + 0.5) / n + rng.uniform(-0.02, 0.02, size=n)
        s = W.Structure(posn=f @ cell.T, species=(np.arange(n) % 2).astype(np.int32), cell=cell)
    elif case == "perfect":
        s = _perfect_lattice()
    elif case == "one_atom":
        s = W.Structure(posn=np.array([[0.3, 0.2, 0.1]]), species=np.array([1], np.int32), cell=np.eye(3) * 4.0)
    elif case == "two_atoms":
        s = W.Structure(posn=np.array([[0.0, 0.0, 0.0], [1.9, 0.4, 0.2]]), species=np.array([0, 1], np.int32),
                        cell=W.lattice(5.0, 5.5, 6.0, 90.0, 95.0, 85.0))
    elif case == "isolated":
        p = np.array([[0, 0, 0], [2.0, 0, 0], [0, 2.1, 0], [30.0, 30.0, 30.0]])
        s = W.Structure(posn=p, species=np.array([0, 1, 1, 0], np.int32), cell=np.zeros((3, 3)))
    else:
        s = W.make_structures("cell1728")[0]
    from oracle import pyoracle
    o_nb = pyoracle.neighbors(oracles["mixed512"].rc, s.posn, s.cell)
    _assert_lists_equal(engines["mixed512"].neighbors(s.posn, s.cell), o_nb)
    eo, Fo, _ = oracles["mixed512"].compute(s.posn, s.species, s.cell, force=True)
    e, F, _ = engines["mixed512"].compute([s], _flags("ENERGY", "FORCE", "BATCHED"))
    _assert_ef(e[0], F[0], eo, Fo, s.natoms)


def _dense_cell(n, rho, seed, angles=(84.0, 97.0, 91.0), wrap=True):
    rng = np.random.default_rng(seed)
    L = (n / rho) ** (1.0 / 3.0)
    cell = W.lattice(L, 1.05 * L, 0.95 * L, *angles)
    f = rng.uniform(0, 1, size=(n, 3))
    if not wrap:  # positions several cells away from the home cell
        f += rng.integers(-3, 4, size=(n, 3))
    return W.Structure(posn=f @ cell.T, species=(rng.uniform(size=n) < 0.33).astype(np.int32), cell=cell)


@pytest.mark.parametrize("case", ["n300", "n700", "n2048", "unwrapped", "lattice_ties", "n5000"])
def test_cell_list_neighbors(engines, case):
    """Structures large enough for the cell-list build (reach 1-3 cells, stencils that wrap,
    positions outside the home cell, atoms exactly on cell faces, more than 4096 atoms): the
    lists equal the oracle's, order and minimum-image flags included."""
    if case == "lattice_ties":
        m, a = 12, 2.2  # 12 cells per axis at reach 3: every atom sits on a cell face
        idx = np.array([(x, y, z) for x in range(m) for y in range(m) for z in range(m)], dtype=float)
        s = W.Structure(posn=idx * a, species=(np.arange(m ** 3) % 2).astype(np.int32), cell=np.eye(3) * m * a)
    elif case == "unwrapped":
        s = _dense_cell(900, 0.07, 5, wrap=False)
    else:
        n = int(case[1:])
        s = _dense_cell(n, {300: 0.09, 700: 0.05, 2048: 0.07, 5000: 0.06}[n], n)
    from oracle import pyoracle
    rc = engines["mixed512"].rc
    _assert_lists_equal(engines["mixed512"].neighbors(s.posn, s.cell), pyoracle.neighbors(rc, s.posn, s.cell))


def test_cell_list_batch_against_oracle(engines, oracles):
    """A batch mixing image-shell, brute-force and cell-list structures: energies and forces.
    (Workload structures: uniform random positions put atoms 0.3 A apart, where FP32 forces
    are not meant to hold 1e-4 eV/A.)"""
    strucs = W.make_structures("mixed512", seed=40, count=4, sizes=[40, 180, 1100, 2048])
    e, F, _ = engines["mixed512"].compute(strucs, _flags("ENERGY", "FORCE", "BATCHED"))
    for k, s in enumerate(strucs):
        eo, Fo, _ = oracles["mixed512"].compute(s.posn, s.species, s.cell, force=True)
        _assert_ef(e[k], F[k], eo, Fo, s.natoms)


def test_far_images_against_oracle(engines, oracles):
    """Atoms moved by up to 400 lattice vectors (so that their integer floors no longer fit the 9
    bits packed beside the wrapped coordinates and come from their own array instead), in
    structures of every neighbour mode (image shells, single image, cell lists) inside one batch:
    neighbour lists equal the oracle's exactly, energies and forces within the tolerances."""
    from oracle import pyoracle
    rng = np.random.default_rng(404)
    strucs = W.make_structures("mixed512", seed=405, count=6, sizes=[20, 60, 150, 400, 900, 1500])
    moved = []
    for k, s in enumerate(strucs):
        shift = rng.integers(-400, 401, size=(s.natoms, 3)) if k % 2 == 0 else np.zeros((s.natoms, 3), dtype=np.int64)
        if k == 1:
            shift[: s.natoms // 2] = 300  # half the atoms far away, half at home
        moved.append(W.Structure(posn=s.posn + shift @ np.asarray(s.cell).T, species=s.species, cell=s.cell))
    eng, orc = engines["mixed512"], oracles["mixed512"]
    e, F, _ = eng.compute(moved, _flags("ENERGY", "FORCE", "BATCHED"))
    for k, s in enumerate(moved):
        eo, Fo, _ = orc.compute(s.posn, s.species, s.cell, force=True)
        _assert_ef(e[k], F[k], eo, Fo, s.natoms)
        _assert_lists_equal(eng.neighbors(s.posn, s.cell), pyoracle.neighbors(orc.rc, s.posn, s.cell))


def test_empty_structures_in_batch(engines, oracles):
    strucs = W.make_structures("mixed512", seed=8, count=3, sizes=[20, 30, 25])
    empty = W.Structure(posn=np.zeros((0, 3)), species=np.zeros(0, np.int32), cell=np.eye(3) * 10)
    batch = [strucs[0], empty, strucs[1], strucs[2]]
    e, F, _ = engines["mixed512"].compute(batch, _flags("ENERGY", "FORCE", "BATCHED"))
    assert e[1] == 0.0 and F[1].shape == (0, 3)
    for k, s in ((0, strucs[0]), (2, strucs[1]), (3, strucs[2])):
        eo, Fo, _ = oracles["mixed512"].compute(s.posn, s.species, s.cell, force=True)
        _assert_ef(e[k], F[k], eo, Fo, s.natoms)
    e0, _, _ = engines["mixed512"].compute([], _flags("ENERGY", "BATCHED"))
    assert len(e0) == 0


def test_capacity_retry(native_lib, oracles):
    """A too-small neighbour capacity overflows on the device, is detected and retried."""
    from atomnn_gb300 import engine
    eng = engine.Engine(os.path.join(GOLDEN, "mixed512.nnp"), max_neighbors=32)
    s2 = W.make_structures("mixed512", seed=31, count=1, sizes=[300])[0]
    e, F, _ = eng.compute([s2], _flags("ENERGY", "FORCE", "BATCHED"))
    eo, Fo, _ = oracles["mixed512"].compute(s2.posn, s2.species, s2.cell, force=True)
    _assert_ef(e[0], F[0], eo, Fo, s2.natoms)
    eng.close()


def test_invalid_inputs_rejected(engines):
    from atomnn_gb300 import engine
    s = W.make_structures("mixed512", seed=8, count=1, sizes=[20])[0]
    bad = W.Structure(posn=s.posn.copy(), species=s.species, cell=s.cell)
    bad.posn[3, 1] = np.nan
    with pytest.raises(engine.NNPGPUError) as ei:
        engines["mixed512"].compute([bad], _flags("ENERGY", "FORCE", "BATCHED"))
    assert ei.value.code == engine.ERR_INVALID
    bad2 = W.Structure(posn=s.posn, species=s.species + 5, cell=s.cell)
    with pytest.raises(engine.NNPGPUError) as ei:
        engines["mixed512"].compute([bad2], _flags("ENERGY", "FORCE", "BATCHED"))
    assert ei.value.code == engine.ERR_INVALID
    bad3 = W.Structure(posn=s.posn, species=s.species, cell=np.array([[1.0, 2, 3], [2, 4, 6], [0, 0, 1]]))
    with pytest.raises(engine.NNPGPUError) as ei:
        engines["mixed512"].compute([bad3], _flags("ENERGY", "FORCE", "BATCHED"))
    assert ei.value.code == engine.ERR_INVALID
    # the context stays usable after rejected input
    e, _, _ = engines["mixed512"].compute([s], _flags("ENERGY", "BATCHED"))
    assert np.isfinite(e[0])


def test_force_range_refused(native_lib, tmp_path):
    """Forces are summed in 64-bit fixed point (2^-32 eV/A): a slot contribution that is not
    finite or not below 1e9 eV/A is refused with an error instead of wrapping the integer sums;
    the next call on the same context is unaffected."""
    from atomnn_gb300 import engine
    pot = W.make_potential("small64")
    pot.nets[0].outw = np.array([1.0e14])  # every force scaled far beyond the range
    path = str(tmp_path / "huge.nnp")
    W.write_potential(pot, path)
    eng = engine.Engine(path)
    try:
        s = W.make_structures("small64")[0]
        for fl in (_flags("ENERGY", "FORCE", "BATCHED"), _flags("ENERGY", "FORCE")):
            with pytest.raises(engine.NNPGPUError) as ei:
                eng.compute([s], fl)
            assert ei.value.code == engine.ERR_INVALID and "fixed-point" in str(ei.value)
        e, _, _ = eng.compute([s], _flags("ENERGY", "BATCHED"))  # no forces: nothing to refuse
        assert np.isfinite(e).all() and abs(e[0]) > 1e10
    finally:
        eng.close()


def test_full_size_properties(engines):
    """At full size (65536-atom cell, 13824-atom supercell) where the oracle is too slow:
    translation invariance, zero net force in wide cells, and extensivity under replication."""
    eng = engines["mixed512"]
    big = W.make_structures("cell65536")[0]
    e1, F1, _ = eng.compute([big], _flags("ENERGY", "FORCE", "BATCHED"))
    assert np.abs(F1[0].sum(axis=0)).max() < 1e-6 * big.natoms
    shifted = W.Structure(posn=big.posn + np.array([1.37, -2.11, 0.53]), species=big.species, cell=big.cell)
    e2, F2, _ = eng.compute([shifted], _flags("ENERGY", "FORCE", "BATCHED"))
    assert abs(e1[0] - e2[0]) / big.natoms < E_TOL
    assert np.abs(F1[0] - F2[0]).max() < F_TOL
    c = W.make_structures("cell1728")[0]
    reps = [(i, j, k) for i in range(2) for j in range(2) for k in range(2)]
    sup = W.Structure(posn=np.concatenate([c.posn + c.cell @ np.array(r, float) for r in reps]),
                      species=np.concatenate([c.species] * 8), cell=c.cell * 2)
    ec, Fc, _ = eng.compute([c], _flags("ENERGY", "FORCE", "BATCHED"))
    es, Fs, _ = eng.compute([sup], _flags("ENERGY", "FORCE", "BATCHED"))
    assert abs(es[0] / sup.natoms - ec[0] / c.natoms) < E_TOL
    for r in range(8):
        assert np.abs(Fs[0][r * 1728:(r + 1) * 1728] - Fc[0]).max() < F_TOL


# ---- BF16 tensor-core networks: the accuracy gate is force RMSE <= 1e-3 eV/A against the
# FP64 oracle; the energy per atom is held to 1e-3 eV/atom.
BF16_F_RMSE = 1e-3
BF16_E_TOL = 1e-3


@pytest.mark.parametrize("name", ["small64", "mixed3"])
def test_bf16_networks_against_golden(engines, name):
    pot = str(np.load(os.path.join(GOLDEN, name + ".npz"))["potential"][0])
    cases = load_golden(name)
    e, F, _ = engines[pot].compute([s for s, _ in cases], _flags("ENERGY", "FORCE", "BATCHED", "BF16"))
    for k, (s, ref) in enumerate(cases):
        assert abs(e[k] - ref["energy"][0]) / s.natoms <= BF16_E_TOL
        assert np.sqrt(((F[k] - ref["force"]) ** 2).mean()) <= BF16_F_RMSE


def test_bf16_networks_mixed_batch(engines, oracles):
    strucs = W.make_structures("mixed512", seed=12, count=6, sizes=[16, 50, 130, 400, 900, 1500])
    e, F, _ = engines["mixed512"].compute(strucs, _flags("ENERGY", "FORCE", "BATCHED", "BF16"))
    e32, F32, _ = engines["mixed512"].compute(strucs, _flags("ENERGY", "FORCE", "BATCHED"))
    for k, s in enumerate(strucs):
        eo, Fo, _ = oracles["mixed512"].compute(s.posn, s.species, s.cell, force=True)
        assert abs(e[k] - eo) / s.natoms <= BF16_E_TOL
        assert np.sqrt(((F[k] - Fo) ** 2).mean()) <= BF16_F_RMSE
        # and the BF16 path really differs from the FP32 one (the tensor-core kernel ran)
        assert not np.array_equal(F[k], F32[k])


def test_autotune_keeps_results(native_lib):
    """The autotuner times every candidate launch shape on a batch and keeps the fastest; launch
    shapes do not change any atom's arithmetic, so results are bit-identical before and after."""
    from atomnn_gb300 import engine
    eng = engine.Engine(os.path.join(GOLDEN, "mixed512.nnp"))
    try:
        strucs = W.make_structures("mixed512", seed=55, count=16)
        flags = _flags("ENERGY", "FORCE", "BATCHED")
        e0, F0, _ = eng.compute(strucs, flags)
        natoms = np.array([s.natoms for s in strucs], np.int32)
        posn = np.concatenate([s.posn for s in strucs])
        spec = np.concatenate([s.species for s in strucs]).astype(np.int32)
        cells = np.concatenate([s.cell_colmajor() for s in strucs])
        shapes, report = eng.autotune(natoms, posn, spec, cells, engine.FORCE)
        for knob in ("warps_nbr", "warps_symm", "nn_tile", "warps_force"):
            assert knob in report
        assert shapes["warps_nbr"] in (1, 2, 4) and shapes["warps_force"] in (1, 2, 4) and shapes["nn_tile"] in (16, 32, 64)
        for tune in (shapes, dict(warps_nbr=1, warps_symm=2, warps_force=1, nn_tile=64)):
            eng.set_tune(**tune)
            e1, F1, _ = eng.compute(strucs, flags)
            np.testing.assert_array_equal(e0, e1)
            for a, b in zip(F0, F1):
                np.testing.assert_array_equal(a, b)
    finally:
        eng.close()


@pytest.mark.parametrize("variant", ["all_moment_blocks", "lambda_above_one", "split_unshared", "split_top8", "split_top32",
                                     "two_high_levels", "mixed_cutoffs"])
def test_angular_paths_against_oracle(native_lib, oracle_lib, tmp_path, variant):
    """Blocks with zeta <= 4 and |lambda| <= 1 run through the moment tensors, the others
    through the triplet loop.  all_moment_blocks: every block (the same-species A-A block
    included) on the moment path; lambda_above_one: lambda = 2 forces the triplet loop on
    low-zeta blocks.  GAUSS blocks whose other functions share the block's largest zeta split (low zeta on the moment path, the top level on the triplet loop):
    split_unshared: two-width A-A blocks with zeta 1, 2, 4, 16 beside blocks of another width,
    so that no moments are shared; split_top8 and split_top32: top levels zeta 8 and 32 (the
    mixed512 potential itself splits its zeta-16 A-A blocks with shared moments);
    two_high_levels: zeta 8 and 16 in one block, which keeps the whole block on the triplet loop;
    mixed_cutoffs: angular blocks with a TANH cutoff at 5.0 A beside COS radial bases at 6.5 A (no
    cutoff shared by the centre's bases; neighbours beyond a block's radius add nothing to it).
    All against the oracle on structures with one, few and many neighbours."""
    from atomnn_gb300 import engine
    pot = W.make_potential("mixed512")
    for (i, j, k), b in list(pot.angular.items()):
        if variant == "all_moment_blocks":
            pot.angular[(i, j, k)] = W._angular(6.5, [0.005, 0.05], [1, 2, 4], [1, -1])
        elif variant == "lambda_above_one":
            if j != k:
                pot.angular[(i, j, k)] = W._angular(6.5, [0.005, 0.05], [1, 2, 4], [2, -1])
        elif variant == "mixed_cutoffs":
            b = pot.angular[(i, j, k)]
            b.rc, b.cutname = W._f6(5.0), "TANH"
        elif variant == "split_unshared":
            pot.angular[(i, j, k)] = (W._angular(6.5, [0.005, 0.05], [1, 2, 4, 16], [1, -1]) if j == k == 0 else
                                      W._angular(6.5, [0.02], [1, 2, 4], [1, -1]))
        elif j == k == 0:
            zetas = {"split_top8": [1, 2, 8], "split_top32": [1, 4, 32], "two_high_levels": [1, 8, 16]}[variant]
            pot.angular[(i, j, k)] = W._angular(6.5, [0.005], zetas, [1, -1])
    for t in range(2):  # input sizes changed: new networks
        means = W._estimate_means(pot, t, 0.07, [1.0 / 3.0, 2.0 / 3.0])
        pot.nets[t] = W._make_network(np.random.default_rng(t), pot.ninput(t), [64, 64], means)
    path = str(tmp_path / "variant.nnp")
    W.write_potential(pot, path)
    eng = engine.Engine(path)
    orc = oracle_lib.OracleNNP(path)
    try:
        strucs = W.make_structures("mixed512", seed=17, count=4, sizes=[20, 90, 400, 1200])
        strucs.append(W.Structure(posn=np.array([[0.0, 0.0, 0.0], [1.9, 0.4, 0.2], [0.3, 2.1, 0.1]]),
                                  species=np.array([0, 1, 0], np.int32), cell=np.zeros((3, 3))))
        e, F, G = eng.compute(strucs, _flags("ENERGY", "FORCE", "SYMM", "BATCHED"))
        off = 0
        for k, s in enumerate(strucs):
            eo, Fo, Go = orc.compute(s.posn, s.species, s.cell, force=True, symm=True)
            _assert_ef(e[k], F[k], eo, Fo, s.natoms)
            Gs = G[off:off + s.natoms, :Go.shape[1]]
            off += s.natoms
            np.testing.assert_allclose(Gs, Go, rtol=0, atol=G_TOL * max(np.abs(Go).max(), 1e-30))
    finally:
        eng.close()


@pytest.mark.parametrize("nsp", [3, 4])
def test_many_species_against_oracle(native_lib, oracle_lib, tmp_path, nsp):
    """Potentials with three and four species: every radial pair and angular block (moment blocks
    over more than two neighbour species, which do not share their moments; the first species'
    own block split at zeta 16), the species carried by the neighbour lists and the species sort
    of the networks, against the oracle: energies and forces on the FP32 path (batched and one
    structure at a time), descriptors, and the BF16 path's force RMSE."""
    from atomnn_gb300 import engine
    rc = 6.0
    names = [("A", 24.305, -0.5), ("B", 15.999, -0.25), ("C", 12.011, -0.1), ("D", 1.008, -0.05)][:nsp]
    pot = W.Potential(rc=W._f6(rc), species=[W.Species(n, m, e) for n, m, e in names])
    for i in range(nsp):
        for j in range(nsp):
            pot.radial[(i, j)] = W.RadialBasis(rc=W._f6(rc), rs=[W._f6(0.0), W._f6(3.0)], eta=[W._f6(0.5), W._f6(0.05)])
        for j in range(nsp):
            for k in range(j, nsp):
                pot.angular[(i, j, k)] = W._angular(rc, [0.005], [1, 2, 4, 16] if j == k == 0 else [1, 2, 4], [1, -1])
    for i in range(nsp):
        means = W._estimate_means(pot, i, 0.07, [1.0 / nsp] * nsp)
        pot.nets[i] = W._make_network(np.random.default_rng(10 + i), pot.ninput(i), [32, 32], means)
    path = str(tmp_path / ("species%d.nnp" % nsp))
    W.write_potential(pot, path)
    eng = engine.Engine(path)
    orc = oracle_lib.OracleNNP(path)
    try:
        rng = np.random.default_rng(100 + nsp)
        strucs = W.make_structures("mixed512", seed=200 + nsp, count=4, sizes=[30, 150, 700, 1300])
        strucs = [W.Structure(posn=s.posn, species=rng.integers(0, nsp, size=s.natoms).astype(np.int32), cell=s.cell) for s in strucs]
        e, F, G = eng.compute(strucs, _flags("ENERGY", "FORCE", "SYMM", "BATCHED"))
        ep, Fp, _ = eng.compute(strucs, _flags("ENERGY", "FORCE"))
        eb, Fb, _ = eng.compute(strucs, _flags("ENERGY", "FORCE", "BATCHED", "BF16"))
        off = 0
        for k, s in enumerate(strucs):
            eo, Fo, Go = orc.compute(s.posn, s.species, s.cell, force=True, symm=True)
            _assert_ef(e[k], F[k], eo, Fo, s.natoms)
            np.testing.assert_array_equal(F[k], Fp[k])
            Gs = G[off:off + s.natoms, :Go.shape[1]]
            off += s.natoms
            np.testing.assert_allclose(Gs, Go, rtol=0, atol=G_TOL * max(np.abs(Go).max(), 1e-30))
            assert np.sqrt(np.mean((Fb[k] - Fo) ** 2)) <= 1e-3
    finally:
        eng.close()


def test_energy_from_stored_descriptors(engines, oracles):
    """nnpgpu_energy_symm: NNP::energy on stored descriptors (nnp.cpp:390-402), as the trainers
    evaluate structures read back from binary files, on the oracle's FP64 descriptors.  With and
    without the vacuum energies, FP32 and BF16 networks, one-atom and empty structures included."""
    from atomnn_gb300 import engine
    eng, orc = engines["mixed512"], oracles["mixed512"]
    strucs = W.make_structures("mixed512", seed=41, count=4, sizes=[30, 300, 1500, 2])
    strucs.insert(1, W.Structure(posn=np.zeros((1, 3)), species=np.array([1], np.int32), cell=np.zeros((3, 3))))
    eo, rows = [], []
    for s in strucs:
        e, _, G = orc.compute(s.posn, s.species, s.cell, force=False, symm=True)
        eo.append(e)
        rows.append(G)
    width = max(eng.ninput)
    symm = np.zeros((sum(s.natoms for s in strucs), width + 3))  # wider rows than needed are fine
    off = 0
    for s, G in zip(strucs, rows):
        symm[off:off + s.natoms, :G.shape[1]] = G
        off += s.natoms
    natoms = [s.natoms for s in strucs] + [0]
    species = np.concatenate([s.species for s in strucs])
    e = eng.energy_symm(natoms, species, symm)
    e_nv = eng.energy_symm(natoms, species, symm, flags=engine.NO_VACUUM)
    e_bf = eng.energy_symm(natoms, species, symm, flags=engine.BF16)
    pot = W.make_potential("mixed512")
    for k, s in enumerate(strucs):
        assert abs(e[k] - eo[k]) / s.natoms <= E_TOL, (k, e[k], eo[k])
        assert abs(e_bf[k] - eo[k]) / s.natoms <= BF16_E_TOL
        evac = sum(pot.species[t].energy for t in s.species)
        assert abs((e[k] - e_nv[k]) - evac) <= 1e-9 * max(1.0, abs(evac))
    assert e[-1] == 0.0 and e_nv[-1] == 0.0
    # the same structures through the positions give the same energies
    ec, _, _ = eng.compute(strucs, _flags("ENERGY", "BATCHED"))
    for k, s in enumerate(strucs):
        assert abs(e[k] - ec[k]) / s.natoms <= E_TOL
    with pytest.raises(engine.NNPGPUError):
        eng.energy_symm(natoms, species, symm[:, :width - 1])
    bad = species.copy()
    bad[3] = 5
    with pytest.raises(engine.NNPGPUError):
        eng.energy_symm(natoms, bad, symm)


@pytest.mark.parametrize("kind,family", [("radial", f) for f in ("TANH", "SOFTPLUS", "LOGCOSH", "SWISH", "MISH")] +
                         [("angular", f) for f in ("IPOWP", "IPOWS", "SECHP", "SECHS")])
def test_basis_families_against_oracle(native_lib, oracle_lib, tmp_path, kind, family):
    """Every radial family of BasisR (basis_radial.cpp:302-444) and angular family of BasisA
    (basis_angular.cpp:406-640) on the GPU against the oracle: descriptors, energies and forces
    (the force terms follow the reference's expressions).  In the angular case the A-A blocks
    (zeta up to 16) take the triplet path and the others, for the product families IPOWP and
    SECHP, the moment path; the sum families IPOWS and SECHS take the triplet path throughout."""
    from atomnn_gb300 import engine
    pot = W.make_potential("mixed512")
    for b in (pot.radial if kind == "radial" else pot.angular).values():
        b.phi = family
    path = str(tmp_path / "family.nnp")
    W.write_potential(pot, path)
    # networks scaled by the inputs' actual means for this family (taken from the oracle)
    orc = oracle_lib.OracleNNP(path)
    sample = W.make_structures("mixed512", seed=23, count=1, sizes=[600])[0]
    _, _, Gs = orc.compute(sample.posn, sample.species, sample.cell, force=False, symm=True)
    for t in range(2):
        means = np.abs(Gs[sample.species == t, :pot.ninput(t)]).mean(axis=0) + 1e-3
        pot.nets[t] = W._make_network(np.random.default_rng(t + 7), pot.ninput(t), [64, 64], means)
    W.write_potential(pot, path)
    orc = oracle_lib.OracleNNP(path)
    eng = engine.Engine(path)
    try:
        strucs = W.make_structures("mixed512", seed=29, count=3, sizes=[30, 250, 900])
        e, F, G = eng.compute(strucs, _flags("ENERGY", "FORCE", "SYMM", "BATCHED"))
        off = 0
        for k, s in enumerate(strucs):
            eo, Fo, Go = orc.compute(s.posn, s.species, s.cell, force=True, symm=True)
            # these untrained potentials give forces up to ~10 eV/A: the FP32 force bound scales
            # with the largest force (F_TOL per 2 eV/A of it)
            assert abs(e[k] - eo) / s.natoms <= E_TOL
            assert np.abs(F[k] - Fo).max() <= F_TOL * max(1.0, np.abs(Fo).max() / 2.0)
            np.testing.assert_allclose(G[off:off + s.natoms, :Go.shape[1]], Go, rtol=0, atol=G_TOL * np.abs(Go).max())
            off += s.natoms
    finally:
        eng.close()


# ---------------------------------------------------------------- against the reference's own outputs
_REF = np.load(os.path.join(GOLDEN, "reference.npz"))
_REF_CASES = [str(c) for c in _REF["cases"]]


@pytest.mark.parametrize("case", _REF_CASES)
def test_against_reference_fixture(native_lib, tmp_path, case):
    """The GPU path against outputs of the reference's own code (tests/golden/reference.npz, from
    tests/golden/make_ref_golden.py): neighbour lists in the reference's order with its minimum
    images (vectors to 2e-5 A), FP32 energies within 1e-5 eV/atom, symmetry functions within 1e-5
    of the largest, forces within 1e-4 eV/A (scaled by the largest force over 2 eV/A for the
    untrained option variants), and the BF16 path's force RMSE within 1e-3 eV/A."""
    import sys
    sys.path.insert(0, GOLDEN)
    import variants as V
    from atomnn_gb300 import engine
    eng = engine.Engine(V.write(str(_REF[case + "/variant"][0]), str(tmp_path)))
    try:
        strucs, prefixes = [], []
        for k in range(int(_REF[case + "/nstruc"][0])):
            p = "%s/%d/" % (case, k)
            strucs.append(W.Structure(posn=_REF[p + "posn"], species=_REF[p + "species"], cell=_REF[p + "cell"]))
            prefixes.append(p)
        e, F, G = eng.compute(strucs, _flags("ENERGY", "FORCE", "SYMM", "BATCHED"))
        ec, _, _ = eng.compute(strucs, _flags("ENERGY", "FORCE", "NO_VACUUM", "BATCHED"))
        eb, Fb, _ = eng.compute(strucs, _flags("ENERGY", "FORCE", "BATCHED", "BF16"))
        off = 0
        for k, (s, p) in enumerate(zip(strucs, prefixes)):
            Fr = _REF[p + "force"]
            fscale = 1.0 if case in ("small64", "mixed3", "cluster20", "edge") else max(1.0, float(np.abs(Fr).max()) / 2.0)
            n = max(s.natoms, 1)
            assert abs(e[k] - _REF[p + "energy"][0]) / n <= E_TOL
            assert abs(ec[k] - _REF[p + "energy_compute"][0]) / n <= E_TOL
            if s.natoms:
                assert np.abs(F[k] - Fr).max() <= F_TOL * fscale
                assert np.sqrt(((Fb[k] - Fr) ** 2).mean()) <= 1e-3 * fscale
            rows, Gr = _REF[p + "symm_atoms"], _REF[p + "symm"]
            if len(rows):
                Gs = G[off + rows, :Gr.shape[1]]
                assert np.abs(Gs - Gr).max() <= G_TOL * max(np.abs(Gr).max(), 1.0)
            off += s.natoms
            if (p + "nb_count") in _REF.files and s.natoms:
                g = eng.neighbors(s.posn, s.cell)
                np.testing.assert_array_equal([len(x["index"]) for x in g], _REF[p + "nb_count"])
                if len(_REF[p + "nb_index"]):
                    np.testing.assert_array_equal(np.concatenate([x["index"] for x in g]), _REF[p + "nb_index"])
                    np.testing.assert_array_equal(np.concatenate([x["min"] for x in g]).astype(np.uint8), _REF[p + "nb_min"])
                    np.testing.assert_allclose(np.concatenate([x["r"] for x in g]), _REF[p + "nb_r"], rtol=0, atol=2e-5)
    finally:
        eng.close()


def test_page_locked_host_buffers(engines):
    """nnpgpu_compute reads and writes page-locked caller buffers by DMA (no staging): the results
    equal those of ordinary (pageable) buffers bit for bit."""
    import torch
    from atomnn_gb300 import engine
    eng = engines["mixed512"]
    strucs = W.make_structures("mixed512", seed=52, count=5, sizes=[30, 400, 90, 1200, 16])
    natoms = np.array([s.natoms for s in strucs], dtype=np.int32)
    posn = np.concatenate([s.posn for s in strucs])
    species = np.concatenate([s.species for s in strucs]).astype(np.int32)
    cells = np.concatenate([s.cell_colmajor() for s in strucs])
    flags = engine.ENERGY | engine.FORCE | engine.BATCHED | engine.BF16
    e0, F0 = np.zeros(len(strucs)), np.zeros((len(posn), 3))
    eng.compute_flat(natoms, posn, species, cells, flags, e0, F0)
    keep = []

    def pinned(a):
        t = torch.empty(a.shape, dtype=torch.from_numpy(np.ascontiguousarray(a)).dtype, pin_memory=True)
        keep.append(t)
        v = t.numpy()
        v[...] = a
        return v

    e1, F1 = pinned(np.zeros(len(strucs))), pinned(np.zeros((len(posn), 3)))
    for _ in range(2):
        eng.compute_flat(natoms, pinned(posn), pinned(species), cells, flags, e1, F1)
        np.testing.assert_array_equal(e1, e0)
        np.testing.assert_array_equal(F1, F0)
