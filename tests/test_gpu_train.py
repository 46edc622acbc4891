"""The trainers' batch error and parameter gradient on the GPU against the FP64 oracle: the energy
trainer (nnpgpu_train_grad; NNPTE::error, src/nnp/nnpte.cpp:870-921, with Cost::grad,
src/ml/nn.cpp:1554-1589) and the force trainer's loss (nnpgpu_train_force_grad; NNPTEF::error,
src/nnp/nnptef.cpp:1043-1135).  The oracle's gradients are themselves checked against finite
differences in tests/test_oracle.py.  Tolerances: losses 1e-5 relative; gradient 1e-4 (energy) and
2e-4 (with forces: FP32 second derivatives) of its largest component."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from atomnn_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pair(native_lib, oracle_lib):
    from atomnn_gb300 import engine
    path = os.path.join(GOLDEN, "mixed512.nnp")
    eng = engine.Engine(path)
    yield eng, oracle_lib.OracleNNP(path)
    eng.close()


@pytest.mark.parametrize("loss,delta", [("MSE", 1.0), ("MAE", 1.0), ("HUBER", 0.05), ("ASINH", 0.05)])
def test_train_grad_matches_oracle(pair, loss, delta):
    eng, orc = pair
    strucs = W.make_structures("mixed512", seed=71, count=6, sizes=[16, 40, 120, 300, 700, 1100])
    e0 = np.array([orc.compute(s.posn, s.species, s.cell, force=False)[0] for s in strucs])
    rng = np.random.default_rng(5)
    eref = e0 + rng.normal(0.0, 0.3, size=len(strucs)) * np.array([s.natoms for s in strucs]) ** 0.5
    codes = {"MSE": 0, "MAE": 1, "HUBER": 2, "ASINH": 3}
    L, r2, g = eng.train_grad(strucs, eref, loss, delta)
    Lo, r2o, go = orc.train_grad(strucs, eref, codes[loss], delta)
    assert g.shape == go.shape and g.size == eng.nparams(0) + eng.nparams(1)
    assert abs(L - Lo) <= 1e-5 * abs(Lo) + 1e-9
    assert abs(r2 - r2o) <= 1e-5 * abs(r2o) + 1e-9
    assert np.abs(g - go).max() <= 1e-4 * np.abs(go).max() + 1e-9


def test_train_grad_two_calls_identical(pair):
    """No atomics in the gradient: repeated calls give bit-identical results."""
    eng, _ = pair
    strucs = W.make_structures("mixed512", seed=72, count=4, sizes=[50, 200, 600, 1500])
    eref = np.zeros(len(strucs))
    a = eng.train_grad(strucs, eref, "MSE")
    b = eng.train_grad(strucs, eref, "MSE")
    assert a[0] == b[0] and a[1] == b[1]
    np.testing.assert_array_equal(a[2], b[2])


def test_train_grad_rejects_bad_loss(pair):
    from atomnn_gb300 import engine
    eng, _ = pair
    s = W.make_structures("mixed512", seed=73, count=1, sizes=[30])
    with pytest.raises(engine.NNPGPUError):
        eng.train_grad(s, np.zeros(1), "HUBER", delta=0.0)


# ---- the force trainer (nnpgpu_train_force_grad): loss of NNPTEF::error (nnptef.cpp:1043-1135),
# exact gradient (the oracle's is checked against finite differences in tests/test_oracle.py)
def _force_batch(orc, seed, sizes):
    strucs = W.make_structures("mixed512", seed=seed, count=len(sizes), sizes=sizes)
    ref = [orc.compute(s.posn, s.species, s.cell, force=True) for s in strucs]
    rng = np.random.default_rng(seed)
    eref = np.array([r[0] for r in ref]) + rng.normal(0.0, 0.3, size=len(strucs)) * np.array([s.natoms for s in strucs]) ** 0.5
    fref = [r[1] + rng.normal(0.0, 0.2, r[1].shape) for r in ref]
    return strucs, eref, fref


@pytest.mark.parametrize("loss,delta", [("MSE", 1.0), ("HUBER", 0.05)])
def test_train_force_grad_matches_oracle(pair, loss, delta):
    eng, orc = pair
    strucs, eref, fref = _force_batch(orc, 81, [16, 40, 120, 300, 600])
    codes = {"MSE": 0, "MAE": 1, "HUBER": 2, "ASINH": 3}
    beta = 2.0
    L, r2, f2, g = eng.train_force_grad(strucs, eref, fref, beta, loss, delta)
    Lo, r2o, f2o, go = orc.train_force_grad(strucs, eref, fref, beta, codes[loss], delta)
    assert abs(L - Lo) <= 1e-5 * abs(Lo) + 1e-9
    assert abs(r2 - r2o) <= 1e-5 * abs(r2o) + 1e-9
    assert abs(f2 - f2o) <= 1e-5 * abs(f2o) + 1e-9
    assert np.abs(g - go).max() <= 2e-4 * np.abs(go).max(), np.abs(g - go).max() / np.abs(go).max()


def test_train_force_grad_reduces_to_energy_gradient(pair):
    """beta = 0 leaves the energy trainer's gradient; repeated calls are bit-identical."""
    eng, orc = pair
    strucs, eref, fref = _force_batch(orc, 82, [30, 200, 900])
    L, r2, f2, g = eng.train_force_grad(strucs, eref, fref, 0.0, "MSE")
    Le, r2e, ge = eng.train_grad(strucs, eref, "MSE")
    assert L == Le and r2 == r2e and f2 > 0
    np.testing.assert_array_equal(g, ge)
    a = eng.train_force_grad(strucs, eref, fref, 1.5, "MSE")
    b = eng.train_force_grad(strucs, eref, fref, 1.5, "MSE")
    assert a[:3] == b[:3]
    np.testing.assert_array_equal(a[3], b[3])


def test_train_force_grad_rejects_bad_input(pair):
    from atomnn_gb300 import engine
    eng, orc = pair
    strucs, eref, fref = _force_batch(orc, 83, [20])
    with pytest.raises(engine.NNPGPUError):
        eng.train_force_grad(strucs, eref, fref, -1.0, "MSE")
    with pytest.raises(engine.NNPGPUError):
        eng.train_force_grad(strucs, eref, fref, 1.0, "ASINH", delta=0.0)


def _three_species_potential(path):
    rc = 6.0
    names = [("A", 24.305, -0.5), ("B", 15.999, -0.25), ("C", 12.011, -0.1)]
    pot = W.Potential(rc=W._f6(rc), species=[W.Species(n, m, e) for n, m, e in names])
    for i in range(3):
        for j in range(3):
            pot.radial[(i, j)] = W.RadialBasis(rc=W._f6(rc), rs=[W._f6(0.0), W._f6(3.0)], eta=[W._f6(0.5), W._f6(0.05)])
        for j in range(3):
            for k in range(j, 3):
                pot.angular[(i, j, k)] = W._angular(rc, [0.005], [1, 2, 4, 16] if j == k == 0 else [1, 2, 4], [1, -1])
    for i in range(3):
        means = W._estimate_means(pot, i, 0.07, [1.0 / 3.0] * 3)
        pot.nets[i] = W._make_network(np.random.default_rng(20 + i), pot.ninput(i), [16, 16], means)
    W.write_potential(pot, path)
    return path


def test_three_species_trainers_match_oracle(native_lib, oracle_lib, tmp_path):
    """Both trainers with a three-species potential (every species' networks and parameter block,
    moment blocks over three neighbour species): loss and gradient against the oracle."""
    from atomnn_gb300 import engine
    path = _three_species_potential(str(tmp_path / "three.nnp"))
    eng = engine.Engine(path)
    orc = oracle_lib.OracleNNP(path)
    try:
        rng = np.random.default_rng(91)
        strucs = W.make_structures("mixed512", seed=92, count=4, sizes=[20, 90, 300, 700])
        strucs = [W.Structure(posn=s.posn, species=rng.integers(0, 3, size=s.natoms).astype(np.int32), cell=s.cell) for s in strucs]
        ref = [orc.compute(s.posn, s.species, s.cell, force=True) for s in strucs]
        eref = np.array([r[0] for r in ref]) + rng.normal(0.0, 0.3, size=len(strucs)) * np.array([s.natoms for s in strucs]) ** 0.5
        fref = [r[1] + rng.normal(0.0, 0.2, r[1].shape) for r in ref]
        L, r2, g = eng.train_grad(strucs, eref, "MSE")
        Lo, r2o, go = orc.train_grad(strucs, eref, 0, 1.0)
        assert g.size == sum(eng.nparams(t) for t in range(3))
        assert abs(L - Lo) <= 1e-5 * abs(Lo) + 1e-9
        assert np.abs(g - go).max() <= 1e-4 * np.abs(go).max() + 1e-9
        L, r2, f2, g = eng.train_force_grad(strucs, eref, fref, 2.0, "MSE")
        Lo, r2o, f2o, go = orc.train_force_grad(strucs, eref, fref, 2.0, 0, 1.0)
        assert abs(L - Lo) <= 1e-5 * abs(Lo) + 1e-9 and abs(f2 - f2o) <= 1e-5 * abs(f2o) + 1e-9
        assert np.abs(g - go).max() <= 2e-4 * np.abs(go).max(), np.abs(g - go).max() / np.abs(go).max()
    finally:
        eng.close()


def test_set_params_updates_the_device_networks(native_lib, oracle_lib, tmp_path):
    """A trainer's update through nnpgpu_set_params reaches the FP32 and tensor-core networks
    (including launch sequences captured before it): energies and forces equal the oracle's on
    the potential that nnpgpu_write_potential writes afterwards."""
    from atomnn_gb300 import engine
    eng = engine.Engine(os.path.join(GOLDEN, "mixed512.nnp"))
    try:
        strucs = W.make_structures("mixed512", seed=91, count=3, sizes=[40, 300, 900])
        for flags in (engine.BF16, 0):
            for _ in range(3):  # the batch shape's launch sequence is captured
                eng.compute(strucs, engine.ENERGY | engine.FORCE | engine.BATCHED | flags)
        rng = np.random.default_rng(7)
        for t in range(eng.ntypes):
            eng.set_params(t, eng.params(t) * (1.0 + 0.05 * rng.normal(size=eng.nparams(t))))
        path = str(tmp_path / "updated.nnp")
        eng.write_potential(path)
        orc = oracle_lib.OracleNNP(path)
        e, F, _ = eng.compute(strucs, engine.ENERGY | engine.FORCE | engine.BATCHED)
        eb, Fb, _ = eng.compute(strucs, engine.ENERGY | engine.FORCE | engine.BATCHED | engine.BF16)
        for k, s in enumerate(strucs):
            eo, Fo, _ = orc.compute(s.posn, s.species, s.cell, force=True)
            assert abs(e[k] - eo) / s.natoms <= 1e-5
            assert np.abs(F[k] - Fo).max() <= 1e-4 * max(1.0, np.abs(Fo).max() / 2.0)
            assert abs(eb[k] - eo) / s.natoms <= 1e-3
            assert np.sqrt(((Fb[k] - Fo) ** 2).mean()) <= 1e-3
    finally:
        eng.close()
