"""The energy trainer's batch error and parameter gradient on the GPU (nnpgpu_train_grad) against
the FP64 oracle (NNPTE::error, src/nnp/nnpte.cpp:870-921, with Cost::grad, src/ml/nn.cpp:1554-1589;
the oracle's gradient is itself checked against finite differences in tests/test_oracle.py).
Tolerances: losses 1e-5 relative; gradient 1e-4 of its largest component (FP32 descriptors and
networks on the GPU)."""
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
