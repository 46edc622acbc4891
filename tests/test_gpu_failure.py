"""Failure detection on the GPU without a fault: the tensor-core network kernel's bounded
mbarrier waits.  With the wait limit set to 0 every wait gives up at once; the kernel must
record the timeout, wait (bounded) for the weight copies it had already issued, free its TMEM
and return, so that the call ends with NNPGPU_ERR_TIMEOUT and the same context then gives the
same results as before.  Nothing here faults, traps or hangs the GPU: the waits that run out are
waits on copies that complete normally."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from atomnn_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def test_tensor_core_wait_timeout_leaves_context_usable(native_lib):
    from atomnn_gb300 import engine
    eng = engine.Engine(os.path.join(GOLDEN, "mixed512.nnp"))
    strucs = W.make_structures("mixed512", seed=91, count=3, sizes=[300, 40, 700])
    flags = engine.ENERGY | engine.FORCE | engine.BATCHED | engine.BF16
    e0, F0, _ = eng.compute(strucs, flags)
    e0b, F0b, _ = eng.compute(strucs, flags)  # second call of the shape: captured launch sequence
    eng.set_wait_limit(0)
    for _ in range(2):  # plain launch, then the launch sequence captured with the new limit
        with pytest.raises(engine.NNPGPUError) as ei:
            eng.compute(strucs, flags)
        assert ei.value.code == engine.ERR_TIMEOUT
        assert "destroy" not in str(ei.value)  # the kernel's own copies finished
    eng.set_wait_limit()  # default bound
    for _ in range(2):
        e1, F1, _ = eng.compute(strucs, flags)
        np.testing.assert_allclose(e1, e0, rtol=0, atol=1e-9)
        for a, b in zip(F1, F0):
            np.testing.assert_allclose(a, b, rtol=0, atol=1e-9)
    # the FP32 path has no such wait and is unaffected by the limit
    eng.set_wait_limit(0)
    e2, _, _ = eng.compute(strucs, engine.ENERGY | engine.BATCHED)
    assert np.all(np.abs(np.asarray(e2) - np.asarray(e0)) / np.array([s.natoms for s in strucs]) < 1e-3)
    with pytest.raises(engine.NNPGPUError):
        eng.set_wait_limit(-1)
    eng.close()
