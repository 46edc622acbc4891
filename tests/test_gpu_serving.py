"""Serving (continuous batching) on the GPU: a request's result is the same alone and in a mix
of concurrent requests, resident MD-style repeat steps equal a fresh evaluation, and requests
beyond the device budget are refused."""
import os
import time

import numpy as np
import pytest

from conftest import GOLDEN
from atomnn_gb300 import workloads as W

pytestmark = pytest.mark.gpu

E_TOL = 1e-5   # eV/atom
F_TOL = 1e-4   # eV/A


def _wait(eng, rid, natoms, timeout=60.0):
    t0 = time.time()
    while time.time() - t0 < timeout:
        r = eng.poll(rid, natoms)
        if r is not None:
            return r
        time.sleep(0.0005)
    raise TimeoutError("request %d not served" % rid)


@pytest.fixture
def served(native_lib):
    from atomnn_gb300 import engine
    eng = engine.Engine(os.path.join(GOLDEN, "mixed512.nnp"))
    eng.serve_start(max_inflight=3, skin=1.0, flags=engine.BF16)
    yield eng
    eng.serve_stop()
    eng.close()


def test_alone_equals_in_the_mix(served):
    target = W.make_structures("mixed512", seed=61, count=1, sizes=[333])[0]
    e_alone, F_alone, _ = _wait(served, served.submit(target), target.natoms)
    others = W.make_structures("mixed512", seed=62, count=40)
    ids = []
    for k, s in enumerate(others):
        ids.append((served.submit(s), s))
        if k == 20:
            tid = served.submit(target)
    res = [_wait(served, rid, s.natoms) for rid, s in ids]
    e_mix, F_mix, _ = _wait(served, tid, target.natoms)
    assert abs(e_mix - e_alone) / target.natoms <= E_TOL
    assert np.abs(F_mix - F_alone).max() <= F_TOL
    # and every result of the mix equals a direct evaluation of that structure
    from atomnn_gb300 import engine
    e_dir, F_dir, _ = served.compute([s for _, s in ids], engine.ENERGY | engine.FORCE | engine.BATCHED | engine.BF16)
    for k, (e, F, lat) in enumerate(res):
        assert abs(e - e_dir[k]) / ids[k][1].natoms <= E_TOL
        assert np.abs(F - F_dir[k]).max() <= F_TOL
        assert lat > 0
    # served results against the FP64 oracle: the target and every fourth structure of the mix
    # (BF16 networks: energy within 1e-3 eV/atom, force RMSE within 1e-3 eV/A)
    from oracle import pyoracle
    orc = pyoracle.OracleNNP(os.path.join(GOLDEN, "mixed512.nnp"))
    for s, (e, F) in [(target, (e_mix, F_mix))] + [(ids[k][1], res[k][:2]) for k in range(0, len(ids), 4)]:
        eo, Fo, _ = orc.compute(s.posn, s.species, s.cell, force=True)
        assert abs(e - eo) / s.natoms <= 1e-3
        assert np.sqrt(((F - Fo) ** 2).mean()) <= 1e-3


def test_unmoved_repeat_served_from_resident_results(served):
    """A keyed request whose inputs equal the key's last evaluated ones is answered from the
    resident results; a moved one is evaluated again."""
    from atomnn_gb300 import engine
    s = W.make_structures("mixed512", seed=66, count=1, sizes=[700])[0]
    e1, F1, _ = _wait(served, served.submit(s, key=11), s.natoms)
    e2, F2, _ = _wait(served, served.submit(s, key=11), s.natoms)
    assert e2 == e1 and np.array_equal(F2, F1)
    moved = W.Structure(posn=s.posn + 0.01, species=s.species, cell=s.cell)
    e3, F3, _ = _wait(served, served.submit(moved, key=11), s.natoms)
    e_ref, F_ref, _ = served.compute([moved], engine.ENERGY | engine.FORCE | engine.BATCHED | engine.BF16)
    assert abs(e3 - e_ref[0]) / s.natoms <= E_TOL and np.abs(F3 - F_ref[0]).max() <= F_TOL
    # a different key with the same inputs is not served from key 11's results, but agrees
    e4, F4, _ = _wait(served, served.submit(s, key=12), s.natoms)
    assert abs(e4 - e1) / s.natoms <= E_TOL and np.abs(F4 - F1).max() <= F_TOL


def test_resident_md_steps_match_fresh_evaluation(served):
    from atomnn_gb300 import engine
    rng = np.random.default_rng(5)
    base = W.make_structures("cell1728")[0]
    posn = base.posn.copy()
    for step in range(4):
        s = W.Structure(posn=posn.copy(), species=base.species, cell=base.cell)
        e, F, _ = _wait(served, served.submit(s, key=7), s.natoms)
        e_ref, F_ref, _ = served.compute([s], engine.ENERGY | engine.FORCE | engine.BATCHED | engine.BF16)
        assert abs(e - e_ref[0]) / s.natoms <= E_TOL
        assert np.abs(F - F_ref[0]).max() <= F_TOL
        posn += rng.uniform(-0.02, 0.02, size=posn.shape)  # MD-style step, well inside skin/2


def test_resident_md_steps_far_images(served, oracle_lib):
    """Resident MD-style steps of a structure whose atoms sit up to 400 cells from the home cell:
    the resident list's lattice translations (kept modulo 1024 in the slot codes) are recovered
    from the atoms' integer floors, so every step equals a fresh evaluation and the oracle."""
    from atomnn_gb300 import engine
    rng = np.random.default_rng(6)
    base = W.make_structures("mixed512", seed=61, count=1, sizes=[400])[0]
    posn = base.posn + rng.integers(-400, 401, size=(base.natoms, 3)) @ np.asarray(base.cell).T
    orc = oracle_lib.OracleNNP(os.path.join(GOLDEN, "mixed512.nnp"))
    for step in range(3):
        s = W.Structure(posn=posn.copy(), species=base.species, cell=base.cell)
        e, F, _ = _wait(served, served.submit(s, key=9), s.natoms)
        e_ref, F_ref, _ = served.compute([s], engine.ENERGY | engine.FORCE | engine.BATCHED | engine.BF16)
        assert abs(e - e_ref[0]) / s.natoms <= E_TOL
        assert np.abs(F - F_ref[0]).max() <= F_TOL
        posn += rng.uniform(-0.02, 0.02, size=posn.shape)
    eo, Fo, _ = orc.compute(s.posn, s.species, s.cell, force=True)
    assert abs(e - eo) / s.natoms <= 1e-3 and np.sqrt(np.mean((F - Fo) ** 2)) <= 1e-3  # BF16 gates


def test_oversized_request_refused(native_lib):
    from atomnn_gb300 import engine
    eng = engine.Engine(os.path.join(GOLDEN, "mixed512.nnp"))
    eng.serve_start(max_inflight=2, max_batch_atoms=1000, skin=0.0)
    s = W.make_structures("mixed512", seed=70, count=1, sizes=[1500])[0]
    with pytest.raises(engine.NNPGPUError) as ei:
        eng.submit(s)
    assert ei.value.code == engine.ERR_OOM
    small = W.make_structures("mixed512", seed=71, count=1, sizes=[200])[0]
    e, F, _ = _wait(eng, eng.submit(small), small.natoms)
    assert np.isfinite(e)
    eng.serve_stop()
    eng.close()
