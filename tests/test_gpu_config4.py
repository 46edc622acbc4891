"""Precision at scale: the 65,536-atom two-species cell at 0.07 atoms/A^3 with its own potential
(32 G2 + 64 G4 per species, networks 96-128-128-1 tanh, rc 6.5 A), on the GPU against the FP64
oracle fixture tests/golden/cell65536.npz (tests/golden/make_cell65536.py; every 8th atom's
force, 64 atoms' descriptors, every atom's neighbour count).

Gates: the plain and batched FP32 paths within 1e-5 eV/atom of the FP64 energy with forces
within 1e-4 eV/A (max abs over the sampled atoms), descriptors within 1e-5 of the largest; the
BF16 tensor-core path within 1e-3 eV/atom with force RMSE within 1e-3 eV/A.  The inputs are
regenerated from the seeded generator and must match the digests stored with the fixture."""
import hashlib
import os
import sys

import numpy as np
import pytest

from conftest import GOLDEN, REPO
from atomnn_gb300 import workloads as W

pytestmark = pytest.mark.gpu

sys.path.insert(0, GOLDEN)
import make_cell65536 as M  # noqa: E402


@pytest.fixture(scope="module")
def case(native_lib):
    fx = np.load(os.path.join(GOLDEN, "cell65536.npz"))
    potfile, s, pot_sha, struc_sha = M.inputs(os.path.join(REPO, "atomnn_gb300", "_build", "workloads"))
    assert pot_sha == str(fx["potential_sha256"][0]), "the seeded generator wrote a different potential on this machine"
    assert struc_sha == str(fx["structure_sha256"][0]), "the seeded generator made a different structure on this machine"
    from atomnn_gb300 import engine
    eng = engine.Engine(potfile)
    yield eng, s, fx
    eng.close()


@pytest.mark.parametrize("path", ["plain_fp32", "batched_fp32", "batched_bf16"])
def test_cell65536_against_fp64(case, path):
    from atomnn_gb300 import engine
    eng, s, fx = case
    flags = engine.ENERGY | engine.FORCE | {"plain_fp32": 0, "batched_fp32": engine.BATCHED,
                                            "batched_bf16": engine.BATCHED | engine.BF16}[path]
    e, F, _ = eng.compute([s], flags)
    de = abs(e[0] - float(fx["energy"][0])) / s.natoms
    dF = F[0][fx["force_atoms"]] - fx["force"]
    if path == "batched_bf16":
        assert de <= 1e-3
        assert np.sqrt((dF ** 2).mean()) <= 1e-3
    else:
        assert de <= 1e-5
        assert np.abs(dF).max() <= 1e-4


def test_cell65536_descriptors_and_lists(case):
    from atomnn_gb300 import engine
    eng, s, fx = case
    e, _, G = eng.compute([s], engine.ENERGY | engine.SYMM | engine.BATCHED | engine.NO_VACUUM)
    assert abs(e[0] - float(fx["energy_compute"][0])) / s.natoms <= 1e-5
    rows = fx["symm_atoms"]
    Gr = fx["symm"]
    assert np.abs(G[rows, :Gr.shape[1]] - Gr).max() <= 1e-5 * np.abs(Gr).max()
    nb = eng.neighbors(s.posn, s.cell, cap=256)
    np.testing.assert_array_equal([len(x["index"]) for x in nb], fx["nb_count"])
