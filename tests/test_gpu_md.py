"""MD on resident device state (nnpgpu_md_*) against velocity-Verlet steps driven by the FP64
oracle: Verlet::compute (src/torch/integrator.cpp:170-193) with the forces and energy of
PotNNPE::compute (src/torch/pot_nnpe.cpp:175-295), i.e. NNP::force and NNP::energy with the
species vacuum energies.  Tolerances: positions 1e-6 A, velocities 1e-5 A/t, potential energy
1e-5 eV/atom after the run (FP32 descriptors on the GPU, FP64 in the oracle)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from atomnn_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _oracle_md(orc, s, mass, vel, dt, nsteps, start_forces=False):
    """The reference's integrator on the oracle's forces; returns per-step pe, ke and the state."""
    x = s.posn.copy()
    v = vel.copy()
    F = np.zeros_like(x)
    if start_forces:
        _, F, _ = orc.compute(x, s.species, s.cell, force=True)
    m = mass[:, None]
    pe, ke = [], []
    for _ in range(nsteps):
        v = v + (0.5 * dt * F) / m
        x = x + v * dt
        e, F, _ = orc.compute(x, s.species, s.cell, force=True)
        v = v + (0.5 * dt * F) / m
        pe.append(e)
        ke.append(0.5 * float(np.sum(mass * np.sum(v * v, axis=1))))
    return np.array(pe), np.array(ke), x, v, F


def _wrap(x, cell):
    f = np.linalg.solve(cell, x.T).T
    f = f - np.floor(f)
    return f @ cell.T


@pytest.fixture(scope="module")
def eng(native_lib):
    from atomnn_gb300 import engine
    e = engine.Engine(os.path.join(GOLDEN, "mixed512.nnp"))
    yield e
    e.close()


@pytest.fixture(scope="module")
def orc(oracle_lib):
    return oracle_lib.OracleNNP(os.path.join(GOLDEN, "mixed512.nnp"))


@pytest.mark.parametrize("case", ["cell_list_skin", "image_shells", "zero_skin"])
def test_md_matches_oracle_integrator(eng, orc, case):
    rng = np.random.default_rng(3)
    # the oracle evaluates about 500 atoms/s on one core: keep atoms x steps small
    size, nsteps = {"cell_list_skin": (600, 20), "image_shells": (40, 40), "zero_skin": (300, 20)}[case]
    s = W.make_structures("mixed512", seed=9, count=1, sizes=[size])[0]
    n = s.natoms
    mass = np.where(s.species == 0, 2.0, 1.5)
    vel = rng.normal(0.0, 0.5, size=(n, 3))
    dt = 0.01
    md = eng.md(s, mass, dt, skin=0.0 if case == "zero_skin" else 0.2, vel=vel)
    try:
        pe, ke = md.run(nsteps)
        x, v, F, rebuilds = md.state()
    finally:
        md.close()
    pe_o, ke_o, x_o, v_o, F_o = _oracle_md(orc, s, mass, vel, dt, nsteps)
    assert np.abs(pe - pe_o).max() / n <= 1e-5
    assert np.abs(ke - ke_o).max() / n <= 1e-5
    np.testing.assert_allclose(x, _wrap(x_o, s.cell), rtol=0, atol=1e-6)
    np.testing.assert_allclose(v, v_o, rtol=0, atol=1e-5)
    assert np.abs(F - F_o).max() <= 1e-4
    if case == "cell_list_skin":
        # the fastest atoms move 0.1 A within about 6 steps: the 0.2 A skin list is rebuilt
        assert rebuilds >= 2


def test_md_start_forces_and_energy_conservation(eng, orc):
    """nnpgpu_md_forces before the run gives the standard velocity-Verlet start; over 300 steps
    of a 1728-atom cell the total energy stays put (a size-independent property)."""
    s = W.make_structures("cell1728")[0]
    n = s.natoms
    mass = np.where(s.species == 0, 24.305, 15.999) * 1.036427e-4  # amu -> eV ps^2 / A^2
    rng = np.random.default_rng(5)
    vel = rng.normal(0.0, 1.0, size=(n, 3)) * np.sqrt(0.025 / mass)[:, None]  # about 300 K
    md = eng.md(s, mass, 0.0005, skin=1.0, vel=vel)
    try:
        pe0 = md.forces()
        eo, _, _ = orc.compute(s.posn, s.species, s.cell, force=True)
        assert abs(pe0 - eo) / n <= 1e-5
        pe, ke = md.run(300)
    finally:
        md.close()
    tot = pe + ke
    assert np.abs(tot - tot[0]).max() / n < 1e-3, (tot.min(), tot.max())
    assert np.abs(pe - pe[0]).max() / n > 1e-4  # the system does evolve


def test_md_bf16_networks_start_and_energy_conservation(native_lib, oracle_lib, tmp_path):
    """The MD run with tensor-core (BF16 split) networks on the 1728-atom cell and its own
    potential: the starting energy against the FP64 oracle (1e-5 eV/atom) and the total energy
    over 300 steps, as for the FP32 networks."""
    from atomnn_gb300 import engine
    pot = W.workload_files("cell1728", str(tmp_path))
    s = W.make_structures("cell1728")[0]
    n = s.natoms
    mass = np.where(s.species == 0, 24.305, 15.999) * 1.036427e-4  # amu -> eV ps^2 / A^2
    rng = np.random.default_rng(5)
    vel = rng.normal(0.0, 1.0, size=(n, 3)) * np.sqrt(0.025 / mass)[:, None]  # about 300 K
    e = engine.Engine(pot)
    try:
        md = e.md(s, mass, 0.0005, skin=1.0, vel=vel, flags=engine.BF16)
        try:
            pe0 = md.forces()
            pe, ke = md.run(300)
        finally:
            md.close()
    finally:
        e.close()
    eo, _, _ = oracle_lib.OracleNNP(pot).compute(s.posn, s.species, s.cell, force=True)
    assert abs(pe0 - eo) / n <= 1e-5
    tot = pe + ke
    assert np.abs(tot - tot[0]).max() / n < 1e-3, (tot.min(), tot.max())
    assert np.abs(pe - pe[0]).max() / n > 1e-6  # the system does evolve


def test_md_invalid_inputs(eng):
    from atomnn_gb300 import engine
    s = W.make_structures("mixed512", seed=9, count=1, sizes=[40])[0]
    with pytest.raises(engine.NNPGPUError):
        eng.md(s, -1.0, 0.01)
    with pytest.raises(engine.NNPGPUError):
        eng.md(s, 1.0, 0.0)
    bad = W.Structure(posn=s.posn, species=np.full(s.natoms, 7, np.int32), cell=s.cell)
    with pytest.raises(engine.NNPGPUError):
        eng.md(bad, 1.0, 0.01)
