"""Host logic of bench.py on the CPU: the size strata the CPU legs time, the trainers' rows (with
an engine stand-in that answers through the oracle, so the GPU-vs-oracle gradient error must be
zero), and the parsing of the clock samples taken during the timed region."""
import os
import sys
import types

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)

import bench  # noqa: E402
from atomnn_gb300 import workloads as W  # noqa: E402


def test_strata_deal_every_structure_once():
    strucs = W.make_structures("mixed512")
    for n in (4, 64):
        parts = bench.strata(strucs, n)
        assert len(parts) == n
        ids = [id(s) for p in parts for s in p]
        assert sorted(ids) == sorted(id(s) for s in strucs)
        # each stratum holds every n-th structure by size rank: its first is no larger than the
        # previous stratum's first, and the atom counts are balanced
        firsts = [p[0].natoms for p in parts]
        assert firsts == sorted(firsts, reverse=True)
        sums = [sum(s.natoms for s in p) for p in parts]
        assert max(sums) - min(sums) <= max(s.natoms for s in strucs)


def test_training_rows_with_an_oracle_engine(oracle_lib):
    pot = W.workload_files("mixed512", bench.WORK_DIR)
    orc = oracle_lib.OracleNNP(pot)
    strucs = sorted(W.make_structures("mixed512"), key=lambda s: s.natoms)[:8]  # the 8 smallest

    class OracleEngine:
        def compute(self, S, flags):
            r = [orc.compute(s.posn, s.species, s.cell, force=True) for s in S]
            return np.array([x[0] for x in r]), [x[1] for x in r], None

        def train_grad(self, S, er, loss):
            return orc.train_grad(S, er, 0, 1.0)

        def train_force_grad(self, S, er, fr, beta, loss):
            return orc.train_force_grad(S, er, fr, beta, 0, 1.0)

    E = types.SimpleNamespace(ENERGY=1, FORCE=2, BATCHED=0x20)
    out = bench.training_lines(E, OracleEngine(), pot, strucs)
    assert set(out) == {"energy", "energy_force"}
    for row in out.values():
        assert row["structures"] == 8 and row["atoms"] == sum(s.natoms for s in strucs)
        assert row["atoms_per_s"] > 0 and row["ms_per_call"] > 0
        assert row["cpu_oracle"]["cores"] == 1 and row["cpu_oracle"]["atoms_per_s"] > 0
        assert row["grad_err_vs_oracle"] == 0.0


def test_clock_samples_parsed(monkeypatch):
    lines = ["0, 2070, 2070, 900.1, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
             "0, 2055, 2070, 1350.0, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
             "0, 2070, 2070, 1300.2, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
             "garbage line"]

    class FakeProc:
        def terminate(self):
            pass

        def communicate(self, timeout=None):
            return "\n".join(lines), ""

    monkeypatch.setattr(bench.subprocess, "Popen", lambda *a, **k: FakeProc())
    clk = bench.ClockSampler(0).stop()
    assert clk["sm_mhz"] == 2070.0 and clk["sm_max_mhz"] == 2070.0
    assert clk["reasons"] == ["sw_power_cap"] and clk["samples"] == 3


def test_reference_arm_line():
    """bench.py --impl reference on the CPU (the oracle over the host cores) prints one JSON line
    with the keys of the benchmark contract; a 32-structure workload keeps it short."""
    import json
    import subprocess
    out = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference", "--steps", "1", "--warmup", "3",
                          "--count", "32"], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "atoms/s" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["steps"] == 1 and d["warmup"] == 3 and d["n_gpus"] == 1
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"] == {"value": d["value"], "unit": "atoms/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert "32 triclinic" in d["config"]["workload"]
