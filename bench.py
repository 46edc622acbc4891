#!/usr/bin/env python3
"""Throughput benchmark of the NNP energy+force path on one GB300 (or N replicas).

A step is one evaluation of energy and forces of every structure of the workload ``mixed512``
(512 seeded triclinic two-species structures, 16-2048 atoms, log-uniform; 24 G2 + 32 G4 per
species; networks 56-64-64-1): neighbour lists, symmetry functions, atomic networks, chain
rule and force sums, all on the GPU.  ``value`` is atoms/s with inputs resident in HBM;
``e2e`` is the same through the host-buffer C API (copies inside the timed region).

``--impl reference`` times the reference algorithm on the host CPU cores instead: the FP64 C++
restatement in oracle/, which reproduces the reference's own code bit for bit on the pinned
fixtures (the reference's sources are not on this machine), over all host cores: each step is
one of four size strata of the workload (every fourth structure by size, largest first), so
four steps cover it once; the GPU arm's ``cpu_baseline`` times the same four strata.

Besides the headline, the line carries per-configuration figures (``configs``) for the 64-atom
one-species cell, the 1728-atom two-species cell and the 65,536-atom cell with its 96-128-128-1
networks: GPU atoms/s of the plain FP32 and the batched BF16 path, the oracle's single-thread
atoms/s, and the energy and force errors against FP64.  ``md`` gives velocity-Verlet step rates
on resident device state for the two cells, ``training`` the trainers' batch error and gradient
over the whole workload, each beside the oracle on one core.
"""
import argparse
import json
import math
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

from atomnn_gb300 import workloads as W  # noqa: E402

METRIC = "atoms/sec E+F (BF16 batched vs plain), p50/p99 latency, at force err ≤1e-3 eV/Å"
WORKLOAD = "mixed512"
KERNELS_PER_BATCH = 12  # frac, cell scan, cell fill, neighbor, symm, 3x type sort, network, force, force conversion, energy
WORK_DIR = os.path.join(REPO, "atomnn_gb300", "_build", "workloads")


# ----------------------------------------------------------------------------- CPU (oracle) leg
_ORC = None


def _oracle_init(potpath):
    global _ORC
    from oracle import pyoracle
    _ORC = pyoracle.OracleNNP(potpath)


def _oracle_eval(args):
    posn, species, cell = args
    e, F, _ = _ORC.compute(posn, species, cell, force=True)
    return e, F


NSTRATA = 4


def strata(strucs, n=NSTRATA):
    """The workload's structures sorted by size (largest first) and dealt into n strata: every
    stratum holds every n-th structure by size rank, so each has the workload's size mix."""
    order = sorted(range(len(strucs)), key=lambda k: -strucs[k].natoms)
    return [[strucs[k] for k in order[q::n]] for q in range(n)]


def largest_first(strucs):
    return sorted(strucs, key=lambda s: -s.natoms)


class OraclePool:
    """Process pool (spawn) running the FP64 oracle on the host cores."""

    def __init__(self, potpath, procs):
        from oracle import pyoracle
        pyoracle.build()
        self.procs = procs
        self.pool = mp.get_context("spawn").Pool(procs, initializer=_oracle_init, initargs=(potpath,))
        self.pool.map(_oracle_eval, [(np.zeros((1, 3)), np.zeros(1, np.int32), np.eye(3) * 20.0)] * procs)

    def run(self, strucs):
        """E+F of every structure, one task per structure in the given order (largest first
        balances the processes); returns (seconds, results)."""
        t0 = time.perf_counter()
        res = self.pool.map(_oracle_eval, [(s.posn, s.species, s.cell) for s in strucs], chunksize=1)
        return time.perf_counter() - t0, res

    def close(self):
        self.pool.terminate()


# ----------------------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.proc = None
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(device), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout=10)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for k, name in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


# ----------------------------------------------------------------------------- helpers
def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def convention_work(eng, strucs, pot):
    """Algorithmic work of one step in the fixed convention: FP32 flops of descriptors+chain rule
    = P*(30 + 13*nR_J) + T*(60 + 25*nA_JK); neighbour bytes = 16N + 16P + 4N; force and energy bytes =
    52N (fixed-point sums in, FP64 forces out, atomic energies in); network flops = 4*sum_l in_l*out_l per atom."""
    nt = pot.ntypes
    nR = [[len(pot.radial[(i, j)].rs) for j in range(nt)] for i in range(nt)]
    nA = {(i, j, k): len(pot.angular[(i, j, k)].eta) for i in range(nt) for j in range(nt) for k in range(j, nt)}
    flops_desc, P, N = 0.0, 0, 0
    for s in strucs:
        nb = eng.neighbors(s.posn, s.cell, cap=256)
        for a, lst in enumerate(nb):
            I = int(s.species[a])
            t = s.species[lst["index"]]
            cnt = [int((t == J).sum()) for J in range(nt)]
            P += len(t)
            for J in range(nt):
                flops_desc += cnt[J] * (30 + 13 * nR[I][J])
                for K in range(J, nt):
                    T = cnt[J] * (cnt[J] - 1) // 2 if J == K else cnt[J] * cnt[K]
                    flops_desc += T * (60 + 25 * nA[(I, J, K)])
        N += s.natoms
    net_flops = 0.0
    for s in strucs:
        for I in range(nt):
            n = int((s.species == I).sum())
            net = pot.nets[I]
            dims = [net.nin] + list(net.nodes)
            net_flops += n * 4 * sum(dims[l] * dims[l + 1] for l in range(len(dims) - 1))
    return dict(pairs=P, atoms=N, desc_flops=flops_desc, nbr_bytes=16 * N + 16 * P + 4 * N, gather_bytes=52 * N,
                net_flops=net_flops)


def peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return d, "measured (MEASURED_PEAKS.json)"
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "sm_max_mhz": 2070.0}, "fallback"


# ----------------------------------------------------------------------------- reference arm
def run_reference(args, ws, rank):
    if rank != 0:
        return 0
    potpath = W.workload_files(WORKLOAD, WORK_DIR)
    strucs = W.make_structures(WORKLOAD)[:args.count]
    procs = os.cpu_count() or 1
    pool = OraclePool(potpath, procs)
    parts = strata(strucs)
    times, atoms = [], []
    for k in range(args.warmup + args.steps):
        sample = parts[k % NSTRATA]
        dt, _ = pool.run(sample)
        if k >= args.warmup:
            times.append(dt)
            atoms.append(sum(s.natoms for s in sample))
    pool.close()
    value = sum(atoms) / sum(times)
    sample_desc = ("each step: one of %d size strata of the %d-structure workload (every %d-th structure by size, %d structures, "
                   "about %d atoms), largest first, one process per core; %d consecutive steps cover the workload once"
                   % (NSTRATA, len(strucs), NSTRATA, len(parts[0]), sum(s.natoms for s in parts[0]), NSTRATA))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "atoms/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000 * statistics.mean(times), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": {"workload": "%s: %d triclinic A/B structures, 16-2048 atoms, 56-64-64-1 networks" % (WORKLOAD, len(strucs)),
                       "parallelism": "host cores (process pool)"},
            "cpu_baseline": {"value": value, "unit": "atoms/s", "cores": procs, "kind": "port", "sample": sample_desc},
            "e2e": {"value": value, "unit": "atoms/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ----------------------------------------------------------------------------- per-configuration lines
CONFIGS = (
    ("c1_small64", "small64", "64-atom one-species cubic cell (8.1 A), 16 G2 + 16 G4, 32-32-32-1 networks, rc 6.0 A"),
    ("c2_cell1728", "cell1728", "1728-atom A:B 1:2 cubic cell at 0.07/A^3, 24 G2 + 32 G4 per species, 56-64-64-1 networks, rc 6.5 A"),
    ("c4_cell65536", "cell65536", "65,536-atom A:B 1:2 cubic cell at 0.07/A^3, 32 G2 + 64 G4 per species, 96-128-128-1 networks, rc 6.5 A"),
)


def cpu_config_baselines(run_cpu):
    """The oracle's single-thread E+F atoms/s per configuration (run before any GPU call).  The
    65,536-atom cell is timed on a sample of 256 centres, each with the reference's full scan
    over all atoms for its neighbour list (NeighborList::build with a subset), its descriptors,
    network and chain rule: the per-atom cost of the whole evaluation."""
    from oracle import pyoracle
    out = {}
    for key, name, _ in CONFIGS:
        if not run_cpu:
            out[key] = None
            continue
        pot = W.workload_files(name, WORK_DIR)
        orc = pyoracle.OracleNNP(pot)
        s = W.make_structures(name)[0]
        if name == "cell65536":
            centres = np.random.default_rng(5).choice(s.natoms, 256, replace=False)
            t0 = time.perf_counter()
            orc.compute_centres(s.posn, s.species, s.cell, centres)
            dt = time.perf_counter() - t0
            out[key] = {"atoms_per_s": len(centres) / dt, "cores": 1, "seconds": dt,
                        "sample": "256 centres of the cell, each scanning all 65,536 atoms (O(N) per centre as in the reference)"}
        else:
            reps = 20 if s.natoms < 500 else 1
            t0 = time.perf_counter()
            for _ in range(reps):
                e, F, _ = orc.compute(s.posn, s.species, s.cell, force=True)
            dt = (time.perf_counter() - t0) / reps
            out[key] = {"atoms_per_s": s.natoms / dt, "cores": 1, "seconds": dt, "sample": "the whole structure",
                        "energy": e, "force": F}
    return out


def gpu_config_lines(E, device, stream, cpu):
    """GPU atoms/s of each configuration through nnpgpu_compute_device (inputs in HBM; CUDA events
    around 10 calls after 3 warm-up calls): the plain FP32 path (the batched flag off) and the
    batched BF16 path, with their energy and force errors against FP64 (the oracle for the small
    cells, the committed oracle fixture tests/golden/cell65536.npz for the large one)."""
    import hashlib
    import torch
    dev = torch.device("cuda", device)
    out = {}
    for key, name, desc in CONFIGS:
        pot = W.workload_files(name, WORK_DIR)
        s = W.make_structures(name)[0]
        eng = E.Engine(pot, device=device)
        try:
            natoms = np.array([s.natoms], dtype=np.int32)
            cells = s.cell_colmajor()
            d_posn = torch.from_numpy(np.ascontiguousarray(s.posn)).to(dev)
            d_spec = torch.from_numpy(np.ascontiguousarray(s.species, dtype=np.int32)).to(dev)
            d_e = torch.zeros(1, dtype=torch.float64, device=dev)
            d_f = torch.zeros((s.natoms, 3), dtype=torch.float64, device=dev)
            line = {"workload": desc, "atoms": s.natoms}
            for tag, flags in (("gpu_plain_fp32", E.ENERGY | E.FORCE), ("gpu_batched_bf16", E.ENERGY | E.FORCE | E.BATCHED | E.BF16)):
                step = lambda: eng.compute_device(natoms, d_posn.data_ptr(), d_spec.data_ptr(), cells, flags, d_e.data_ptr(), d_f.data_ptr(),
                                                  0, stream.cuda_stream)
                for _ in range(3):
                    step()
                torch.cuda.synchronize()
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                for _ in range(10):
                    step()
                b.record(stream)
                torch.cuda.synchronize()
                ms = a.elapsed_time(b) / 10
                e = float(d_e.cpu()[0])
                F = d_f.cpu().numpy()
                err = None
                if name == "cell65536":
                    fx = os.path.join(REPO, "tests", "golden", "cell65536.npz")
                    if os.path.exists(fx):
                        g = np.load(fx)
                        h = hashlib.sha256()
                        for arr in (np.ascontiguousarray(s.posn, dtype=np.float64), np.ascontiguousarray(s.species, dtype=np.int32),
                                    np.ascontiguousarray(s.cell, dtype=np.float64)):
                            h.update(arr.tobytes())
                        if h.hexdigest() == str(g["structure_sha256"][0]):
                            dF = F[g["force_atoms"]] - g["force"]
                            err = {"energy_err_per_atom": abs(e - float(g["energy"][0])) / s.natoms,
                                   "force_rmse": float(np.sqrt((dF ** 2).mean())), "force_err_max": float(np.abs(dF).max()),
                                   "against": "FP64 oracle fixture (every 8th atom's force)"}
                elif cpu.get(key):
                    dF = F - cpu[key]["force"]
                    err = {"energy_err_per_atom": abs(e - cpu[key]["energy"]) / s.natoms, "force_rmse": float(np.sqrt((dF ** 2).mean())),
                           "force_err_max": float(np.abs(dF).max()), "against": "FP64 oracle"}
                line[tag] = {"atoms_per_s": s.natoms / (ms / 1000.0), "ms": ms, "errors": err}
            if cpu.get(key):
                line["cpu_oracle"] = {k: v for k, v in cpu[key].items() if k not in ("energy", "force")}
            out[key] = line
        finally:
            eng.close()
    return out


def md_lines(E, device, bf16, cpu):
    """Velocity-Verlet MD on resident device state (nnpgpu_md_run; the reference's MD job,
    src/torch/torch.cpp:267-275, with Verlet::compute and PotNNPE::compute) on the 1728-atom and
    the 65,536-atom cells with their own potentials: host wall clock around nnpgpu_md_run, which
    returns every step's potential and kinetic energy.  The CPU figure is one force evaluation of
    the oracle per step on one core (the reference's MD job evaluates one structure in one process),
    from the per-configuration CPU timings."""
    out = {}
    for key, name, nsteps in (("c2_cell1728", "cell1728", 500), ("c4_cell65536", "cell65536", 50)):
        pot = W.workload_files(name, WORK_DIR)
        s = W.make_structures(name)[0]
        n = s.natoms
        mass = np.where(s.species == 0, 24.305, 15.999) * 1.036427e-4  # amu -> eV ps^2 / A^2
        vel = np.random.default_rng(5).normal(0.0, 1.0, size=(n, 3)) * np.sqrt(0.025 / mass)[:, None]  # about 300 K
        eng = E.Engine(pot, device=device)
        try:
            md = eng.md(s, mass, 0.0005, skin=1.0, vel=vel, flags=E.BF16 if bf16 else 0)
            try:
                md.forces()
                md.run(20)
                t0 = time.perf_counter()
                pe, ke = md.run(nsteps)
                dt = time.perf_counter() - t0
                _, _, _, rebuilds = md.state()
            finally:
                md.close()
        finally:
            eng.close()
        tot = pe + ke
        line = {"atoms": n, "steps": nsteps, "ms_per_step": 1000.0 * dt / nsteps, "atom_steps_per_s": n * nsteps / dt,
                "list_rebuilds": rebuilds, "energy_drift_per_atom": float(np.abs(tot - tot[0]).max() / n),
                "networks": "BF16 tensor cores" if bf16 else "FP32",
                "desc": "dt 0.5 fs, 1.0 A skin (the rc+skin list re-decided at rc every step, rebuilt after skin/2), about 300 K"}
        c = cpu.get(key)
        if c:
            per_atom = 1.0 / c["atoms_per_s"]
            line["cpu_oracle"] = {"atom_steps_per_s": c["atoms_per_s"], "ms_per_step": 1000.0 * per_atom * n, "cores": 1,
                                  "sample": "one E+F evaluation of the cell per step (" + c["sample"] + ")"}
        out[key] = line
    return out


def training_lines(E, eng, potpath, strucs):
    """The trainers' batch error and gradient (nnpgpu_train_grad: NNPTE::error with Cost::grad,
    src/nnp/nnpte.cpp:870-921; nnpgpu_train_force_grad: NNPTEF::error, src/nnp/nnptef.cpp:1043-1135)
    over the whole workload through the host-buffer API (host wall clock, mean of 3 calls after one),
    and the FP64 oracle's same call on one core over every 64th structure by size, with the
    gradients' agreement on that sample."""
    from oracle import pyoracle
    rng = np.random.default_rng(11)
    e0, F0, _ = eng.compute(strucs, E.ENERGY | E.FORCE | E.BATCHED)
    eref = np.array(e0) + rng.normal(0.0, 0.3, size=len(strucs)) * np.array([s.natoms for s in strucs]) ** 0.5
    fref = [F + rng.normal(0.0, 0.2, F.shape) for F in F0]
    atoms = sum(s.natoms for s in strucs)
    one = strata(strucs, 64)[0]
    pick = [next(k for k, s in enumerate(strucs) if s is x) for x in one]
    orc = pyoracle.OracleNNP(potpath)
    out = {}
    for tag, gpu_call, cpu_call in (
            ("energy", lambda S, er, fr: eng.train_grad(S, er, "MSE")[-1],
             lambda S, er, fr: orc.train_grad(S, er, 0, 1.0)[-1]),
            ("energy_force", lambda S, er, fr: eng.train_force_grad(S, er, fr, 1.0, "MSE")[-1],
             lambda S, er, fr: orc.train_force_grad(S, er, fr, 1.0, 0, 1.0)[-1])):
        gpu_call(strucs, eref, fref)
        ts = []
        for _ in range(3):
            t0 = time.perf_counter()
            gpu_call(strucs, eref, fref)
            ts.append(time.perf_counter() - t0)
        er1, fr1 = eref[pick], [fref[k] for k in pick]
        t0 = time.perf_counter()
        go = cpu_call(one, er1, fr1)
        tc = time.perf_counter() - t0
        g = gpu_call(one, er1, fr1)
        n1 = sum(s.natoms for s in one)
        out[tag] = {"atoms_per_s": atoms / statistics.mean(ts), "ms_per_call": 1000.0 * statistics.mean(ts),
                    "structures": len(strucs), "atoms": atoms,
                    "cpu_oracle": {"atoms_per_s": n1 / tc, "cores": 1,
                                   "sample": "every 64th structure by size (%d structures, %d atoms), one process" % (len(one), n1)},
                    "grad_err_vs_oracle": float(np.abs(g - go).max() / np.abs(go).max()),
                    "desc": "loss MSE%s; batch error and gradient of every network parameter, FP64 reduction" %
                            (", force weight 1.0" if tag == "energy_force" else "")}
    return out


# ----------------------------------------------------------------------------- native arm
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="native", choices=["native", "reference"])
    ap.add_argument("--plain-steps", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-configs", action="store_true", help="skip the per-configuration lines")
    ap.add_argument("--shard", action="store_true",
                    help="N > 1: split the structures over the ranks (strong scaling) instead of replicating them (weak)")
    ap.add_argument("--count", type=int, default=512, help="structures of the workload (512 = the full workload)")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch shapes (profiling runs)")
    ap.add_argument("--serve-rate", type=float, default=2000.0)
    ap.add_argument("--serve-seconds", type=float, default=60.0)
    ap.add_argument("--no-md", action="store_true", help="skip the MD step rates")
    ap.add_argument("--no-train", action="store_true", help="skip the trainers' timings")
    ap.add_argument("--training-only", action="store_true", help="print only the trainers' timings (one JSON line)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    ws, rank, local = dist_info()
    if args.impl == "reference":
        return run_reference(args, ws, rank)
    if args.training_only:
        if rank == 0:
            import torch
            torch.cuda.set_device(local)
            from atomnn_gb300 import engine as E
            potpath = W.workload_files(WORKLOAD, WORK_DIR)
            eng = E.Engine(potpath, device=local)
            try:
                print(json.dumps({"workload": WORKLOAD, "training": training_lines(E, eng, potpath, W.make_structures(WORKLOAD)[:args.count])}),
                      flush=True)
            finally:
                eng.close()
        return 0

    pot = W.make_potential(WORKLOAD)
    potpath = W.workload_files(WORKLOAD, WORK_DIR)
    strucs = W.make_structures(WORKLOAD)[:args.count]
    job_atoms = sum(s.natoms for s in strucs)
    if args.shard and ws > 1:
        from atomnn_gb300 import replicas
        off, cnt = replicas.shard(len(strucs), rank, ws)  # contiguous blocks, as the compute tool distributes them
        strucs = strucs[off:off + cnt]
    natoms = np.array([s.natoms for s in strucs], dtype=np.int32)
    total_atoms = int(natoms.sum())

    # CPU baselines first: the spawn pool starts before any GPU call.  All cores: the workload's
    # four size strata (the reference arm's steps), each timed on its own, largest first; one
    # core: one size stratum of a 64-way split.
    cpu = None
    cpu_cfg = {}
    if rank == 0 and not args.no_cpu_baseline:
        procs = os.cpu_count() or 1
        pool = OraclePool(potpath, procs)
        sample, res, dt = [], [], 0.0
        for part in strata(strucs):
            t_part, r_part = pool.run(part)
            sample += part
            res += r_part
            dt += t_part
        tot = sum(x.natoms for x in sample)
        pool.close()
        one = strata(strucs, 64)[0]
        from oracle import pyoracle
        orc1 = pyoracle.OracleNNP(potpath)
        t0 = time.perf_counter()
        for x in one:
            orc1.compute(x.posn, x.species, x.cell, force=True)
        dt1 = time.perf_counter() - t0
        cpu = dict(value=tot / dt, unit="atoms/s", cores=procs, kind="port",
                   sample="all %d structures of the workload (%d atoms) once, as %d size strata timed one after the other "
                          "(each largest first), E+F, FP64 oracle, one process per core" % (len(sample), tot, NSTRATA),
                   single_thread={"value": sum(x.natoms for x in one) / dt1, "unit": "atoms/s", "cores": 1,
                                  "sample": "every 64th structure by size (%d structures, %d atoms), E+F, one process"
                                            % (len(one), sum(x.natoms for x in one))},
                   sample_structs=sample, sample_results=res, seconds=dt)
    if rank == 0 and not args.no_configs:
        cpu_cfg = cpu_config_baselines(not args.no_cpu_baseline)

    import torch
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    from atomnn_gb300 import engine as E
    eng = E.Engine(potpath, device=local)
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream

    posn = np.concatenate([s.posn for s in strucs])
    species = np.concatenate([s.species for s in strucs]).astype(np.int32)
    cells = np.concatenate([s.cell_colmajor() for s in strucs])
    d_posn = torch.from_numpy(posn).to(dev)
    d_spec = torch.from_numpy(species).to(dev)
    d_energy = torch.zeros(len(strucs), dtype=torch.float64, device=dev)
    d_force = torch.zeros((total_atoms, 3), dtype=torch.float64, device=dev)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def barrier():
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    def device_step(flags):
        eng.compute_device(natoms, d_posn.data_ptr(), d_spec.data_ptr(), cells, flags, d_energy.data_ptr(), d_force.data_ptr(), 0, sptr)

    def timed(flags, steps, warmup, profile=False):
        for _ in range(warmup):
            device_step(flags)
        if profile:
            eng.profile_enable(True)
            for _ in range(2):  # first traced run is uncaptured, the second one is captured
                device_step(flags)
            eng.profile_enable(True)  # reset the counters
        barrier()
        evs = []
        for _ in range(steps):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            device_step(flags)
            b.record(stream)
            evs.append((a, b))
        barrier()
        ms = [a.elapsed_time(b) for a, b in evs]
        prof = eng.profile_read() if profile else None
        if profile:
            eng.profile_enable(False)
        return ms, prof

    batched = E.ENERGY | E.FORCE | E.BATCHED
    bf16_ok = True
    try:
        device_step(batched | E.BF16)
    except E.NNPGPUError:
        bf16_ok = False
    head_flags = batched | (E.BF16 if bf16_ok else 0)
    # launch shapes (atoms per CTA of the neighbour / descriptor / chain-rule kernels) picked by
    # the engine's autotuner on this workload before anything is timed
    if args.no_autotune:
        tune_shapes, tune_report = eng.get_tune(), "not run (--no-autotune)"
    else:
        tune_shapes, tune_report = eng.autotune(natoms, posn, species, cells, (E.BF16 if bf16_ok else 0) | E.FORCE)

    clocks = ClockSampler(local)
    # keep the GPU busy for ~0.6 s (untimed) while the clock sampler starts, so that its samples
    # fall under load; the warm-up steps of timed() follow
    t_settle = time.perf_counter()
    while time.perf_counter() - t_settle < 0.6:
        device_step(head_flags)
        torch.cuda.synchronize()
    ms, prof = timed(head_flags, args.steps, args.warmup, profile=True)
    clk = clocks.stop()
    t_step = statistics.mean(ms) / 1000.0
    if ws > 1:
        t = torch.tensor([t_step], dtype=torch.float64, device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        t_step = float(t.item())
    value = (job_atoms if (args.shard and ws > 1) else ws * total_atoms) / t_step

    # batched FP32 (when the headline is BF16) and the plain path (one structure at a time)
    fp32_ms, _ = timed(batched, args.steps, 1) if bf16_ok else (ms, None)
    plain_ms, _ = timed(E.ENERGY | E.FORCE, args.plain_steps, 1) if args.plain_steps > 0 else (None, None)

    # end to end through the host-buffer API with page-locked host arrays (the library copies
    # them by DMA, no staging), copies inside the timed region
    keep = []

    def pinned(a):
        t = torch.empty(a.shape, dtype=torch.from_numpy(np.ascontiguousarray(a)).dtype, pin_memory=True)
        keep.append(t)
        v = t.numpy()
        v[...] = a
        return v

    posn_h, species_h = pinned(posn), pinned(species)
    h_energy = pinned(np.zeros(len(strucs)))
    h_force = pinned(np.zeros((total_atoms, 3)))
    for _ in range(2):
        eng.compute_flat(natoms, posn_h, species_h, cells, head_flags, h_energy, h_force)
    barrier()
    e2e_t = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        eng.compute_flat(natoms, posn_h, species_h, cells, head_flags, h_energy, h_force)
        e2e_t.append(time.perf_counter() - t0)
    barrier()
    e2e_step = statistics.mean(e2e_t)
    if ws > 1:
        t = torch.tensor([e2e_step], dtype=torch.float64, device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_step = float(t.item())
    job = job_atoms if (args.shard and ws > 1) else ws * total_atoms

    # serving: Poisson stream of 16-4096-atom requests with 20% resident MD-style repeat steps,
    # then a saturating burst; latencies are measured by the engine (submission -> completion)
    serve_out = None
    if not args.no_serving:
        from atomnn_gb300 import serving as SV
        pool = SV.make_pool()
        eng.serve_start(max_inflight=3, skin=1.0, flags=(E.BF16 if bf16_ok else 0), hbm_budget_bytes=40 << 30)
        SV.run_stream(eng, pool, rate=args.serve_rate, duration=1.0, seed=1)
        st = SV.run_stream(eng, pool, rate=args.serve_rate, duration=args.serve_seconds, seed=2)
        bu = SV.run_stream(eng, pool, rate=2000.0, duration=1.0, burst=True, repeat_frac=0.0, seed=3)
        eng.serve_stop()
        # the plain FP32 path (one structure per call, inputs in HBM) on the same size mix: every
        # structure of the request pool once
        p_nat = np.array([x.natoms for x in pool], dtype=np.int32)
        p_pos = torch.from_numpy(np.concatenate([x.posn for x in pool])).to(dev)
        p_spe = torch.from_numpy(np.concatenate([x.species for x in pool]).astype(np.int32)).to(dev)
        p_cel = np.concatenate([x.cell_colmajor() for x in pool])
        p_e = torch.zeros(len(pool), dtype=torch.float64, device=dev)
        p_f = torch.zeros((int(p_nat.sum()), 3), dtype=torch.float64, device=dev)
        pstep = lambda: eng.compute_device(p_nat, p_pos.data_ptr(), p_spe.data_ptr(), p_cel, E.ENERGY | E.FORCE, p_e.data_ptr(),
                                           p_f.data_ptr(), 0, sptr)
        pstep()
        torch.cuda.synchronize()
        pa, pb = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        pa.record(stream)
        for _ in range(2):
            pstep()
        pb.record(stream)
        torch.cuda.synchronize()
        plain_serve = 2 * int(p_nat.sum()) / (pa.elapsed_time(pb) / 1000.0)
        pct = lambda a, q: float(np.percentile(a, q) * 1000.0) if len(a) else None
        serve_out = {
            "offered_req_per_s": args.serve_rate, "seconds": args.serve_seconds, "requests": st["requests"], "repeat_steps": st["repeats"],
            "p50_ms": pct(st["latencies"], 50), "p99_ms": pct(st["latencies"], 99), "atoms_per_s": st["atoms"] / st["wall"],
            "saturated": {"requests": bu["requests"], "atoms_per_s": bu["atoms"] / bu["wall"], "p50_ms": pct(bu["latencies"], 50),
                          "p99_ms": pct(bu["latencies"], 99)},
            "plain_same_mix": {"atoms_per_s": plain_serve, "desc": "plain FP32 path, one structure per call, on the request pool's "
                                                                   "%d structures (16-4096 atoms)" % len(pool)},
            "saturated_vs_plain_same_mix": (bu["atoms"] / bu["wall"]) / plain_serve,
            "desc": "nnpgpu_serve_*: 3 slots, continuous batching, 40 GB admission budget, 1.0 A skin for resident keys, "
                    "sizes log-uniform 16-4096 atoms",
        }
    h2d = posn.nbytes + species.nbytes + cells.nbytes + natoms.nbytes
    d2h = 8 * len(strucs) + 24 * total_atoms + 32

    out = None
    if rank == 0:
        pk, pk_src = peaks()
        work = convention_work(eng, strucs, pot)
        stage = {k: (v[0] / max(v[1], 1)) for k, v in prof.items()}
        if min(stage.values()) <= 0:
            raise RuntimeError("stage tracing returned no timings: %r" % prof)
        t_desc = (stage["descriptors"] + stage["chain_rule"]) / 1000.0
        sms = torch.cuda.get_device_properties(dev).multi_processor_count
        fp32_peak = sms * 128 * 2 * pk.get("sm_max_mhz", 2070.0) * 1e6 / 1e12
        ach = work["desc_flops"] / t_desc / 1e12
        executed = None
        ffile = os.path.join(REPO, "profiles", "flops.json")
        if os.path.exists(ffile):
            with open(ffile) as f:
                fpa = json.load(f).get(WORKLOAD, {}).get("executed_fp32_flops_per_atom")
            if fpa:
                ex = fpa * total_atoms / t_desc / 1e12
                executed = {"achieved": ex, "frac": ex / fp32_peak, "unit": "TFLOP/s",
                            "work": "%d FP32 flops per atom executed (2 FFMA + FADD + FMUL, ncu instruction counts, "
                                    "profiles/flops.json)" % fpa}
        roof = {"bound": "fp32", "kernel": "symm_kernel + force_kernel (descriptor and chain-rule triplet passes)",
                "achieved": ach, "peak": fp32_peak, "unit": "TFLOP/s", "frac": ach / fp32_peak, "traffic": None,
                "peak_source": "derived: %d SMs (from the device) x 128 FP32 lanes x 2 x sm_max_mhz from MEASURED_PEAKS.json "
                               "(no FP32 figure is measured)" % sms,
                "work": "convention flops P*(30+13 nR) + T*(60+25 nA) = %.4g per step" % work["desc_flops"],
                "kernel_ms": t_desc * 1000.0, "executed": executed,
                "note": "achieved/frac count the fixed convention's flops, which the moment-tensor blocks no longer execute; "
                        "executed.frac is the FP32 work the kernels actually issue"}
        tfile = os.path.join(REPO, "profiles", "traffic.json")
        if os.path.exists(tfile):
            with open(tfile) as f:
                roof["traffic"] = json.load(f).get(WORKLOAD)
        hbm = pk["hbm_gbs"]
        kernels = {
            "neighbors": {"bound": "hbm", "achieved_gbs": work["nbr_bytes"] / (stage["neighbors"] / 1000) / 1e9, "peak_gbs": hbm,
                          "ms": stage["neighbors"]},
            "forces_energy": {"bound": "hbm", "achieved_gbs": work["gather_bytes"] / (stage["forces_energy"] / 1000) / 1e9,
                              "peak_gbs": hbm, "ms": stage["forces_energy"]},
            "networks": {"bound": "tensor" if bf16_ok else "fp32", "achieved_tflops": work["net_flops"] / (stage["networks"] / 1000) / 1e12,
                         "peak_tflops": pk["bf16_tflops"] if bf16_ok else fp32_peak, "ms": stage["networks"]},
            "descriptors": {"ms": stage["descriptors"]}, "chain_rule": {"ms": stage["chain_rule"]}, "force_clear": {"ms": stage["force_clear"]},
        }
        acc = None
        if cpu is not None:
            acc = {}
            for tag, fl in (("bf16" if bf16_ok else "fp32", head_flags), ("fp32", batched)):
                e, F, _ = eng.compute(cpu["sample_structs"], fl)
                de = max(abs(e[k] - cpu["sample_results"][k][0]) / s.natoms for k, s in enumerate(cpu["sample_structs"]))
                dF = np.concatenate([F[k] - cpu["sample_results"][k][1] for k in range(len(F))])
                acc[tag] = {"energy_err_per_atom_max": de, "force_rmse": float(np.sqrt((dF ** 2).mean())),
                            "force_err_max": float(np.abs(dF).max())}
        out = {
            "metric": METRIC, "value": value, "unit": "atoms/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": t_step * 1000.0, "higher_is_better": True, "scaling": "strong" if (args.shard and ws > 1) else "weak",
            "vs_baseline": None,
            "dtype": "bf16" if bf16_ok else "f32", "data": "synthetic (seeded generator, atomnn_gb300/workloads.py)",
            "config": {"workload": "%s: %d triclinic A/B structures (%d atoms), N log-uniform 16-2048, density 0.05-0.09/A^3, "
                                   "24 G2 + 32 G4 per species, networks 56-64-64-1 tanh, rc 6.5 A" % (WORKLOAD, len(strucs), total_atoms),
                       "structures": len(strucs), "atoms": total_atoms, "path": "batched (one launch sequence per step, CUDA graph)",
                       "networks": "BF16 tensor cores" if bf16_ok else "FP32", "parallelism": "replicas" if ws > 1 else "single GPU",
                       "l2": "flushed between timed steps (512 MiB write, outside the step events)",
                       "launch_shapes": tune_shapes},
            "autotune": tune_report,
            "clocks": clk,
            "e2e": {"value": job / e2e_step, "unit": "atoms/s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                    "ms_per_step": e2e_step * 1000,
                    "path": "nnpgpu_compute on page-locked host arrays (positions, species, cells in; energies, forces out)"},
            "gpu_launches": KERNELS_PER_BATCH * args.steps,
            "roofline": roof,
            "kernels": kernels,
            "plain": None if plain_ms is None else {
                "value": total_atoms / (statistics.mean(plain_ms) / 1000), "unit": "atoms/s", "ms_per_step": statistics.mean(plain_ms),
                "desc": "one structure at a time (12 launches per structure), FP32 networks"},
            "batched_fp32": {"value": total_atoms / (statistics.mean(fp32_ms) / 1000), "unit": "atoms/s", "ms_per_step": statistics.mean(fp32_ms)},
            "accuracy_vs_fp64_oracle": acc,
            "accuracy_sample": None if cpu is None else "all %d structures of the workload" % len(cpu["sample_structs"]),
            "serving": serve_out,
        }
        if cpu is not None:
            out["cpu_baseline"] = {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample", "single_thread")}
        if not args.no_configs:
            out["configs"] = gpu_config_lines(E, local, stream, cpu_cfg)
        if not args.no_md:
            try:
                out["md"] = md_lines(E, local, bf16_ok, cpu_cfg)
            except Exception as ex:  # reported in the line; the headline stands on its own
                out["md"] = {"error": repr(ex)}
        if not args.no_train:
            try:
                out["training"] = training_lines(E, eng, potpath, strucs)
            except Exception as ex:
                out["training"] = {"error": repr(ex)}
        print(json.dumps(out), flush=True)
    eng.close()
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
