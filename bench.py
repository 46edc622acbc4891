#!/usr/bin/env python3
"""Throughput benchmark of the NNP energy+force path on one GB300 (or N replicas).

A step is one evaluation of energy and forces of every structure of the workload ``mixed512``
(512 seeded triclinic two-species structures, 16-2048 atoms, log-uniform; 24 G2 + 32 G4 per
species; networks 56-64-64-1): neighbour lists, symmetry functions, atomic networks, chain
rule and force gather, all on the GPU.  ``value`` is atoms/s with inputs resident in HBM;
``e2e`` is the same through the host-buffer C API (copies inside the timed region).

``--impl reference`` times the reference algorithm on the host CPU cores instead: the FP64 C++
restatement in oracle/ (the reference itself cannot be built here: Eigen and MPI are absent),
over all host cores, on bounded samples of the same workload.
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
KERNELS_PER_BATCH = 15  # frac, cell scan, cell fill, neighbor, 2x reverse, symm, 3x type sort, network, force, gather, orphan, energy
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


def cpu_sample(strucs, target_atoms, offset=0):
    out, tot, k = [], 0, offset
    while tot < target_atoms:
        s = strucs[k % len(strucs)]
        out.append(s)
        tot += s.natoms
        k += 1
    return out, tot


class OraclePool:
    """Process pool (spawn) running the FP64 oracle on the host cores."""

    def __init__(self, potpath, procs):
        from oracle import pyoracle
        pyoracle.build()
        self.procs = procs
        self.pool = mp.get_context("spawn").Pool(procs, initializer=_oracle_init, initargs=(potpath,))
        self.pool.map(_oracle_eval, [(np.zeros((1, 3)), np.zeros(1, np.int32), np.eye(3) * 20.0)] * procs)

    def run(self, strucs):
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
    = P*(30 + 13*nR_J) + T*(60 + 25*nA_JK); neighbour bytes = 16N + 16P + 4N; gather bytes =
    28P + 24N; network flops = 4*sum_l in_l*out_l per atom."""
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
    return dict(pairs=P, atoms=N, desc_flops=flops_desc, nbr_bytes=16 * N + 16 * P + 4 * N, gather_bytes=28 * P + 24 * N,
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
    pot = W.make_potential(WORKLOAD)
    potpath = W.workload_files(WORKLOAD, WORK_DIR)
    strucs = W.make_structures(WORKLOAD)
    procs = os.cpu_count() or 1
    pool = OraclePool(potpath, procs)
    per_step_atoms = int(args.ref_step_atoms or 600 * procs)
    times, atoms = [], []
    off = 0
    for k in range(args.warmup + args.steps):
        sample, tot = cpu_sample(strucs, per_step_atoms, off)
        off += len(sample)
        dt, _ = pool.run(sample)
        if k >= args.warmup:
            times.append(dt)
            atoms.append(tot)
    pool.close()
    value = sum(atoms) / sum(times)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "atoms/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000 * statistics.mean(times), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": {"workload": "%s: %s" % (WORKLOAD, "512 triclinic A/B structures, 16-2048 atoms, 56-64-64-1 networks"),
                       "parallelism": "host cores (process pool)"},
            "cpu_baseline": {"value": value, "unit": "atoms/s", "cores": procs, "kind": "port",
                             "sample": "each step: consecutive structures of the workload totalling >= %d atoms" % per_step_atoms},
            "e2e": {"value": value, "unit": "atoms/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ----------------------------------------------------------------------------- native arm
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="native", choices=["native", "reference"])
    ap.add_argument("--plain-steps", type=int, default=3)
    ap.add_argument("--cpu-atoms-per-core", type=int, default=4000)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ref-step-atoms", type=int, default=0)
    ap.add_argument("--count", type=int, default=512, help="structures of the workload (512 = the full workload)")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch shapes (profiling runs)")
    ap.add_argument("--serve-rate", type=float, default=2000.0)
    ap.add_argument("--serve-seconds", type=float, default=5.0)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    ws, rank, local = dist_info()
    if args.impl == "reference":
        return run_reference(args, ws, rank)

    pot = W.make_potential(WORKLOAD)
    potpath = W.workload_files(WORKLOAD, WORK_DIR)
    strucs = W.make_structures(WORKLOAD)[:args.count]
    natoms = np.array([s.natoms for s in strucs], dtype=np.int32)
    total_atoms = int(natoms.sum())

    # CPU baseline first: the spawn pool starts before any GPU call
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        procs = os.cpu_count() or 1
        pool = OraclePool(potpath, procs)
        sample, tot = cpu_sample(strucs, args.cpu_atoms_per_core * procs)
        dt, res = pool.run(sample)
        pool.close()
        cpu = dict(value=tot / dt, unit="atoms/s", cores=procs, kind="port",
                   sample="first %d structures of the workload (%d atoms), E+F, FP64 oracle, one process per core" % (len(sample), tot),
                   sample_structs=sample, sample_results=res, seconds=dt)

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
    ms, prof = timed(head_flags, args.steps, args.warmup, profile=True)
    clk = clocks.stop()
    t_step = statistics.mean(ms) / 1000.0
    if ws > 1:
        t = torch.tensor([t_step], dtype=torch.float64, device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        t_step = float(t.item())
    value = ws * total_atoms / t_step

    # batched FP32 (when the headline is BF16) and the plain path (one structure at a time)
    fp32_ms, _ = timed(batched, args.steps, 1) if bf16_ok else (ms, None)
    plain_ms, _ = timed(E.ENERGY | E.FORCE, args.plain_steps, 1) if args.plain_steps > 0 else (None, None)

    # end to end through the host-buffer API (pinned staging, copies inside the timed region)
    h_energy = np.zeros(len(strucs))
    h_force = np.zeros((total_atoms, 3))
    for _ in range(2):
        eng.compute_flat(natoms, posn, species, cells, head_flags, h_energy, h_force)
    barrier()
    e2e_t = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        eng.compute_flat(natoms, posn, species, cells, head_flags, h_energy, h_force)
        e2e_t.append(time.perf_counter() - t0)
    barrier()
    e2e_step = statistics.mean(e2e_t)

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
        pct = lambda a, q: float(np.percentile(a, q) * 1000.0) if len(a) else None
        serve_out = {
            "offered_req_per_s": args.serve_rate, "seconds": args.serve_seconds, "requests": st["requests"], "repeat_steps": st["repeats"],
            "p50_ms": pct(st["latencies"], 50), "p99_ms": pct(st["latencies"], 99), "atoms_per_s": st["atoms"] / st["wall"],
            "saturated": {"requests": bu["requests"], "atoms_per_s": bu["atoms"] / bu["wall"], "p50_ms": pct(bu["latencies"], 50),
                          "p99_ms": pct(bu["latencies"], 99)},
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
        fp32_peak = 152 * 128 * 2 * pk.get("sm_max_mhz", 2070.0) * 1e6 / 1e12
        ach = work["desc_flops"] / t_desc / 1e12
        roof = {"bound": "fp32", "kernel": "symm_kernel + force_kernel (descriptor and chain-rule triplet passes)",
                "achieved": ach, "peak": fp32_peak, "unit": "TFLOP/s", "frac": ach / fp32_peak, "traffic": None,
                "peak_source": "derived: 152 SMs x 128 FP32 lanes x 2 x sm_max_mhz from MEASURED_PEAKS.json (no FP32 figure is measured)",
                "work": "convention flops P*(30+13 nR) + T*(60+25 nA) = %.4g per step" % work["desc_flops"],
                "kernel_ms": t_desc * 1000.0}
        tfile = os.path.join(REPO, "profiles", "traffic.json")
        if os.path.exists(tfile):
            with open(tfile) as f:
                roof["traffic"] = json.load(f).get(WORKLOAD)
        hbm = pk["hbm_gbs"]
        kernels = {
            "neighbors": {"bound": "hbm", "achieved_gbs": work["nbr_bytes"] / (stage["neighbors"] / 1000) / 1e9, "peak_gbs": hbm,
                          "ms": stage["neighbors"]},
            "gather_energy": {"bound": "hbm", "achieved_gbs": work["gather_bytes"] / (stage["gather_energy"] / 1000) / 1e9,
                              "peak_gbs": hbm, "ms": stage["gather_energy"]},
            "networks": {"bound": "tensor" if bf16_ok else "fp32", "achieved_tflops": work["net_flops"] / (stage["networks"] / 1000) / 1e12,
                         "peak_tflops": pk["bf16_tflops"] if bf16_ok else fp32_peak, "ms": stage["networks"]},
            "descriptors": {"ms": stage["descriptors"]}, "chain_rule": {"ms": stage["chain_rule"]}, "transpose": {"ms": stage["transpose"]},
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
            "ms_per_step": t_step * 1000.0, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16" if bf16_ok else "f32", "data": "synthetic (seeded generator, atomnn_gb300/workloads.py)",
            "config": {"workload": "%s: %d triclinic A/B structures (%d atoms), N log-uniform 16-2048, density 0.05-0.09/A^3, "
                                   "24 G2 + 32 G4 per species, networks 56-64-64-1 tanh, rc 6.5 A" % (WORKLOAD, len(strucs), total_atoms),
                       "structures": len(strucs), "atoms": total_atoms, "path": "batched (one launch sequence per step, CUDA graph)",
                       "networks": "BF16 tensor cores" if bf16_ok else "FP32", "parallelism": "replicas" if ws > 1 else "single GPU",
                       "l2": "flushed between timed steps (512 MiB write, outside the step events)",
                       "launch_shapes": tune_shapes},
            "autotune": tune_report,
            "clocks": clk,
            "e2e": {"value": ws * total_atoms / e2e_step, "unit": "atoms/s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                    "ms_per_step": e2e_step * 1000},
            "gpu_launches": KERNELS_PER_BATCH * args.steps,
            "roofline": roof,
            "kernels": kernels,
            "plain": None if plain_ms is None else {
                "value": total_atoms / (statistics.mean(plain_ms) / 1000), "unit": "atoms/s", "ms_per_step": statistics.mean(plain_ms),
                "desc": "one structure at a time (12 launches per structure), FP32 networks"},
            "batched_fp32": {"value": total_atoms / (statistics.mean(fp32_ms) / 1000), "unit": "atoms/s", "ms_per_step": statistics.mean(fp32_ms)},
            "accuracy_vs_fp64_oracle": acc,
            "serving": serve_out,
        }
        if serve_out is not None and out["plain"] is not None:
            serve_out["saturated_vs_plain"] = serve_out["saturated"]["atoms_per_s"] / out["plain"]["value"]
        if cpu is not None:
            out["cpu_baseline"] = {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")}
        print(json.dumps(out), flush=True)
    eng.close()
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
