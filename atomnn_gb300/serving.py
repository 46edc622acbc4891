"""Serving load generator: a Poisson stream of energy+force requests against nnpgpu_serve_*.

Requests draw their structure from a pool of seeded structures (sizes log-uniform over 16-4096
atoms, built as the ``serve`` workload).  A fraction of the requests are MD-style repeat steps of
a resident structure: the same key, positions moved by at most ``max_disp`` per component from
that key's previous step, so the engine can refresh its resident neighbour list (skin) instead
of rebuilding it.  Latency is measured by the engine from submission to completion.
"""
import threading
import time

import numpy as np

from . import workloads as W


def make_pool(n=256, seed=4242, hi=4096):
    rng = np.random.default_rng(seed)
    sizes = [int(round(np.exp(rng.uniform(np.log(16), np.log(hi))))) for _ in range(n)]
    return W.make_structures("serve", seed=seed + 1, count=n, sizes=sizes)


def run_stream(eng, pool, rate, duration, repeat_frac=0.2, n_resident=32, max_disp=0.02, seed=7, burst=False):
    """Submit requests (Poisson arrivals at ``rate`` per second for ``duration`` seconds, or all
    at once when ``burst``) and wait for all of them.  Returns a dict of latencies (s), served
    atoms, requests, wall time and the number of repeat steps."""
    rng = np.random.default_rng(seed)
    n_req = int(rate * duration)
    arrivals = np.zeros(n_req) if burst else np.cumsum(rng.exponential(1.0 / rate, size=n_req))
    resident = {}  # key -> current positions
    outstanding = {}
    lock = threading.Lock()
    done = []
    finished = threading.Event()

    def poller():
        while True:
            with lock:
                items = list(outstanding.items())
            for rid, natoms in items:
                r = eng.poll(rid, natoms)
                if r is not None:
                    with lock:
                        del outstanding[rid]
                    done.append((natoms, r[2]))
            if finished.is_set():
                with lock:
                    if not outstanding:
                        return
            time.sleep(0.0002)

    th = threading.Thread(target=poller, daemon=True)
    th.start()
    t0 = time.perf_counter()
    repeats = 0
    for k in range(n_req):
        wait = t0 + arrivals[k] - time.perf_counter()
        if wait > 0:
            time.sleep(wait)
        if rng.random() < repeat_frac:
            key = int(rng.integers(n_resident))
            base = pool[key % len(pool)]
            if key in resident:
                posn = resident[key] + rng.uniform(-max_disp, max_disp, size=resident[key].shape)
                repeats += 1
            else:
                posn = base.posn.copy()
            resident[key] = posn
            s = W.Structure(posn=posn, species=base.species, cell=base.cell)
        else:
            key = -1
            s = pool[int(rng.integers(len(pool)))]
        rid = eng.submit(s, key=key)
        with lock:
            outstanding[rid] = s.natoms
    finished.set()
    th.join(timeout=600)
    wall = time.perf_counter() - t0
    lat = np.array([x[1] for x in done])
    atoms = int(sum(x[0] for x in done))
    return dict(latencies=lat, atoms=atoms, requests=len(done), wall=wall, repeats=repeats)
