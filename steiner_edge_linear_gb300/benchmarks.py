"""Batched and serving workloads of bench.py.

batched: 4096 independent instances of the mixed distribution (n log-uniform
  in [64, 4096], degree {3,4,6,8}, k uniform in [4, 10], weights [1, 1000],
  about 10% group instances; instance i is generated from seed base + i),
  solved by one persistent, graph-captured launch; compared with the plain
  one-instance-at-a-time GPU solve.
serve: Poisson arrivals of instances from the same distribution plus 2%
  large ones (n = 2^17, degree 8, k = 12), admitted by table footprint
  against a 150 GB budget; p50/p99 latency and solves/s per arrival rate,
  and the plain sequential GPU solves/s of the same stream.
"""
from __future__ import annotations

import contextlib
import random
import statistics
import time

import numpy as np

from . import Csr, Server, Solver, StpInstance

MIXED_BASE = 20250301
LARGE = dict(n=1 << 17, degree=8, wmin=1, wmax=1000, k=12)


def shard(count: int, rank: int, world: int) -> range:
    """Contiguous share of `count` instances for `rank` of `world` replicas."""
    per, rem = divmod(count, world)
    start = rank * per + min(rank, rem)
    return range(start, start + per + (1 if rank < rem else 0))


def mixed_instances(indices) -> list[Csr]:
    return [Csr.from_stp(StpInstance.mixed(MIXED_BASE, i)) for i in indices]


def percentile(xs, q):
    xs = sorted(xs)
    if not xs:
        return None
    i = min(len(xs) - 1, max(0, int(round(q / 100.0 * (len(xs) - 1)))))
    return xs[i]


class _NoClock:
    def summary(self) -> dict:
        return {}


@contextlib.contextmanager
def _no_clock():
    yield _NoClock()


def run_batched(args, dist, clock=_no_clock) -> dict:
    """`clock()` is a context manager that samples the GPU clocks while the
    timed steps run; its summary() goes into the line's "clocks"."""
    import torch

    dev = torch.device("cuda", dist.local)
    torch.cuda.set_device(dev)
    idx = shard(args.batch_count * dist.world, dist.rank, dist.world)  # weak scaling: count per GPU
    graphs = mixed_instances(idx)
    stream = torch.cuda.current_stream(dev).cuda_stream
    solver = Solver(dist.local)
    tuning, tuning_mw = solver.batch_autotune_tiles(graphs, stream=stream)
    for _ in range(max(3, args.warmup)):
        costs, st = solver.batch_solve(graphs, stream=stream)
    dist.barrier()
    dev_ms, wall = [], []
    with clock() as clk:
        for _ in range(args.steps):
            t0 = time.perf_counter()
            c2, st = solver.batch_solve(graphs, stream=stream)
            wall.append(time.perf_counter() - t0)
            dev_ms.append(st["total_ms"])
            assert np.array_equal(c2, costs)
    dist.barrier()
    ms = dist.max(statistics.median(dev_ms))
    e2e_s = dist.max(statistics.median(wall))
    # plain one-at-a-time GPU solves on a sample, same instances
    sample = graphs[:256]
    for g in sample[:8]:
        solver.solve(g, check=False, stream=stream)
    t0 = time.perf_counter()
    plain_costs = [solver.solve(g, check=False, stream=stream).cost for g in sample]
    plain_rate = len(sample) / (time.perf_counter() - t0)
    assert plain_costs == [int(x) for x in costs[:len(sample)]]
    solver.close()
    count = len(graphs) * dist.world
    out = {"metric": "solves/s", "value": round(count / (ms / 1000.0), 1), "unit": "solves/s",
           "n_gpus": dist.world, "steps": args.steps, "warmup": max(3, args.warmup),
           "ms_per_step": round(ms, 3), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "int32", "data": "synthetic (seeded mixed distribution)",
           "config": {"workload": f"batched: {len(graphs)} mixed instances per GPU in one persistent launch",
                      "table_bytes": st["table_bytes"], "relax_rows": st["relax_rows"],
                      "autotuned_rcap_by_class": [int(x) for x in tuning],
                      "autotuned_merge_width_by_class": [int(x) for x in tuning_mw]},
           "e2e": {"value": round(count / e2e_s, 1), "unit": "solves/s",
                   "h2d_bytes_per_step": int(sum(4 * (g.n + 1) + 8 * g.arcs + 4 * g.k for g in graphs)),
                   "d2h_bytes_per_step": 8 * len(graphs) + 4},
           "plain_gpu_one_at_a_time": {"value": round(plain_rate, 1), "unit": "solves/s",
                                       "sample": f"first {len(sample)} instances, emv_solve each"},
           "batched_vs_plain": round(count / (ms / 1000.0) / plain_rate, 1),
           "clocks": clk.summary()}
    return out


def run_serve(args, dist, clock=_no_clock) -> dict | None:
    """Poisson request stream against the continuous-batching server; the
    clocks are sampled while the requests are served."""
    import torch

    if dist.rank != 0:
        return None
    torch.cuda.set_device(dist.local)
    rng = random.Random(12345)
    nreq = args.serve_requests
    kinds = ["large" if rng.random() < 0.02 else "mixed" for _ in range(nreq)]
    large_cache = {}
    stream = []
    for i, kd in enumerate(kinds):
        if kd == "large":
            key = len(large_cache) % 4  # four distinct large instances, reused
            if key not in large_cache:
                large_cache[key] = Csr.from_stp(StpInstance.regular(seed=1000 + key, **LARGE))
            stream.append(large_cache[key])
        else:
            stream.append(Csr.from_stp(StpInstance.mixed(MIXED_BASE, i)))
    # plain sequential solves of the whole stream (its mix of small and large
    # requests), after a warm-up; every served cost must equal its plain one
    with Solver(dist.local) as s:
        for g in stream[:64]:
            s.solve(g, check=False)
        t0 = time.perf_counter()
        want = [s.solve(g, check=False).cost for g in stream]
        plain_rate = len(stream) / (time.perf_counter() - t0)
    results = []
    with clock() as clk:
        for rate in [float(x) for x in args.serve_rates.split(",")]:
            with Server(dist.local, hbm_budget_bytes=150 * 10**9, max_slots=4096, large_n=65536) as srv:
                ids = []
                t_start = time.perf_counter()
                next_t = t_start
                for g in stream:
                    next_t += rng.expovariate(rate)
                    delay = next_t - time.perf_counter()
                    if delay > 0:
                        time.sleep(delay)
                    ids.append(srv.submit(g))
                lat = []
                costs = []
                for r in ids:
                    c, l_ms = srv.wait(r, 3600)
                    costs.append(c)
                    lat.append(l_ms)
                wall = time.perf_counter() - t_start
                st = srv.stats()
            assert costs == want, "served costs differ from single solves"
            small = [l for l, kd in zip(lat, kinds) if kd == "mixed"]
            results.append({"arrival_rate": rate, "solves_per_s": round(len(ids) / wall, 1),
                            "p50_ms": round(percentile(lat, 50), 3), "p99_ms": round(percentile(lat, 99), 3),
                            "p99_small_ms": round(percentile(small, 99), 3), "waves": st["waves"],
                            "peak_resident": st["peak_resident"], "peak_bytes": st["peak_bytes"]})
    best = max(r["solves_per_s"] for r in results)
    return {"metric": "solves/s", "value": best, "unit": "solves/s", "n_gpus": 1, "steps": len(results),
            "warmup": 0, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic (mixed distribution + 2% n=2^17 k=12)",
            "config": {"workload": f"serving: {nreq} Poisson arrivals per rate, budget 150 GB"},
            "rates": results,
            "plain_gpu_sequential": {"value": round(plain_rate, 1), "unit": "solves/s",
                                     "sample": f"all {len(stream)} requests of the stream, emv_solve each"},
            "served_vs_plain": round(best / plain_rate, 1),
            "clocks": clk.summary()}
