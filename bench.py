#!/usr/bin/env python3
"""Benchmark of the GB300 EMV Steiner solver.

Default workload (one JSON line): the single large plain solve -- random
20-regular graph, n = 100000, m = 10^6, weights uniform in [1, 100], k = 12
terminals, seed 123456789 (table 2^12 x 10^5 int32 = 1.64 GB).  A step is one
complete solve (table init, k level-1 closures, 11 merge levels, all
relaxations, cost read) with the CSR already resident in HBM; the working set
(1.7 GB) is larger than L2, so no flush is needed between steps.

  value  solves/s with device-resident inputs (CUDA events, max over ranks)
  e2e    solves/s through the public C ABI (emv_solve) from pinned host CSR,
         host->device copies and the cost read inside the timed region
  roofline  the dominant kernel against the measured HBM copy bandwidth
  cpu_baseline  the reference's own emv_kernel (oracle/_ref) on the box's
         host cores, on a bounded sample of the same workload
  batched, serve  the batching and serving paths measured in the same
         run: 4096 mixed instances in one persistent launch, and a Poisson
         request stream through the continuous-batching server, each against
         plain one-instance-at-a-time GPU solves
  roofline_scale  two timed solves of the n = 2^20, k = 14 instance (64 GiB
         table) with their phases and the relaxation's roofline
         (--no-extras leaves batched, serve and roofline_scale out)

Other workloads alone: --workload batched, --workload serve, --workload
roofline (n = 2^20, k = 14).  --impl reference times the reference instead
(its process never loads the solver's library: the instance comes from the
stand-alone generator executable).
Multi-GPU (torchrun): independent replicas, one per rank.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SINGLE = dict(n=100000, degree=20, wmin=1, wmax=100, k=12, seed=123456789)
SINGLE_NAME = "single large plain solve: random 20-regular n=100000 m=1e6 w=[1,100] k=12 seed=123456789"
ROOFLINE = dict(n=1 << 20, degree=10, wmin=1, wmax=1024, k=14, seed=123456789)
ROOFLINE_NAME = "roofline-scale solve: random 10-regular n=2^20 m=5*2^20 w=[1,1024] k=14 seed=123456789 (64 GiB table)"
PROFILES = os.path.join(ROOT, "profiles")


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    p.add_argument("--workload", choices=["single", "roofline", "batched", "serve"], default="single")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-extras", action="store_true", help="single workload without the batched/serve sub-objects")
    p.add_argument("--batch-count", type=int, default=4096)
    p.add_argument("--serve-rates", type=str, default="2000,8000")
    p.add_argument("--serve-requests", type=int, default=4000)
    return p.parse_args()


# --------------------------------------------------------------- plumbing

class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            import torch
            backend = "nccl" if torch.cuda.is_available() else "gloo"
            if backend == "nccl":
                torch.cuda.set_device(self.local)
            dist.init_process_group(backend=backend)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x: float) -> float:
        if not self.pg:
            return x
        import torch
        dev = torch.device("cuda", self.local) if torch.cuda.is_available() else torch.device("cpu")
        t = torch.tensor([x], dtype=torch.float64, device=dev)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while running."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            if self.thread:
                self.thread.join(timeout=2)

    def summary(self) -> dict:
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = max(smax, float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks() -> dict:
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def profile_traffic(name: str):
    """DRAM bytes per launch from a committed ncu summary (profiles/<name>.json), or None."""
    path = os.path.join(PROFILES, name + ".json")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        return json.load(f)


# ------------------------------------------------------------- workloads

def merge_bytes(n: int, k: int) -> float:
    """12 bytes per (X, Y, v) triple, Y a proper non-empty subset of X (reader-el.c:2294 accounting)."""
    return 12.0 * n * (3 ** k - 2 ** (k + 1) + 1)


def relax_bytes_per_row(n: int, m: int) -> float:
    """One read of row_ptr/col/w and one read + one write of the row, int32."""
    return 12.0 * n + 16.0 * m + 4.0 * (n + 1)


GEN_PATH = os.path.join(ROOT, "steiner_edge_linear_gb300", "lib", "emv-gen")


def write_instance(path: str, *args) -> None:
    """Writes a generated instance as STP with the stand-alone generator
    executable (the same generator as the library, without loading the
    library), e.g. write_instance(p, "regular", n, d, wmin, wmax, k, seed)."""
    if not os.path.exists(GEN_PATH):
        from steiner_edge_linear_gb300 import build as _b  # compiles only; loads nothing
        _b.build()
    subprocess.run([GEN_PATH] + [str(a) for a in args] + [path], check=True, stdout=subprocess.DEVNULL)


def _single_args(cfg: dict) -> list:
    return ["regular", cfg["n"], cfg["degree"], cfg["wmin"], cfg["wmax"], cfg["k"], cfg["seed"]]


def cpu_reference_runs(steps: int, warmup: int, threads: int | None = None) -> dict:
    """Times complete solves of the benchmark instance with the reference's own
    emv_kernel (oracle/_ref, built from the reference source with -O3 and
    OpenMP) on the host cores; falls back to the oracle's C restatement where
    the reference leg is not built.  Warm-up runs use the first 8 terminals.
    Nothing here loads the solver's library: the instance comes from the
    stand-alone generator."""
    import oracle

    oracle.build(reference=True)
    threads = threads or os.cpu_count() or 1
    runs, cost = [], None
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "single.stp")
        write_instance(path, *_single_args(SINGLE))
        kind = "reference" if oracle.reference_available() else "port"
        csr = None if kind == "reference" else oracle.read_stp_csr(path)
        for i in range(warmup + steps):
            kp = 8 if i < warmup else 0
            if kind == "reference":
                r = oracle.ref_emv(path, kprefix=kp, threads=threads)
                t = (r["zero_ms"] + r["kernel_ms"]) / 1000.0
                c = r["cost"]
            else:
                n, row, col, w, terms = csr
                t0 = time.perf_counter()
                _, c = oracle.emv_table(n, row, col, w, terms[:kp] if kp else terms, threads=threads)
                t = time.perf_counter() - t0
            if i >= warmup:
                runs.append(t)
                cost = c
    return {"kind": kind, "threads": threads, "runs_s": runs, "cost": cost}


def reference_throughput(indices, base_seed: int) -> dict:
    """The reference's emv_kernel (oracle/_ref) in throughput mode: one
    single-threaded process per host core over a sample of the batched
    distribution (instances written by the stand-alone generator)."""
    import oracle
    from concurrent.futures import ThreadPoolExecutor

    oracle.build(reference=True)
    cores = os.cpu_count() or 1
    with tempfile.TemporaryDirectory() as tmp:
        paths = []
        for i in indices:
            p = os.path.join(tmp, f"i{i}.stp")
            write_instance(p, "mixed", base_seed, i)
            paths.append(p)
        kind = "reference" if oracle.reference_available() else "port"

        def one(p):
            if kind == "reference":
                oracle.ref_emv(p, threads=1)
            else:
                n, row, col, w, terms = oracle.read_stp_csr(p)
                oracle.emv_table(n, row, col, w, terms, threads=1)

        t0 = time.perf_counter()
        with ThreadPoolExecutor(max_workers=cores) as ex:
            done = sum(1 for _ in ex.map(one, paths))
        wall = time.perf_counter() - t0
    return {"value": round(done / wall, 2), "unit": "solves/s", "cores": cores, "kind": kind,
            "sample": f"{done} instances of the same distribution, one single-threaded process per core"}


def run_single(args, dist: Dist, cfg: dict = SINGLE, cfg_name: str = SINGLE_NAME, with_e2e: bool = True) -> dict:
    import numpy as np
    import torch

    import steiner_edge_linear_gb300 as E

    E.build()
    dev = torch.device("cuda", dist.local)
    torch.cuda.set_device(dev)
    inst = E.StpInstance.regular(**cfg)
    csr = E.Csr.from_stp(inst)
    n, m, k = csr.n, inst.m, csr.k
    row = torch.from_numpy(csr.row_ptr).to(dev)
    col = torch.from_numpy(csr.col).to(dev)
    w = torch.from_numpy(csr.w).to(dev)
    stream = torch.cuda.current_stream(dev)
    sp = stream.cuda_stream
    solver = E.Solver(dist.local)

    def step():
        return solver.solve_dev(n, csr.arcs, row.data_ptr(), col.data_ptr(), w.data_ptr(), csr.terminals,
                                stream=sp)

    for _ in range(max(3, args.warmup)):
        r0 = step()
    cost = r0.cost
    timings = []
    dist.barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dist.local) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            r = step()
            timings.append(r.timing)
            assert r.cost == cost
        ev1.record(stream)
        torch.cuda.synchronize()
    dist.barrier()
    ms = ev0.elapsed_time(ev1)
    ms = dist.max(ms)
    value = args.steps * dist.world / (ms / 1000.0)

    # e2e through emv_solve with pinned host CSR: H2D of the graph + D2H of the cost per step;
    # the default call (admission checks on), and the same call without the host-side checks
    pin = [torch.from_numpy(a).pin_memory() for a in (csr.row_ptr, csr.col, csr.w)]
    hcsr = E.Csr(n, pin[0].numpy(), pin[1].numpy(), pin[2].numpy(), csr.terminals)
    e2e = {}
    for check in ((True, False) if with_e2e else ()):
        for _ in range(2):
            solver.solve(hcsr, check=check, stream=sp)
        dist.barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            r = solver.solve(hcsr, check=check, stream=sp)
            assert r.cost == cost
        torch.cuda.synchronize()
        e2e[check] = dist.max(time.perf_counter() - t0)
    e2e_s = e2e.get(True)
    h2d = 4 * (n + 1) + 8 * csr.arcs + 4 * k
    d2h = 4 + 16

    # roofline of the dominant kernel (by device time)
    merge_ms = statistics.median(t["merge_ms"] for t in timings)
    relax_ms = statistics.median(t["relax_ms"] + t["level1_ms"] for t in timings)
    kernel_ms = statistics.median(t["kernel_ms"] for t in timings)
    launches = int(statistics.median(t["launches"] for t in timings))
    rows = (1 << k) - 1
    relax_launches = int(statistics.median(t["relax_launches"] for t in timings))
    peak = measured_peaks()
    if relax_ms >= merge_ms:
        kname, kms, launches_k = "k_relax", relax_ms, relax_launches
        alg = rows * relax_bytes_per_row(n, m)
        unit_note = f"12n+16m+4(n+1) bytes per row closure x {rows} rows"
    else:
        kname, kms, launches_k = ("k_merge_stream16" if cfg is SINGLE else "merge"), merge_ms, k - 1
        alg = merge_bytes(n, k)
        unit_note = "12 bytes per (X,Y,v) triple x n(3^k-2^(k+1)+1)"
    achieved = alg / (kms / 1000.0) / 1e9
    prof = profile_traffic(f"{kname}_single") if cfg is SINGLE else None
    traffic = None
    if prof and "dram_bytes_per_launch" in prof:
        traffic = float(prof["dram_bytes_per_launch"])
    elif prof and "dram_bytes_per_solve" in prof:
        traffic = prof["dram_bytes_per_solve"] / launches_k
    roofline = {"bound": "hbm", "kernel": kname, "achieved": round(achieved, 1), "peak": peak["hbm_gbs"],
                "unit": "GB/s", "frac": round(achieved / peak["hbm_gbs"], 4),
                "traffic": traffic, "algorithmic_bytes_per_launch": alg / launches_k,
                "avg_launch_ms": kms / launches_k, "launches_per_solve": launches_k,
                "peak_source": f"{peak['source']} hbm_gbs (copy)", "work_unit": unit_note}

    out = {"metric": "solves/s", "value": round(value, 4), "unit": "solves/s", "n_gpus": dist.world,
           "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": round(ms / args.steps, 3),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
           "data": "synthetic (seeded generator, configuration-model random regular graph)",
           "config": single_config(cfg, cfg_name, dist.world),
           "cost": cost,
           "e2e": ({"value": round(args.steps * dist.world / e2e_s, 4), "unit": "solves/s",
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "call": "emv_solve, default flags (host admission checks on)",
                    "without_host_checks": round(args.steps * dist.world / e2e[False], 4)} if with_e2e else None),
           "gpu_launches": launches * args.steps,
           "phases_ms": {"merge": round(merge_ms, 3), "relax_incl_level1": round(relax_ms, 3),
                         "kernel": round(kernel_ms, 3)},
           "relax_sweeps_per_solve": int(statistics.median(t["relax_sweeps"] for t in timings)),
           # levels (of k - 1 relaxed, k - 2 merged from level 3) that ran on 16-bit values; the table is int32
           "levels_16bit": {"relax": timings[-1]["relax16_levels"], "merge": timings[-1]["merge16_levels"]},
           "gcell_per_s": round(((1 << k) * n) / (kernel_ms / 1000.0) / 1e9, 3),
           "merge_gbs_algorithmic": round(merge_bytes(n, k) / (merge_ms / 1000.0) / 1e9, 1),
           "relax_gbs_algorithmic": round(rows * relax_bytes_per_row(n, m) / (relax_ms / 1000.0) / 1e9, 1),
           "roofline": roofline,
           "clocks": clk.summary()}
    solver.close()
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline and cfg is SINGLE:
        c = cpu_reference_runs(steps=1, warmup=0)
        t = statistics.median(c["runs_s"])
        out["cpu_baseline"] = {"value": round(1.0 / t, 5), "unit": "solves/s", "cores": c["threads"],
                               "kind": c["kind"], "cost": c["cost"],
                               "sample": (f"one complete solve of the same instance (all 4096 rows, {t:.2f} s) by the "
                                          f"reference's emv_kernel, -O3, {c['threads']} OpenMP threads")}
    return out


def extras(args, dist) -> dict:
    """The batched and serving workloads of the default line, each with its
    own clocks: batched and served solves/s against plain
    one-instance-at-a-time GPU solves (config: 4096 mixed instances; a
    Poisson stream at one saturating arrival rate)."""
    from steiner_edge_linear_gb300 import benchmarks

    out = {}
    b = benchmarks.run_batched(args, dist, clock=lambda: ClockSampler(dist.local))
    out["batched"] = {k: b[k] for k in ("value", "unit", "ms_per_step", "e2e", "plain_gpu_one_at_a_time",
                                        "batched_vs_plain", "clocks")}
    out["batched"]["workload"] = b["config"]["workload"]
    out["batched"]["autotuned"] = {k: b["config"][k] for k in b["config"] if k != "workload"}
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        out["batched"]["cpu_baseline"] = reference_throughput(range(0, 256), benchmarks.MIXED_BASE)
    # the roofline-scale solve (n = 2^20, k = 14, 64 GiB table): two timed solves
    short = argparse.Namespace(**vars(args))
    short.steps, short.warmup = 2, 1
    rf = run_single(short, dist, ROOFLINE, ROOFLINE_NAME, with_e2e=False)
    if rf is not None:
        out["roofline_scale"] = {k: rf[k] for k in ("value", "unit", "ms_per_step", "cost", "phases_ms",
                                                    "relax_sweeps_per_solve", "levels_16bit", "relax_gbs_algorithmic",
                                                    "merge_gbs_algorithmic", "roofline", "clocks")}
        out["roofline_scale"]["workload"] = ROOFLINE_NAME
    one_rate = argparse.Namespace(**vars(args))
    one_rate.serve_rates = args.serve_rates.split(",")[-1]  # the saturating rate only
    sv = benchmarks.run_serve(one_rate, dist, clock=lambda: ClockSampler(dist.local))
    if sv is not None:
        out["serve"] = {k: sv[k] for k in ("value", "unit", "rates", "plain_gpu_sequential", "served_vs_plain",
                                           "clocks")}
        out["serve"]["workload"] = sv["config"]["workload"]
    return out


def single_config(cfg: dict, name: str, world: int) -> dict:
    """The `config` object of a single-solve line (both arms)."""
    n, k = cfg["n"], cfg["k"]
    return {"workload": name, "n": n, "m": n * cfg["degree"] // 2, "k": k, "table_bytes": 4 * n << k,
            "parallelism": f"replicas x{world}",
            "l2": f"no flush: {4 * (n << k) / 1e9:.1f} GB table per step > 129 MB L2"}


def run_reference(args, dist: Dist) -> dict | None:
    """The reference arm: each timed step is one complete solve of the benchmark
    instance by the reference's own emv_kernel on all host cores (about 20 s on
    16 Neoverse-V2 cores); warm-up steps solve the first 8 terminals only."""
    if dist.rank != 0:
        return None
    c = cpu_reference_runs(steps=args.steps, warmup=args.warmup)
    t = statistics.median(c["runs_s"])
    value = 1.0 / t
    return {"metric": "solves/s", "value": round(value, 5), "unit": "solves/s", "n_gpus": dist.world,
            "cost": c["cost"],
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1000.0 * t, 1), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int64",
            "data": "synthetic (seeded generator, configuration-model random regular graph)",
            "impl": "reference",
            "config": single_config(SINGLE, SINGLE_NAME, dist.world),
            "cpu_baseline": {"value": round(value, 5), "unit": "solves/s", "cores": c["threads"], "kind": c["kind"],
                             "sample": "complete solves of the benchmark instance, median of the timed steps"},
            "e2e": {"value": round(value, 5), "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    args = parse_args()
    dist = Dist()
    try:
        if args.impl == "reference":
            out = run_reference(args, dist)
        elif args.workload == "single":
            out = run_single(args, dist)
            if not args.no_extras:
                ex = extras(args, dist)
                if out is not None:
                    out.update(ex)
        elif args.workload == "roofline":
            out = run_single(args, dist, ROOFLINE, ROOFLINE_NAME)
        elif args.workload == "batched":
            from steiner_edge_linear_gb300 import benchmarks
            out = benchmarks.run_batched(args, dist, clock=lambda: ClockSampler(dist.local))
            if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
                out["cpu_baseline"] = reference_throughput(range(0, 256), benchmarks.MIXED_BASE)
        else:
            from steiner_edge_linear_gb300 import benchmarks
            out = benchmarks.run_serve(args, dist, clock=lambda: ClockSampler(dist.local))
        if out is not None and dist.rank == 0:
            print(json.dumps(out), flush=True)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
