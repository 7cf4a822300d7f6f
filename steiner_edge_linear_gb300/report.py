"""Experiment runs of the command line and their result table.

A Python 3.12 replacement of the run-and-parse part of the reference's
experiments/report.py (its gnuplot plotting is not reproduced): it generates
instances (the reference calls graph-gen/gen-unique; here the solver's own
generators, emv_gen_regular / _powlaw / _clique, which use a different PRNG),
runs ``reader-el-gpu -el`` on each, parses every output line with the
reference's patterns (report.py:61-127) and writes one whitespace-separated row
per run with report.py's columns (report.py:180-205), followed by roofline
columns: merge and relaxation time and their algorithmic bytes per second
against the measured HBM copy bandwidth.

    python -m steiner_edge_linear_gb300.report --run -n 1024 4096 -d 4 -k 6 8 -o runs/
    python -m steiner_edge_linear_gb300.report --parse runs/*.out
"""
from __future__ import annotations

import argparse
import json
import os
import re
import subprocess
import sys
from typing import Optional, Sequence

from .verify import parse_output

RE_SEED = re.compile(r"random seed = (.*)", re.M | re.I)
RE_ROOT = re.compile(r"root build:(.*)\[zero:(.*)ms\] \[pos:(.*)ms\] \[adj:(.*)ms\] \[term:(.*)ms\] done. \[(.*)ms\] "
                     r"{peak:(.*)GiB} {curr:(.*)GiB}", re.M)
RE_TOTAL = re.compile(r"grand total \[(.*)ms\] {peak:(.*)GiB}(.*)", re.M)
RE_HOST = re.compile(r"host:(.*)", re.M)
RE_BUILD = re.compile(r"build:(.*), (.*)", re.M)
RE_COMPILER = re.compile(r"compiler:(.*)", re.M)

COLUMNS = ["n", "m", "k", "in_cost", "seed", "in_peak", "in_curr",
           "r_zero", "r_pos", "r_adj", "r_term", "r_total", "r_peak", "r_curr",
           "e_zero", "e_kernel", "e_kernel_gibs", "e_total", "e_cost", "e_peak", "e_curr",
           "g_total", "g_peak",
           "merge_ms", "merge_gbs", "merge_frac", "relax_ms", "relax_gbs", "relax_frac", "sweeps"]


def merge_bytes(n: int, k: int) -> float:
    """12 bytes per (X, Y, v) triple: read d[Y][v], d[X\\Y][v], update d[X][v] (R:2068-2088)."""
    return 12.0 * n * (3 ** k - 2 ** (k + 1) + 1)


def relax_bytes(n: int, m: int, k: int) -> float:
    """One read of row/col/w and a read and a write of d per row closure, 2^k - 1 rows."""
    return (2 ** k - 1) * (12.0 * n + 16.0 * m + 4.0 * (n + 1))


def hbm_peak_gbs() -> Optional[float]:
    here = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    path = os.path.join(here, "MEASURED_PEAKS.json")
    try:
        return float(json.load(open(path))["hbm_gbs"])
    except (OSError, KeyError, ValueError):
        return None


def parse_run(text: str, list_solution: bool = False) -> dict:
    """All fields of one run's stdout, report.py's names plus the roofline columns."""
    f = parse_output(text, list_solution)
    row: dict = {c: None for c in COLUMNS}
    row.update(n=f.get("n"), m=f.get("m"), k=f.get("k"), in_cost=f.get("in_cost"), in_peak=f.get("in_peak"),
               in_curr=f.get("in_curr"), e_zero=f.get("zero_ms"), e_kernel=f.get("kernel_ms"),
               e_kernel_gibs=f.get("kernel_gibs"), e_total=f.get("total_ms"), e_cost=f.get("el_cost"),
               e_peak=f.get("el_peak"), e_curr=f.get("el_curr"), merge_ms=f.get("merge_ms"),
               relax_ms=f.get("relax_ms"), sweeps=f.get("relax_sweeps"))
    for line in text.splitlines():
        if line.startswith("random seed"):
            row["seed"] = int(RE_SEED.search(line).group(1))
        elif line.startswith("root build"):
            mt = RE_ROOT.search(line)
            if mt:
                vals = [float(x) for x in mt.groups()[1:8]]
                for c, v in zip(("r_zero", "r_pos", "r_adj", "r_term", "r_total", "r_peak", "r_curr"), vals):
                    row[c] = v
        elif line.startswith("grand total"):
            mt = RE_TOTAL.search(line)
            row["g_total"], row["g_peak"] = float(mt.group(1)), float(mt.group(2))
        elif line.startswith("host"):
            row["host"] = RE_HOST.search(line).group(1).strip()
        elif line.startswith("build"):
            mt = RE_BUILD.search(line)
            row["build"] = mt.group(1).strip() + ", " + mt.group(2).strip()
        elif line.startswith("compiler"):
            row["compiler"] = RE_COMPILER.search(line).group(1).strip()
    peak = hbm_peak_gbs()
    n, m, k = row["n"], row["m"], row["k"]
    if row["merge_ms"] and n and k:
        row["merge_gbs"] = merge_bytes(n, k) / (row["merge_ms"] * 1e6)
        row["merge_frac"] = row["merge_gbs"] / peak if peak else None
    if row["relax_ms"] and n and k:
        relax_all = row["relax_ms"] + (f.get("level1_ms") or 0.0)
        row["relax_gbs"] = relax_bytes(n, m, k) / (relax_all * 1e6)
        row["relax_frac"] = row["relax_gbs"] / peak if peak else None
    return row


def format_row(row: dict) -> str:
    out = []
    for c in COLUMNS:
        v = row.get(c)
        out.append("-" if v is None else (f"{v:.4f}" if isinstance(v, float) else str(v)))
    return " ".join(out)


def write_table(rows: Sequence[dict], path: Optional[str]) -> str:
    text = "# " + " ".join(COLUMNS) + "\n" + "".join(format_row(r) + "\n" for r in rows)
    if path:
        with open(path, "w") as fh:
            fh.write(text)
    return text


def run_experiments(out_dir: str, graph_type: str, nodes: Sequence[int], degrees: Sequence[int],
                    terms: Sequence[int], ew: int, seed: int, repeats: int, exe: Optional[str] = None,
                    list_solution: bool = False, alpha: float = -0.5, classes: int = 10) -> list[dict]:
    """report.py's run loop (generate, solve, parse) over n x d x k x repeats."""
    from . import CLI_PATH, StpInstance
    exe = exe or CLI_PATH
    os.makedirs(out_dir, exist_ok=True)
    rows = []
    for n in nodes:
        for d in degrees:
            for k in terms:
                for r in range(repeats):
                    s = seed + r
                    if graph_type == "regular":
                        g = StpInstance.regular(n, d, 1, ew, k, s)
                    elif graph_type == "powlaw":
                        g = StpInstance.powlaw(n, d, alpha, classes, 1, ew, k, s)
                    elif graph_type == "clique":
                        g = StpInstance.clique(n, 1, ew, k, s)
                    else:
                        raise ValueError(f"unknown graph type {graph_type}")
                    base = os.path.join(out_dir, f"{graph_type}-n{n}-d{d}-k{k}-s{s}")
                    g.write(base + ".stp")
                    cmd = [exe, "-in", base + ".stp", "-seed", str(s), "-el"] + (["-list"] if list_solution else [])
                    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
                    with open(base + ".out", "w") as fh:
                        fh.write(proc.stdout)
                    if proc.returncode != 0:
                        raise RuntimeError(f"{' '.join(cmd)} failed:\n{proc.stdout[-2000:]}")
                    row = parse_run(proc.stdout, list_solution)
                    row.update(g_type=graph_type, g_n=n, g_m=g.m, g_k=k, g_seed=s)
                    rows.append(row)
    return rows


def main(argv: Optional[Sequence[str]] = None) -> int:
    p = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    p.add_argument("--run", action="store_true", help="generate instances and run the command line")
    p.add_argument("--parse", nargs="*", default=[], help="outputs of earlier runs to tabulate")
    p.add_argument("-o", "--out-dir", default="report")
    p.add_argument("-gt", "--graph-type", default="regular", choices=["regular", "powlaw", "clique"])
    p.add_argument("-n", "--nodes", nargs="+", type=int, default=[1024])
    p.add_argument("-d", "--deg", nargs="+", type=int, default=[20])
    p.add_argument("-k", "--terminals", nargs="+", type=int, default=[10])
    p.add_argument("-ew", "--edge-weight", type=int, default=10000)
    p.add_argument("-al", "--alpha", type=float, default=-0.5)
    p.add_argument("-r", "--repeats", type=int, default=1)
    p.add_argument("-s", "--seed", type=int, default=123456789)
    p.add_argument("-e", "--exe", default=None)
    p.add_argument("-list", "--list-solution", action="store_true")
    p.add_argument("--table", default=None, help="write the rows here (default <out-dir>/report.dat)")
    a = p.parse_args(argv)
    rows = []
    if a.run:
        rows += run_experiments(a.out_dir, a.graph_type, a.nodes, a.deg, a.terminals, a.edge_weight, a.seed,
                                a.repeats, a.exe, a.list_solution, a.alpha)
    for path in a.parse:
        rows.append(parse_run(open(path).read(), a.list_solution))
    if not rows:
        p.error("nothing to do: give --run or --parse")
    table = a.table or (os.path.join(a.out_dir, "report.dat") if a.run else None)
    sys.stdout.write(write_table(rows, table))
    return 0


if __name__ == "__main__":
    sys.exit(main())
