"""Correctness runs of the command line on STP instances.

A Python 3.12 replacement of the reference's experiments/verify.py (which uses
``re.L`` on str patterns and so no longer runs).  For every instance it runs
``reader-el-gpu -in <file> -el [-list]``, fails on ``ERROR``/``assert`` in the
output (verify.py:219-226), parses the ``input``/``erickson``/``terminals``/
``solution`` lines with the reference's own patterns (verify.py:126-147) and
compares the instance's cost line with the computed cost (verify.py:228-230).
With ``--list`` the tree check is stricter than verify.py:104-118 (which only
asks the listed edges to connect the terminals): every listed pair must be an
input edge, the pairs must form a tree that spans all terminals, and the sum of
their weights (the lightest parallel edge of each pair) must equal the cost.

    python -m steiner_edge_linear_gb300.verify --testset DIR     # DIR/*/*.stp
    python -m steiner_edge_linear_gb300.verify a.stp b.stp --list
"""
from __future__ import annotations

import argparse
import glob
import os
import re
import subprocess
import sys
import time
from typing import Optional, Sequence

# The reference's line patterns (experiments/verify.py:126-147), without re.L.
RE_INPUT = re.compile(r"(.*)n = (.*), m = (.*), k = (.*), cost = (.*) \[(.*)ms\] {peak:(.*)GiB} {curr:(.*)GiB}",
                      re.M | re.I)
RE_ERICKSON = re.compile(r"erickson: \[zero:(.*)ms\] \[kernel:(.*)ms (.*)GiB/s\] done. \[(.*)ms\] \[cost:(.*)] "
                         r"{peak:(.*)GiB} {curr:(.*)GiB}", re.M)
RE_ERICKSON_LIST = re.compile(r"erickson: \[zero:(.*)ms\] \[kernel:(.*)ms (.*)GiB/s\] \[traceback: (.*)ms\] done. "
                              r"\[(.*)ms\] \[cost:(.*)] {peak:(.*)GiB} {curr:(.*)GiB}", re.M)
# k == 2 prints the path line without the zero field (reader-el.c:2171)
RE_ERICKSON_K2 = re.compile(r"erickson: \[kernel:(.*)ms (.*)GiB/s\] done. \[(.*)ms\] \[cost:(.*)] "
                            r"{peak:(.*)GiB} {curr:(.*)GiB}", re.M)
RE_TERMINALS = re.compile(r"terminals:(.*)", re.M)
RE_SOLUTION = re.compile(r'"([^"]*)"')
# the solver's own extra line
RE_GPU = re.compile(r"gpu: \[level1: (.*) ms\] \[merge: (.*) ms (.*) GB/s\] \[relax: (.*) ms (.*) GB/s (\d+) sweeps\] "
                    r"\[(.*) Gcell/s\] \[launches: (\d+)\]")


def parse_output(text: str, list_solution: bool = False) -> dict:
    """Fields of one run's stdout (the keys follow verify.py's variable names)."""
    out: dict = {}
    for line in text.splitlines():
        if line.startswith("input"):
            mt = RE_INPUT.search(line)
            if not mt:
                raise ValueError(f"unparsable input line: {line!r}")
            n, m, k, cost, ms, peak, curr = (g.strip() for g in mt.groups()[1:8])
            out.update(n=int(n), m=int(m), k=int(k), in_cost=int(cost), input_ms=float(ms), in_peak=float(peak),
                       in_curr=float(curr))
        elif line.startswith("erickson"):
            mt = (RE_ERICKSON_LIST if list_solution else RE_ERICKSON).search(line)
            if mt:
                g = [x.strip() for x in mt.groups()]
                if list_solution:
                    zero, kernel, gibs, tb, total, cost, peak, curr = g
                    out["traceback_ms"] = float(tb)
                else:
                    zero, kernel, gibs, total, cost, peak, curr = g
                out["zero_ms"] = float(zero)
            else:
                mt = RE_ERICKSON_K2.search(line)
                if not mt:
                    raise ValueError(f"unparsable erickson line: {line!r}")
                kernel, gibs, total, cost, peak, curr = (x.strip() for x in mt.groups())
            out.update(kernel_ms=float(kernel), kernel_gibs=float(gibs), total_ms=float(total), el_cost=int(cost),
                       el_peak=float(peak), el_curr=float(curr))
        elif line.startswith("solution"):
            out["solution"] = [tuple(int(x) for x in p.split()) for p in RE_SOLUTION.findall(line)]
        elif line.startswith("terminals"):
            out["terminals"] = [int(x) for x in RE_TERMINALS.search(line).group(1).split()]
        elif line.startswith("gpu:"):
            mt = RE_GPU.search(line)
            if mt:
                l1, mg, mgbs, rx, rxgbs, sw, gc, la = mt.groups()
                out.update(level1_ms=float(l1), merge_ms=float(mg), merge_gbs=float(mgbs), relax_ms=float(rx),
                           relax_gbs=float(rxgbs), relax_sweeps=int(sw), gcell_s=float(gc), launches=int(la))
    return out


def check_solution(edges, terminals: Sequence[int], pairs: Sequence[tuple], cost: int) -> Optional[str]:
    """None when `pairs` (1-based vertex pairs) is a tree of input edges that
    spans `terminals` (1-based) with weight `cost`, else the reason.  `edges`
    is the instance's (m, 3) 0-based u, v, w list."""
    lightest: dict = {}
    for u, v, w in edges:
        key = (min(int(u), int(v)), max(int(u), int(v)))
        lightest[key] = min(int(w), lightest.get(key, int(w)))
    parent: dict = {}

    def find(x):
        while parent.setdefault(x, x) != x:
            parent[x] = parent[parent[x]]
            x = parent[x]
        return x

    weight = 0
    for a, b in pairs:
        u, v = a - 1, b - 1
        key = (min(u, v), max(u, v))
        if key not in lightest:
            return f"listed pair {a} {b} is not an input edge"
        ru, rv = find(u), find(v)
        if ru == rv:
            return f"listed pair {a} {b} closes a cycle"
        parent[ru] = rv
        weight += lightest[key]
    terms = [t - 1 for t in terminals]
    if len(set(terms)) > 1:
        if any(t not in parent for t in terms):
            return "a terminal is not covered"
        roots = {find(t) for t in terms}
        if len(roots) != 1:
            return "the listed edges do not connect the terminals"
        if len({find(x) for x in parent}) != 1:
            return "the listed edges are not one tree"
    if weight != cost:
        return f"tree weight {weight} differs from cost {cost}"
    return None


def default_exe() -> str:
    from . import CLI_PATH
    return CLI_PATH


def verify_file(path: str, exe: str, arg_cmd: str = "el", list_solution: bool = False,
                extra: Sequence[str] = ()) -> tuple[bool, str, dict]:
    """Runs the command line on one instance; returns (passed, message, fields)."""
    cmd = [exe, "-in", path, f"-{arg_cmd}"] + (["-list"] if list_solution else []) + list(extra)
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    text = proc.stdout
    if "ERROR" in text:
        return False, "error: testing failed", {}
    if "assert" in text or "Assert" in text:
        return False, "assert: testing failed", {}
    if proc.returncode != 0:
        return False, f"exit status {proc.returncode}", {}
    try:
        f = parse_output(text, list_solution)
    except ValueError as e:
        return False, str(e), {}
    if "el_cost" not in f:
        return False, "no erickson line", f
    if f.get("in_cost", -1) != -1 and f["in_cost"] != f["el_cost"]:
        return False, f"fail inCost = {f['in_cost']} elCost = {f['el_cost']}", f
    if list_solution:
        if "-bin" in extra:
            from . import BinContainer
            idx = int(extra[extra.index("-index") + 1]) if "-index" in extra else 0
            with BinContainer(path) as b:
                inst = b.stp(idx)
        else:
            from . import StpInstance
            inst = StpInstance.from_file(path)
        why = check_solution(inst.edges, f.get("terminals", []), f.get("solution", []), f["el_cost"])
        if why:
            return False, f"fail, {why}", f
    note = "" if f.get("in_cost", -1) != -1 else " (no cost line to compare)"
    return True, "pass" + note, f


def run(files: Sequence[str], exe: str, arg_cmd: str = "el", list_solution: bool = False, print_only: bool = False,
        log=None, extra: Sequence[str] = ()) -> bool:
    """verify.py's loop over instances, with its PASS/FAIL banner."""
    logs = [sys.stdout] + ([log] if log else [])

    def emit(msg: str) -> None:
        for s in logs:
            s.write(msg)
            s.flush()

    emit(f"date: {time.strftime('%d/%m/%y')}\ntime: {time.strftime('%H:%M:%S')}\n\n")
    emit(f"exe: {exe}\narg cmd: {arg_cmd}\n\n")
    failed = False
    for path in files:
        if print_only:
            emit(" ".join([exe, "-in", path, f"-{arg_cmd}"] + (["-list"] if list_solution else [])) + "\n\n")
            continue
        ok, msg, _ = verify_file(path, exe, arg_cmd, list_solution, extra)
        emit(f"STP instance: {path} {msg}\n")
        failed |= not ok
    banner = "FAIL\nFAIL\nFAIL" if failed else "PASS\nPASS\nPASS"
    emit("\n*********************************************\n" + banner +
         "\n*********************************************\n")
    return not failed


def main(argv: Optional[Sequence[str]] = None) -> int:
    p = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    p.add_argument("files", nargs="*", help="STP files (or EMVBIN01 containers with --bin)")
    p.add_argument("--testset", help="directory searched as <dir>/*/*.stp, like verify.py")
    p.add_argument("--exe", default=None, help="command line to run (default: the built reader-el-gpu)")
    p.add_argument("-c", "--arg-cmd", default="el", choices=["el", "erickson"])
    p.add_argument("--list", action="store_true", help="also check the listed Steiner tree")
    p.add_argument("--bin", action="store_true", help="inputs are EMVBIN01 containers (instance 0)")
    p.add_argument("--print", action="store_true", help="print the commands only")
    p.add_argument("--log", help="also write the report to this file")
    a = p.parse_args(argv)
    files = list(a.files)
    if a.testset:
        files += sorted(glob.glob(os.path.join(a.testset, "*", "*.stp")))
    if not files:
        p.error("no instances given")
    log = open(a.log, "w") if a.log else None
    try:
        ok = run(files, a.exe or default_exe(), a.arg_cmd, a.list, a.print, log, ["-bin"] if a.bin else [])
    finally:
        if log:
            log.close()
    return 0 if ok else 1


if __name__ == "__main__":
    sys.exit(main())
