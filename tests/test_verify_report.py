"""The verify/report replacements: line parsing with the reference's patterns,
the strict tree check, the verify loop over a stand-in command, and GPU runs
of both tools on real instances."""
import os
import stat

import numpy as np
import pytest

from steiner_edge_linear_gb300 import report, verify
from tests.golden.cases import CASES, instance_for

# lines in the command line's format (cli.cpp), instance B01_LIKE below
CANNED = """invoked as: reader-el-gpu -in x.stp -el -list
random seed = 123456789
input: n = 5, m = 6, k = 3, cost = {in_cost} [0.05 ms] {peak: 0.00GiB} {curr: 0.00GiB}
terminals: 1 3 5
root build: [zero: 0.00 ms] [pos: 0.01 ms] [adj: 0.01 ms] [term: 0.00 ms] done. [0.03 ms] {peak: 0.00GiB} {curr: 0.00GiB}
command: Erickson-Monma-Veinott
erickson: [zero: 0.01 ms] [kernel: 1.25 ms 0.01GiB/s] [traceback: 0.10 ms] done. [3.00 ms] [cost: {cost}] {peak: 0.01GiB} {curr: 0.01GiB}
solution: [{solution}]
gpu: [level1: 0.100 ms] [merge: 0.200 ms 0.5 GB/s] [relax: 0.300 ms 0.6 GB/s 12 sweeps] [0.004 Gcell/s] [launches: 9]
command done [5.00 ms]
grand total [6.00 ms] {peak: 0.01GiB}
host: box
build: edge-linear kernel, gb300 cuda sm_103a, frontier relaxation
list solution: true
num threads: 1
compiler: gcc 13.3.0
"""

B01_LIKE = """section graph
nodes 5
edges 6
e 1 2 3
e 2 3 4
e 3 4 5
e 4 5 6
e 5 1 7
e 2 4 1
end

section terminals
terminals 3
t 1
t 3
t 5
end

cost 11
eof
"""
EDGES = np.array([[0, 1, 3], [1, 2, 4], [2, 3, 5], [3, 4, 6], [4, 0, 7], [1, 3, 1]])


def canned(cost=11, solution='"1 2", "2 4", "4 5", "2 3"', in_cost=None):
    in_cost = cost if in_cost is None else in_cost
    return CANNED.replace("{cost}", str(cost)).replace("{solution}", solution).replace("{in_cost}", str(in_cost))


def test_parse_output_fields():
    f = verify.parse_output(canned(), list_solution=True)
    assert (f["n"], f["m"], f["k"], f["in_cost"], f["el_cost"]) == (5, 6, 3, 11, 11)
    assert f["terminals"] == [1, 3, 5] and f["solution"] == [(1, 2), (2, 4), (4, 5), (2, 3)]
    assert f["traceback_ms"] == pytest.approx(0.10) and f["kernel_ms"] == pytest.approx(1.25)
    assert f["relax_sweeps"] == 12 and f["launches"] == 9
    k2 = "erickson: [kernel: 0.50 ms 0.10GiB/s] done. [0.70 ms] [cost: 9] {peak: 0.00GiB} {curr: 0.00GiB}"
    assert verify.parse_output(k2)["el_cost"] == 9


def test_check_solution_strict():
    t = [1, 3, 5]
    # 1-2 (3), 2-3 (4), 2-4 (1), 4-5 (6) = 14
    assert verify.check_solution(EDGES, t, [(1, 2), (2, 3), (2, 4), (4, 5)], 14) is None
    assert "weight" in verify.check_solution(EDGES, t, [(1, 2), (2, 3), (2, 4), (4, 5)], 11)
    assert "not an input edge" in verify.check_solution(EDGES, t, [(1, 3), (3, 5)], 0)
    assert "cycle" in verify.check_solution(EDGES, t, [(1, 2), (2, 4), (4, 5), (5, 1)], 17)
    assert "not covered" in verify.check_solution(EDGES, t, [(1, 2), (2, 3)], 7)
    assert verify.check_solution(EDGES, t, [(1, 2), (2, 3), (4, 5)], 13) is not None


def _fake_exe(tmp_path, outputs: dict) -> str:
    """A stand-in command line printing a canned output per input file."""
    for path, text in outputs.items():
        with open(path + ".canned", "w") as fh:
            fh.write(text)
    exe = str(tmp_path / "fake-reader")
    with open(exe, "w") as fh:
        fh.write('#!/bin/sh\ncat "$2.canned"\n')
    os.chmod(exe, os.stat(exe).st_mode | stat.S_IEXEC)
    return exe


def test_verify_loop_pass_and_fail(tmp_path, capsys):
    good, bad_cost, bad_tree, err = (str(tmp_path / f"{x}.stp") for x in ("good", "cost", "tree", "err"))
    for p in (good, bad_cost, bad_tree, err):
        open(p, "w").write(B01_LIKE.replace("cost 11", "cost 14"))
    exe = _fake_exe(tmp_path, {
        good: canned(14, '"1 2", "2 3", "2 4", "4 5"'),
        bad_cost: canned(13, '"1 2", "2 3", "2 4", "4 5"', in_cost=14),
        bad_tree: canned(14, '"1 2", "2 3", "4 5"'),
        err: "ERROR [file = cli.cpp, line = 1] main: min_cost != cost\n",
    })
    assert verify.run([good], exe, list_solution=True)
    assert "PASS" in capsys.readouterr().out
    for p in (bad_cost, bad_tree, err):
        assert not verify.run([p], exe, list_solution=True), p
    out = capsys.readouterr().out
    assert "fail inCost = 14 elCost = 13" in out and "error: testing failed" in out and "FAIL" in out
    assert verify.main([good, "--exe", exe, "--list"]) == 0
    assert verify.main([good, bad_cost, "--exe", exe]) == 1


def test_report_row_columns():
    row = report.parse_run(canned(), list_solution=True)
    assert (row["n"], row["m"], row["k"], row["e_cost"], row["seed"]) == (5, 6, 3, 11, 123456789)
    assert row["r_total"] == pytest.approx(0.03) and row["g_total"] == pytest.approx(6.0)
    assert row["merge_gbs"] == pytest.approx(report.merge_bytes(5, 3) / 0.2e6)
    line = report.format_row(row)
    assert len(line.split()) == len(report.COLUMNS)
    assert report.write_table([row], None).startswith("# n m k")


@pytest.mark.gpu
def test_verify_golden_files_on_gpu(emv, golden, tmp_path, capsys):
    files = []
    for name, spec in sorted(CASES.items()):
        if spec.get("kind") != "file":
            continue
        inst = instance_for(spec)
        inst.cost = golden["cases"][name]["cost"]
        path = str(tmp_path / f"{name}.stp")
        inst.write(path)
        files.append(path)
    assert files and verify.run(files, emv.CLI_PATH, list_solution=True)
    wrong = instance_for(CASES["path_n3000_k5"])
    wrong.cost = golden["cases"]["path_n3000_k5"]["cost"] + 1
    wrong.write(str(tmp_path / "wrong.stp"))
    assert not verify.run([str(tmp_path / "wrong.stp")], emv.CLI_PATH)
    # container input through the same loop
    binf = str(tmp_path / "g.bin")
    emv.BinContainer.write(binf, [emv.StpInstance.from_file(files[0])])
    assert verify.main([binf, "--bin", "--list"]) == 0


@pytest.mark.gpu
def test_report_runs_generated_instances(emv, orc, tmp_path):
    rows = report.run_experiments(str(tmp_path / "rep"), "regular", [1024, 2048], [4], [5, 7], 1000, 123456789, 1)
    assert len(rows) == 4
    for r in rows:
        g = emv.StpInstance.regular(r["g_n"], 4, 1, 1000, r["g_k"], r["g_seed"])
        c = emv.Csr.from_stp(g)
        assert r["e_cost"] == orc.emv_table(c.n, c.row_ptr, c.col, c.w, c.terminals)[1]
        assert r["merge_gbs"] > 0 and r["relax_gbs"] > 0 and r["sweeps"] > 0
    text = open(str(tmp_path / "rep" / "regular-n1024-d4-k5-s123456789.out")).read()
    assert report.parse_run(text)["e_cost"] == rows[0]["e_cost"]
