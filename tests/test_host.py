"""Host side of the solver, no GPU: STP reader, CSR builder, admission checks,
generator, C-ABI exports and the command line's no-GPU paths."""
import os
import re
import subprocess

import numpy as np
import pytest

from tests.golden.cases import CASES, instance_for, instance_fnv

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

B01_LIKE = """33d32945 stp file, stp format version 1.0

section comment
name    "tiny"
end

section graph
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


def test_parse_like_graph_load(emv):
    g = emv.StpInstance.from_text(B01_LIKE)
    assert (g.n, g.m, g.k, g.cost) == (5, 6, 3, 11)
    assert g.edges[0].tolist() == [0, 1, 3]
    assert g.terminals.tolist() == [0, 2, 4]


def test_parse_crlf_data_lines_and_blank_lines(emv):
    # the reference reads "e 1 2 3\r\n" through sscanf (R:560), so CR on data lines is fine
    text = B01_LIKE.replace("e 1 2 3\n", "e 1 2 3\r\n").replace("\n\n", "\n\n\n")
    g = emv.StpInstance.from_text(text)
    assert g.m == 6 and g.edges[0].tolist() == [0, 1, 3]


@pytest.mark.parametrize("mutate,why", [
    (lambda t: t.replace("section graph", "section graph\nsection comment"), "nested sections"),
    (lambda t: t.replace("edges 6", "edges 7"), "edge count"),
    (lambda t: t.replace("terminals 3", "terminals 4"), "terminal count"),
    (lambda t: t.replace("e 1 2 3", "e 1 9 3"), "endpoint out of range"),
    (lambda t: t.replace("e 1 2 3", "e 1 x 3"), "invalid edge line"),
    (lambda t: t.replace("section terminals\nterminals 3\n", "section terminals\n"), "terminals not initialised"),
    (lambda t: t.replace("section comment", "section bogus"), "invalid section"),
    (lambda t: t.replace("nodes 5", "nodes five"), "invalid nodes line"),
    (lambda t: t.replace("cost 11", "coordinates 3"), "coordinates"),
])
def test_parse_errors_are_status_codes(emv, mutate, why):
    with pytest.raises(emv.EmvError) as ei:
        emv.StpInstance.from_text(mutate(B01_LIKE))
    assert ei.value.status == 2, why


def test_parse_ignores_unknown_and_dd_lines(emv):
    text = B01_LIKE.replace("cost 11", "dd 1 2 3\nremark whatever\ncost 11")
    assert emv.StpInstance.from_text(text).cost == 11


def test_stp_write_roundtrip(emv, tmp_path):
    inst = emv.StpInstance.regular(300, 4, 1, 50, 6, 17)
    path = str(tmp_path / "x.stp")
    inst.write(path)
    back = emv.StpInstance.from_file(path)
    assert back.n == inst.n and np.array_equal(back.edges, inst.edges)
    assert np.array_equal(back.terminals, inst.terminals)


def test_csr_both_arcs_and_self_loops(emv):
    g = emv.StpInstance.from_text(B01_LIKE.replace("e 2 4 1", "e 2 2 1"))
    c = emv.Csr.from_stp(g)
    assert c.arcs == 12
    assert np.array_equal(np.diff(c.row_ptr), [2, 4, 2, 2, 2])  # self-loop counts twice at vertex 2
    for u in range(c.n):
        for e in range(c.row_ptr[u], c.row_ptr[u + 1]):
            v, w = c.col[e], c.w[e]
            back = [c.w[f] for f in range(c.row_ptr[v], c.row_ptr[v + 1]) if c.col[f] == u]
            assert w in back


def test_graph_check_rejects_disconnected_and_overflow(emv):
    disc = emv.StpInstance.from_text(B01_LIKE.replace("e 5 1 7\n", "").replace("e 4 5 6\n", "")
                                     .replace("edges 6", "edges 4"))
    with pytest.raises(emv.EmvError) as ei:
        emv.Csr.from_stp(disc).check()
    assert ei.value.status == 7
    big = emv.StpInstance.from_text(B01_LIKE.replace("e 1 2 3", "e 1 2 900000000")
                                    .replace("e 2 3 4", "e 2 3 900000000"))
    with pytest.raises(emv.EmvError) as ei:
        emv.Csr.from_stp(big).check()
    assert ei.value.status == 8
    assert emv.Csr.from_stp(emv.StpInstance.from_text(B01_LIKE)).check() > 0


def test_generator_regular_properties(emv):
    inst = emv.StpInstance.regular(5000, 6, 1, 1000, 12, 5)
    assert inst.m == 5000 * 6 // 2
    deg = np.bincount(inst.edges[:, :2].reshape(-1), minlength=inst.n)
    assert (deg == 6).all()
    assert len(set(inst.terminals.tolist())) == 12
    assert inst.edges[:, 2].min() >= 1 and inst.edges[:, 2].max() <= 1000
    emv.Csr.from_stp(inst).check()  # connected
    again = emv.StpInstance.regular(5000, 6, 1, 1000, 12, 5)
    assert np.array_equal(again.edges, inst.edges)
    other = emv.StpInstance.regular(5000, 6, 1, 1000, 12, 6)
    assert not np.array_equal(other.edges, inst.edges)


def test_generator_mixed_distribution(emv):
    ns, ks, groups = [], [], 0
    for i in range(400):
        inst = emv.StpInstance.mixed(99, i)
        zero = (inst.edges[:, 2] == 0).any()
        groups += int(zero)
        ns.append(inst.n - (6 if zero else 0))
        ks.append(inst.k)
        assert 64 <= ns[-1] <= 4096
        emv.Csr.from_stp(inst).check()
    assert 4 <= min(ks) and max(ks) <= 10
    assert 20 <= groups <= 70  # about 10%
    ln = np.log(ns)
    assert abs(np.median(ln) - (np.log(64) + np.log(4096)) / 2) < 0.4  # log-uniform


@pytest.mark.parametrize("name", sorted(CASES))
def test_generator_reproduces_golden_instances(emv, golden, name):
    """The committed fixtures pin the generator's output on this platform."""
    assert instance_fnv(instance_for(CASES[name])) == golden["cases"][name]["instance_fnv"]


def test_library_exports_every_declared_symbol(emv):
    header = open(os.path.join(ROOT, "include", "emv.h")).read()
    names = sorted(set(re.findall(r"^\s*(?:int|void|const char \*)\s*\**\s*(emv_\w+)\s*\(", header, re.M)))
    assert len(names) >= 25
    lib = emv.load_library()
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) <= set(emv.SIGNATURES)


def test_status_strings(emv):
    lib = emv.load_library()
    assert lib.emv_status_str(0) == b"ok"
    assert lib.emv_status_str(7) == b"graph not connected"
    assert b"sm_103a" in lib.emv_version()


def test_cli_help_and_nop_run_without_gpu(emv, tmp_path):
    out = subprocess.run([emv.CLI_PATH, "-h"], stdout=subprocess.PIPE, text=True, check=True).stdout
    assert "-el : Erickson-Monma-Veinott algorithm" in out
    path = str(tmp_path / "t.stp")
    with open(path, "w") as f:
        f.write(B01_LIKE)
    out = subprocess.run([emv.CLI_PATH, "-in", path], stdout=subprocess.PIPE, text=True, check=True).stdout
    assert "command: no operation" in out
    assert re.search(r"input: n = 5, m = 6, k = 3, cost = 11 \[(.*)ms\] {peak:(.*)GiB} {curr:(.*)GiB}", out)
    assert "terminals: 1 3 5" in out
    assert re.search(r"root build:(.*)\[zero:(.*)ms\] \[pos:(.*)ms\] \[adj:(.*)ms\] \[term:(.*)ms\] done. "
                     r"\[(.*)ms\] {peak:(.*)GiB} {curr:(.*)GiB}", out)
    assert re.search(r"grand total \[(.*)ms\] {peak:(.*)GiB}", out)


def test_cli_parse_error_exits_nonzero(emv, tmp_path):
    path = str(tmp_path / "bad.stp")
    with open(path, "w") as f:
        f.write(B01_LIKE.replace("edges 6", "edges 9"))
    r = subprocess.run([emv.CLI_PATH, "-in", path, "-el"], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    assert r.returncode != 0 and "ERROR" in r.stderr


def test_generator_powlaw_and_clique(emv):
    g = emv.StpInstance.powlaw(20000, 6, -0.5, 10, 1, 100, 8, 5)
    deg = np.bincount(g.edges[:, :2].reshape(-1), minlength=g.n)
    assert abs(deg.mean() - 6) < 0.2 and deg.max() > 20 * deg.min()  # heavy tail
    emv.Csr.from_stp(g).check()
    again = emv.StpInstance.powlaw(20000, 6, -0.5, 10, 1, 100, 8, 5)
    assert np.array_equal(again.edges, g.edges) and np.array_equal(again.terminals, g.terminals)
    q = emv.StpInstance.clique(60, 1, 50, 6, 3)
    assert q.m == 60 * 59 // 2 and len(set(q.terminals.tolist())) == 6
    with pytest.raises(emv.EmvError):
        emv.StpInstance.powlaw(100, 4, 0.5, 5, 1, 10, 3, 1)  # alpha must be negative
