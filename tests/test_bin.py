"""EMVBIN01 instance container (emv_bin_*): round trips, corrupt files, the
command line's -bin input, and GPU solves from a container."""
import os
import re
import struct
import subprocess

import numpy as np
import pytest

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


def _instances(emv):
    return [emv.StpInstance.from_text(B01_LIKE),
            emv.StpInstance.regular(3000, 6, 1, 1000, 7, 11),
            emv.StpInstance.mixed(5, 0),
            emv.StpInstance.mixed(5, 17),
            emv.StpInstance.powlaw(2000, 6, -0.5, 8, 1, 50, 5, 3)]


def test_round_trip_csr_and_stp(emv, tmp_path):
    insts = _instances(emv)
    path = str(tmp_path / "a.bin")
    emv.BinContainer.write(path, insts)
    with emv.BinContainer(path) as b:
        assert len(b) == len(insts)
        for i, g in enumerate(insts):
            want = emv.Csr.from_stp(g)
            got = b.csr(i)
            assert got.n == want.n and got.cost == g.cost
            for a in ("row_ptr", "col", "w", "terminals"):
                assert np.array_equal(getattr(got, a), getattr(want, a)), a
            back = b.stp(i)
            assert back.n == g.n and back.cost == g.cost
            assert np.array_equal(back.edges, g.edges) and np.array_equal(back.terminals, g.terminals)


def test_without_edges_has_no_stp_form(emv, tmp_path):
    path = str(tmp_path / "b.bin")
    g = emv.StpInstance.regular(500, 4, 1, 10, 4, 2)
    emv.BinContainer.write(path, [g], with_edges=False)
    with emv.BinContainer(path) as b:
        assert np.array_equal(b.csr(0).col, emv.Csr.from_stp(g).col)
        with pytest.raises(emv.EmvError) as ei:
            b.stp(0)
        assert ei.value.status == 1
        with pytest.raises(emv.EmvError) as ei:
            b.csr(1)
        assert ei.value.status == 1


def _corrupt(src: str, dst: str, fn) -> None:
    data = bytearray(open(src, "rb").read())
    fn(data)
    open(dst, "wb").write(bytes(data))


def _first_record(data: bytearray) -> int:
    return struct.unpack_from("<Q", data, 16)[0]


@pytest.mark.parametrize("what", ["magic", "count", "offset", "truncate", "head", "row_ptr", "weight",
                                  "terminal", "edge"])
def test_corrupt_containers_are_parse_errors(emv, tmp_path, what):
    src = str(tmp_path / "ok.bin")
    emv.BinContainer.write(src, [emv.StpInstance.from_text(B01_LIKE)])
    dst = str(tmp_path / "bad.bin")
    n, m, k = 5, 6, 3

    def rec(d):
        return _first_record(d)

    def arr(d, which):  # byte offset of an int32 array inside record 0
        o = rec(d) + 40
        pad = lambda b: (b + 7) // 8 * 8
        sizes = {"row_ptr": 4 * (n + 1), "col": 8 * m, "w": 8 * m, "terms": 4 * k, "edges": 12 * m}
        for name in ("row_ptr", "col", "w", "terms", "edges"):
            if name == which:
                return o
            o += pad(sizes[name])

    edits = {
        "magic": lambda d: d.__setitem__(slice(0, 8), b"NOTEMVB!"),
        "count": lambda d: struct.pack_into("<Q", d, 8, 10**6),
        "offset": lambda d: struct.pack_into("<Q", d, 16, len(d) + 8),
        "truncate": lambda d: d.__delitem__(slice(len(d) - 16, len(d))),
        "head": lambda d: struct.pack_into("<q", d, rec(d), -4),
        "row_ptr": lambda d: struct.pack_into("<i", d, arr(d, "row_ptr") + 8, 99),
        "weight": lambda d: struct.pack_into("<i", d, arr(d, "w"), -1),
        "terminal": lambda d: struct.pack_into("<i", d, arr(d, "terms"), n),
        "edge": lambda d: struct.pack_into("<i", d, arr(d, "edges"), 2),
    }
    _corrupt(src, dst, edits[what])
    with pytest.raises(emv.EmvError) as ei:
        with emv.BinContainer(dst) as b:
            b.csr(0)
    assert ei.value.status == 2, what


def test_not_a_container(emv, tmp_path):
    path = str(tmp_path / "t.stp")
    open(path, "w").write(B01_LIKE)
    with pytest.raises(emv.EmvError) as ei:
        emv.BinContainer(path)
    assert ei.value.status == 2


def test_cli_bin_input_lines_match_stp_input(emv, tmp_path):
    g = emv.StpInstance.regular(2000, 4, 1, 100, 6, 9)
    g.cost = 1234
    stp = str(tmp_path / "g.stp")
    g.write(stp)
    other = emv.StpInstance.regular(300, 4, 1, 100, 3, 1)
    binf = str(tmp_path / "g.bin")
    emv.BinContainer.write(binf, [other, g])

    def lines(args):
        out = subprocess.run([emv.CLI_PATH] + args, stdout=subprocess.PIPE, text=True, check=True).stdout
        inp = next(ln for ln in out.splitlines() if ln.startswith("input"))
        ter = next(ln for ln in out.splitlines() if ln.startswith("terminals"))
        return re.sub(r"\[.*", "", inp), ter

    assert lines(["-in", stp]) == lines(["-in", binf, "-bin", "-index", "1"])
    r = subprocess.run([emv.CLI_PATH, "-in", binf, "-bin", "-index", "2"], stdout=subprocess.PIPE,
                       stderr=subprocess.PIPE, text=True)
    assert r.returncode != 0 and "ERROR" in r.stderr


@pytest.mark.gpu
def test_gpu_solves_from_container(emv, orc, tmp_path):
    insts = [emv.StpInstance.mixed(77, i) for i in range(40)] + [emv.StpInstance.regular(4000, 6, 1, 1000, 8, 5)]
    path = str(tmp_path / "s.bin")
    emv.BinContainer.write(path, insts, with_edges=False)
    with emv.BinContainer(path) as b:
        graphs = [b.csr(i) for i in range(len(b))]
    with emv.Solver(0) as s:
        costs, _ = s.batch_solve(graphs)
        single = [s.solve(g).cost for g in graphs]
    want = [orc.emv_table(g.n, g.row_ptr, g.col, g.w, g.terminals)[1] for g in graphs]
    assert list(costs) == single == want
    # the command line solves container input and keeps the cost-line check
    big = insts[-1]
    big.cost = want[-1]
    emv.BinContainer.write(path, [big])
    out = subprocess.run([emv.CLI_PATH, "-in", path, "-bin", "-el", "-list"], stdout=subprocess.PIPE, text=True,
                         check=True).stdout
    assert f"[cost: {want[-1]}]" in out
    big.cost = want[-1] + 1
    emv.BinContainer.write(path, [big])
    r = subprocess.run([emv.CLI_PATH, "-in", path, "-bin", "-el"], stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                       text=True)
    assert r.returncode != 0 and "min_cost != cost" in r.stderr
