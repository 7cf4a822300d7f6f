"""GPU parity: the sm_103a solver against the oracle and the reference's golden tables.

The bar is bit-exact: the whole int32 DP table and the cost equal the
oracle's on the same instance and the reference's golden hashes; the tree is a
valid Steiner tree of real edges whose weight equals the cost.
"""
import os
import subprocess

import numpy as np
import pytest

from tests.golden.cases import CASES, instance_for, instance_fnv
from tests.helpers import check_tree, table_row_fnv

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def solver(emv):
    s = emv.Solver(0)
    yield s
    s.close()


@pytest.mark.parametrize("name", sorted(CASES))
def test_table_and_cost_match_oracle_and_golden(name, emv, orc, golden, solver):
    g = golden["cases"][name]
    inst = instance_for(CASES[name])
    assert instance_fnv(inst) == g["instance_fnv"]
    csr = emv.Csr.from_stp(inst)
    res = solver.solve(csr, tree=True, table=True)
    want, want_cost = orc.emv_table(csr.n, csr.row_ptr, csr.col, csr.w, csr.terminals, threads=8)
    assert res.cost == want_cost == g["cost"]
    mism = np.argwhere(res.table != want)
    assert mism.size == 0, f"{len(mism)} cells differ, first (X, v) = {mism[:5].tolist()}"
    assert f"{orc.fnv64(res.table):016x}" == g["table_fnv"]
    if "row_fnv" in g and csr.k <= 8:
        assert table_row_fnv(res.table) == g["row_fnv"]
    check_tree(csr.n, inst.edges, res.tree, csr.terminals, res.cost)
    assert res.tree_weight == res.cost or csr.k == 1


def test_repeat_solves_identical(emv, solver):
    inst = emv.StpInstance.regular(5000, 6, 1, 1000, 9, 77)
    csr = emv.Csr.from_stp(inst)
    a = solver.solve(csr, table=True)
    b = solver.solve(csr, table=True)
    assert a.cost == b.cost and np.array_equal(a.table, b.table)


def test_kernel_dev_on_caller_table(emv, orc, solver):
    torch = pytest.importorskip("torch")
    inst = emv.StpInstance.regular(3000, 8, 1, 1000, 7, 31337)
    csr = emv.Csr.from_stp(inst)
    dev = torch.device("cuda:0")
    row = torch.from_numpy(csr.row_ptr).to(dev)
    col = torch.from_numpy(csr.col).to(dev)
    w = torch.from_numpy(csr.w).to(dev)
    ld = csr.n + 5  # any stride >= n
    table = torch.full(((1 << csr.k), ld), -7, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream().cuda_stream
    cost = solver.kernel_dev(csr.n, csr.arcs, row.data_ptr(), col.data_ptr(), w.data_ptr(), csr.terminals,
                             table.data_ptr(), ld, stream)
    torch.cuda.synchronize()
    want, want_cost = orc.emv_table(csr.n, csr.row_ptr, csr.col, csr.w, csr.terminals, threads=8)
    got = table[:, :csr.n].cpu().numpy()
    assert cost == want_cost
    assert np.array_equal(got, want)
    assert (table[:, csr.n:].cpu().numpy() == -7).all(), "padding columns must stay untouched"


def test_solve_dev_matches_solve(emv, solver):
    torch = pytest.importorskip("torch")
    inst = emv.StpInstance.regular(2500, 4, 1, 100, 8, 5)
    csr = emv.Csr.from_stp(inst)
    dev = torch.device("cuda:0")
    row, col, w = (torch.from_numpy(a).to(dev) for a in (csr.row_ptr, csr.col, csr.w))
    torch.cuda.synchronize()
    r1 = solver.solve_dev(csr.n, csr.arcs, row.data_ptr(), col.data_ptr(), w.data_ptr(), csr.terminals, tree=True)
    r2 = solver.solve(csr)
    assert r1.cost == r2.cost
    check_tree(csr.n, inst.edges, r1.tree, csr.terminals, r1.cost)


def test_sssp_matches_oracle(emv, orc, solver):
    inst = emv.StpInstance.regular(20000, 6, 1, 1000, 2, 8)
    csr = emv.Csr.from_stp(inst)
    for s in (0, 12345, 19999):
        d, _ = solver.sssp(csr, s)
        assert np.array_equal(d, orc.sssp(csr.n, csr.row_ptr, csr.col, csr.w, s))


def test_large_single_solve_properties(emv, orc, solver):
    """n = 1e5, degree 20, k = 12 (the single large solve): the full table is
    too slow for the oracle here, so check it through size-independent
    properties plus exact rows over the first 5 terminals (d[X][v] depends on
    the terminals of X only; the oracle computes those 32 rows)."""
    inst = emv.StpInstance.regular(100000, 20, 1, 100, 12, 123456789)
    csr = emv.Csr.from_stp(inst)
    res = solver.solve(csr, tree=True, table=True)
    t = res.table
    sub, _ = orc.emv_table(csr.n, csr.row_ptr, csr.col, csr.w, csr.terminals[:5], threads=16)
    assert np.array_equal(t[:32], sub)
    assert (t[0] == emv.INF32).all() and (t[1:] < emv.INF32).all()
    rng = np.random.default_rng(0)
    src = np.repeat(np.arange(csr.n), np.diff(csr.row_ptr))
    for X in rng.integers(1, 1 << 12, size=24):
        row = t[X]
        # closure: d[X][v] <= d[X][u] + w(u, v) for every arc
        assert (row[csr.col] <= row[src] + csr.w).all()
        # monotone in X and bounded by every split
        for b in range(12):
            if X >> b & 1:
                assert (t[X ^ (1 << b)] <= row).all()
                Y = X & ~(1 << b)
                if Y:
                    assert (row <= t[Y] + t[1 << b]).all()
    assert res.cost == int(t[(1 << 11) - 1, csr.terminals[11]])
    check_tree(csr.n, inst.edges, res.tree, csr.terminals, res.cost)


@pytest.mark.parametrize("n,degree,k", [(700, 6, 13), (300, 4, 14), (120, 4, 15)])
def test_large_k_whole_table(emv, orc, solver, n, degree, k):
    """k = 13..15 run the streamed merge in subset groups with row tiles; the
    whole table must still equal the oracle's."""
    inst = emv.StpInstance.regular(n, degree, 1, 1000, k, 4242 + k)
    csr = emv.Csr.from_stp(inst)
    res = solver.solve(csr, tree=True, table=True)
    want, want_cost = orc.emv_table(csr.n, csr.row_ptr, csr.col, csr.w, csr.terminals, threads=8)
    assert res.cost == want_cost
    mism = np.argwhere(res.table != want)
    assert mism.size == 0, f"{len(mism)} cells differ, first (X, v) = {mism[:5].tolist()}"
    check_tree(csr.n, inst.edges, res.tree, csr.terminals, res.cost)


def _narrow_levels(table, terms):
    """Levels the solver takes with 16-bit values, recomputed from the
    oracle's table: M(j) is the largest value level j's merge writes (from the
    lower levels, terminal override included), M(1) the largest single-source
    distance.  Level m >= 2 relaxes with 16-bit records when M(m-1) + M(1) <=
    32767; level m >= 3 merges from 16-bit rows when every M(j) + M(m-j) <=
    65533.  Returns (relaxed, merged) level counts."""
    k = len(terms)
    M = {1: int(max(table[1 << i].max() for i in range(k)))}
    for m in range(2, k):
        mx = 0
        for X in range(1, 1 << k):
            if bin(X).count("1") != m:
                continue
            best = None
            Y = (X - 1) & X
            while Y:
                if Y < (X ^ Y):
                    s = table[Y].astype(np.int64) + table[X ^ Y]
                    best = s if best is None else np.minimum(best, s)
                Y = (Y - 1) & X
            for t in range(k):
                if X >> t & 1:
                    best[terms[t]] = table[X ^ (1 << t)][terms[t]]
            mx = max(mx, int(best.max()))
        M[m] = mx
    relaxed = sum(1 for m in range(2, k + 1) if M[m - 1] + M[1] <= 32767)
    merged = sum(1 for m in range(3, k + 1) if max(M[j] + M[m - j] for j in range(1, m // 2 + 1)) <= 65533)
    return relaxed, merged


# weight range -> which levels take 16-bit relaxation records and merge rows
WIDTH_CASES = {100: ("all", "all"), 3000: ("some", "all"), 5000: ("some", "some"), 8000: ("none", "none")}


@pytest.mark.parametrize("ew", sorted(WIDTH_CASES))
def test_value_widths_match_oracle(emv, orc, ew):
    """16-bit values are taken per level only where the level maxima bound
    them: weights up to 100 keep every level 16-bit, larger weights the lower
    levels only or none.  The level counts equal the rule's, and the table
    equals the oracle's with automatic and with 32-bit values."""
    k = 10
    inst = emv.StpInstance.regular(6000, 6, 1, ew, k, 515)
    csr = emv.Csr.from_stp(inst)
    want, want_cost = orc.emv_table(csr.n, csr.row_ptr, csr.col, csr.w, csr.terminals, threads=8)
    relaxed, merged = _narrow_levels(want, list(csr.terminals))
    kinds = tuple("all" if c == top else "none" if c == 0 else "some" for c, top in ((relaxed, k - 1), (merged, k - 2)))
    assert kinds == WIDTH_CASES[ew]
    with emv.Solver(0) as s:
        for bits in (0, 32):
            s.set_value_bits(bits)
            res = s.solve(csr, tree=True, table=True)
            assert res.timing["relax16_levels"] == (relaxed if bits == 0 else 0)
            assert res.timing["merge16_levels"] == (merged if bits == 0 else 0)
            assert res.cost == want_cost
            mism = np.argwhere(res.table != want)
            assert mism.size == 0, f"bits {bits}: {len(mism)} cells differ, first (X, v) = {mism[:5].tolist()}"
            check_tree(csr.n, inst.edges, res.tree, csr.terminals, res.cost)
        with pytest.raises(emv.EmvError):
            s.set_value_bits(16)


def test_wide_records_and_partial_merge_block_equal_32_bit_values(emv):
    """Records past three quarters of L2 (n = 2^18 + 40) take 1 KB per vertex:
    512 rows of 16 bits against 256 of 32; the last 64-vertex merge block is
    partial.  Both tables are identical."""
    inst = emv.StpInstance.regular((1 << 18) + 40, 6, 1, 100, 11, 2718)
    csr = emv.Csr.from_stp(inst)
    with emv.Solver(0) as s:
        a = s.solve(csr, table=True)
        s.set_value_bits(32)
        b = s.solve(csr, table=True)
    assert a.timing["relax16_levels"] == 10 and a.timing["merge16_levels"] == 9
    assert b.timing["relax16_levels"] == 0 and b.timing["merge16_levels"] == 0
    assert a.cost == b.cost and np.array_equal(a.table, b.table)


def test_640_byte_records_match_oracle(emv, orc):
    """k = 12 with weights up to 8000 keeps 32-bit values: levels 5..7 (792,
    924, 792 subsets) relax in 5, 6 and 5 chunks of 640-byte records instead
    of 7, 8 and 7 of 512 bytes.  Whole table against the oracle, and the
    launch count of that chunk rule."""
    inst = emv.StpInstance.regular(2000, 6, 1, 8000, 12, 606)
    csr = emv.Csr.from_stp(inst)
    want, want_cost = orc.emv_table(csr.n, csr.row_ptr, csr.col, csr.w, csr.terminals, threads=8)
    with emv.Solver(0) as s:
        res = s.solve(csr, tree=True, table=True)
    assert res.timing["relax16_levels"] == 0
    # level 1, then per level m: 66 -> 1, 220 -> 2, 495 -> 4, 792 -> 5, 924 -> 6, 792 -> 5, 495 -> 4, 220 -> 2,
    # 66, 12, 1 -> 1 each
    assert res.timing["relax_launches"] == 1 + 1 + 2 + 4 + 5 + 6 + 5 + 4 + 2 + 1 + 1 + 1
    assert res.cost == want_cost
    mism = np.argwhere(res.table != want)
    assert mism.size == 0, f"{len(mism)} cells differ, first (X, v) = {mism[:5].tolist()}"
    check_tree(csr.n, inst.edges, res.tree, csr.terminals, res.cost)


def test_bad_inputs_report_status(emv, solver):
    disc = emv.StpInstance.from_text(
        "section graph\nnodes 4\nedges 2\ne 1 2 3\ne 3 4 5\nend\nsection terminals\nterminals 2\nt 1\nt 3\nend\n")
    csr = emv.Csr.from_stp(disc)
    with pytest.raises(emv.EmvError) as ei:
        solver.solve(csr)
    assert ei.value.status == 7  # EMV_ERR_DISCONNECTED
    inst = emv.StpInstance.regular(100, 4, 1, 10, 5, 1)
    csr = emv.Csr.from_stp(inst)
    with pytest.raises(emv.EmvError) as ei:
        solver.solve(csr, terminals=[0, 1, 200])
    assert ei.value.status == 1
    with pytest.raises(emv.EmvError):
        solver.solve(csr, terminals=list(range(21)))
    # the context stays usable after errors
    assert solver.solve(csr).cost > 0


def test_admission_checks_on_every_entry_point(emv, solver):
    """Weights near 2^30 are EMV_ERR_OVERFLOW, a head out of range
    EMV_ERR_BAD_INPUT and a disconnected graph EMV_ERR_DISCONNECTED, from the
    host entry point with its default flags and from both device entry
    points (the device check of k_pack_scan and the level-1 connectivity
    test), and from emv_closure_noalloc; the context solves again after each."""
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream().cuda_stream
    base = emv.Csr.from_stp(emv.StpInstance.regular(300, 4, 1, 100, 5, 21))
    heavy = emv.Csr(base.n, base.row_ptr, base.col, np.full_like(base.w, 1 << 28), base.terminals)
    bad_head = emv.Csr(base.n, base.row_ptr, base.col.copy(), base.w, base.terminals)
    bad_head.col[11] = base.n + 5
    disc_inst = emv.StpInstance(8, np.array([[0, 1, 3], [1, 2, 4], [3, 4, 1], [4, 5, 2], [6, 7, 1], [5, 6, 9]],
                                            np.int64), np.array([0, 2, 4], np.int64))
    disc = emv.Csr.from_stp(disc_inst)
    disc = emv.Csr(disc.n, disc.row_ptr, disc.col, disc.w, disc.terminals)
    # vertices 0-2 and 3-7 are two components
    assert disc.n == 8
    cases = [(heavy, 8), (bad_head, 1), (disc, 7)]
    for g, status in cases:
        with pytest.raises(emv.EmvError) as ei:
            solver.solve(g)
        assert ei.value.status == status
        row, col, w = (torch.from_numpy(a).to(dev) for a in (g.row_ptr, g.col, g.w))
        with pytest.raises(emv.EmvError) as ei:
            solver.solve_dev(g.n, g.arcs, row.data_ptr(), col.data_ptr(), w.data_ptr(), g.terminals, stream=stream)
        assert ei.value.status == status
        table = torch.empty(((1 << g.k), g.n), dtype=torch.int32, device=dev)
        with pytest.raises(emv.EmvError) as ei:
            solver.kernel_dev(g.n, g.arcs, row.data_ptr(), col.data_ptr(), w.data_ptr(), g.terminals,
                              table.data_ptr(), g.n, stream)
        assert ei.value.status == status
        torch.cuda.synchronize()
    # the closure entry point: a single weight of 2^30 or more, and a head out of range
    huge = emv.Csr(base.n, base.row_ptr, base.col, base.w.copy(), base.terminals)
    huge.w[3] = 1 << 30
    init = torch.full((1, base.n), emv.INF32, dtype=torch.int32, device=dev)
    init[0, 0] = 0
    for g, status in ((huge, 8), (bad_head, 1)):
        row, col, w = (torch.from_numpy(a).to(dev) for a in (g.row_ptr, g.col, g.w))
        with pytest.raises(emv.EmvError) as ei:
            emv.Solver.closure_noalloc(g.n, g.arcs, row.data_ptr(), col.data_ptr(), w.data_ptr(), init.data_ptr(), 1,
                                       g.n, init.data_ptr(), stream)
        assert ei.value.status == status
    # still usable
    assert solver.solve(base).cost == solver.solve(base, check=False).cost > 0


def test_sweep_limit_is_a_timeout_status_and_context_survives(emv, orc):
    """A bounded device loop that runs out reports EMV_ERR_TIMEOUT through the
    status word; nothing traps and the same context solves again."""
    inst = emv.StpInstance.regular(3000, 4, 1, 1000, 6, 99)
    csr = emv.Csr.from_stp(inst)
    want = orc.emv_table(csr.n, csr.row_ptr, csr.col, csr.w, csr.terminals)[1]
    with emv.Solver(0) as s:
        s.set_sweep_limit(2)
        with pytest.raises(emv.EmvError) as ei:
            s.solve(csr)
        assert ei.value.status == 5  # EMV_ERR_TIMEOUT
        s.set_sweep_limit(0)
        assert s.solve(csr).cost == want
        with pytest.raises(emv.EmvError):
            s.set_sweep_limit(-1)


def test_table_beyond_device_memory_is_oom_and_context_survives(emv, solver):
    """A table larger than the device (n * 2^k * 4 bytes well above its memory)
    fails its allocation with EMV_ERR_OOM; the context is usable afterwards."""
    torch = pytest.importorskip("torch")
    total = torch.cuda.get_device_properties(0).total_memory
    k = 20
    n = 1 << 14
    while n * (4 << k) < 2 * total:
        n <<= 1
    inst = emv.StpInstance.regular(n, 4, 1, 10, k, 5)
    csr = emv.Csr.from_stp(inst)
    with pytest.raises(emv.EmvError) as ei:
        solver.solve(csr)
    assert ei.value.status == 3  # EMV_ERR_OOM
    small = emv.Csr.from_stp(emv.StpInstance.regular(500, 4, 1, 10, 5, 5))
    assert solver.solve(small).cost > 0


def test_cli_reference_lines(emv, tmp_path):
    """reader-el-gpu -el -list prints the reference's lines; the regexes are
    those of the reference's scripts (experiments/verify.py:126-147)."""
    import re

    inst = emv.StpInstance.regular(3000, 4, 1, 1000, 9, 2718)
    csr = emv.Csr.from_stp(inst)
    cost = emv.Solver().solve(csr).cost
    inst.cost = cost
    path = str(tmp_path / "i.stp")
    inst.write(path)
    out = subprocess.run([emv.CLI_PATH, "-in", path, "-el", "-list"], stdout=subprocess.PIPE, text=True,
                         check=True).stdout
    line = next(ln for ln in out.splitlines() if ln.startswith("erickson"))
    mt = re.search(r"erickson: \[zero:(.*)ms\] \[kernel:(.*)ms (.*)GiB/s\] \[traceback: (.*)ms\] done. "
                   r"\[(.*)ms\] \[cost:(.*)] {peak:(.*)GiB} {curr:(.*)GiB}", line)
    assert mt and int(mt.group(6)) == cost
    inp = next(ln for ln in out.splitlines() if ln.startswith("input"))
    assert re.search(r"(.*)n = (.*), m = (.*), k = (.*), cost = (.*) \[(.*)ms\] {peak:(.*)GiB} {curr:(.*)GiB}", inp)
    sol = next(ln for ln in out.splitlines() if ln.startswith("solution"))
    pairs = re.findall(r'"([^"]*)"', sol)
    lookup = {}
    for u, v, w in inst.edges:
        lookup.setdefault((min(u, v), max(u, v)), set()).add(int(w))
    tree = []
    for p in pairs:
        u, v = (int(x) - 1 for x in p.split())
        tree.append((u, v, min(lookup[(min(u, v), max(u, v))])))
    check_tree(inst.n, inst.edges, np.array(tree), inst.terminals, cost)
    # a wrong cost line in the input ends the run with ERROR, as in the reference
    inst.cost = cost + 1
    inst.write(path)
    r = subprocess.run([emv.CLI_PATH, "-in", path, "-el"], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    assert r.returncode != 0 and "min_cost != cost" in r.stderr


def test_cli_dijkstra_command(emv, orc, tmp_path):
    """-dijkstra (R:2454-2484): source = rand() % n after srand(seed), distances on the GPU."""
    import ctypes
    import re

    inst = emv.StpInstance.regular(5000, 6, 1, 1000, 3, 4)
    path = str(tmp_path / "d.stp")
    inst.write(path)
    out = subprocess.run([emv.CLI_PATH, "-in", path, "-dijkstra", "-seed", "77"], stdout=subprocess.PIPE, text=True,
                         check=True).stdout
    mt = re.search(r"dijkstra: \[source: (\d+)\] \[total: (.*) ms (.*)GiB/s\] \[reached: (\d+)\] \[max: (\d+)\]", out)
    assert mt, out
    libc = ctypes.CDLL(None)
    libc.srand(77)
    src = libc.rand() % inst.n
    assert int(mt.group(1)) == src + 1
    csr = emv.Csr.from_stp(inst)
    d = orc.sssp(csr.n, csr.row_ptr, csr.col, csr.w, src)
    assert int(mt.group(4)) == inst.n and int(mt.group(5)) == int(d.max())


def test_roofline_scale_solve(emv, orc, tmp_path):
    """n = 2^20, degree 10, k = 14 (the 64 GiB table).  With the fixture of
    tests/golden/make_roofline_golden.py (the reference's own complete run on
    the host cores): the whole table hashes to the reference's table and the
    costs are equal.  Without it: d[X][v] depends only on the terminals in X,
    so the reference's run on the first 10 terminals (ref_emv -kprefix 10:
    the 1024 rows X < 2^10) pins those rows bit for bit (the oracle's first 6
    terminals where the reference leg is not built).  Closure and
    monotonicity on sampled rows either way."""
    import json

    torch = pytest.importorskip("torch")
    from tests.golden.make_roofline_golden import OUT as GOLDEN, SPEC, instance_fnv_fast

    inst = emv.StpInstance.regular(SPEC["n"], SPEC["degree"], SPEC["wmin"], SPEC["wmax"], SPEC["k"], SPEC["seed"])
    csr = emv.Csr.from_stp(inst)
    dev = torch.device("cuda:0")
    row, col, w = (torch.from_numpy(a).to(dev) for a in (csr.row_ptr, csr.col, csr.w))
    n, k = csr.n, csr.k
    table = torch.empty(((1 << k), n), dtype=torch.int32, device=dev)
    with emv.Solver(0) as s:
        cost = s.kernel_dev(n, csr.arcs, row.data_ptr(), col.data_ptr(), w.data_ptr(), csr.terminals,
                            table.data_ptr(), n, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert cost == int(table[(1 << (k - 1)) - 1, int(csr.terminals[k - 1])])

    def rows_fnv(x0, x1, h=orc.FNV_BASIS, per_row=False):
        rows = []
        for X0 in range(x0, x1, 256):
            part = table[X0:min(x1, X0 + 256)].cpu().numpy()
            h = orc.fnv64(part, h)
            if per_row:
                rows += [orc.fnv64(part[i]) for i in range(part.shape[0])]
        return h, rows

    if os.path.exists(GOLDEN):
        with open(GOLDEN) as f:
            gold = json.load(f)
        assert instance_fnv_fast(orc, inst) == gold["instance_fnv"]
        assert cost == gold["cost"]
        h, _ = rows_fnv(0, 1 << k)
        assert f"{h:016x}" == gold["table_fnv"], "whole table differs from the reference's"
    elif orc.reference_available():
        kp = 10
        path = str(tmp_path / "roofline.stp")
        inst.write(path)
        rowfnv = str(tmp_path / "rows.bin")
        r = orc.ref_emv(path, kprefix=kp, rowfnv_out=rowfnv, threads=os.cpu_count())
        ref_rows = np.fromfile(rowfnv, dtype="<u8")
        assert r["k"] == kp and ref_rows.size == 1 << kp
        h, got_rows = rows_fnv(0, 1 << kp, per_row=True)
        bad = np.nonzero(np.array(got_rows, dtype=np.uint64) != ref_rows)[0]
        assert bad.size == 0, f"{bad.size} rows differ from the reference, first subsets {bad[:8].tolist()}"
        assert h == r["fnv"]
        # the cost of the 10-terminal prefix instance is a cell of the full table
        assert r["cost"] == int(table[(1 << (kp - 1)) - 1, int(csr.terminals[kp - 1])])
    else:
        want, _ = orc.emv_table(n, csr.row_ptr, csr.col, csr.w, csr.terminals[:6], threads=16)
        assert np.array_equal(table[:64].cpu().numpy(), want)
    src = np.repeat(np.arange(n), np.diff(csr.row_ptr))
    rng = np.random.default_rng(3)
    for X in rng.integers(1 << 10, 1 << k, size=4):
        r = table[int(X)].cpu().numpy()
        assert (r[csr.col] <= r[src] + csr.w).all()
        for b in range(k):
            if X >> b & 1 and X ^ (1 << b):
                assert (table[int(X) ^ (1 << b)].cpu().numpy() <= r).all()
    del table
    torch.cuda.empty_cache()
