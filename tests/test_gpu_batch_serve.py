"""Batched launch and continuous-batching server: every cost equals the
single-instance solve and the oracle, alone and in the mix; the batched
launch's whole tables equal the reference-written golden tables."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mixed(emv):
    """80 instances of the mixed distribution (n log-uniform in [64, 4096],
    degree {3,4,6,8}, k in [4, 10], about 10% group instances)."""
    return [emv.Csr.from_stp(emv.StpInstance.mixed(777, i)) for i in range(80)]


@pytest.fixture(scope="module")
def mixed_oracle(orc, mixed):
    """The oracle's cost of every instance of `mixed`."""
    return [orc.emv_table(g.n, g.row_ptr, g.col, g.w, g.terminals, threads=16)[1] for g in mixed]


def test_batch_costs_equal_single_and_oracle(emv, mixed, mixed_oracle):
    with emv.Solver(0) as s:
        costs, stats = s.batch_solve(mixed)
        single = [s.solve(g).cost for g in mixed]
    assert list(costs) == single == mixed_oracle
    assert stats["work_items"] == len(mixed) and stats["total_ms"] > 0


def test_batch_tables_equal_reference_golden(emv, orc, golden):
    """The 24 mixed golden cases (5 of them group instances with zero-weight
    root arcs) in one batched launch: every instance's whole table hashes to
    the table the reference's own emv_kernel wrote (tests/golden/golden.json),
    and equals the oracle's cell by cell; costs equal the golden costs."""
    from tests.golden.cases import CASES, instance_for, instance_fnv

    names = sorted(n for n in CASES if n.startswith("mixed_"))
    insts = [instance_for(CASES[n]) for n in names]
    graphs = [emv.Csr.from_stp(i) for i in insts]
    with emv.Solver(0) as s:
        costs, _, tables = s.batch_solve(graphs, tables=True)
        again, _, tables2 = s.batch_solve(graphs[::-1], tables=True)  # another launch order
    groups = 0
    for name, inst, g, c, t in zip(names, insts, graphs, costs, tables):
        gold = golden["cases"][name]
        assert instance_fnv(inst) == gold["instance_fnv"]
        assert c == gold["cost"], name
        assert f"{orc.fnv64(t):016x}" == gold["table_fnv"], name
        want, _ = orc.emv_table(g.n, g.row_ptr, g.col, g.w, g.terminals, threads=8)
        assert np.array_equal(t, want), name
        groups += bool((inst.edges[:, 2] == 0).any())
    assert groups >= 3
    assert list(again[::-1]) == list(costs)
    assert all(np.array_equal(a, b) for a, b in zip(tables, tables2[::-1]))


def test_batch_merge_tile_widths_equal_reference_golden(emv, orc, golden):
    """The merge's vertex-block width (32 * mw vertices, tuned per class) and
    the relaxation's rows per chunk change only the order of the work: with
    every width forced for every class, and with the tuned tables, every
    mixed golden instance's whole table still hashes to the reference's."""
    from tests.golden.cases import CASES, instance_for

    names = sorted(n for n in CASES if n.startswith("mixed_"))
    graphs = [emv.Csr.from_stp(instance_for(CASES[n])) for n in names]
    classes = emv.BATCH_CLASSES
    with emv.Solver(0) as s:
        for mw, rcap in ((1, 32), (2, 8), (4, 128), (8, 4)):
            s.batch_set_tiles([rcap] * classes, [mw] * classes)
            costs, _, tables = s.batch_solve(graphs, tables=True)
            for name, c, t in zip(names, costs, tables):
                gold = golden["cases"][name]
                assert c == gold["cost"], (name, mw)
                assert f"{orc.fnv64(t):016x}" == gold["table_fnv"], (name, mw)
        rcap_t, mw_t = s.batch_autotune_tiles(graphs)
        costs, _, tables = s.batch_solve(graphs, tables=True)
    assert set(int(x) for x in rcap_t) <= {0, 4, 8, 16, 32, 64, 128} and rcap_t.max() > 0
    assert set(int(x) for x in mw_t) <= {0, 1, 2, 4, 8} and mw_t.max() > 0
    assert all((r > 0) == (w > 0) for r, w in zip(rcap_t, mw_t))
    for name, c, t in zip(names, costs, tables):
        assert f"{orc.fnv64(t):016x}" == golden["cases"][name]["table_fnv"], name


def test_batch_repeat_and_autotune(emv, mixed):
    with emv.Solver(0) as s:
        a, _ = s.batch_solve(mixed)
        b, _ = s.batch_solve(mixed)  # replays the captured graph
        table = s.batch_autotune(mixed)
        c, st = s.batch_solve(mixed)
    assert np.array_equal(a, b) and np.array_equal(a, c)
    assert set(int(x) for x in table) <= {0, 4, 8, 16, 32, 64, 128} and table.max() > 0


def test_batch_group_instances(emv, orc):
    groups = []
    i = 0
    while len(groups) < 6:
        inst = emv.StpInstance.mixed(4242, i)
        i += 1
        if (inst.edges[:, 2] == 0).any():
            groups.append(emv.Csr.from_stp(inst))
    with emv.Solver(0) as s:
        costs, _ = s.batch_solve(groups)
    for g, c in zip(groups, costs):
        _, want = orc.emv_table(g.n, g.row_ptr, g.col, g.w, g.terminals, threads=8)
        assert c == want


def test_batch_rejects_out_of_range(emv):
    big_k = emv.Csr.from_stp(emv.StpInstance.regular(200, 4, 1, 10, 11, 1))
    with emv.Solver(0) as s:
        with pytest.raises(emv.EmvError) as ei:
            s.batch_solve([big_k])
        assert ei.value.status == 1


@pytest.mark.parametrize("wave_sms", [0, -1, 3])
def test_server_result_same_alone_and_in_mix(emv, orc, mixed, mixed_oracle, wave_sms):
    """Continuous batching: a request's cost is the same when it runs alone
    and when it shares waves with 80 others plus a large request that runs on
    the multi-CTA path concurrently, and every served cost equals the
    oracle's (the large one's: equal to the plain GPU solve, whose table is
    pinned to the reference elsewhere).  wave_sms: the default split of the
    SMs beside a large solve, none (waves and the large solve take turns),
    and a narrow one (waves on 3 SMs, the large solve's relaxation grids on
    the rest)."""
    probe = mixed[5]
    large = emv.Csr.from_stp(emv.StpInstance.regular(70000, 8, 1, 1000, 9, 99))
    with emv.Solver(0) as s:
        want = {i: s.solve(g).cost for i, g in enumerate(mixed)}
        want_large = s.solve(large).cost
    assert [want[i] for i in range(len(mixed))] == mixed_oracle
    with emv.Server(0, hbm_budget_bytes=20 * 10**9, max_slots=256, large_n=65536, wave_sms=wave_sms) as srv:
        rid = srv.submit(probe)
        alone, _ = srv.wait(rid)
        assert alone == want[5]
        ids = {}
        lid = None
        for i, g in enumerate(mixed):
            ids[srv.submit(g)] = i
            if i == 20:
                lid = srv.submit(large)  # starts with small requests resident: the SMs are split
            if i % 10 == 0:
                time.sleep(0.002)  # arrivals while earlier requests are on the GPU
        for r, i in ids.items():
            cost, lat = srv.wait(r)
            assert cost == want[i], i
            assert lat >= 0
        assert srv.wait(lid)[0] == want_large
        st = srv.stats()
    assert st["completed"] == len(mixed) + 2
    assert st["peak_resident"] > 1 and st["waves"] >= 10


def test_server_admission_budget_and_cancel(emv, mixed):
    one = mixed[0]
    need = (one.n << one.k) * 4
    with emv.Server(0, hbm_budget_bytes=need // 2, max_slots=8) as srv:
        with pytest.raises(emv.EmvError) as ei:
            srv.submit(one)
        assert ei.value.status == 4  # EMV_ERR_OVER_BUDGET
        assert srv.stats()["rejected"] == 1
    budget = 3 * max((g.n << g.k) * 4 + 64 * g.n for g in mixed[:20])
    with emv.Server(0, hbm_budget_bytes=budget, max_slots=4) as srv:
        ids = [srv.submit(g) for g in mixed[:20]]
        srv.cancel(ids[-1])
        done = 0
        for r in ids[:-1]:
            srv.wait(r)
            done += 1
        try:
            srv.wait(ids[-1])  # finished before the cancel reached it
        except emv.EmvError as e:
            assert e.status == 10  # EMV_ERR_CANCELLED
        assert done == 19
        st = srv.stats()
    assert st["peak_resident"] <= 4 and st["peak_bytes"] <= budget


def test_autotune_first_on_fresh_context(emv):
    """Autotune samples instances by class; their cost slots are the callers'
    indices, which can exceed the sample size (a fresh context has no larger
    cost buffer from an earlier batch)."""
    graphs = [emv.Csr.from_stp(emv.StpInstance.mixed(31, i)) for i in range(300)]
    with emv.Solver(0) as s:
        table = s.batch_autotune(graphs)
        costs, _ = s.batch_solve(graphs)
        ref = [s.solve(g).cost for g in graphs[::25]]
    assert table.max() > 0
    assert list(costs[::25]) == ref
