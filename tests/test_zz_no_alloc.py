"""The allocation-free closure entry point (emv_closure_noalloc).

Callers that cannot allocate device memory -- their framework owns the
device's memory through its own pool, or a latency-critical loop must not pay
the device-wide synchronisation of cudaMalloc/cudaFree -- call this entry
point, whose working memory is a fixed array inside the library.  The tests
call it through the C ABI and compare it bit for bit, as every integer test
here, with the oracle's multi-source closure (one Dijkstra per row from a
virtual source) and with the solver's existing single-source entry point
(emv_sssp), on two calls in a row: the second call runs on the array the first
one left behind.  Also: the documented size limits (n = 131072, 32 rows), an
all-INF row, unreachable vertices, an odd stride, in-place use, and the input
checks (bad CSR, init above INF, a finite value reaching 2^30, a capturing
stream), after each of which the entry point still works.  The file sits on
its own and pytest collects it last.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev(torch, *arrays):
    dev = torch.device("cuda:0")
    return [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in arrays]


def _call(emv, torch, csr_t, n, arcs, init_t, rows, ld, out_t):
    row, col, w = csr_t
    stream = torch.cuda.current_stream().cuda_stream
    emv.Solver.closure_noalloc(n, arcs, row.data_ptr(), col.data_ptr(), w.data_ptr(), init_t.data_ptr(), rows, ld,
                               out_t.data_ptr(), stream)
    torch.cuda.synchronize()


def test_closure_noalloc_matches_oracle_and_sssp_on_two_calls(emv, orc):
    torch = pytest.importorskip("torch")
    inst = emv.StpInstance.regular(20000, 6, 1, 1000, 4, 2024)
    csr = emv.Csr.from_stp(inst)
    n = csr.n
    rng = np.random.default_rng(7)
    sources = rng.choice(n, size=12, replace=False)
    with emv.Solver(0) as s:
        dists = np.stack([s.sssp(csr, int(x))[0] for x in sources])
    rows = 14
    init = np.full((rows, n), emv.INF32, np.int32)
    for r in range(12):
        init[r, sources[r]] = 0
    offs = rng.integers(0, 500, size=12)
    init[12, sources] = offs  # one row seeded at all twelve sources
    init[13, sources[:3]] = offs[:3]
    want = orc.closure(n, csr.row_ptr, csr.col, csr.w, init)
    # the oracle agrees with the existing single-source entry point
    assert np.array_equal(want[:12], dists)
    assert np.array_equal(want[12], np.min(dists + offs[:, None], axis=0))

    csr_t = _dev(torch, csr.row_ptr, csr.col, csr.w)
    (d_init,) = _dev(torch, init)
    for _ in range(2):
        out = torch.full_like(d_init, -1)
        _call(emv, torch, csr_t, n, csr.arcs, d_init, rows, n, out)
        assert np.array_equal(out.cpu().numpy().astype(np.int64), want)

    # in place (out == init), with a stride larger than n
    ld = n + 3
    wide = torch.full((rows, ld), -5, dtype=torch.int32, device="cuda:0")
    wide[:, :n] = d_init
    _call(emv, torch, csr_t, n, csr.arcs, wide, rows, ld, wide)
    got = wide.cpu().numpy()
    assert np.array_equal(got[:, :n].astype(np.int64), want) and (got[:, n:] == -5).all()


def test_closure_noalloc_at_its_limits(emv, orc):
    """n = 131072 and 32 rows fill the fixed array (records, both flag arrays,
    then the control and status words); odd stride; row 31 all INF."""
    torch = pytest.importorskip("torch")
    n, rows = 131072, 32
    inst = emv.StpInstance.regular(n, 4, 1, 1000, 2, 99)
    csr = emv.Csr.from_stp(inst)
    rng = np.random.default_rng(11)
    ld = n + 1
    init = np.full((rows, ld), emv.INF32, np.int32)
    for r in range(rows - 1):
        seeds = rng.choice(n, size=1 + r % 5, replace=False)
        init[r, seeds] = rng.integers(0, 2000, size=seeds.size)
    init[:, n] = 77  # the padding column is never read
    want = orc.closure(n, csr.row_ptr, csr.col, csr.w, init[:, :n])
    assert (want[rows - 1] == emv.INF32).all()
    csr_t = _dev(torch, csr.row_ptr, csr.col, csr.w)
    (d_init,) = _dev(torch, init)
    for _ in range(2):
        out = torch.full((rows, ld), -9, dtype=torch.int32, device="cuda:0")
        _call(emv, torch, csr_t, n, csr.arcs, d_init, rows, ld, out)
        got = out.cpu().numpy()
        assert np.array_equal(got[:, :n].astype(np.int64), want)
        assert (got[:, n] == -9).all()


def test_closure_noalloc_unreachable_vertices_stay_inf(emv, orc):
    """Two components: seeds in the first leave the second at INF."""
    torch = pytest.importorskip("torch")
    a = emv.StpInstance.regular(3000, 4, 1, 100, 2, 5)
    b = emv.StpInstance.regular(2000, 6, 1, 100, 2, 6)
    edges = np.concatenate([a.edges, b.edges + np.array([a.n, a.n, 0])])
    inst = emv.StpInstance(a.n + b.n, edges, np.array([0, a.n], np.int64))
    csr = emv.Csr.from_stp(inst)
    n, rows = csr.n, 3
    init = np.full((rows, n), emv.INF32, np.int32)
    init[0, 10] = 0
    init[1, [5, 2999]] = [3, 1]
    want = orc.closure(n, csr.row_ptr, csr.col, csr.w, init)
    assert (want[:2, a.n:] == emv.INF32).all() and (want[:2, :a.n] < emv.INF32).all()
    assert (want[2] == emv.INF32).all()
    csr_t = _dev(torch, csr.row_ptr, csr.col, csr.w)
    (d_init,) = _dev(torch, init)
    out = torch.empty_like(d_init)
    _call(emv, torch, csr_t, n, csr.arcs, d_init, rows, n, out)
    assert np.array_equal(out.cpu().numpy().astype(np.int64), want)


def test_closure_noalloc_checks_its_inputs(emv, orc):
    """A head out of range and an init value above INF are EMV_ERR_BAD_INPUT;
    a finite value that would reach 2^30 is EMV_ERR_OVERFLOW, never a wrapped
    or silently INF result; a capturing stream is refused before the call
    touches it.  The entry point works again after each."""
    torch = pytest.importorskip("torch")
    big = (1 << 30) - 3
    # path 0 - 1 - 2 - 3: from vertex 0, d(0, 1) = 2^30 - 3 is finite but d(0, 2) would reach 2^30
    edges = np.array([[0, 1, big], [1, 2, 5], [2, 3, 1]], np.int64)
    path = emv.Csr.from_stp(emv.StpInstance(4, edges, np.array([0, 3], np.int64)))
    init = np.full((1, 4), emv.INF32, np.int32)
    init[0, 0] = 0
    csr_t = _dev(torch, path.row_ptr, path.col, path.w)
    (d_init,) = _dev(torch, init)
    out = torch.empty_like(d_init)
    with pytest.raises(emv.EmvError) as ei:
        _call(emv, torch, csr_t, 4, path.arcs, d_init, 1, 4, out)
    assert ei.value.status == 8  # EMV_ERR_OVERFLOW
    # seeded at vertex 1 instead, every value stays below 2^30
    init2 = np.full((1, 4), emv.INF32, np.int32)
    init2[0, 1] = 0
    (d_init2,) = _dev(torch, init2)
    _call(emv, torch, csr_t, 4, path.arcs, d_init2, 1, 4, out)
    assert out.cpu().numpy().tolist() == [[big, 0, 5, 6]]
    assert orc.closure(4, path.row_ptr, path.col, path.w, init2).tolist() == [[big, 0, 5, 6]]

    small = emv.Csr.from_stp(emv.StpInstance.regular(500, 4, 1, 50, 2, 3))
    init3 = np.full((2, 500), emv.INF32, np.int32)
    init3[0, 7] = 0
    init3[1, 9] = 4
    want = orc.closure(500, small.row_ptr, small.col, small.w, init3)
    bad_col = small.col.copy()
    bad_col[17] = 500
    for col, ini, status in ((bad_col, init3, 1), (small.col, np.where(init3 == 4, emv.INF32 + 1, init3), 1)):
        t = _dev(torch, small.row_ptr, col, small.w)
        (di,) = _dev(torch, ini.astype(np.int32))
        o = torch.empty_like(di)
        with pytest.raises(emv.EmvError) as ei:
            _call(emv, torch, t, 500, small.arcs, di, 2, 500, o)
        assert ei.value.status == status
    t = _dev(torch, small.row_ptr, small.col, small.w)
    (di,) = _dev(torch, init3)
    o = torch.empty_like(di)
    _call(emv, torch, t, 500, small.arcs, di, 2, 500, o)
    assert np.array_equal(o.cpu().numpy().astype(np.int64), want)

    # a capturing stream: refused with a status, the capture itself stays valid
    side = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    refused = None
    with torch.cuda.graph(graph, stream=side, capture_error_mode="thread_local"):
        o.add_(0)  # something for the graph to hold
        try:
            emv.Solver.closure_noalloc(500, small.arcs, t[0].data_ptr(), t[1].data_ptr(), t[2].data_ptr(),
                                       di.data_ptr(), 2, 500, o.data_ptr(), side.cuda_stream)
        except emv.EmvError as e:
            refused = e
    assert refused is not None and refused.status == 1 and "capturing" in str(refused)
    torch.cuda.synchronize()
    o.fill_(-1)
    _call(emv, torch, t, 500, small.arcs, di, 2, 500, o)
    assert np.array_equal(o.cpu().numpy().astype(np.int64), want)


def test_closure_noalloc_rejects_sizes_beyond_its_array(emv):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    dummy = torch.zeros(64, dtype=torch.int32, device=dev)
    p = dummy.data_ptr()
    with pytest.raises(emv.EmvError) as ei:
        emv.Solver.closure_noalloc(131073, 10, p, p, p, p, 1, 131073, p)
    assert ei.value.status == 1 and "exceed" in str(ei.value)
    with pytest.raises(emv.EmvError):
        emv.Solver.closure_noalloc(16, 10, p, p, p, p, 33, 16, p)
