"""The allocation-free closure entry point (emv_closure_noalloc).

Callers that cannot allocate device memory -- their framework owns the
device's memory through its own pool, or a latency-critical loop must not pay
the device-wide synchronisation of cudaMalloc/cudaFree -- call this entry
point, whose working memory is a fixed array inside the library.  The test
checks it through the C ABI against the solver's existing single-source entry
point (emv_sssp), bit for bit as every integer test here, on two calls in a
row: the second call runs on the array the first one left behind.  It sits in
a file of its own that pytest collects last.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_closure_noalloc_matches_sssp_on_two_calls(emv):
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
    want = np.empty((rows, n), np.int64)
    for r in range(12):
        init[r, sources[r]] = 0
        want[r] = dists[r]
    offs = rng.integers(0, 500, size=12)
    init[12, sources] = offs  # one row seeded at all twelve sources
    want[12] = np.min(dists + offs[:, None], axis=0)
    init[13, sources[:3]] = offs[:3]
    want[13] = np.min(dists[:3] + offs[:3, None], axis=0)

    dev = torch.device("cuda:0")
    row, col, w = (torch.from_numpy(a).to(dev) for a in (csr.row_ptr, csr.col, csr.w))
    d_init = torch.from_numpy(init).to(dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    for _ in range(2):
        out = torch.full_like(d_init, -1)
        emv.Solver.closure_noalloc(n, csr.arcs, row.data_ptr(), col.data_ptr(), w.data_ptr(), d_init.data_ptr(),
                                   rows, n, out.data_ptr(), stream)
        torch.cuda.synchronize()
        assert np.array_equal(out.cpu().numpy().astype(np.int64), want)

    # in place (out == init), with a stride larger than n
    ld = n + 3
    wide = torch.full((rows, ld), -5, dtype=torch.int32, device=dev)
    wide[:, :n] = d_init
    emv.Solver.closure_noalloc(n, csr.arcs, row.data_ptr(), col.data_ptr(), w.data_ptr(), wide.data_ptr(), rows, ld,
                               wide.data_ptr(), stream)
    torch.cuda.synchronize()
    got = wide.cpu().numpy()
    assert np.array_equal(got[:, :n].astype(np.int64), want) and (got[:, n:] == -5).all()


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
