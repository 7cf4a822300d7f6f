// emv_batch.cu -- many independent instances in one persistent launch (C ABI),
// and the autotuner that picks the per-class tile shapes.
//
// No counterpart in the reference, which solves one instance per process
// (reader/reader-el.c:2355-2536); each instance's values are those of its
// emv_kernel (R:1966-2139).
#include "emv_batch.cuh"
#include "emv_solver.h"
#include "emv_batch_host.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

namespace {

// f(i) for i in [0, count) on up to 16 host threads (chunks of 16 indices).
template <class F> void host_parallel_for(int64_t count, F f)
{
    const unsigned hw = std::thread::hardware_concurrency();
    const int64_t T = std::min<int64_t>({16, (int64_t)(hw ? hw : 1), (count + 63) / 64});
    if (T <= 1) {
        for (int64_t i = 0; i < count; i++) f(i);
        return;
    }
    std::atomic<int64_t> next{0};
    auto work = [&]() {
        for (;;) {
            const int64_t i0 = next.fetch_add(16);
            if (i0 >= count) return;
            for (int64_t i = i0; i < std::min(count, i0 + 16); i++) f(i);
        }
    };
    std::vector<std::thread> th;
    for (int64_t t = 1; t < T; t++) th.emplace_back(work);
    work();
    for (std::thread &t : th) t.join();
}

}  // namespace

using namespace emv;

namespace {

int32_t pow2_floor(int32_t x)
{
    int32_t p = 1;
    while (p * 2 <= x) p *= 2;
    return p;
}

}  // namespace

int32_t batch_class_of(int32_t n, int32_t k)
{
    const int32_t nb = n <= 256 ? 0 : n <= 1024 ? 1 : n <= 4096 ? 2 : 3;
    const int32_t kb = k <= 6 ? 0 : k <= 8 ? 1 : 2;
    return nb * 3 + kb;
}

// Largest rows-per-chunk whose vertex-major buffer fits the shared memory.
int32_t batch_rcap_max(int32_t n)
{
    int32_t r = BATCH_RCAP_MAX;
    while (r > 1 && (int64_t)n * batch_stride(r) * 4 > BATCH_SMEM_BYTES) r /= 2;
    return r;
}

bool batch_fits(int32_t n, int32_t k)
{
    return k >= 1 && k <= BATCH_KMAX && (int64_t)n * 2 * 4 <= BATCH_SMEM_BYTES &&
           ((int64_t)32 << k) * 4 <= BATCH_SMEM_BYTES;
}

int32_t batch_rcap_for(const emv_ctx *c, int32_t n, int32_t k)
{
    const int32_t cap = batch_rcap_max(n);
    const int32_t cls = batch_class_of(n, k);
    int32_t r = (cls >= 0 && cls < BATCH_CLASSES && c->tune_rcap[cls] > 0) ? c->tune_rcap[cls] : 32;
    return std::min(cap, pow2_floor(std::max(1, r)));
}

// Largest merge block width (in 32-vertex columns) whose staged rows fit the
// shared memory, and no wider than the instance.
int32_t batch_mw_max(int32_t n, int32_t k)
{
    int32_t mw = BATCH_MW_MAX;
    while (mw > 1 && (((int64_t)32 * mw << k) * 4 > BATCH_SMEM_BYTES || 32 * (mw / 2) >= n)) mw /= 2;
    return mw;
}

int32_t batch_mw_for(const emv_ctx *c, int32_t n, int32_t k)
{
    const int32_t cls = batch_class_of(n, k);
    const int32_t w = (cls >= 0 && cls < BATCH_CLASSES && c->tune_mw[cls] > 0) ? c->tune_mw[cls] : 1;
    return std::min(batch_mw_max(n, k), pow2_floor(std::max(1, w)));
}

int prepare_batch_subsets(emv_ctx *c, cudaStream_t st)
{
    if (c->bxs_ready) return EMV_OK;
    std::vector<uint32_t> all;
    std::vector<int32_t> off((size_t)(BATCH_KMAX + 1) * (BATCH_KMAX + 2), 0);
    for (int32_t k = 1; k <= BATCH_KMAX; k++) {
        std::vector<uint32_t> xs;
        std::vector<int64_t> lo;
        subset_levels(k, xs, lo);
        const int32_t base = (int32_t)all.size();
        for (int32_t m = 0; m <= k + 1; m++) off[(size_t)k * (BATCH_KMAX + 2) + m] = base + (int32_t)lo[(size_t)m];
        all.insert(all.end(), xs.begin(), xs.end());
    }
    int r = dev_reserve(c->bxs, sizeof(uint32_t) * all.size());
    if (!r) r = dev_reserve(c->bxs_off, sizeof(int32_t) * off.size());
    if (r) return r;
    CUDA_TRY(cudaMemcpyAsync(c->bxs.ptr, all.data(), sizeof(uint32_t) * all.size(), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(c->bxs_off.ptr, off.data(), sizeof(int32_t) * off.size(), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    c->bxs_ready = true;
    return EMV_OK;
}

int batch_kernel_setup(emv_ctx *c)
{
    if (c->batch_blocks > 0) return EMV_OK;
    CUDA_TRY(cudaFuncSetAttribute(k_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, BATCH_SMEM_BYTES));
    int per_sm = 0;
    CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch, BATCH_THREADS, BATCH_SMEM_BYTES));
    c->batch_blocks = std::max(1, per_sm) * c->sms;
    return EMV_OK;
}

// Launches k_batch over `count` prepared descriptors (device arrays already set).
int launch_batch(emv_ctx *c, const BatchArgs &args, int32_t count, cudaStream_t st, int32_t max_blocks)
{
    int r = batch_kernel_setup(c);
    if (r) return r;
    CUDA_TRY(cudaMemsetAsync(args.queue, 0, sizeof(uint32_t), st));
    const int cap = max_blocks > 0 ? std::min(max_blocks, c->batch_blocks) : c->batch_blocks;
    const int blocks = std::min(cap, std::max(1, count));
    BatchArgs a = args;
    k_batch<<<blocks, BATCH_THREADS, BATCH_SMEM_BYTES, st>>>(a);
    CUDA_TRY(cudaGetLastError());
    return EMV_OK;
}

// Estimated device work of one instance, for largest-first ordering.
double batch_work(int32_t n, int32_t k, int64_t arcs)
{
    return std::pow(3.0, k) * n * 0.5 + std::pow(2.0, k) * (double)arcs * 6.0;
}

// emv_batch_solve and emv_batch_solve_tables: tables_out (or null) receives
// the finished table of every instance whose entry is not null.
static int batch_solve(emv_ctx *c, const emv_instance *inst, int32_t count, int64_t *costs_out,
                       int32_t *const *tables_out, emv_batch_stats *stats, void *stream)
{
    if (!c || (count > 0 && (!inst || !costs_out)) || count < 0)
        return emv_fail(EMV_ERR_BAD_INPUT, "emv_batch_solve: bad arguments");
    if (count == 0) return EMV_OK;
    CUDA_TRY(cudaSetDevice(c->device));
    cudaStream_t st = (cudaStream_t)stream;
    const auto t0 = std::chrono::steady_clock::now();
    // Admission checks of every instance, in parallel on the host; the first
    // failing instance (lowest index) is reported.
    std::vector<int> bad((size_t)count, 0);
    std::vector<std::string> why((size_t)count);
    host_parallel_for(count, [&](int64_t i) {
        const emv_instance &I = inst[i];
        int r = emv_graph_validate(&I.g);
        if (!r && !batch_fits(I.g.n, I.k))
            r = emv_fail(EMV_ERR_BAD_INPUT, "n = %d, k = %d outside the batched range (k <= %d)", I.g.n, I.k, BATCH_KMAX);
        if (!r && !I.terminals) r = emv_fail(EMV_ERR_BAD_INPUT, "null terminals");
        for (int32_t t = 0; !r && t < I.k; t++)
            if (I.terminals[t] < 0 || I.terminals[t] >= I.g.n) r = emv_fail(EMV_ERR_BAD_INPUT, "terminal out of range");
        if (!r) r = emv_graph_check(&I.g, nullptr);
        if (r) {
            bad[(size_t)i] = r;
            why[(size_t)i] = emv_last_error();
        }
    });
    for (int32_t i = 0; i < count; i++)
        if (bad[(size_t)i]) return emv_fail(bad[(size_t)i], "instance %d: %s", i, why[(size_t)i].c_str());
    // Largest first, so the persistent CTAs finish together.
    std::vector<int32_t> order((size_t)count);
    for (int32_t i = 0; i < count; i++) order[(size_t)i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int32_t x, int32_t y) {
        return batch_work(inst[x].g.n, inst[x].k, inst[x].g.arcs) > batch_work(inst[y].g.n, inst[y].k, inst[y].g.arcs);
    });
    BatchPack pk;
    int r = batch_pack(c, inst, order, 1, -1, pk);
    if (r) return r;
    r = batch_upload(c, pk, st);
    if (r) return r;
    CUDA_TRY(cudaEventRecord(c->ev[0], st));
    BatchArgs a = batch_args(c, pk);
    // The queue reset and the persistent launch are replayed as one CUDA graph.
    r = batch_graph_launch(c, a, count, st);
    if (r) return r;
    CUDA_TRY(cudaEventRecord(c->ev[1], st));
    CUDA_TRY(cudaMemcpyAsync(costs_out, a.costs, sizeof(int64_t) * (size_t)count, cudaMemcpyDeviceToHost, st));
    uint32_t err = 0;
    CUDA_TRY(cudaMemcpyAsync(&err, a.err, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    if (err) return emv_dev_status_to_emv(err);
    if (tables_out) {
        // instance order[j] ran in launch slot j; its table (ld = n) is at table_off[j]
        for (int32_t j = 0; j < count; j++) {
            const int32_t i = order[(size_t)j];
            if (!tables_out[i]) continue;
            const size_t words = (size_t)inst[i].g.n << inst[i].k;
            CUDA_TRY(cudaMemcpyAsync(tables_out[i], (const int32_t *)c->b_table.ptr + pk.table_off[(size_t)j],
                                     sizeof(int32_t) * words, cudaMemcpyDeviceToHost, st));
        }
        CUDA_TRY(cudaStreamSynchronize(st));
    }
    if (stats) {
        float ms = 0;
        cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]);
        stats->total_ms = ms;
        stats->upload_ms = (float)std::chrono::duration<double, std::milli>(pk.t_upload_end - t0).count();
        stats->work_items = count;
        stats->table_bytes = pk.table_words * 4;
        stats->merge_tile = 32;
        stats->relax_rows = pk.rcap_used;
    }
    return EMV_OK;
}

extern "C" int emv_batch_solve(emv_ctx *c, const emv_instance *inst, int32_t count, int64_t *costs_out,
                               emv_batch_stats *stats, void *stream)
{
    return batch_solve(c, inst, count, costs_out, nullptr, stats, stream);
}

extern "C" int emv_batch_solve_tables(emv_ctx *c, const emv_instance *inst, int32_t count, int64_t *costs_out,
                                      int32_t *const *tables_out, emv_batch_stats *stats, void *stream)
{
    if (!tables_out) return emv_fail(EMV_ERR_BAD_INPUT, "emv_batch_solve_tables: null table list");
    return batch_solve(c, inst, count, costs_out, tables_out, stats, stream);
}

// ---------------------------------------------------------------- packing

int batch_pack(emv_ctx *c, const emv_instance *inst, const std::vector<int32_t> &order, int32_t lo, int32_t hi,
               BatchPack &pk)
{
    const int32_t count = (int32_t)order.size();
    pk.desc.resize((size_t)count);
    pk.row_off.resize((size_t)count);
    pk.arc_off.resize((size_t)count);
    pk.term_off.resize((size_t)count);
    pk.table_off.resize((size_t)count);
    int64_t rows = 0, arcs = 0, terms = 0, words = 0;
    for (int32_t j = 0; j < count; j++) {
        const emv_instance &I = inst[order[(size_t)j]];
        BatchInst &d = pk.desc[(size_t)j];
        std::memset(&d, 0, sizeof(d));
        d.n = I.g.n;
        d.k = I.k;
        d.rcap = batch_rcap_for(c, I.g.n, I.k);
        d.mw = batch_mw_for(c, I.g.n, I.k);
        d.orig = order[(size_t)j];
        d.lo = lo;
        d.hi = hi < 0 ? I.k : hi;
        pk.row_off[(size_t)j] = rows;
        pk.arc_off[(size_t)j] = arcs;
        pk.term_off[(size_t)j] = terms;
        pk.table_off[(size_t)j] = words;
        rows += I.g.n + 1;
        arcs += I.g.arcs;
        terms += I.k;
        words += ((int64_t)I.g.n << I.k);
        pk.rcap_used = std::max(pk.rcap_used, d.rcap);
        pk.cost_slots = std::max<int64_t>(pk.cost_slots, (int64_t)d.orig + 1);
    }
    pk.rows = rows;
    pk.arcs = arcs;
    pk.terms = terms;
    pk.table_words = words;
    pk.count = count;
    // Host staging (pinned, reused): row_ptr | adj | terms | desc
    const size_t bytes = sizeof(int32_t) * (size_t)rows + sizeof(int2) * (size_t)arcs + sizeof(int32_t) * (size_t)terms +
                         sizeof(BatchInst) * (size_t)count + 64;
    if (c->bstage_bytes < bytes) {
        if (c->bstage) cudaFreeHost(c->bstage);
        c->bstage = nullptr;
        c->bstage_bytes = 0;
        if (cudaMallocHost(&c->bstage, bytes) != cudaSuccess) {
            cudaGetLastError();
            return emv_fail(EMV_ERR_OOM, "pinned staging of %zu bytes", bytes);
        }
        c->bstage_bytes = bytes;
    }
    char *p = (char *)c->bstage;
    int32_t *hrow = (int32_t *)p;
    int2 *hadj = (int2 *)(hrow + rows);
    int32_t *hterm = (int32_t *)(hadj + arcs);
    BatchInst *hdesc = (BatchInst *)(((uintptr_t)(hterm + terms) + 15) & ~(uintptr_t)15);
    host_parallel_for(count, [&](int64_t j) {  // disjoint ranges of the staging buffer
        const emv_instance &I = inst[order[(size_t)j]];
        std::memcpy(hrow + pk.row_off[(size_t)j], I.g.row_ptr, sizeof(int32_t) * ((size_t)I.g.n + 1));
        int2 *ha = hadj + pk.arc_off[(size_t)j];
        for (int64_t e = 0; e < I.g.arcs; e++) ha[e] = make_int2(I.g.col[e], I.g.w[e]);
        std::memcpy(hterm + pk.term_off[(size_t)j], I.terminals, sizeof(int32_t) * (size_t)I.k);
    });
    std::memcpy(hdesc, pk.desc.data(), sizeof(BatchInst) * (size_t)count);
    pk.h_row = hrow;
    pk.h_adj = hadj;
    pk.h_term = hterm;
    pk.h_desc = hdesc;
    return EMV_OK;
}

int batch_upload(emv_ctx *c, BatchPack &pk, cudaStream_t st)
{
    int r = dev_reserve(c->b_row, sizeof(int32_t) * (size_t)pk.rows);
    if (!r) r = dev_reserve(c->b_adj, sizeof(int2) * (size_t)std::max<int64_t>(pk.arcs, 1));
    if (!r) r = dev_reserve(c->b_term, sizeof(int32_t) * (size_t)std::max<int64_t>(pk.terms, 1));
    if (!r) r = dev_reserve(c->b_desc, sizeof(BatchInst) * (size_t)pk.count);
    if (!r) r = dev_reserve(c->b_table, sizeof(int32_t) * (size_t)pk.table_words);
    // costs are written at index orig (the caller's instance index), which can
    // exceed the number of instances in this launch when it is a sample
    if (!r) r = dev_reserve(c->b_costs, sizeof(int64_t) * (size_t)std::max<int64_t>(pk.cost_slots, 1));
    if (!r) r = dev_reserve(c->b_ctrl, 64);
    if (!r) r = prepare_batch_subsets(c, st);
    if (r) return r;
    for (int32_t j = 0; j < pk.count; j++) {
        BatchInst &d = pk.h_desc[j];
        if (d.orig < 0 || d.orig >= pk.cost_slots) return emv_fail(EMV_ERR_INTERNAL, "batch: cost slot out of range");
        d.row_ptr = (const int32_t *)c->b_row.ptr + pk.row_off[(size_t)j];
        d.adj = (const int2 *)c->b_adj.ptr + pk.arc_off[(size_t)j];
        d.terms = (const int32_t *)c->b_term.ptr + pk.term_off[(size_t)j];
        d.table = (int32_t *)c->b_table.ptr + pk.table_off[(size_t)j];
        pk.desc[(size_t)j] = d;
    }
    CUDA_TRY(cudaMemcpyAsync(c->b_row.ptr, pk.h_row, sizeof(int32_t) * (size_t)pk.rows, cudaMemcpyHostToDevice, st));
    if (pk.arcs > 0)
        CUDA_TRY(cudaMemcpyAsync(c->b_adj.ptr, pk.h_adj, sizeof(int2) * (size_t)pk.arcs, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(c->b_term.ptr, pk.h_term, sizeof(int32_t) * (size_t)pk.terms, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(c->b_desc.ptr, pk.h_desc, sizeof(BatchInst) * (size_t)pk.count, cudaMemcpyHostToDevice,
                             st));
    CUDA_TRY(cudaMemsetAsync(c->b_ctrl.ptr, 0, 64, st));
    pk.t_upload_end = std::chrono::steady_clock::now();
    return EMV_OK;
}

BatchArgs batch_args(emv_ctx *c, const BatchPack &pk)
{
    BatchArgs a;
    std::memset(&a, 0, sizeof(a));  // padding included: the graph cache compares bytes
    a.inst = (const BatchInst *)c->b_desc.ptr;
    a.count = pk.count;
    a.xs = (const uint32_t *)c->bxs.ptr;
    a.xs_off = (const int32_t *)c->bxs_off.ptr;
    a.costs = (int64_t *)c->b_costs.ptr;
    a.queue = (uint32_t *)c->b_ctrl.ptr;
    a.err = (uint32_t *)c->b_ctrl.ptr + 8;
    return a;
}

// Captures {queue reset, persistent kernel} once per argument set and replays it.
int batch_graph_launch(emv_ctx *c, const BatchArgs &a, int32_t count, cudaStream_t st)
{
    int r = batch_kernel_setup(c);
    if (r) return r;
    static_assert(sizeof(BatchArgs) <= sizeof(c->bgraph_args), "graph key too small");
    const bool same = c->bgraph_exec && std::memcmp(c->bgraph_args, &a, sizeof(a)) == 0;
    if (!same) {
        if (c->bgraph_exec) cudaGraphExecDestroy(c->bgraph_exec);
        c->bgraph_exec = nullptr;
        cudaStream_t cap;
        CUDA_TRY(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            r = launch_batch(c, a, count, cap);
            e = cudaStreamEndCapture(cap, &g);
        }
        cudaStreamDestroy(cap);
        if (r) return r;
        if (e != cudaSuccess) {
            cudaGetLastError();
            return emv_fail(EMV_ERR_CUDA, "batch graph capture: %s", cudaGetErrorString(e));
        }
        e = cudaGraphInstantiate(&c->bgraph_exec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            cudaGetLastError();
            c->bgraph_exec = nullptr;
            return emv_fail(EMV_ERR_CUDA, "batch graph instantiate: %s", cudaGetErrorString(e));
        }
        std::memcpy(c->bgraph_args, &a, sizeof(a));
    }
    CUDA_TRY(cudaGraphLaunch(c->bgraph_exec, st));
    return EMV_OK;
}

// --------------------------------------------------------------- autotuner

namespace {

// Device time of one batched launch over the sample `ids` with the current
// tuning, at about four sample instances per block, as in a full batch where
// every block solves many: the time then follows a block's throughput, not
// the single slowest instance.  Best of three.
int time_sample(emv_ctx *c, const emv_instance *inst, const std::vector<int32_t> &ids, cudaStream_t st, float &ms)
{
    BatchPack pk;
    int r = batch_pack(c, inst, ids, 1, -1, pk);
    if (!r) r = batch_upload(c, pk, st);
    if (r) return r;
    BatchArgs a = batch_args(c, pk);
    const int32_t blocks = std::max<int32_t>(1, (pk.count + 3) / 4);
    ms = 1e30f;
    for (int rep = 0; rep < 3; rep++) {
        CUDA_TRY(cudaEventRecord(c->ev[0], st));
        r = launch_batch(c, a, pk.count, st, blocks);
        if (r) return r;
        CUDA_TRY(cudaEventRecord(c->ev[1], st));
        CUDA_TRY(cudaStreamSynchronize(st));
        float t = 0;
        cudaEventElapsedTime(&t, c->ev[0], c->ev[1]);
        ms = std::min(ms, t);
    }
    return EMV_OK;
}

}  // namespace

// For every instance class present in `inst`, times the relaxation's
// rows-per-chunk candidates on a sample of that class and keeps the fastest,
// then, with it, the merge's vertex-block widths (32, 64, 128 or 256
// vertices; candidates whose staged rows do not fit are skipped) and keeps
// the fastest (in the context, and in out_rcap / out_mw[class] when given).
static int batch_autotune(emv_ctx *c, const emv_instance *inst, int32_t count, int32_t *out_rcap, int32_t *out_mw,
                   cudaStream_t st)
{
    std::vector<std::vector<int32_t>> by_class(BATCH_CLASSES);
    for (int32_t i = 0; i < count; i++) {
        if (!batch_fits(inst[i].g.n, inst[i].k)) continue;
        const int32_t cls = batch_class_of(inst[i].g.n, inst[i].k);
        if (by_class[(size_t)cls].size() < 64) by_class[(size_t)cls].push_back(i);
    }
    for (int32_t cls = 0; cls < BATCH_CLASSES; cls++) {
        auto &ids = by_class[(size_t)cls];
        if (ids.empty()) continue;
        int32_t nmax = 0, kmin = BATCH_KMAX;
        for (int32_t i : ids) {
            nmax = std::max(nmax, inst[i].g.n);
            kmin = std::min(kmin, inst[i].k);
        }
        c->tune_mw[cls] = 1;
        float best_ms = 1e30f;
        int32_t best = 0;
        for (int32_t cand : {4, 8, 16, 32, 64, 128}) {
            c->tune_rcap[cls] = cand;
            float ms = 0;
            const int r = time_sample(c, inst, ids, st, ms);
            if (r) return r;
            if (ms < best_ms) {
                best_ms = ms;
                best = cand;
            }
        }
        c->tune_rcap[cls] = best;
        int32_t best_mw = 1;
        for (int32_t mw = 2; mw <= BATCH_MW_MAX && mw <= batch_mw_max(nmax, kmin); mw *= 2) {
            c->tune_mw[cls] = mw;
            float ms = 0;
            const int r = time_sample(c, inst, ids, st, ms);
            if (r) return r;
            if (ms < best_ms) {
                best_ms = ms;
                best_mw = mw;
            }
        }
        c->tune_mw[cls] = best_mw;
    }
    if (out_rcap)
        for (int32_t cls = 0; cls < BATCH_CLASSES; cls++) out_rcap[cls] = c->tune_rcap[cls];
    if (out_mw)
        for (int32_t cls = 0; cls < BATCH_CLASSES; cls++) out_mw[cls] = c->tune_mw[cls];
    return EMV_OK;
}

extern "C" int emv_batch_autotune(emv_ctx *c, const emv_instance *inst, int32_t count, int32_t *out_rcap,
                                  void *stream)
{
    if (!c || (count > 0 && !inst)) return emv_fail(EMV_ERR_BAD_INPUT, "emv_batch_autotune: bad arguments");
    CUDA_TRY(cudaSetDevice(c->device));
    return batch_autotune(c, inst, count, out_rcap, nullptr, (cudaStream_t)stream);
}

extern "C" int emv_batch_autotune2(emv_ctx *c, const emv_instance *inst, int32_t count, int32_t *out_rcap,
                                   int32_t *out_mw, void *stream)
{
    if (!c || (count > 0 && !inst)) return emv_fail(EMV_ERR_BAD_INPUT, "emv_batch_autotune2: bad arguments");
    CUDA_TRY(cudaSetDevice(c->device));
    return batch_autotune(c, inst, count, out_rcap, out_mw, (cudaStream_t)stream);
}

extern "C" int emv_batch_set_tuning2(emv_ctx *c, const int32_t *rcap, const int32_t *mw, int32_t classes)
{
    if (!c || !rcap || !mw || classes != BATCH_CLASSES)
        return emv_fail(EMV_ERR_BAD_INPUT, "emv_batch_set_tuning2: bad arguments");
    for (int32_t i = 0; i < classes; i++)
        if (rcap[i] < 0 || mw[i] < 0) return emv_fail(EMV_ERR_BAD_INPUT, "emv_batch_set_tuning2: negative entry");
    for (int32_t i = 0; i < classes; i++) {
        c->tune_rcap[i] = rcap[i];
        c->tune_mw[i] = mw[i];
    }
    return EMV_OK;
}

extern "C" int emv_batch_set_tuning(emv_ctx *c, const int32_t *rcap, int32_t classes)
{
    if (!c || !rcap || classes != BATCH_CLASSES) return emv_fail(EMV_ERR_BAD_INPUT, "emv_batch_set_tuning: bad arguments");
    for (int32_t i = 0; i < classes; i++) c->tune_rcap[i] = rcap[i];
    return EMV_OK;
}
