// emv_server.cpp -- continuous-batching request loop on one GPU (C ABI).
//
// No counterpart in the reference (one instance per process, reader-el.c:2355).
// Requests are admitted by their device footprint (table 2^k*n*4 bytes plus
// the graph) against a byte budget and a slot limit.  A scheduler thread runs
// "waves": one launch of the persistent CTA-resident solver (emv_batch.cuh)
// in which every resident request advances by exactly one DP level, so
// requests that arrive while others are on the GPU join at the next wave and
// levels of different requests interleave.  Tables stay resident in HBM
// across levels (stream-ordered allocations).  Requests too large for one
// CTA (n above large_n, or k above the batched range) go to a second worker
// that runs the multi-CTA solver on its own stream, concurrently with the
// waves.  A wave block takes a whole SM, and a relaxation grid must be
// resident at once, so while a large request runs with small ones resident
// the two split the SMs: the large solve's relaxation grids are sized for
// all but wave_sms SMs, and the waves launch at most wave_sms blocks (one per
// SM).  Neither then waits for the other's blocks to drain.  Every call is
// thread-safe.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "emv_batch_host.h"
#include "emv_solver.h"

using namespace emv;
using Clock = std::chrono::steady_clock;

int solve_on_device(emv_ctx *c, int32_t n, int64_t arcs, const int32_t *row_ptr, const int32_t *col,
                    const int32_t *w, const int32_t *terms, int32_t k, int32_t flags, emv_result *out,
                    cudaStream_t st);

namespace {

enum ReqState { Q_QUEUED, Q_RESIDENT, Q_DONE, Q_FAILED, Q_CANCELLED };

struct Req {
    int64_t id = 0;
    int32_t n = 0, k = 0;
    int64_t arcs = 0;
    std::vector<int32_t> row, col, w, terms;
    int64_t bytes = 0;
    bool large = false;
    int state = Q_QUEUED;
    bool cancel = false;
    int32_t next_level = 1;
    int32_t slot = -1;
    int64_t cost = 0;
    int status = EMV_OK;
    Clock::time_point t_submit, t_done;
    // device (small requests)
    int32_t *d_row = nullptr;
    int2 *d_adj = nullptr;
    int32_t *d_terms = nullptr;
    int32_t *d_table = nullptr;
};

int64_t footprint(int32_t n, int32_t k, int64_t arcs)
{
    return ((int64_t)n << k) * 4 + (int64_t)(n + 1) * 4 + arcs * 8 + (int64_t)k * 4;
}

}  // namespace

struct emv_server {
    emv_server_opts opts{};
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Req *> queue_small, queue_large;
    std::vector<Req *> resident;     // small requests on the GPU
    std::unordered_map<int64_t, Req *> reqs;
    int64_t next_id = 1;
    int64_t resident_bytes = 0;
    int64_t resident_count = 0;
    bool stop = false;
    emv_server_stats stats{};
    std::thread sched, large_worker;
    emv_ctx *ctx_small = nullptr;
    emv_ctx *ctx_large = nullptr;
    cudaStream_t st_small = nullptr, st_large = nullptr;
    // wave buffers
    std::vector<int32_t> free_slots;
    DevBuf d_desc, d_costs, d_ctrl;
    BatchInst *h_desc = nullptr;
    int64_t *h_costs = nullptr;
    int32_t cap_slots = 0;
    int32_t wave_sms = 0;                  // SMs the waves keep while a large request runs (0: no split)
    std::atomic<bool> large_sharing{false};  // a large solve runs on the other SMs
};

namespace {

void finish(emv_server *s, Req *r, int status, int64_t cost)
{
    r->status = status;
    r->cost = cost;
    r->state = status == EMV_OK ? Q_DONE : (status == EMV_ERR_CANCELLED ? Q_CANCELLED : Q_FAILED);
    r->t_done = Clock::now();
    if (status == EMV_OK) s->stats.completed++;
}

void release_device(emv_server *s, Req *r)
{
    cudaStream_t st = s->st_small;
    if (r->d_row) cudaFreeAsync(r->d_row, st);
    if (r->d_adj) cudaFreeAsync(r->d_adj, st);
    if (r->d_terms) cudaFreeAsync(r->d_terms, st);
    if (r->d_table) cudaFreeAsync(r->d_table, st);
    r->d_row = nullptr;
    r->d_adj = nullptr;
    r->d_terms = nullptr;
    r->d_table = nullptr;
}

// Device set-up of a newly admitted small request (stream-ordered).  The
// packed arcs are written into `adj`, which must live until the stream syncs.
int stage_small(emv_server *s, Req *r, std::vector<int2> &adj)
{
    cudaStream_t st = s->st_small;
    const size_t arcs = (size_t)std::max<int64_t>(r->arcs, 1);
    if (cudaMallocAsync((void **)&r->d_row, sizeof(int32_t) * ((size_t)r->n + 1), st) != cudaSuccess ||
        cudaMallocAsync((void **)&r->d_adj, sizeof(int2) * arcs, st) != cudaSuccess ||
        cudaMallocAsync((void **)&r->d_terms, sizeof(int32_t) * (size_t)r->k, st) != cudaSuccess ||
        cudaMallocAsync((void **)&r->d_table, sizeof(int32_t) * ((size_t)r->n << r->k), st) != cudaSuccess) {
        cudaGetLastError();
        return emv_fail(EMV_ERR_OOM, "server: device allocation for request %lld", (long long)r->id);
    }
    adj.resize(arcs);
    for (int64_t e = 0; e < r->arcs; e++) adj[(size_t)e] = make_int2(r->col[(size_t)e], r->w[(size_t)e]);
    CUDA_TRY(cudaMemcpyAsync(r->d_row, r->row.data(), sizeof(int32_t) * ((size_t)r->n + 1), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(r->d_adj, adj.data(), sizeof(int2) * (size_t)r->arcs, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(r->d_terms, r->terms.data(), sizeof(int32_t) * (size_t)r->k, cudaMemcpyHostToDevice, st));
    return EMV_OK;
}

// Admits queued requests in arrival order while the budget and the slots allow.
void admit_locked(emv_server *s, std::vector<Req *> &admitted)
{
    while (!s->queue_small.empty()) {
        Req *r = s->queue_small.front();
        if (r->cancel) {
            s->queue_small.pop_front();
            finish(s, r, EMV_ERR_CANCELLED, 0);
            s->cv_done.notify_all();
            continue;
        }
        if (s->free_slots.empty() || s->resident_count >= s->opts.max_slots ||
            s->resident_bytes + r->bytes > s->opts.hbm_budget_bytes)
            break;
        s->queue_small.pop_front();
        r->slot = s->free_slots.back();
        s->free_slots.pop_back();
        r->state = Q_RESIDENT;
        s->resident_bytes += r->bytes;
        s->resident_count++;
        admitted.push_back(r);
    }
    s->stats.peak_resident = std::max<int64_t>(s->stats.peak_resident, s->resident_count);
    s->stats.peak_bytes = std::max<int64_t>(s->stats.peak_bytes, s->resident_bytes);
}

void scheduler(emv_server *s)
{
    cudaSetDevice(s->opts.device);
    for (;;) {
        std::vector<Req *> admitted;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv_work.wait(lk, [&] { return s->stop || !s->queue_small.empty() || !s->resident.empty(); });
            if (s->stop && s->queue_small.empty() && s->resident.empty()) return;
            admit_locked(s, admitted);
        }
        std::vector<std::vector<int2>> staging(admitted.size());
        std::vector<int> staged(admitted.size(), EMV_OK);
        for (size_t i = 0; i < admitted.size(); i++) staged[i] = stage_small(s, admitted[i], staging[i]);
        if (!admitted.empty() && cudaStreamSynchronize(s->st_small) != cudaSuccess) {
            cudaGetLastError();
            for (int &x : staged) x = EMV_ERR_CUDA;
        }
        for (size_t i = 0; i < admitted.size(); i++) {
            Req *r = admitted[i];
            std::lock_guard<std::mutex> lk(s->mu);
            if (staged[i]) {
                release_device(s, r);
                s->free_slots.push_back(r->slot);
                s->resident_bytes -= r->bytes;
                s->resident_count--;
                finish(s, r, staged[i], 0);
                s->cv_done.notify_all();
            } else {
                s->resident.push_back(r);
            }
        }
        // One wave: every resident request advances by one level.
        std::vector<Req *> wave;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            for (Req *r : s->resident) wave.push_back(r);
        }
        if (wave.empty()) continue;
        for (size_t j = 0; j < wave.size(); j++) {
            Req *r = wave[j];
            BatchInst &d = s->h_desc[j];
            std::memset(&d, 0, sizeof(d));
            d.row_ptr = r->d_row;
            d.adj = r->d_adj;
            d.terms = r->d_terms;
            d.table = r->d_table;
            d.n = r->n;
            d.k = r->k;
            d.rcap = batch_rcap_for(s->ctx_small, r->n, r->k);
            d.mw = batch_mw_for(s->ctx_small, r->n, r->k);
            d.orig = r->slot;
            d.lo = d.hi = r->next_level;
        }
        int st = EMV_OK;
        BatchArgs a;
        std::memset(&a, 0, sizeof(a));
        a.inst = (const BatchInst *)s->d_desc.ptr;
        a.count = (int32_t)wave.size();
        a.xs = (const uint32_t *)s->ctx_small->bxs.ptr;
        a.xs_off = (const int32_t *)s->ctx_small->bxs_off.ptr;
        a.costs = (int64_t *)s->d_costs.ptr;
        a.queue = (uint32_t *)s->d_ctrl.ptr;
        a.err = (uint32_t *)s->d_ctrl.ptr + 8;
        uint32_t err = 0;
        if (cudaMemcpyAsync(s->d_desc.ptr, s->h_desc, sizeof(BatchInst) * wave.size(), cudaMemcpyHostToDevice,
                            s->st_small) != cudaSuccess)
            st = emv_fail(EMV_ERR_CUDA, "server: descriptor upload");
        // beside a large solve the wave stays on its share of the SMs
        const int32_t wave_blocks = s->large_sharing.load() ? s->wave_sms : 0;
        if (!st) st = launch_batch(s->ctx_small, a, a.count, s->st_small, wave_blocks);
        if (!st && cudaMemcpyAsync(s->h_costs, s->d_costs.ptr, sizeof(int64_t) * (size_t)s->cap_slots,
                                   cudaMemcpyDeviceToHost, s->st_small) != cudaSuccess)
            st = emv_fail(EMV_ERR_CUDA, "server: cost read");
        if (!st && cudaMemcpyAsync(&err, a.err, sizeof(uint32_t), cudaMemcpyDeviceToHost, s->st_small) != cudaSuccess)
            st = emv_fail(EMV_ERR_CUDA, "server: status read");
        if (!st && cudaStreamSynchronize(s->st_small) != cudaSuccess) {
            cudaGetLastError();
            st = emv_fail(EMV_ERR_CUDA, "server: wave failed");
        }
        if (!st && err) st = emv_dev_status_to_emv(err);
        if (!st) cudaMemsetAsync(a.err, 0, sizeof(uint32_t), s->st_small);
        std::lock_guard<std::mutex> lk(s->mu);
        s->stats.waves++;
        for (Req *r : wave) {
            bool done = false;
            if (st) {
                finish(s, r, st, 0);
                done = true;
            } else if (r->cancel) {
                finish(s, r, EMV_ERR_CANCELLED, 0);
                done = true;
            } else if (r->next_level == r->k) {
                finish(s, r, EMV_OK, s->h_costs[r->slot]);
                done = true;
            } else {
                r->next_level++;
            }
            if (done) {
                release_device(s, r);
                s->free_slots.push_back(r->slot);
                s->resident_bytes -= r->bytes;
                s->resident_count--;
                s->resident.erase(std::find(s->resident.begin(), s->resident.end(), r));
            }
        }
        s->cv_done.notify_all();
    }
}

void large_loop(emv_server *s)
{
    cudaSetDevice(s->opts.device);
    for (;;) {
        Req *r = nullptr;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv_work.wait(lk, [&] {
                if (s->stop) return true;
                if (s->queue_large.empty()) return false;
                return s->resident_bytes + s->queue_large.front()->bytes <= s->opts.hbm_budget_bytes ||
                       s->resident_count == 0;
            });
            if (s->stop && s->queue_large.empty()) return;
            if (s->queue_large.empty()) continue;
            r = s->queue_large.front();
            s->queue_large.pop_front();
            if (r->cancel) {
                finish(s, r, EMV_ERR_CANCELLED, 0);
                s->cv_done.notify_all();
                continue;
            }
            r->state = Q_RESIDENT;
            s->resident_bytes += r->bytes;
            s->resident_count++;
            s->stats.peak_resident = std::max<int64_t>(s->stats.peak_resident, s->resident_count);
            s->stats.peak_bytes = std::max<int64_t>(s->stats.peak_bytes, s->resident_bytes);
            // split the SMs only when there are small requests to run beside it
            const bool share = s->wave_sms > 0 && (!s->resident.empty() || !s->queue_small.empty());
            s->ctx_large->relax_sm_cap = share ? s->ctx_large->sms - s->wave_sms : 0;
            s->large_sharing = share;
        }
        emv_graph g{r->n, r->arcs, r->row.data(), r->col.data(), r->w.data()};
        emv_result res;
        std::memset(&res, 0, sizeof(res));
        int st = emv_solve(s->ctx_large, &g, r->terms.data(), r->k, EMV_SOLVE_NOCHECK, &res, s->st_large);
        s->large_sharing = false;
        std::lock_guard<std::mutex> lk(s->mu);
        s->resident_bytes -= r->bytes;
        s->resident_count--;
        finish(s, r, st, res.cost);
        s->cv_done.notify_all();
        s->cv_work.notify_all();
    }
}

void server_free(emv_server *s)
{
    if (s->ctx_small) emv_destroy(s->ctx_small);
    if (s->ctx_large) emv_destroy(s->ctx_large);
    dev_release(s->d_desc);
    dev_release(s->d_costs);
    dev_release(s->d_ctrl);
    if (s->h_desc) cudaFreeHost(s->h_desc);
    if (s->h_costs) cudaFreeHost(s->h_costs);
    if (s->st_small) cudaStreamDestroy(s->st_small);
    if (s->st_large) cudaStreamDestroy(s->st_large);
    for (auto &kv : s->reqs) delete kv.second;
    delete s;
}

}  // namespace

extern "C" int emv_server_create(emv_server **out, const emv_server_opts *opts)
{
    if (!out || !opts || opts->max_slots <= 0 || opts->hbm_budget_bytes <= 0)
        return emv_fail(EMV_ERR_BAD_INPUT, "emv_server_create: bad options");
    *out = nullptr;
    emv_server *s = new (std::nothrow) emv_server();
    if (!s) return emv_fail(EMV_ERR_OOM, "server");
    s->opts = *opts;
    if (s->opts.large_n <= 0) s->opts.large_n = 1 << 16;
    int st = emv_create(&s->ctx_small, opts->device);
    if (!st) st = emv_create(&s->ctx_large, opts->device);
    if (st) {
        server_free(s);
        return st;
    }
    s->cap_slots = opts->max_slots;
    {
        const int sms = s->ctx_large->sms;
        const int want = opts->wave_sms == 0 ? std::max(1, sms / 6) : opts->wave_sms;
        s->wave_sms = (want > 0 && want < sms) ? want : 0;
    }
    // The large requests bound the stream's throughput (each needs the whole
    // GPU for tens of milliseconds), so their stream gets the highest
    // priority: when a wave and a large solve both have blocks waiting for
    // SMs, the large solve's go first and its cooperative grids are not held
    // back behind a wave.
    int prio_least = 0, prio_greatest = 0;
    if (cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest) != cudaSuccess) {
        cudaGetLastError();
        prio_least = prio_greatest = 0;
    }
    if (cudaStreamCreateWithPriority(&s->st_small, cudaStreamNonBlocking, prio_least) != cudaSuccess ||
        cudaStreamCreateWithPriority(&s->st_large, cudaStreamNonBlocking, prio_greatest) != cudaSuccess ||
        cudaMallocHost((void **)&s->h_desc, sizeof(BatchInst) * (size_t)s->cap_slots) != cudaSuccess ||
        cudaMallocHost((void **)&s->h_costs, sizeof(int64_t) * (size_t)s->cap_slots) != cudaSuccess) {
        cudaGetLastError();
        server_free(s);
        return emv_fail(EMV_ERR_CUDA, "server: stream or pinned buffer");
    }
    st = dev_reserve(s->d_desc, sizeof(BatchInst) * (size_t)s->cap_slots);
    if (!st) st = dev_reserve(s->d_costs, sizeof(int64_t) * (size_t)s->cap_slots);
    if (!st) st = dev_reserve(s->d_ctrl, 64);
    if (!st) st = prepare_batch_subsets(s->ctx_small, s->st_small);
    if (!st) st = batch_kernel_setup(s->ctx_small);
    if (!st && cudaMemsetAsync(s->d_ctrl.ptr, 0, 64, s->st_small) != cudaSuccess) st = EMV_ERR_CUDA;
    // keep freed pool memory cached in the process (no release at stream syncs)
    cudaMemPool_t pool;
    if (!st && cudaDeviceGetDefaultMemPool(&pool, opts->device) == cudaSuccess) {
        uint64_t thr = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    if (st) {
        server_free(s);
        return st;
    }
    for (int32_t i = s->cap_slots - 1; i >= 0; i--) s->free_slots.push_back(i);
    s->sched = std::thread(scheduler, s);
    s->large_worker = std::thread(large_loop, s);
    *out = s;
    return EMV_OK;
}

extern "C" int emv_server_submit(emv_server *s, const emv_graph *g, const int32_t *terminals, int32_t k,
                                 int64_t *req_id)
{
    if (!s || !req_id) return emv_fail(EMV_ERR_BAD_INPUT, "emv_server_submit: null argument");
    int st = emv_graph_validate(g);
    if (st) return st;
    if (k < 1 || k > EMV_MAX_K || !terminals) return emv_fail(EMV_ERR_BAD_INPUT, "k = %d out of range", k);
    for (int32_t i = 0; i < k; i++)
        if (terminals[i] < 0 || terminals[i] >= g->n) return emv_fail(EMV_ERR_BAD_INPUT, "terminal out of range");
    st = emv_graph_check(g, nullptr);
    if (st) return st;
    const int64_t bytes = footprint(g->n, k, g->arcs);
    if (bytes > s->opts.hbm_budget_bytes) {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stats.rejected++;
    }
    if (bytes > s->opts.hbm_budget_bytes)
        return emv_fail(EMV_ERR_OVER_BUDGET, "request needs %lld bytes, budget %lld", (long long)bytes,
                        (long long)s->opts.hbm_budget_bytes);
    Req *r = new (std::nothrow) Req();
    if (!r) return emv_fail(EMV_ERR_OOM, "request");
    r->n = g->n;
    r->k = k;
    r->arcs = g->arcs;
    r->row.assign(g->row_ptr, g->row_ptr + g->n + 1);
    r->col.assign(g->col, g->col + g->arcs);
    r->w.assign(g->w, g->w + g->arcs);
    r->terms.assign(terminals, terminals + k);
    r->bytes = bytes;
    r->large = g->n >= s->opts.large_n || !batch_fits(g->n, k);
    r->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        r->id = s->next_id++;
        s->reqs[r->id] = r;
        (r->large ? s->queue_large : s->queue_small).push_back(r);
        s->stats.submitted++;
        *req_id = r->id;
    }
    s->cv_work.notify_all();
    return EMV_OK;
}

static int result_locked(emv_server *s, Req *r, int64_t *cost, double *latency_ms)
{
    if (r->state == Q_QUEUED || r->state == Q_RESIDENT) return EMV_ERR_NOT_READY;
    if (cost) *cost = r->cost;
    if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
    if (r->status != EMV_OK) return emv_fail(r->status, "request %lld failed: %s", (long long)r->id,
                                             emv_status_str(r->status));
    return EMV_OK;
}

extern "C" int emv_server_poll(emv_server *s, int64_t id, int64_t *cost, double *latency_ms)
{
    if (!s) return emv_fail(EMV_ERR_BAD_INPUT, "null server");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return emv_fail(EMV_ERR_BAD_INPUT, "unknown request %lld", (long long)id);
    return result_locked(s, it->second, cost, latency_ms);
}

extern "C" int emv_server_wait(emv_server *s, int64_t id, int64_t *cost, double *latency_ms, double timeout_s)
{
    if (!s) return emv_fail(EMV_ERR_BAD_INPUT, "null server");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return emv_fail(EMV_ERR_BAD_INPUT, "unknown request %lld", (long long)id);
    Req *r = it->second;
    const auto until = Clock::now() + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(timeout_s));
    s->cv_done.wait_until(lk, until, [&] { return r->state != Q_QUEUED && r->state != Q_RESIDENT; });
    return result_locked(s, r, cost, latency_ms);
}

extern "C" int emv_server_cancel(emv_server *s, int64_t id)
{
    if (!s) return emv_fail(EMV_ERR_BAD_INPUT, "null server");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return emv_fail(EMV_ERR_BAD_INPUT, "unknown request %lld", (long long)id);
    it->second->cancel = true;
    s->cv_work.notify_all();
    return EMV_OK;
}

extern "C" int emv_server_stats_get(emv_server *s, emv_server_stats *out)
{
    if (!s || !out) return emv_fail(EMV_ERR_BAD_INPUT, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->stats;
    return EMV_OK;
}

extern "C" int emv_server_destroy(emv_server *s)
{
    if (!s) return EMV_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        for (Req *r : s->queue_small) r->cancel = true;
        for (Req *r : s->queue_large) r->cancel = true;
        for (Req *r : s->resident) r->cancel = true;
    }
    s->cv_work.notify_all();
    if (s->sched.joinable()) s->sched.join();
    if (s->large_worker.joinable()) s->large_worker.join();
    cudaSetDevice(s->opts.device);
    cudaDeviceSynchronize();
    server_free(s);
    return EMV_OK;
}
