// emv_device.cu -- solver context and the single-instance GPU DP (C ABI).
//
// Reference counterparts (reader/reader-el.c):
//   emv_kernel              R:1966-2139  -> emv_kernel_dev
//   erickson_monma_veinott  R:2141-2343  -> emv_solve / emv_solve_dev
//   dijkstra (-dijkstra)    R:1762-1880, R:2454-2484 -> emv_sssp
#include "emv_kernels.cuh"
#include "emv_solver.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <numeric>
#include <vector>

using namespace emv;

int emv_dev_status_to_emv(uint32_t s)
{
    if (s == 0) return EMV_OK;
    if (s & (EMV_DEV_BARRIER_TIMEOUT | EMV_DEV_SWEEP_LIMIT | EMV_DEV_TB_STEPS | EMV_DEV_QUEUE_TIMEOUT))
        return emv_fail(EMV_ERR_TIMEOUT, "device loop bound reached (status 0x%x)", s);
    if (s & EMV_DEV_BAD_VALUE) return emv_fail(EMV_ERR_BAD_INPUT, "an input value is above 2^30 (status 0x%x)", s);
    if (s & EMV_DEV_OVERFLOW)
        return emv_fail(EMV_ERR_OVERFLOW, "a finite value plus an arc weight reached 2^30 (status 0x%x)", s);
    return emv_fail(EMV_ERR_INTERNAL, "device status 0x%x", s);
}

extern "C" const char *emv_version(void) { return "emv-gb300 1.0 sm_103a"; }

// ------------------------------------------------------------ buffers

int dev_reserve(DevBuf &b, size_t bytes)
{
    if (b.bytes >= bytes) return EMV_OK;
    if (b.ptr) cudaFree(b.ptr);
    b.ptr = nullptr;
    b.bytes = 0;
    size_t want = std::max<size_t>(bytes, 256);
    cudaError_t e = cudaMalloc(&b.ptr, want);
    if (e != cudaSuccess) {
        cudaGetLastError();
        b.ptr = nullptr;
        return emv_fail(e == cudaErrorMemoryAllocation ? EMV_ERR_OOM : EMV_ERR_CUDA,
                        "cudaMalloc(%zu): %s", want, cudaGetErrorString(e));
    }
    b.bytes = want;
    return EMV_OK;
}

void dev_release(DevBuf &b)
{
    if (b.ptr) cudaFree(b.ptr);
    b.ptr = nullptr;
    b.bytes = 0;
}

// ------------------------------------------------------------ context

// Relaxation kernels by record width: k_relax<1, 2, 4, 5, 8> with 32-bit,
// then with 16-bit records (32 * VEC words a vertex).
static const void *const relax_fns[RELAX_VARIANTS] = {
    (const void *)k_relax<1>,       (const void *)k_relax<2>,       (const void *)k_relax<4>,
    (const void *)k_relax<5>,       (const void *)k_relax<8>,       (const void *)k_relax<1, true>,
    (const void *)k_relax<2, true>, (const void *)k_relax<4, true>, (const void *)k_relax<5, true>,
    (const void *)k_relax<8, true>};

extern "C" int emv_create(emv_ctx **out, int32_t device)
{
    if (!out) return emv_fail(EMV_ERR_BAD_INPUT, "null ctx pointer");
    *out = nullptr;
    int ndev = 0;
    CUDA_TRY(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) return emv_fail(EMV_ERR_BAD_INPUT, "device %d of %d", device, ndev);
    CUDA_TRY(cudaSetDevice(device));
    cudaDeviceProp prop;
    CUDA_TRY(cudaGetDeviceProperties(&prop, device));
    if (!prop.cooperativeLaunch) return emv_fail(EMV_ERR_CUDA, "device lacks cooperative launch");
    emv_ctx *c = new (std::nothrow) emv_ctx();
    if (!c) return emv_fail(EMV_ERR_OOM, "ctx");
    c->device = device;
    c->sms = prop.multiProcessorCount;
    c->l2_bytes = prop.l2CacheSize;
    for (int i = 0; i < RELAX_VARIANTS; i++) {
        int per_sm = 0;
        CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, relax_fns[i], RELAX_THREADS, 0));
        c->relax_blocks_max[i] = std::max(1, per_sm) * c->sms;
    }
    int st = dev_reserve(c->ctrl, sizeof(uint32_t) * C_WORDS);
    if (!st) st = dev_reserve(c->stat, sizeof(DevStat));
    if (!st) st = dev_reserve(c->lvlmax, sizeof(uint32_t) * (EMV_MAX_K + 1));
    if (!st) st = dev_reserve(c->gscan, sizeof(GraphScan));
    if (!st) {
        if (cudaMallocHost(&c->pinned, 4096) != cudaSuccess) { cudaGetLastError(); st = emv_fail(EMV_ERR_OOM, "pinned"); }
    }
    for (int i = 0; !st && i < MAX_EVENTS; i++)
        if (cudaEventCreate(&c->ev[i]) != cudaSuccess) st = emv_fail(EMV_ERR_CUDA, "event create");
    for (int i = 0; !st && i <= EMV_MAX_K; i++)
        if (cudaEventCreateWithFlags(&c->evmax[i], cudaEventDisableTiming) != cudaSuccess)
            st = emv_fail(EMV_ERR_CUDA, "event create");
    if (st) {
        emv_destroy(c);
        return st;
    }
    *out = c;
    return EMV_OK;
}

extern "C" int emv_set_sweep_limit(emv_ctx *c, int64_t limit)
{
    if (!c || limit < 0) return emv_fail(EMV_ERR_BAD_INPUT, "emv_set_sweep_limit: bad arguments");
    c->sweep_limit = limit;
    return EMV_OK;
}

extern "C" int emv_set_value_bits(emv_ctx *c, int32_t bits)
{
    if (!c || (bits != 0 && bits != 32)) return emv_fail(EMV_ERR_BAD_INPUT, "emv_set_value_bits: bits 0 or 32");
    c->value_bits = bits;
    return EMV_OK;
}

extern "C" int emv_destroy(emv_ctx *c)
{
    if (!c) return EMV_OK;
    cudaSetDevice(c->device);
    cudaDeviceSynchronize();
    for (DevBuf *b : {&c->ctrl, &c->stat, &c->lvlmax, &c->gscan, &c->shadow, &c->scratch, &c->act, &c->adj, &c->stamp, &c->terms, &c->g_row,
                      &c->g_col, &c->g_w, &c->table, &c->tb_edges, &c->tb_out, &c->tb_work})
        dev_release(*b);
    for (KPlan *p : c->kplans) {
        if (!p) continue;
        for (DevBuf *b : {&p->xs, &p->mpairs, &p->movr, &p->mstream_data, &p->mstream_phases}) dev_release(*b);
        delete p;
    }
    for (int i = 0; i < MAX_EVENTS; i++)
        if (c->ev[i]) cudaEventDestroy(c->ev[i]);
    for (int i = 0; i <= EMV_MAX_K; i++)
        if (c->evmax[i]) cudaEventDestroy(c->evmax[i]);
    if (c->pinned) cudaFreeHost(c->pinned);
    delete c;
    return EMV_OK;
}

// ------------------------------------------------------------ the DP

static int grid_for(int64_t work, int threads, int cap)
{
    int64_t g = (work + threads - 1) / threads;
    return (int)std::max<int64_t>(1, std::min<int64_t>(g, cap));
}

// Launches the relaxation of one chunk of at most CHUNK_ROWS rows (2 *
// CHUNK_ROWS with 16-bit records, which the caller takes only for rows whose
// values are all at most 32767) as one cooperative, persistent kernel; the
// record width follows the row count.  vmax (or null) receives the largest
// value written.
int launch_relax(emv_ctx *c, const int32_t *row_ptr, const int2 *adj, int32_t n, int64_t ld, int32_t *table,
                 const uint32_t *rows, int32_t nrows, const int32_t *terms, int32_t level1, cudaStream_t st,
                 bool u16 = false, uint32_t *vmax = nullptr, uint16_t *shadow = nullptr, int64_t shadow_ld = 0)
{
    RelaxArgs a;
    a.stamp = (int32_t *)c->stamp.ptr;
    a.row_ptr = row_ptr;
    a.adj = adj;
    a.n = n;
    a.ld = ld;
    a.table = table;
    a.rows = rows;
    a.nrows = nrows;
    a.terms = terms;
    a.level1 = level1;
    a.scratch = (int32_t *)c->scratch.ptr;
    a.act0 = (uint8_t *)c->act.ptr;
    a.act1 = (uint8_t *)c->act.ptr + ((size_t)n + 255) / 256 * 256;
    a.ctrl = (uint32_t *)c->ctrl.ptr;
    a.stat = (DevStat *)c->stat.ptr;
    a.max_sweeps = (c->sweep_limit > 0 && c->sweep_limit < (int64_t)n + 1) ? (int32_t)c->sweep_limit : n + 1;
    // Dense sweeps pay off while almost every vertex has a changed neighbour:
    // with mean degree d and a fraction f of vertices changed, a vertex has none
    // with probability (1 - f)^d; take every vertex while that is below 10 %.
    const double deg = (double)c->relax_arcs / (double)n;
    a.dense_min = deg > 0 ? (int32_t)std::min<double>((double)n, (double)n * (1.0 - std::pow(0.1, 1.0 / deg))) : n;
    a.vmax = vmax;
    a.shadow = shadow;
    a.shadow_ld = shadow_ld;
    const int32_t words = u16 ? (nrows + 1) / 2 : nrows;  // int32 words a vertex record needs
    // Without stamps a sweep pulls every arc, also from heads that did not
    // change: worth it once most heads changed while the records are L2 hits
    // (from 75 % of the vertices), only at 97 % when they stream from HBM.
    const int wi = words <= 32 ? 0 : words <= 64 ? 1 : words <= 128 ? 2 : words <= 160 ? 3 : 4;
    const int64_t rec_words = (int64_t)32 * (wi == 3 ? 5 : 1 << (wi < 3 ? wi : 3));
    const bool resident = (int64_t)n * rec_words * 4 <= c->l2_bytes * 3 / 4;
    a.pull_all_min = n - n / (resident ? 4 : 32);
    const int vi = wi + (u16 ? 5 : 0);
    const void *fn = relax_fns[vi];
    // A warp per 8 vertices is enough; small graphs use fewer blocks (cheaper barriers).
    const int vpb = 8 * (RELAX_THREADS / 32);
    int bmax = c->relax_blocks_max[vi];
    if (c->relax_sm_cap > 0 && c->relax_sm_cap < c->sms) bmax = std::max(1, bmax / c->sms * c->relax_sm_cap);
    const int blocks = std::min(bmax, std::max(1, (n + vpb - 1) / vpb));
    CUDA_TRY(cudaMemsetAsync(a.ctrl, 0, sizeof(uint32_t) * C_WORDS, st));
    void *args[] = {&a};
    CUDA_TRY(cudaLaunchCooperativeKernel(fn, dim3(blocks), dim3(RELAX_THREADS), args, 0, st));
    c->launches += 1;  // the kernel (the control-word memset is not a kernel)
    return EMV_OK;
}

int32_t relax_chunk_rows(const emv_ctx *c, int32_t n, bool u16) { return relax_rows_per_chunk(n, c->l2_bytes, u16); }

int32_t relax_chunk_rows_level(const emv_ctx *c, int32_t n, bool u16, int64_t cnt)
{
    return relax_rows_per_level_chunk(n, c->l2_bytes, u16, cnt);
}

int reserve_relax(emv_ctx *c, int32_t n)
{
    const size_t npad = ((size_t)n + 31) / 32 * 32;
    int st = dev_reserve(c->scratch, npad * CHUNK_ROWS * sizeof(int32_t));
    if (!st) st = dev_reserve(c->act, 2 * (((size_t)n + 255) / 256 * 256));
    if (!st) st = dev_reserve(c->stamp, sizeof(int32_t) * (size_t)n);
    return st;
}

constexpr int32_t MERGE_SMEM_BYTES = 220 * 1024;
constexpr int32_t MERGE_SMEM_KMAX = 15;  // staged slots must fit 16 bits

constexpr int32_t STREAM_SMEM_BYTES = 224 * 1024;

// Plans the streamed merge of every level of k on the host (emv_plan.cpp)
// and uploads the plan data and the per-launch phase descriptors.
int plan_stream_merge(emv_ctx *c, int32_t k, cudaStream_t st)
{
    const std::vector<uint32_t> &xs = c->kp->xs_host;
    const std::vector<int64_t> &off = c->kp->xs_off;
    c->kp->mstream_groups.assign((size_t)k + 2, {});
    if (k > MERGE_SMEM_KMAX) return EMV_OK;
    std::vector<uint32_t> data;
    std::vector<std::vector<HostGroup>> plan;
    plan_stream_levels(k, xs, off, STREAM_SMEM_BYTES, data, plan);
    if (data.empty()) return EMV_OK;
    int r = dev_reserve(c->kp->mstream_data, sizeof(uint32_t) * data.size());
    if (r) return r;
    std::vector<MergePhase> phases;
    const uint32_t *base = (const uint32_t *)c->kp->mstream_data.ptr;
    for (int32_t m = 2; m <= k; m++)
        for (const HostGroup &G : plan[(size_t)m]) {
            StreamGroup sg;
            sg.x0 = G.x0;
            sg.cnt = G.cnt;
            sg.smem = G.smem;
            sg.phase_off = (int64_t)phases.size();
            sg.nphase = (int64_t)G.phases.size();
            if (sg.smem > STREAM_SMEM_BYTES) return emv_fail(EMV_ERR_INTERNAL, "merge plan: %lld bytes of shared memory",
                                                             (long long)sg.smem);
            for (const HostPhase &hp : G.phases) {
                if (hp.pairs_at % 4 != 0) return emv_fail(EMV_ERR_INTERNAL, "merge plan: pair block not 16-byte aligned");
                MergePhase mp;
                mp.rows = base + hp.rows_at;
                mp.qoff = base + hp.qoff_at;
                mp.pairs = base + hp.pairs_at;
                mp.nrows = hp.nrows;
                mp.pad_ = 0;
                phases.push_back(mp);
            }
            c->kp->mstream_groups[(size_t)m].push_back(sg);
        }
    r = dev_reserve(c->kp->mstream_phases, sizeof(MergePhase) * std::max<size_t>(1, phases.size()));
    if (r) return r;
    CUDA_TRY(cudaMemcpyAsync(c->kp->mstream_data.ptr, data.data(), sizeof(uint32_t) * data.size(), cudaMemcpyHostToDevice,
                             st));
    if (!phases.empty())
        CUDA_TRY(cudaMemcpyAsync(c->kp->mstream_phases.ptr, phases.data(), sizeof(MergePhase) * phases.size(),
                                 cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    return EMV_OK;
}

static int build_plan(emv_ctx *c, int32_t k, cudaStream_t st);

int prepare_subsets(emv_ctx *c, int32_t k, cudaStream_t st)
{
    if (c->xs_k == k) return EMV_OK;
    if (k < 1 || k > EMV_MAX_K) return emv_fail(EMV_ERR_BAD_INPUT, "k = %d", k);
    if (c->kplans[k]) {  // built before on this context
        c->kp = c->kplans[k];
        c->xs_k = k;
        return EMV_OK;
    }
    KPlan *plan = new (std::nothrow) KPlan();
    if (!plan) return emv_fail(EMV_ERR_OOM, "plan");
    c->kp = plan;
    c->xs_k = -1;
    const int r0 = build_plan(c, k, st);
    if (r0) {
        for (DevBuf *b : {&plan->xs, &plan->mpairs, &plan->movr, &plan->mstream_data, &plan->mstream_phases})
            dev_release(*b);
        delete plan;
        c->kp = nullptr;
        return r0;
    }
    c->kplans[k] = plan;
    c->xs_k = k;
    return EMV_OK;
}

// Builds c->kp for k: subsets, slot lists and the streamed merge plan.
static int build_plan(emv_ctx *c, int32_t k, cudaStream_t st)
{
    subset_levels(k, c->kp->xs_host, c->kp->xs_off);
    int r = dev_reserve(c->kp->xs, sizeof(uint32_t) * std::max<size_t>(1, c->kp->xs_host.size()));
    if (r) return r;
    CUDA_TRY(cudaMemcpyAsync(c->kp->xs.ptr, c->kp->xs_host.data(), sizeof(uint32_t) * c->kp->xs_host.size(),
                             cudaMemcpyHostToDevice, st));
    r = plan_stream_merge(c, k, st);
    if (r) return r;
    // Pair and override slot lists of the staged-all-rows merge, for the levels
    // the streamed merge has no plan for (level order).
    c->kp->mpair_base.assign((size_t)k + 2, 0);
    c->kp->movr_base.assign((size_t)k + 2, 0);
    std::vector<uint32_t> pairs, ovr;
    if (k <= MERGE_SMEM_KMAX) {
        std::vector<uint32_t> lidx((size_t)1 << k, 0);
        for (size_t i = 0; i < c->kp->xs_host.size(); i++) lidx[c->kp->xs_host[i]] = (uint32_t)i;
        for (int32_t m = 2; m <= k; m++) {
            c->kp->mpair_base[(size_t)m] = (int64_t)pairs.size();
            c->kp->movr_base[(size_t)m] = (int64_t)ovr.size();
            if (!c->kp->mstream_groups[(size_t)m].empty()) continue;
            for (int64_t i = c->kp->xs_off[(size_t)m]; i < c->kp->xs_off[(size_t)m + 1]; i++) {
                const uint32_t X = c->kp->xs_host[(size_t)i];
                const uint32_t low = X & (0u - X), rest = X ^ low;
                uint32_t sm = 0;
                do {
                    const uint32_t Y = low | sm;
                    pairs.push_back(lidx[Y] | (lidx[X ^ Y] << 16));
                    sm = (sm - rest) & rest;
                } while (sm != rest);
                for (int32_t t = 0; t < k; t++)
                    if (X >> t & 1u) ovr.push_back(((uint32_t)t << 16) | lidx[X ^ (1u << t)]);
            }
        }
    }
    if (!pairs.empty()) {
        r = dev_reserve(c->kp->mpairs, sizeof(uint32_t) * pairs.size());
        if (!r) r = dev_reserve(c->kp->movr, sizeof(uint32_t) * ovr.size());
        if (r) return r;
        CUDA_TRY(cudaMemcpyAsync(c->kp->mpairs.ptr, pairs.data(), sizeof(uint32_t) * pairs.size(), cudaMemcpyHostToDevice,
                                 st));
        CUDA_TRY(cudaMemcpyAsync(c->kp->movr.ptr, ovr.data(), sizeof(uint32_t) * ovr.size(), cudaMemcpyHostToDevice, st));
    }
    CUDA_TRY(cudaStreamSynchronize(st));
    return EMV_OK;
}

template <int VB>
static cudaError_t merge_smem_launch(emv_ctx *c, int32_t *table, int64_t ld, int32_t n, int32_t k, int32_t m,
                                     const int32_t *d_terms, cudaStream_t st)
{
    const int64_t b = c->kp->xs_off[(size_t)m], cnt = c->kp->xs_off[(size_t)m + 1] - b;
    const int32_t nstage = (int32_t)c->kp->xs_off[(size_t)m];
    const uint32_t *xs = (const uint32_t *)c->kp->xs.ptr;
    const size_t smem = sizeof(int32_t) * (size_t)nstage * VB;
    const int32_t npairs = (1 << (m - 1)) - 1;
    k_merge_smem<VB><<<(unsigned)((n + VB - 1) / VB), 1024, smem, st>>>(
        table, ld, n, xs + b, (int32_t)cnt, xs, nstage, (const uint32_t *)c->kp->mpairs.ptr + c->kp->mpair_base[(size_t)m],
        npairs, (const uint32_t *)c->kp->movr.ptr + c->kp->movr_base[(size_t)m], m, d_terms);
    (void)k;
    return cudaGetLastError();
}

// Merge of level m: the shared-memory kernel with the widest vertex block
// whose staging fits, else the direct kernel (k above MERGE_SMEM_KMAX).
int launch_merge(emv_ctx *c, int32_t *table, int64_t ld, int32_t n, int32_t k, int32_t m, const int32_t *d_terms,
                 cudaStream_t st, bool u16 = false, const uint16_t *shadow = nullptr, int64_t shadow_ld = 0)
{
    if (!c->merge_attr) {
        const void *fns[6] = {(const void *)k_merge_smem<32>, (const void *)k_merge_smem<16>,
                              (const void *)k_merge_smem<8>, (const void *)k_merge_smem<4>,
                              (const void *)k_merge_smem<2>, (const void *)k_merge_smem<1>};
        for (const void *f : fns)
            CUDA_TRY(cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, MERGE_SMEM_BYTES));
        CUDA_TRY(cudaFuncSetAttribute((const void *)k_merge_stream, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      STREAM_SMEM_BYTES));
        CUDA_TRY(cudaFuncSetAttribute((const void *)k_merge_stream16, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      STREAM_SMEM_BYTES));
        c->merge_attr = true;
    }
    const int64_t nstage = c->kp->xs_off[(size_t)m];
    cudaError_t e = cudaSuccess;
    c->merge16_last = false;
    c->launches++;
    if (k <= MERGE_SMEM_KMAX && !c->kp->mstream_groups[(size_t)m].empty()) {
        // the streamed merge records the level's largest value (other kernels leave it unknown)
        CUDA_TRY(cudaMemsetAsync((uint32_t *)c->lvlmax.ptr + m, 0, sizeof(uint32_t), st));
        const int64_t b = c->kp->xs_off[(size_t)m];
        c->launches += (int64_t)c->kp->mstream_groups[(size_t)m].size() - 1;
        // 16-bit staging reads int2 pairs of vertices: even stride and base
        u16 = u16 && ld % 2 == 0 && ((uintptr_t)table & 7) == 0;
        c->merge16_last = u16;
        for (const StreamGroup &g : c->kp->mstream_groups[(size_t)m]) {
            const uint32_t *xg = (const uint32_t *)c->kp->xs.ptr + b + g.x0;
            const MergePhase *pg = (const MergePhase *)c->kp->mstream_phases.ptr + g.phase_off;
            if (u16)
                k_merge_stream16<<<(unsigned)((n + 63) / 64), 1024, (size_t)g.smem, st>>>(
                    table, ld, n, xg, (int32_t)g.cnt, pg, (int32_t)g.nphase, d_terms, k, (uint32_t *)c->lvlmax.ptr + m,
                    shadow, shadow_ld);
            else
                k_merge_stream<<<(unsigned)((n + 31) / 32), 1024, (size_t)g.smem, st>>>(
                    table, ld, n, xg, (int32_t)g.cnt, pg, (int32_t)g.nphase, d_terms, k, (uint32_t *)c->lvlmax.ptr + m);
            e = cudaGetLastError();
            if (e != cudaSuccess) break;
        }
    } else if (k <= MERGE_SMEM_KMAX) {
        const int64_t row_bytes = nstage * 4;
        if (row_bytes * 32 <= MERGE_SMEM_BYTES) e = merge_smem_launch<32>(c, table, ld, n, k, m, d_terms, st);
        else if (row_bytes * 16 <= MERGE_SMEM_BYTES) e = merge_smem_launch<16>(c, table, ld, n, k, m, d_terms, st);
        else if (row_bytes * 8 <= MERGE_SMEM_BYTES) e = merge_smem_launch<8>(c, table, ld, n, k, m, d_terms, st);
        else if (row_bytes * 4 <= MERGE_SMEM_BYTES) e = merge_smem_launch<4>(c, table, ld, n, k, m, d_terms, st);
        else if (row_bytes * 2 <= MERGE_SMEM_BYTES) e = merge_smem_launch<2>(c, table, ld, n, k, m, d_terms, st);
        else e = merge_smem_launch<1>(c, table, ld, n, k, m, d_terms, st);
    } else {
        const int64_t b = c->kp->xs_off[(size_t)m], cnt = c->kp->xs_off[(size_t)m + 1] - b;
        const int32_t xper = (int32_t)std::min<int64_t>(cnt, 64);
        dim3 grid((unsigned)((n + 31) / 32), (unsigned)((cnt + xper - 1) / xper));
        k_merge<<<grid, 256, 0, st>>>(table, ld, n, (const uint32_t *)c->kp->xs.ptr + b, (int32_t)cnt, xper, d_terms, k);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) return emv_fail(EMV_ERR_CUDA, "merge launch: %s", cudaGetErrorString(e));
    return EMV_OK;
}

// Status of a device CSR check: the same statuses, bound and messages as the
// host check emv_graph_check, whose connectivity part comes from the level-1
// closures instead (run_dp).
static int scan_status(const GraphScan &s, int32_t n)
{
    if (s.bad & SCAN_BAD_ROWS) return emv_fail(EMV_ERR_BAD_INPUT, "graph: row_ptr not from 0 to arcs, non-decreasing");
    if (s.bad & SCAN_BAD_HEAD) return emv_fail(EMV_ERR_BAD_INPUT, "graph: arc head out of range");
    if (s.bad & SCAN_BAD_WEIGHT) return emv_fail(EMV_ERR_BAD_INPUT, "graph: negative weight");
    if (s.bad & SCAN_BIG_WEIGHT) return emv_fail(EMV_ERR_OVERFLOW, "graph: an arc weight reaches 2^30");
    // every finite d[X][v] is a Steiner tree's weight: at most (n-1) * max_w
    // and at most the weight of all edges (two arcs each)
    const int64_t bound = std::min<int64_t>((int64_t)(n - 1) * (int64_t)s.maxw, (int64_t)(s.sumw / 2));
    if (bound >= INF)
        return emv_fail(EMV_ERR_OVERFLOW, "graph: table values may reach 2^30 (bound %lld)", (long long)bound);
    return EMV_OK;
}

// Packs the arcs as int2 (c->adj) and checks the device CSR in the same
// kernel.  With check set, waits for the check and returns its status before
// any kernel of the DP reads the graph; the scan result stays in c->gscan.
static int pack_and_check(emv_ctx *c, int32_t n, int64_t arcs, const int32_t *row_ptr, const int32_t *col,
                          const int32_t *w, bool check, cudaStream_t st)
{
    int r = dev_reserve(c->adj, sizeof(int2) * (size_t)std::max<int64_t>(arcs, 1));
    if (r) return r;
    c->relax_arcs = arcs;
    GraphScan *d_scan = (GraphScan *)c->gscan.ptr;
    CUDA_TRY(cudaMemsetAsync(d_scan, 0, sizeof(GraphScan), st));
    k_pack_scan<<<grid_for(std::max<int64_t>(arcs, (int64_t)n + 1), 256, 4096), 256, 0, st>>>(
        row_ptr, n, col, w, (int2 *)c->adj.ptr, arcs, d_scan);
    CUDA_TRY(cudaGetLastError());
    c->launches++;
    if (!check) return EMV_OK;
    GraphScan *h = (GraphScan *)((char *)c->pinned + 1024);
    CUDA_TRY(cudaMemcpyAsync(h, d_scan, sizeof(GraphScan), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    return scan_status(*h, n);
}

// The DP proper on device data with packed arcs; fills the whole table.
// With check set, a level-1 closure that left a vertex unreached (the graph
// is not connected: the reference's table is undefined there, R:2077) makes
// the solve EMV_ERR_DISCONNECTED; the table is then not meaningful.
int run_dp(emv_ctx *c, int32_t n, const int32_t *row_ptr, const int2 *adj, int32_t k, const int32_t *terms_host,
           int32_t *table, int64_t ld, cudaStream_t st, int64_t *cost_out, emv_timing *tm, bool check)
{
    int r = prepare_subsets(c, k, st);
    if (!r) r = reserve_relax(c, n);
    if (!r) r = dev_reserve(c->terms, sizeof(int32_t) * (size_t)k);
    if (r) return r;
    int32_t *d_terms = (int32_t *)c->terms.ptr;
    CUDA_TRY(cudaMemcpyAsync(d_terms, terms_host, sizeof(int32_t) * (size_t)k, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemsetAsync(c->stat.ptr, 0, sizeof(DevStat), st));
    const uint32_t *xs = (const uint32_t *)c->kp->xs.ptr;
    int ev = 0;
    cudaEvent_t *E = c->ev;
    CUDA_TRY(cudaEventRecord(E[ev++], st));  // 0: start

    // Row 0 is the only row no level writes (R:2243-2259 fills every row).
    k_fill<<<grid_for(n, 256, 1024), 256, 0, st>>>(table, n, INF);
    c->launches++;
    CUDA_TRY(cudaEventRecord(E[ev++], st));  // 1: after fill

    // Level maxima: lvlmax[m] = largest value the merge of level m wrote
    // (level 1: its relaxation), all ones where the kernel does not record it.
    // They reach the host one level late, so no wait idles the device.
    uint32_t *d_max = (uint32_t *)c->lvlmax.ptr, *h_max = (uint32_t *)c->pinned + 64;
    // 16-bit shadow of the relaxed rows (stride a multiple of 64 vertices):
    // the 16-bit merge stages from it with 16-byte asynchronous copies.  Taken
    // when 16-bit values are allowed and the memory is free (with 1 GiB to
    // spare); without it the merge packs the int32 rows itself.
    uint16_t *shadow = nullptr;
    const int64_t sld = ((int64_t)n + 63) / 64 * 64;
    if (c->value_bits == 0 && k >= 3 && k <= MERGE_SMEM_KMAX) {  // the streamed merge's k
        const size_t need = sizeof(uint16_t) * (size_t)sld << k;
        size_t fr = 0, tot = 0;
        if (c->shadow.bytes >= need ||
            (cudaMemGetInfo(&fr, &tot) == cudaSuccess && need + ((size_t)1 << 30) < fr && dev_reserve(c->shadow, need) == EMV_OK))
            shadow = (uint16_t *)c->shadow.ptr;
        cudaGetLastError();
    }
    int64_t levels16 = 0, merges16 = 0, relax_launches = 1;
    CUDA_TRY(cudaMemsetAsync(d_max, 0xff, sizeof(uint32_t) * (EMV_MAX_K + 1), st));
    CUDA_TRY(cudaMemsetAsync(d_max + 1, 0, sizeof(uint32_t), st));

    // Level 1: k single-source closures (R:1988-2031).
    r = launch_relax(c, row_ptr, adj, n, ld, table, xs + c->kp->xs_off[1], k, d_terms, 1, st, false, d_max + 1,
                     shadow, sld);
    if (r) return r;
    CUDA_TRY(cudaEventRecord(E[ev++], st));  // 2: after level 1
    CUDA_TRY(cudaMemcpyAsync(h_max + 1, d_max + 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaEventRecord(c->evmax[1], st));

    for (int32_t m = 2; m <= k; m++) {
        const int64_t b = c->kp->xs_off[(size_t)m], cnt = c->kp->xs_off[(size_t)m + 1] - b;
        // 16-bit merge staging when every sum of two lower-level values is
        // at most 65533 (M(j) bounds level j's values); from level 3 on, where
        // waiting for level m-1's maximum leaves its relaxation queued.
        // 16-bit relaxation records when M(m-1) + M(1) <= 32767: the split
        // {X \ t, t} bounds every merged value of level m by it, and relaxed
        // values never exceed merged ones (level 2 decides after its merge is
        // queued, so that no wait idles the device).
        bool m16 = false, u16 = false;
        if (c->value_bits == 0 && m >= 3) {
            CUDA_TRY(cudaEventSynchronize(c->evmax[m - 1]));
            m16 = merge16_allowed(h_max, m);
            u16 = relax16_allowed(h_max, m);
        }
        r = launch_merge(c, table, ld, n, k, m, d_terms, st, m16, shadow, sld);
        if (r) return r;
        merges16 += c->merge16_last;
        CUDA_TRY(cudaEventRecord(E[ev++], st));  // merge end of level m
        CUDA_TRY(cudaMemcpyAsync(h_max + m, d_max + m, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaEventRecord(c->evmax[m], st));
        if (c->value_bits == 0 && m == 2) {
            CUDA_TRY(cudaEventSynchronize(c->evmax[m - 1]));
            u16 = relax16_allowed(h_max, m);
        }
        levels16 += u16;
        const int32_t chunk = relax_chunk_rows_level(c, n, u16, cnt);
        for (int64_t off = 0; off < cnt; off += chunk) {
            const int32_t rows = (int32_t)std::min<int64_t>(chunk, cnt - off);
            r = launch_relax(c, row_ptr, adj, n, ld, table, xs + b + off, rows, d_terms, 0, st, u16, nullptr, shadow,
                             sld);
            if (r) return r;
            relax_launches++;
        }
        CUDA_TRY(cudaEventRecord(E[ev++], st));  // relax end of level m
    }

    // Cost d[C][q] (R:2137-2138) and the device status, then one host sync.
    int32_t *hp = (int32_t *)c->pinned;
    if (k >= 2) {
        const int64_t C = ((int64_t)1 << (k - 1)) - 1;
        CUDA_TRY(cudaMemcpyAsync(hp, table + C * ld + terms_host[k - 1], sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    } else {
        hp[0] = INF;
    }
    CUDA_TRY(cudaMemcpyAsync(hp + 2, c->stat.ptr, sizeof(DevStat), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    CUDA_TRY(cudaGetLastError());
    DevStat ds;
    std::memcpy(&ds, hp + 2, sizeof(ds));
    if (ds.err) return emv_dev_status_to_emv(ds.err);
    if (check && h_max[1] >= (uint32_t)INF)
        return emv_fail(EMV_ERR_DISCONNECTED, "graph: not connected (a vertex is unreachable from terminal 1)");
    *cost_out = (k >= 2 && hp[0] < INF) ? (int64_t)hp[0] : INT64_MAX;
    if (tm) {
        float ms = 0;
        cudaEventElapsedTime(&ms, E[0], E[1]);
        tm->zero_ms = ms;
        cudaEventElapsedTime(&ms, E[1], E[2]);
        tm->level1_ms = ms;
        tm->merge_ms = tm->relax_ms = 0;
        for (int32_t m = 2; m <= k; m++) {
            const int b = 2 + 2 * (m - 2);  // E[b] merge start, E[b+1] relax start, E[b+2] level end
            cudaEventElapsedTime(&ms, E[b], E[b + 1]);
            tm->merge_ms += ms;
            cudaEventElapsedTime(&ms, E[b + 1], E[b + 2]);
            tm->relax_ms += ms;
        }
        cudaEventElapsedTime(&ms, E[1], E[ev - 1]);
        tm->kernel_ms = ms;
        tm->relax_sweeps = (int64_t)ds.sweeps;
        tm->relax16_levels = levels16;
        tm->merge16_levels = merges16;
        tm->relax_launches = relax_launches;
    }
    return EMV_OK;
}

static int check_k(int32_t n, int32_t k, const int32_t *terms)
{
    if (k < 1 || k > EMV_MAX_K) return emv_fail(EMV_ERR_BAD_INPUT, "k = %d outside [1, %d]", k, EMV_MAX_K);
    if (!terms) return emv_fail(EMV_ERR_BAD_INPUT, "null terminals");
    for (int32_t i = 0; i < k; i++)
        if (terms[i] < 0 || terms[i] >= n) return emv_fail(EMV_ERR_BAD_INPUT, "terminal %d out of range", i);
    return EMV_OK;
}

extern "C" int emv_kernel_dev(emv_ctx *c, int32_t n, int64_t arcs, const int32_t *d_row_ptr, const int32_t *d_col,
                              const int32_t *d_w, int32_t k, const int32_t *terminals, int32_t *d_table, int64_t ld,
                              int64_t *cost_out, void *stream)
{
    if (!c || !d_row_ptr || (arcs > 0 && (!d_col || !d_w)) || !d_table || !cost_out || n <= 0 || arcs < 0 ||
        arcs >= INT32_MAX || ld < n)
        return emv_fail(EMV_ERR_BAD_INPUT, "emv_kernel_dev: bad arguments");
    int r = check_k(n, k, terminals);
    if (r) return r;
    CUDA_TRY(cudaSetDevice(c->device));
    cudaStream_t st = (cudaStream_t)stream;
    c->launches = 0;
    r = pack_and_check(c, n, arcs, d_row_ptr, d_col, d_w, true, st);
    if (r) return r;
    return run_dp(c, n, d_row_ptr, (const int2 *)c->adj.ptr, k, terminals, d_table, ld, st, cost_out, nullptr, true);
}

// Runs the traceback kernel and reduces its edge list to a tree on the host.
int run_traceback(emv_ctx *c, int32_t n, const int32_t *row_ptr, const int2 *adj, int32_t k, const int32_t *table,
                  int64_t ld, cudaStream_t st, emv_result *out)
{
    const int32_t cap = std::max(64, 2 * n);
    int r = dev_reserve(c->tb_edges, sizeof(int32_t) * 3 * (size_t)cap);
    if (!r) r = dev_reserve(c->tb_out, sizeof(int32_t) * 2);
    if (!r) r = dev_reserve(c->tb_work, sizeof(int32_t) * 3 * (size_t)n);
    if (r) return r;
    int32_t *work = (int32_t *)c->tb_work.ptr;
    CUDA_TRY(cudaMemsetAsync(work + 2 * (size_t)n, 0xff, sizeof(int32_t) * (size_t)n, st));
    CUDA_TRY(cudaMemsetAsync(c->tb_out.ptr, 0, sizeof(int32_t) * 2, st));
    TbArgs a;
    a.table = table;
    a.ld = ld;
    a.n = n;
    a.k = k;
    a.row_ptr = row_ptr;
    a.adj = adj;
    a.terms = (const int32_t *)c->terms.ptr;
    a.edges = (int32_t *)c->tb_edges.ptr;
    a.cap = cap;
    a.out = (int32_t *)c->tb_out.ptr;
    a.queue = work;
    a.parent = work + n;
    a.stamp = work + 2 * (size_t)n;
    a.max_steps = 4 * n + 64 * k + 1024;
    CUDA_TRY(cudaEventRecord(c->ev[MAX_EVENTS - 2], st));
    k_traceback<<<1, 32, 0, st>>>(a);
    c->launches++;
    CUDA_TRY(cudaEventRecord(c->ev[MAX_EVENTS - 1], st));
    int32_t hout[2];
    CUDA_TRY(cudaMemcpyAsync(hout, a.out, sizeof(hout), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    float ms = 0;
    cudaEventElapsedTime(&ms, c->ev[MAX_EVENTS - 2], c->ev[MAX_EVENTS - 1]);
    out->timing.traceback_ms = ms;
    if (hout[1]) return emv_dev_status_to_emv((uint32_t)hout[1]);
    std::vector<int32_t> e((size_t)hout[0] * 3);
    if (hout[0] > 0)
        CUDA_TRY(cudaMemcpy(e.data(), a.edges, sizeof(int32_t) * e.size(), cudaMemcpyDeviceToHost));
    // Keep a spanning forest of the emitted edges: duplicates and zero-weight
    // cycles (possible only through zero-weight arcs) are dropped.
    std::vector<int32_t> parent((size_t)n);
    std::iota(parent.begin(), parent.end(), 0);
    auto find = [&](int32_t x) {
        while (parent[(size_t)x] != x) {
            parent[(size_t)x] = parent[(size_t)parent[(size_t)x]];
            x = parent[(size_t)x];
        }
        return x;
    };
    int64_t count = 0, weight = 0;
    for (int32_t i = 0; i < hout[0]; i++) {
        int32_t u = e[(size_t)3 * i], v = e[(size_t)3 * i + 1], wt = e[(size_t)3 * i + 2];
        int32_t ru = find(u), rv = find(v);
        if (ru == rv) continue;
        parent[(size_t)ru] = rv;
        if (out->tree && count < out->tree_cap) {
            out->tree[3 * count] = u;
            out->tree[3 * count + 1] = v;
            out->tree[3 * count + 2] = wt;
        }
        count++;
        weight += wt;
    }
    out->tree_count = count;
    out->tree_weight = weight;
    if (out->tree && count > out->tree_cap)
        return emv_fail(EMV_ERR_BAD_INPUT, "tree buffer holds %lld edges, need %lld", (long long)out->tree_cap,
                        (long long)count);
    return EMV_OK;
}

int solve_on_device(emv_ctx *c, int32_t n, int64_t arcs, const int32_t *row_ptr, const int32_t *col,
                    const int32_t *w, const int32_t *terms, int32_t k, int32_t flags, emv_result *out,
                    cudaStream_t st)
{
    const bool check = !(flags & EMV_SOLVE_NOCHECK);
    int r = pack_and_check(c, n, arcs, row_ptr, col, w, check, st);
    if (r) return r;
    const int64_t ld = ((int64_t)n + 31) / 32 * 32;
    const size_t tbytes = sizeof(int32_t) * (size_t)ld << k;
    r = dev_reserve(c->table, tbytes);
    if (r) return r;
    int32_t *table = (int32_t *)c->table.ptr;
    std::memset(&out->timing, 0, sizeof(out->timing));
    r = run_dp(c, n, row_ptr, (const int2 *)c->adj.ptr, k, terms, table, ld, st, &out->cost, &out->timing, check);
    if (r) return r;
    out->tree_count = 0;
    out->tree_weight = 0;
    if ((flags & EMV_SOLVE_TREE) && k >= 2) {
        r = run_traceback(c, n, row_ptr, (const int2 *)c->adj.ptr, k, table, ld, st, out);
        if (r) return r;
    }
    if ((flags & EMV_SOLVE_TABLE) && out->table) {
        CUDA_TRY(cudaMemcpy2DAsync(out->table, sizeof(int32_t) * (size_t)n, table, sizeof(int32_t) * (size_t)ld,
                                   sizeof(int32_t) * (size_t)n, (size_t)1 << k, cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
    }
    out->timing.launches = c->launches;
    return EMV_OK;
}

extern "C" int emv_solve(emv_ctx *c, const emv_graph *g, const int32_t *terminals, int32_t k, int32_t flags,
                         emv_result *out, void *stream)
{
    if (!c || !out) return emv_fail(EMV_ERR_BAD_INPUT, "null argument");
    int r = emv_graph_validate(g);
    if (r) return r;
    r = check_k(g->n, k, terminals);
    if (r) return r;
    CUDA_TRY(cudaSetDevice(c->device));
    cudaStream_t st = (cudaStream_t)stream;
    c->launches = 0;
    const int32_t n = g->n;
    const int64_t arcs = g->arcs;
    r = dev_reserve(c->g_row, sizeof(int32_t) * ((size_t)n + 1));
    if (!r) r = dev_reserve(c->g_col, sizeof(int32_t) * (size_t)std::max<int64_t>(arcs, 1));
    if (!r) r = dev_reserve(c->g_w, sizeof(int32_t) * (size_t)std::max<int64_t>(arcs, 1));
    if (r) return r;
    CUDA_TRY(cudaMemcpyAsync(c->g_row.ptr, g->row_ptr, sizeof(int32_t) * ((size_t)n + 1), cudaMemcpyHostToDevice, st));
    if (arcs > 0) {
        CUDA_TRY(cudaMemcpyAsync(c->g_col.ptr, g->col, sizeof(int32_t) * (size_t)arcs, cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaMemcpyAsync(c->g_w.ptr, g->w, sizeof(int32_t) * (size_t)arcs, cudaMemcpyHostToDevice, st));
    }
    return solve_on_device(c, n, arcs, (const int32_t *)c->g_row.ptr, (const int32_t *)c->g_col.ptr,
                           (const int32_t *)c->g_w.ptr, terminals, k, flags, out, st);
}

extern "C" int emv_solve_dev(emv_ctx *c, const emv_graph *d_g, const int32_t *terminals, int32_t k, int32_t flags,
                             emv_result *out, void *stream)
{
    if (!c || !out) return emv_fail(EMV_ERR_BAD_INPUT, "null argument");
    int r = emv_graph_validate(d_g);
    if (r) return r;
    r = check_k(d_g->n, k, terminals);
    if (r) return r;
    CUDA_TRY(cudaSetDevice(c->device));
    c->launches = 0;
    return solve_on_device(c, d_g->n, d_g->arcs, d_g->row_ptr, d_g->col, d_g->w, terminals, k, flags, out,
                           (cudaStream_t)stream);
}

extern "C" int emv_sssp(emv_ctx *c, const emv_graph *g, int32_t source, int64_t *dist_out, float *ms_out, void *stream)
{
    if (!c || !dist_out) return emv_fail(EMV_ERR_BAD_INPUT, "null argument");
    int r = emv_graph_validate(g);
    if (r) return r;
    if (source < 0 || source >= g->n) return emv_fail(EMV_ERR_BAD_INPUT, "source out of range");
    CUDA_TRY(cudaSetDevice(c->device));
    cudaStream_t st = (cudaStream_t)stream;
    const int32_t n = g->n;
    const int64_t arcs = g->arcs;
    r = dev_reserve(c->g_row, sizeof(int32_t) * ((size_t)n + 1));
    if (!r) r = dev_reserve(c->g_col, sizeof(int32_t) * (size_t)std::max<int64_t>(arcs, 1));
    if (!r) r = dev_reserve(c->g_w, sizeof(int32_t) * (size_t)std::max<int64_t>(arcs, 1));
    if (!r) r = dev_reserve(c->table, sizeof(int32_t) * 2 * (size_t)n);  // row 1 = {source}
    if (!r) r = dev_reserve(c->terms, sizeof(int32_t));
    if (!r) r = prepare_subsets(c, 1, st);
    if (!r) r = reserve_relax(c, n);
    if (r) return r;
    CUDA_TRY(cudaMemcpyAsync(c->g_row.ptr, g->row_ptr, sizeof(int32_t) * ((size_t)n + 1), cudaMemcpyHostToDevice, st));
    if (arcs > 0) {
        CUDA_TRY(cudaMemcpyAsync(c->g_col.ptr, g->col, sizeof(int32_t) * (size_t)arcs, cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaMemcpyAsync(c->g_w.ptr, g->w, sizeof(int32_t) * (size_t)arcs, cudaMemcpyHostToDevice, st));
    }
    CUDA_TRY(cudaMemcpyAsync(c->terms.ptr, &source, sizeof(int32_t), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemsetAsync(c->stat.ptr, 0, sizeof(DevStat), st));
    r = pack_and_check(c, n, arcs, (const int32_t *)c->g_row.ptr, (const int32_t *)c->g_col.ptr,
                       (const int32_t *)c->g_w.ptr, true, st);
    if (r) return r;
    CUDA_TRY(cudaEventRecord(c->ev[0], st));
    r = launch_relax(c, (const int32_t *)c->g_row.ptr, (const int2 *)c->adj.ptr, n, n, (int32_t *)c->table.ptr,
                     (const uint32_t *)c->kp->xs.ptr, 1, (const int32_t *)c->terms.ptr, 1, st);
    if (r) return r;
    CUDA_TRY(cudaEventRecord(c->ev[1], st));
    std::vector<int32_t> d((size_t)n);
    CUDA_TRY(cudaMemcpyAsync(d.data(), (int32_t *)c->table.ptr + n, sizeof(int32_t) * (size_t)n,
                             cudaMemcpyDeviceToHost, st));
    DevStat ds;
    CUDA_TRY(cudaMemcpyAsync(&ds, c->stat.ptr, sizeof(ds), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    if (ds.err) return emv_dev_status_to_emv(ds.err);
    if (ms_out) cudaEventElapsedTime(ms_out, c->ev[0], c->ev[1]);
    for (int32_t v = 0; v < n; v++) dist_out[v] = d[(size_t)v] >= INF ? INT64_MAX : (int64_t)d[(size_t)v];
    return EMV_OK;
}
