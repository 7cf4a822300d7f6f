// emv_noalloc.cu -- a shortest-path closure entry point that allocates no
// device memory (C ABI, include/emv.h: emv_closure_noalloc).
//
// Some callers of this library cannot allocate device memory at the time they
// call it: code that runs while another framework owns every byte of the
// device through its own pool, code that must not trigger the device-wide
// synchronisation of cudaMalloc/cudaFree in a latency-critical loop, and
// plug-ins whose host application forbids allocation after start-up.  For
// them this file keeps the closure's working memory in one file-scope device
// array of fixed size, reserved when the library is loaded on a device and
// held until the process exits, and reuses it on every call.
//
// The computation is the same multi-source closure as the relaxation kernel
// of emv_kernels.cuh (the reference's dijkstra run from a virtual source,
// reader/reader-el.c:1762-1880 and 2109-2130), in a variant that reads the
// CSR's col and w arrays as given instead of a packed copy:
//   out[r][v] = min over u of init[r][u] + dist(u, v),  r < rows <= 32.
// Each call first checks the CSR on the device (k_noalloc_scan) and returns
// EMV_ERR_BAD_INPUT / EMV_ERR_OVERFLOW before the closure reads it; in the
// closure a value plus a weight saturates at EMV_INF32 instead of wrapping,
// and a finite candidate that saturates where no smaller one exists is
// reported as EMV_ERR_OVERFLOW.
#include <algorithm>
#include <mutex>

#include "emv_device_util.cuh"
#include "emv_solver.h"

using namespace emv;

namespace {

constexpr int32_t NOALLOC_MAX_N = 131072;      // vertices
constexpr int32_t NOALLOC_MAX_ROWS = 32;       // rows per call (one per lane)
constexpr size_t REC_BYTES = (size_t)NOALLOC_MAX_N * NOALLOC_MAX_ROWS * sizeof(int32_t);  // 16 MiB
constexpr size_t FLAG_BYTES = (size_t)NOALLOC_MAX_N;                                     // per flag array
constexpr size_t CTRL_OFF = REC_BYTES + 2 * FLAG_BYTES;
constexpr size_t STAT_OFF = CTRL_OFF + (sizeof(uint32_t) * C_WORDS + 255) / 256 * 256;
static_assert(CTRL_OFF % 128 == 0, "control words on their own lines");
constexpr size_t SCAN_OFF = STAT_OFF + 64;
constexpr size_t NOALLOC_BYTES = STAT_OFF + 256;
static_assert(SCAN_OFF + sizeof(GraphScan) <= NOALLOC_BYTES, "scan words inside the status area");
constexpr int NOALLOC_THREADS = 512;
constexpr int MAX_DEVICES = 64;

// The scratch of every call on this device: vertex-major records, two
// active-flag arrays, the barrier words and the status words.
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

std::mutex g_setup_mu;
unsigned char *g_scratch_ptr[MAX_DEVICES] = {};
int g_blocks[MAX_DEVICES] = {};

struct NoallocArgs {
    const int32_t *row_ptr;
    const int32_t *col;
    const int32_t *w;
    const int32_t *init;
    int32_t *out;
    int64_t ld;
    int32_t n;
    int32_t rows;
    int32_t *rec;
    uint8_t *act0;
    uint8_t *act1;
    uint32_t *ctrl;
    DevStat *stat;
};

// The device check of the caller's CSR, into the scratch's status area.
__global__ void k_noalloc_scan(const int32_t *__restrict__ row_ptr, int32_t n, const int32_t *__restrict__ col,
                               const int32_t *__restrict__ w, int64_t arcs, GraphScan *__restrict__ scan)
{
    scan_csr(row_ptr, n, col, w, nullptr, arcs, scan);
}

// val + wt saturated at INF (wt is in [0, INF) after the scan, val <= INF);
// *sat is set when a finite val saturated.
__device__ __forceinline__ int32_t sat_add(int32_t val, int32_t wt, bool *sat)
{
    const int32_t room = INF - wt;
    *sat |= (val < INF) & (val >= room);
    return min(val, room) + wt;
}

// Same phases as k_relax<1>: rows -> records, frontier sweeps, records -> rows.
__global__ void __launch_bounds__(NOALLOC_THREADS, 2) k_closure_noalloc(NoallocArgs a)
{
    __shared__ int32_t tile[32][33];
    __shared__ int s_ok;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwb = blockDim.x >> 5;
    const int32_t n = a.n, ntiles = (n + 31) >> 5;
    bool bad_value = false;
    for (int32_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int32_t v = t * 32 + lane;
        for (int r = warp; r < 32; r += nwb) {
            const int32_t x = (r < a.rows && v < n) ? a.init[(int64_t)r * a.ld + v] : INF;
            bad_value |= x > INF;
            tile[r][lane] = min(x, INF);
        }
        __syncthreads();
        for (int vv = warp; vv < 32; vv += nwb) {
            const int32_t v2 = t * 32 + vv;
            if (v2 < n) __stcg(a.rec + (int64_t)v2 * 32 + lane, tile[lane][vv]);
        }
        __syncthreads();
    }
    for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        a.act0[v] = 1;
        a.act1[v] = 0;
    }
    if (__any_sync(FULL, bad_value) && lane == 0) atomicOr(&a.stat->err, (uint32_t)EMV_DEV_BAD_VALUE);
    bool overflow = false;
    if (!grid_barrier(a.ctrl, &s_ok)) {
        if (threadIdx.x == 0) atomicOr(&a.stat->err, a.ctrl[C_ERR]);
        return;
    }
    const int32_t gw = (int32_t)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int32_t nwg = (int32_t)((gridDim.x * blockDim.x) >> 5);
    volatile uint32_t *vctrl = a.ctrl;
    int32_t s = 0;
    bool converged = false;
    for (; s <= n; s++) {
        uint8_t *cur = (s & 1) ? a.act1 : a.act0;
        uint8_t *nxt = (s & 1) ? a.act0 : a.act1;
        if (blockIdx.x == 0 && threadIdx.x == 0) vctrl[C_SLOT0 + (s + 1) % 3] = 0;
        bool any = false;
        for (int32_t blk = gw; blk < ntiles; blk += nwg) {
            const int32_t v = blk * 32 + lane;
            const bool f = v < n && __ldcg(cur + v) != 0;
            unsigned act = __ballot_sync(FULL, f);
            if (!act) continue;
            if (f) cur[v] = 0;
            const int32_t rp0 = v < n ? __ldg(a.row_ptr + v) : 0;
            const int32_t rp1 = v < n ? __ldg(a.row_ptr + v + 1) : 0;
            while (act) {
                const int j = __ffs(act) - 1;
                act &= act - 1;
                const int32_t vv = blk * 32 + j;
                const int32_t beg = __shfl_sync(FULL, rp0, j), end = __shfl_sync(FULL, rp1, j);
                int32_t *mine = a.rec + (int64_t)vv * 32 + lane;
                const int32_t old = __ldcg(mine);
                int32_t acc = old;
                bool sat = false;
                for (int32_t e0 = beg; e0 < end; e0 += 32) {
                    int32_t cu = 0, cw = 0;
                    if (e0 + lane < end) {
                        cu = __ldg(a.col + e0 + lane);
                        cw = __ldg(a.w + e0 + lane);
                    }
                    const int cnt = min(32, end - e0);
                    for (int g = 0; g < cnt; g += 8) {
                        int32_t val[8], wt[8];
#pragma unroll
                        for (int i = 0; i < 8; i++) {
                            const int32_t u = __shfl_sync(FULL, cu, (g + i) & 31);
                            wt[i] = __shfl_sync(FULL, cw, (g + i) & 31);
                            val[i] = (g + i < cnt) ? __ldcg(a.rec + (int64_t)u * 32 + lane) : INF;
                        }
#pragma unroll
                        for (int i = 0; i < 8; i++) acc = min(acc, sat_add(val[i], wt[i], &sat));
                    }
                }
                overflow |= sat & (acc >= INF);
                const bool dec = acc < old;
                if (dec) __stcg(mine, acc);
                if (__ballot_sync(FULL, dec)) {
                    any = true;
                    for (int32_t e = beg + lane; e < end; e += 32) nxt[__ldg(a.col + e)] = 1;
                }
            }
        }
        any = __syncthreads_or(any);
        if (any && threadIdx.x == 0) vctrl[C_SLOT0 + s % 3] = 1;
        if (!grid_barrier(a.ctrl, &s_ok)) {
            if (threadIdx.x == 0) atomicOr(&a.stat->err, a.ctrl[C_ERR]);
            return;
        }
        if (vctrl[C_SLOT0 + s % 3] == 0) {
            converged = true;
            break;
        }
    }
    if (__any_sync(FULL, overflow) && lane == 0) atomicOr(&a.stat->err, (uint32_t)EMV_DEV_OVERFLOW);
    if (!converged) {
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(&a.stat->err, (uint32_t)EMV_DEV_SWEEP_LIMIT);
        return;
    }
    for (int32_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        for (int vv = warp; vv < 32; vv += nwb) {
            const int32_t v2 = t * 32 + vv;
            tile[vv][lane] = (v2 < n) ? __ldcg(a.rec + (int64_t)v2 * 32 + lane) : INF;
        }
        __syncthreads();
        const int32_t v = t * 32 + lane;
        if (v < n)
            for (int r = warp; r < a.rows; r += nwb) a.out[(int64_t)r * a.ld + v] = tile[lane][r];
        __syncthreads();
    }
}

// Per-device set-up, done once with that device current: the device address
// of the scratch array (its host-side name is only a stand-in) and the
// cooperative grid size.  No allocation happens here either.
int setup_device(int dev)
{
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (g_scratch_ptr[dev]) return EMV_OK;
    int coop = 0;
    cudaError_t ec = cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    if (ec != cudaSuccess || !coop) {
        cudaGetLastError();
        return emv_fail(EMV_ERR_CUDA, "emv_closure_noalloc: device %d does not support cooperative launches", dev);
    }
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
        cudaGetLastError();
        return emv_fail(EMV_ERR_CUDA, "scratch symbol address: %s", cudaGetErrorString(e));
    }
    int per_sm = 0, sms = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_closure_noalloc, NOALLOC_THREADS, 0);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return emv_fail(EMV_ERR_CUDA, "occupancy query: %s", cudaGetErrorString(e));
    }
    g_blocks[dev] = std::max(1, per_sm) * std::max(1, sms);
    g_scratch_ptr[dev] = (unsigned char *)p;
    return EMV_OK;
}

}  // namespace

extern "C" int emv_closure_noalloc(int32_t n, int64_t arcs, const int32_t *d_row_ptr, const int32_t *d_col,
                                   const int32_t *d_w, const int32_t *d_init, int32_t rows, int64_t ld,
                                   int32_t *d_out, void *stream)
{
    if (n <= 0 || arcs < 0 || arcs >= INT32_MAX || !d_row_ptr || (arcs > 0 && (!d_col || !d_w)) || !d_init ||
        !d_out || rows < 1 || ld < n)
        return emv_fail(EMV_ERR_BAD_INPUT, "emv_closure_noalloc: bad arguments");
    if (n > NOALLOC_MAX_N || rows > NOALLOC_MAX_ROWS)
        return emv_fail(EMV_ERR_BAD_INPUT,
                        "emv_closure_noalloc: n = %d, rows = %d exceed the fixed scratch (n <= %d, rows <= %d)", n,
                        rows, NOALLOC_MAX_N, NOALLOC_MAX_ROWS);
    int dev = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= MAX_DEVICES) return emv_fail(EMV_ERR_BAD_INPUT, "device %d", dev);
    int r = setup_device(dev);
    if (r) return r;
    unsigned char *base = g_scratch_ptr[dev];
    cudaStream_t st = (cudaStream_t)stream;
    // The call waits on the stream (the check and the status reads), which a
    // capturing stream does not allow: refuse before touching the stream.
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    CUDA_TRY(cudaStreamIsCapturing(st, &cap));
    if (cap != cudaStreamCaptureStatusNone)
        return emv_fail(EMV_ERR_BAD_INPUT, "emv_closure_noalloc: the stream is capturing; this call cannot be captured");
    NoallocArgs a;
    a.row_ptr = d_row_ptr;
    a.col = d_col;
    a.w = d_w;
    a.init = d_init;
    a.out = d_out;
    a.ld = ld;
    a.n = n;
    a.rows = rows;
    a.rec = (int32_t *)base;
    a.act0 = base + REC_BYTES;
    a.act1 = base + REC_BYTES + FLAG_BYTES;
    a.ctrl = (uint32_t *)(base + CTRL_OFF);
    a.stat = (DevStat *)(base + STAT_OFF);
    // The array keeps the last call's contents: the barrier, status and check
    // words must start at zero (records and flags are rewritten by the kernel).
    CUDA_TRY(cudaMemsetAsync(base + CTRL_OFF, 0, NOALLOC_BYTES - CTRL_OFF, st));
    // Check the CSR before the closure reads it (heads index the records).
    GraphScan *d_scan = (GraphScan *)(base + SCAN_OFF), hs;
    const int64_t scan_work = std::max<int64_t>(arcs, (int64_t)n + 1);
    k_noalloc_scan<<<(unsigned)std::min<int64_t>(1024, (scan_work + 255) / 256), 256, 0, st>>>(d_row_ptr, n, d_col,
                                                                                                  d_w, arcs, d_scan);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaMemcpyAsync(&hs, d_scan, sizeof(hs), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    if (hs.bad & SCAN_BAD_ROWS) return emv_fail(EMV_ERR_BAD_INPUT, "emv_closure_noalloc: row_ptr not from 0 to arcs, non-decreasing");
    if (hs.bad & SCAN_BAD_HEAD) return emv_fail(EMV_ERR_BAD_INPUT, "emv_closure_noalloc: arc head out of range");
    if (hs.bad & SCAN_BAD_WEIGHT) return emv_fail(EMV_ERR_BAD_INPUT, "emv_closure_noalloc: negative weight");
    if (hs.bad & SCAN_BIG_WEIGHT) return emv_fail(EMV_ERR_OVERFLOW, "emv_closure_noalloc: an arc weight reaches 2^30");
    const int vpb = NOALLOC_THREADS;  // 32 vertices per warp
    const int blocks = std::min(g_blocks[dev], std::max(1, (n + vpb - 1) / vpb));
    void *args[] = {&a};
    CUDA_TRY(cudaLaunchCooperativeKernel((const void *)k_closure_noalloc, dim3(blocks), dim3(NOALLOC_THREADS), args, 0,
                                         st));
    DevStat ds;
    CUDA_TRY(cudaMemcpyAsync(&ds, a.stat, sizeof(ds), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    if (ds.err) return emv_dev_status_to_emv(ds.err);
    return EMV_OK;
}
