// emv_batch.cuh -- the CTA-resident EMV solver used by batching and serving.
//
// One CTA owns one instance at a time and runs a window of its DP levels with
// CTA barriers only, so no grid-wide synchronisation is needed and thousands
// of independent instances of uneven n and k share one persistent launch.
// Per level m of an instance (reader/reader-el.c:2033-2131):
//   merge  -- vertex blocks of 32 * mw (mw autotuned per class): every row of
//             size < m is staged in shared memory as S[Y][32 * mw], a
//             quarter-warp computes one subset X on one 32-vertex column of
//             the block at a time with 4 vertices per lane (R:2068-2107);
//   relax  -- chunks of R rows are loaded into shared memory vertex-major
//             (stride R+1, or R+4 with 4 rows per lane), and in-place sweeps pull
//             min(d[u] + w) over the CSR until a sweep changes nothing
//             (R:2109-2130), then the rows go back to the table.
// The table of an instance is int32 row-major with ld = n.
#pragma once

#include "emv_batch_types.h"
#include "emv_common.cuh"
#include "emv_device_util.cuh"

namespace emv {

__device__ __forceinline__ int32_t xs_start(const BatchArgs &a, int32_t k, int32_t m)
{
    return __ldg(a.xs_off + k * (BATCH_KMAX + 2) + m);
}

// Merge of level m for one instance; S holds 2^k * 32 * mw int32 (staged
// rows of a block of 32 * mw vertices).  The pair loop runs on quarter-warps:
// the 8 lanes of a quarter hold 4 vertices each of one 32-vertex column (one
// 16-byte shared load per staged row and lane), and the four quarters of a
// warp take four (subset, column) tasks of the level, whose subsets all have
// 2^(m-1) - 1 pairs.  Wider blocks (mw > 1) give the low levels, which have
// few subsets, enough tasks for every quarter-warp and stage less often.
__device__ void batch_merge(const BatchArgs &a, int32_t *table, int32_t n, int32_t k, int32_t m,
                            const int32_t *terms, int32_t *S, int32_t mw)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int ql = lane & 7, nq = nw * 4;
    const int32_t lo_b = xs_start(a, k, 1), lo_e = xs_start(a, k, m);       // rows of size 1..m-1
    const int32_t x_b = xs_start(a, k, m), x_e = xs_start(a, k, m + 1);     // rows of size m
    const uint32_t *xs = a.xs;
    const int32_t bw = 32 * mw;                                   // staged words of a row
    const int32_t tasks = (x_e - x_b) * mw;                       // (subset, column) pairs
    const uint4 *S4 = reinterpret_cast<const uint4 *>(S) + ql;  // row Y, column c, this lane: S4[Y * 8 * mw + c * 8]
    for (int32_t vb = 0; vb < n; vb += bw) {
        // staging: 4-byte asynchronous copies, so a warp has all its rows in flight
        for (int32_t i = lo_b + warp; i < lo_e; i += nw) {
            const uint32_t Y = __ldg(xs + i);
            for (int32_t c = 0; c < mw; c++) {
                const int32_t v = vb + c * 32 + lane;
                if (v < n) cp_async4(S + Y * bw + c * 32 + lane, table + (int64_t)Y * n + v);
                else S[Y * bw + c * 32 + lane] = INF;
            }
        }
        cp_async_wait_all();
        __syncthreads();
        for (int32_t t0 = warp * 4; t0 < tasks; t0 += nq) {
            const int32_t t = t0 + (lane >> 3);
            const bool live = t < tasks;
            const int32_t xi = live ? t / mw : 0, c = live ? t - xi * mw : 0;
            const uint32_t X = __ldg(xs + x_b + xi);
            const uint32_t low = X & (0u - X), rest = X ^ low;
            const uint4 *Sc = S4 + c * 8;
            uint4 acc = make_uint4((uint32_t)INF, (uint32_t)INF, (uint32_t)INF, (uint32_t)INF);
            uint32_t sub = 0;
            do {  // 2^(m-1) - 1 pairs {Y, X\Y}, Y holding X's lowest terminal
                const uint32_t Y = low | sub;
                const uint4 y = Sc[Y * 8 * mw], z = Sc[(X ^ Y) * 8 * mw];
                acc.x = min(acc.x, y.x + z.x);
                acc.y = min(acc.y, y.y + z.y);
                acc.z = min(acc.z, y.z + z.z);
                acc.w = min(acc.w, y.w + z.w);
                sub = (sub - rest) & rest;
            } while (sub != rest);
            if (!live) continue;
            const int32_t v4 = vb + c * 32 + ql * 4;
            for (uint32_t bits = X; bits; bits &= bits - 1) {  // terminal override (R:2099-2107)
                const int ti = __ffs(bits) - 1;
                const int32_t d = terms[ti] - v4;
                if (d < 0 || d >= 4) continue;
                const uint32_t o = (uint32_t)S[(X ^ (1u << ti)) * bw + c * 32 + ql * 4 + d];
                if (d == 0) acc.x = o;
                else if (d == 1) acc.y = o;
                else if (d == 2) acc.z = o;
                else acc.w = o;
            }
            int32_t *row = table + (int64_t)X * n + v4;
            if (v4 < n) row[0] = (int32_t)acc.x;
            if (v4 + 1 < n) row[1] = (int32_t)acc.y;
            if (v4 + 2 < n) row[2] = (int32_t)acc.z;
            if (v4 + 3 < n) row[3] = (int32_t)acc.w;
        }
        __syncthreads();
    }
}

// Closure of the rows xs[b, e) (level-1 mode: row r is {r} with source terms[r]).
// Returns false if the sweep bound was hit.
__device__ bool batch_relax(const BatchArgs &a, int32_t *table, int32_t n, const int32_t *row_ptr, const int2 *adj,
                            const int32_t *terms, int32_t b, int32_t e, int32_t rcap, bool level1, int32_t *S)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int32_t cnt = e - b;
    int32_t R = 1;
    while (R < cnt && R < rcap) R <<= 1;
    const int32_t stride = batch_stride(R);
    // R >= 4: a lane holds 4 consecutive rows of a vertex (16-byte shared loads);
    // else a lane holds one row
    const int32_t RV = R >= 4 ? 4 : 1;
    const int32_t LPV = R / RV;            // lanes per vertex
    const int32_t G = 32 / LPV;            // vertices per warp task
    const int32_t vs = lane / LPV, r = (lane % LPV) * RV;
    bool ok = true;
    for (int32_t c0 = 0; c0 < cnt; c0 += R) {
        const int32_t nr = min(R, cnt - c0);
        auto row_in = [&](int32_t rr, int32_t v) -> int32_t {
            if (rr >= nr) return INF;
            if (level1) return (v == terms[c0 + rr]) ? 0 : INF;
            return table[(int64_t)__ldg(a.xs + b + c0 + rr) * n + v];
        };
        if (RV == 4) {
            // a thread moves 4 rows of one vertex (one 16-byte shared store; with a
            // stride of R + 4 the 8 lanes of a store phase hit distinct banks)
            for (int32_t idx = threadIdx.x; idx < (R / 4) * n; idx += blockDim.x) {
                const int32_t g = idx / n, v = idx - g * n;
                const int4 x = make_int4(row_in(4 * g, v), row_in(4 * g + 1, v), row_in(4 * g + 2, v),
                                         row_in(4 * g + 3, v));
                *reinterpret_cast<int4 *>(S + v * stride + 4 * g) = x;
            }
        } else {
            for (int32_t idx = threadIdx.x; idx < R * n; idx += blockDim.x) {
                const int32_t rr = idx / n, v = idx - rr * n;
                S[v * stride + rr] = row_in(rr, v);
            }
        }
        __syncthreads();
        const int32_t tasks = (n + G - 1) / G;
        int32_t sweep = 0;
        for (;; sweep++) {
            if (sweep > n + 1) { ok = false; break; }
            bool changed = false;
            for (int32_t t = warp; t < tasks; t += nw) {
                const int32_t v = t * G + vs;
                if (v >= n || r >= nr) continue;
                const int32_t beg = __ldg(row_ptr + v), end = __ldg(row_ptr + v + 1);
                if (RV == 4) {  // rows r..r+3 (rows past nr are INF and never written back)
                    int4 *mine = reinterpret_cast<int4 *>(S + v * stride + r);
                    const int4 old = *mine;
                    int4 acc = old;
                    for (int32_t q = beg; q < end; q++) {
                        const int2 arc = __ldg(adj + q);
                        acc = vmin(acc, vadd(*reinterpret_cast<const int4 *>(S + arc.x * stride + r), arc.y));
                    }
                    if (vlt(acc, old)) {
                        *mine = acc;
                        changed = true;
                    }
                } else {
                    const int32_t old = S[v * stride + r];
                    int32_t acc = old;
                    for (int32_t q = beg; q < end; q++) {
                        const int2 arc = __ldg(adj + q);
                        acc = min(acc, S[arc.x * stride + r] + arc.y);
                    }
                    if (acc < old) {
                        S[v * stride + r] = acc;
                        changed = true;
                    }
                }
            }
            if (!__syncthreads_or(changed)) break;
        }
        if (RV == 4) {
            for (int32_t idx = threadIdx.x; idx < ((nr + 3) / 4) * n; idx += blockDim.x) {
                const int32_t g = idx / n, v = idx - g * n;
                const int4 x = *reinterpret_cast<const int4 *>(S + v * stride + 4 * g);
                const int32_t r0 = 4 * g;
                table[(int64_t)__ldg(a.xs + b + c0 + r0) * n + v] = x.x;
                if (r0 + 1 < nr) table[(int64_t)__ldg(a.xs + b + c0 + r0 + 1) * n + v] = x.y;
                if (r0 + 2 < nr) table[(int64_t)__ldg(a.xs + b + c0 + r0 + 2) * n + v] = x.z;
                if (r0 + 3 < nr) table[(int64_t)__ldg(a.xs + b + c0 + r0 + 3) * n + v] = x.w;
            }
        } else {
            for (int32_t idx = threadIdx.x; idx < nr * n; idx += blockDim.x) {
                const int32_t rr = idx / n, v = idx - rr * n;
                table[(int64_t)__ldg(a.xs + b + c0 + rr) * n + v] = S[v * stride + rr];
            }
        }
        __syncthreads();
        if (!ok) break;
    }
    return ok;
}

// Runs levels [lo, hi] of one instance with the whole CTA.
__device__ void batch_solve_one(const BatchArgs &a, const BatchInst &I, int32_t *S)
{
    const int32_t n = I.n, k = I.k;
    int32_t *table = I.table;
    const int32_t *row_ptr = I.row_ptr;
    const int2 *adj = I.adj;
    const int32_t *terms = I.terms;
    bool ok = true;
    for (int32_t m = I.lo; m <= I.hi && ok; m++) {
        if (m == 1) {
            for (int32_t v = threadIdx.x; v < n; v += blockDim.x) table[v] = INF;  // row 0
            ok = batch_relax(a, table, n, row_ptr, adj, terms, xs_start(a, k, 1), xs_start(a, k, 2), I.rcap, true, S);
        } else {
            batch_merge(a, table, n, k, m, terms, S, I.mw);
            ok = batch_relax(a, table, n, row_ptr, adj, terms, xs_start(a, k, m), xs_start(a, k, m + 1), I.rcap,
                             false, S);
        }
    }
    if (threadIdx.x == 0) {
        if (!ok) atomicOr(a.err, (uint32_t)EMV_DEV_SWEEP_LIMIT);
        if (I.hi == k) {
            int64_t cost = INT64_MAX;
            if (k >= 2) {
                const int32_t x = table[(int64_t)((1 << (k - 1)) - 1) * n + terms[k - 1]];
                if (x < INF) cost = x;
            }
            a.costs[I.orig] = cost;
        }
    }
}

// Persistent kernel: CTAs pull work items (instances in the given order,
// largest first) from a device counter until the queue is empty.
__global__ void __launch_bounds__(BATCH_THREADS, 1) k_batch(BatchArgs a)
{
    extern __shared__ __align__(16) int32_t S[];
    __shared__ int32_t s_idx;
    for (;;) {
        if (threadIdx.x == 0) s_idx = (int32_t)atomicAdd(a.queue, 1u);
        __syncthreads();
        const int32_t idx = s_idx;
        __syncthreads();
        if (idx >= a.count) break;
        const BatchInst I = a.inst[idx];
        batch_solve_one(a, I, S);
        __syncthreads();
    }
}

}  // namespace emv
