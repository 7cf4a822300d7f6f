// emv_kernels.cuh -- sm_103a kernels of the EMV dynamic program.
//
// Table: int32 d[X * ld + v], subset-major like the reference's FV_INDEX
// (reader/reader-el.c:691), EMV_INF32 = 2^30 for "no value".  All finite
// values are below 2^30 (checked before the DP runs), so a + b of two table values
// fits in uint32 and a value + an arc weight fits in int32.
//
// Kernels (reference step each one replaces):
//   k_fill        f_v = INF                          R:2243-2259
//   k_pack_scan   (col, w) arcs packed as int2        R:794-826 (adjacency fill)
//                 and the device CSR checked
//   k_merge, k_merge_smem, k_merge_stream, k_merge_stream16
//                 subset merge of one level           R:2068-2107
//   k_relax<VEC, U16>  multi-source closure of <= 32*VEC rows (64*VEC with
//                 16-bit records; VEC = 1, 2, 4, 5, 8) R:2109-2130, R:1762-1880
//                 (also the k level-1 SSSPs,          R:1988-2031)
//   k_traceback   tree recovery by recomputation      R:1907-1944
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "emv_common.cuh"
#include "emv_device_util.cuh"

namespace emv {

struct RelaxArgs {
    const int32_t *row_ptr;
    const int2 *adj;
    int32_t n;
    int64_t ld;
    int32_t *table;
    const uint32_t *rows;   // subsets of this chunk
    int32_t nrows;          // <= 32 * VEC of the launch
    const int32_t *terms;   // level-1 mode: row r is {r}, source terms[r]
    int32_t level1;
    int32_t *scratch;       // vertex-major records, n * 32 * VEC int32
    uint8_t *act0;          // active flags, n bytes each
    uint8_t *act1;
    uint32_t *ctrl;         // C_WORDS words
    DevStat *stat;
    int32_t max_sweeps;
    int32_t *stamp;         // n: last sweep in which the vertex changed (-1 none)
    int32_t dense_min;      // a sweep after one with more changed vertices takes every vertex
    int32_t pull_all_min;   // a sweep after one with at least this many changed vertices reads no stamps
    uint32_t *vmax;         // if set: atomicMax of every value phase C writes
    uint16_t *shadow;       // if set: phase C also writes min(value, 0xffff) to shadow[X * shadow_ld + v]
    int64_t shadow_ld;
};

__global__ void k_fill(int32_t *__restrict__ p, int64_t count, int32_t value)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (; i < count; i += stride) p[i] = value;
}

// Packs the (col, w) arcs as int2 and checks the device CSR on the way (the
// admission check of the device entry points; the reference reads only
// well-formed STP, R:473-618): heads in [0, n), weights in [0, 2^30), row_ptr
// from 0 to arcs and non-decreasing.  Reduces the largest weight and the
// weight sum for the value bound.  *scan must be zero before the launch.
__global__ void k_pack_scan(const int32_t *__restrict__ row_ptr, int32_t n, const int32_t *__restrict__ col,
                            const int32_t *__restrict__ w, int2 *__restrict__ adj, int64_t arcs,
                            GraphScan *__restrict__ scan)
{
    scan_csr(row_ptr, n, col, w, adj, arcs, scan);
}

// Subset merge of one level m (R:2068-2088) plus the terminal override of
// the virtual-source arcs (R:2099-2107).  Block (vertex block of 32, group
// of subsets); a warp takes one subset X at a time and its lanes 32 vertices.
// The unordered pairs {Y, X\Y} are enumerated once each (Y holds the lowest
// terminal of X); min is order-independent, so the values equal the
// reference's ordered-pair loop.  Lower-level rows are read-only here.
__global__ void __launch_bounds__(256) k_merge(int32_t *__restrict__ table, int64_t ld, int32_t n,
                                               const uint32_t *__restrict__ xs, int32_t cnt, int32_t xper,
                                               const int32_t *__restrict__ terms, int32_t k)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int32_t v = blockIdx.x * 32 + lane;
    const int32_t xb = blockIdx.y * xper, xe = min(cnt, xb + xper);
    if (v >= n) return;
    for (int32_t xi = xb + warp; xi < xe; xi += nw) {
        const uint32_t X = __ldg(xs + xi);
        const uint32_t low = X & (0u - X), rest = X ^ low;
        uint32_t acc = (uint32_t)INF;
        uint32_t s = 0;
        do {
            const uint32_t Y = low | s, Z = X ^ Y;
            const uint32_t a = (uint32_t)__ldg(table + (int64_t)Y * ld + v);
            const uint32_t b = (uint32_t)__ldg(table + (int64_t)Z * ld + v);
            acc = min(acc, a + b);
            s = (s - rest) & rest;
        } while (s != rest);
        for (uint32_t bits = X; bits; bits &= bits - 1) {
            const int t = __ffs(bits) - 1;
            if (__ldg(terms + t) == v) acc = (uint32_t)__ldg(table + (int64_t)(X ^ (1u << t)) * ld + v);
        }
        table[(int64_t)X * ld + v] = (int32_t)acc;
    }
}

// Shared-memory subset merge of one level m (R:2068-2107).  Block = VB
// consecutive vertices; it stages every row of size 1..m-1 for them once
// (S[slot][VB], slot = position in level order), then computes all C(k,m)
// rows of the level: a warp takes one subset X at a time, lane = (slice,
// vertex) with 32/VB slices splitting X's pair list, combined by shuffles.
// pairs[x * npairs + p] packs the staged slots of Y and X\Y of the p-th
// unordered pair {Y, X\Y} of the x-th subset (Y holds the lowest terminal of
// X); ovr[x * m + i] packs (terminal index << 16 | slot of X\{t}) for the
// override of the virtual-source arcs (R:2099-2107).
template <int VB>
__global__ void __launch_bounds__(1024) k_merge_smem(int32_t *__restrict__ table, int64_t ld, int32_t n,
                                                     const uint32_t *__restrict__ xs_level, int32_t cnt,
                                                     const uint32_t *__restrict__ stage_rows, int32_t nstage,
                                                     const uint32_t *__restrict__ pairs, int32_t npairs,
                                                     const uint32_t *__restrict__ ovr, int32_t m,
                                                     const int32_t *__restrict__ terms)
{
    extern __shared__ int32_t S[];
    __shared__ uint32_t red[32 * 32];  // per-subset partial minima when warps share a subset
    constexpr int G = 32 / VB;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int32_t v0 = blockIdx.x * VB;
    for (int32_t idx = threadIdx.x; idx < nstage * VB; idx += blockDim.x) {
        const int32_t i = idx / VB, j = idx - i * VB;
        const int32_t v = v0 + j;
        S[idx] = (v < n) ? __ldg(table + (int64_t)__ldg(stage_rows + i) * ld + v) : INF;
    }
    // Few subsets (the top levels): split each subset's pairs over `parts` warps.
    const int parts = cnt >= nw ? 1 : nw / cnt;
    if (parts > 1)
        for (int i = threadIdx.x; i < cnt * VB; i += blockDim.x) red[i] = (uint32_t)INF;
    __syncthreads();
    const int slice = lane / VB, j = lane % VB;
    const int32_t v = v0 + j;
    const int32_t tasks = cnt * parts;
    for (int32_t t = warp; t < tasks; t += nw) {
        const int32_t xi = t / parts, part = t - xi * parts;
        const uint32_t *P = pairs + (int64_t)xi * npairs;
        const int32_t step = G * parts;
        uint32_t acc = (uint32_t)INF, acc2 = (uint32_t)INF;
        int32_t p = part * G + slice;
        for (; p + step < npairs; p += 2 * step) {
            const uint32_t q0 = __ldg(P + p), q1 = __ldg(P + p + step);
            acc = min(acc, (uint32_t)S[(q0 & 0xffffu) * VB + j] + (uint32_t)S[(q0 >> 16) * VB + j]);
            acc2 = min(acc2, (uint32_t)S[(q1 & 0xffffu) * VB + j] + (uint32_t)S[(q1 >> 16) * VB + j]);
        }
        if (p < npairs) {
            const uint32_t q0 = __ldg(P + p);
            acc = min(acc, (uint32_t)S[(q0 & 0xffffu) * VB + j] + (uint32_t)S[(q0 >> 16) * VB + j]);
        }
        acc = min(acc, acc2);
#pragma unroll
        for (int off = 16; off >= VB; off >>= 1) acc = min(acc, __shfl_xor_sync(FULL, acc, off));
        if (parts > 1) {
            if (slice == 0) atomicMin(&red[xi * VB + j], acc);
            continue;
        }
        if (slice == 0 && v < n) {
            const uint32_t *O = ovr + (int64_t)xi * m;
            for (int i = 0; i < m; i++) {
                const uint32_t o = __ldg(O + i);
                if (__ldg(terms + (o >> 16)) == v) acc = (uint32_t)S[(o & 0xffffu) * VB + j];
            }
            table[(int64_t)__ldg(xs_level + xi) * ld + v] = (int32_t)acc;
        }
    }
    if (parts > 1) {
        __syncthreads();
        for (int32_t xi = warp; xi < cnt; xi += nw) {
            if (slice != 0 || v >= n) continue;
            uint32_t acc = red[xi * VB + j];
            const uint32_t *O = ovr + (int64_t)xi * m;
            for (int i = 0; i < m; i++) {
                const uint32_t o = __ldg(O + i);
                if (__ldg(terms + (o >> 16)) == v) acc = (uint32_t)S[(o & 0xffffu) * VB + j];
            }
            table[(int64_t)__ldg(xs_level + xi) * ld + v] = (int32_t)acc;
        }
    }
}

// One phase of the streamed merge: a set of staged rows (of sizes j and m-j)
// and, for every subset X of the launch's group, the pairs {Y, X\Y} whose
// halves are both staged, as staged positions (posY | posZ << 16) padded with
// (pad, pad) to whole quads (pad = nrows, a staged row of INF).  X's quads are
// pairs[4 * qoff[x] .. 4 * qoff[x + 1]).
struct MergePhase {
    const uint32_t *rows;   // staged subsets
    const uint32_t *pairs;  // 16-byte aligned
    const uint32_t *qoff;   // cnt + 1 quad offsets
    int32_t nrows;
    int32_t pad_;
};

// Streamed subset merge of level m (R:2068-2107).  Block = 32 consecutive
// vertices; the minima of a group of the level's subsets (all C(k,m) when
// they fit) live in shared memory (acc) while the phases stage only rows of
// sizes j and m-j (all of them, or tiles of them for large k).
// The pair loop runs on quarter-warps: the 8 lanes of a quarter hold 4
// vertices each, so one 16-byte shared load per lane brings a whole staged
// row (128 bytes, one conflict-free wavefront per quarter) and one decoded
// pair serves 32 vertices; the four quarters of a warp take four different
// subsets.  Subsets with few pairs (the top levels) split their list over
// several quarters; partial minima meet in acc through shared-memory
// atomicMin.  The terminal override of the virtual-source arcs
// (R:2099-2107) is applied last, from the finished level m-1 rows.

__device__ __forceinline__ void merge_pair4(uint4 &a, const uint4 *__restrict__ S4, uint32_t pr)
{
    const uint4 y = S4[(pr & 0xffffu) * 8];
    const uint4 z = S4[(pr >> 16) * 8];
    a.x = min(a.x, y.x + z.x);
    a.y = min(a.y, y.y + z.y);
    a.z = min(a.z, y.z + z.z);
    a.w = min(a.w, y.w + z.w);
}

__global__ void __launch_bounds__(1024) k_merge_stream(int32_t *__restrict__ table, int64_t ld, int32_t n,
                                                       const uint32_t *__restrict__ xs_level, int32_t cnt,
                                                       const MergePhase *__restrict__ phases, int32_t nphase,
                                                       const int32_t *__restrict__ terms, int32_t k,
                                                       uint32_t *__restrict__ level_max)
{
    extern __shared__ __align__(16) uint32_t sm[];
    uint32_t *acc = sm;
    uint32_t *S = sm + (size_t)cnt * 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int nq = nw * 4, qid = warp * 4 + (lane >> 3), ql = lane & 7;
    const int32_t v0 = blockIdx.x * 32, v = v0 + lane;
    __shared__ uint32_t s_max;
    if (threadIdx.x == 0) s_max = 0;
    for (int32_t i = threadIdx.x; i < cnt * 32; i += blockDim.x) acc[i] = (uint32_t)INF;
    const int parts = cnt >= nq ? 1 : nq / cnt;
    const uint4 *S4 = reinterpret_cast<const uint4 *>(S) + ql;  // staged row r, this lane's 4 vertices: S4[r * 8]
    const uint4 inf4 = make_uint4((uint32_t)INF, (uint32_t)INF, (uint32_t)INF, (uint32_t)INF);
    for (int32_t ph = 0; ph < nphase; ph++) {
        const MergePhase P = phases[ph];
        __syncthreads();
        if (v0 + 32 <= n) {
            // staging of a full vertex block: 4-byte asynchronous copies, so a
            // warp has all its rows in flight at once (row ids 32 at a time)
            for (int32_t c0 = warp * 32; c0 < P.nrows; c0 += nw * 32) {
                const uint32_t myr = c0 + lane < P.nrows ? __ldg(P.rows + c0 + lane) : 0u;
                const int32_t nr = min(32, P.nrows - c0);
                for (int32_t j = 0; j < nr; j++) {
                    const uint32_t r = __shfl_sync(FULL, myr, j);
                    cp_async4(S + (c0 + j) * 32 + lane, table + (int64_t)r * ld + v);
                }
            }
            if (warp == nw - 1) S[P.nrows * 32 + lane] = (uint32_t)INF;
            cp_async_wait_all();
        } else {
            for (int32_t i = warp; i <= P.nrows; i += nw)
                S[i * 32 + lane] = (i < P.nrows && v < n)
                                       ? (uint32_t)__ldg(table + (int64_t)__ldg(P.rows + i) * ld + v)
                                       : (uint32_t)INF;
        }
        __syncthreads();
        for (int32_t t = qid; t < cnt * parts; t += nq) {
            const int32_t xi = t / parts, part = t - xi * parts;
            const uint32_t qb = __ldg(P.qoff + xi);
            const int32_t quads = (int32_t)(__ldg(P.qoff + xi + 1) - qb);
            const uint4 *Q = reinterpret_cast<const uint4 *>(P.pairs) + qb;
            uint4 a0 = inf4, a1 = inf4;
            int32_t qi = part;
            // two quads of pairs in flight ahead of the one being reduced
            const uint4 zq = make_uint4(0, 0, 0, 0);
            uint4 q = qi < quads ? __ldg(Q + qi) : zq;
            uint4 q1 = qi + parts < quads ? __ldg(Q + qi + parts) : zq;
            while (qi < quads) {
                const int32_t q2i = qi + 2 * parts;
                const uint4 q2 = q2i < quads ? __ldg(Q + q2i) : zq;
                merge_pair4(a0, S4, q.x);
                merge_pair4(a1, S4, q.y);
                merge_pair4(a0, S4, q.z);
                merge_pair4(a1, S4, q.w);
                q = q1;
                q1 = q2;
                qi += parts;
            }
            uint32_t *A = acc + xi * 32 + ql * 4;
            const uint4 r = make_uint4(min(a0.x, a1.x), min(a0.y, a1.y), min(a0.z, a1.z), min(a0.w, a1.w));
            if (parts == 1) {
                uint4 *A4 = reinterpret_cast<uint4 *>(A);
                const uint4 o = *A4;
                *A4 = make_uint4(min(o.x, r.x), min(o.y, r.y), min(o.z, r.z), min(o.w, r.w));
            } else {
                atomicMin(A + 0, r.x);
                atomicMin(A + 1, r.y);
                atomicMin(A + 2, r.z);
                atomicMin(A + 3, r.w);
            }
        }
    }
    __syncthreads();
    bool has_term = false;
    for (int t = 0; t < k; t++) {
        const int32_t tv = __ldg(terms + t);
        has_term |= (tv >= v0 && tv < v0 + 32);
    }
    uint32_t vmax = 0;  // largest value written: the relaxation's record width follows it
    if (v < n)
        for (int32_t xi = warp; xi < cnt; xi += nw) {
            const uint32_t X = __ldg(xs_level + xi);
            uint32_t a = acc[xi * 32 + lane];
            if (has_term)
                for (uint32_t bits = X; bits; bits &= bits - 1) {
                    const int t = __ffs(bits) - 1;
                    if (__ldg(terms + t) == v) a = (uint32_t)table[(int64_t)(X ^ (1u << t)) * ld + v];
                }
            table[(int64_t)X * ld + v] = (int32_t)a;
            vmax = max(vmax, a);
        }
    vmax = __reduce_max_sync(FULL, vmax);
    if (lane == 0) atomicMax(&s_max, vmax);
    __syncthreads();
    if (threadIdx.x == 0) atomicMax(level_max, s_max);
}

// 16-bit streamed merge: the same plan and phases as k_merge_stream, for a
// level whose sums of two staged values are all at most 65533 (the host
// checks the level maxima).  A block takes 64 vertices; a staged row holds
// them as 32 words of two 16-bit values (the same 128 bytes per row), so one
// 16-byte shared load brings 8 vertices and one min(y + z, a) per halfword
// (__viaddmin_u16x2) serves two.  The pad row is all ones: a pad pair sums to
// at least 0xfffe, above every real candidate.  Rows are staged through
// registers (int2 loads, packed to 16 bits), so the table stride and base
// must be even.  Minima live in acc as 16-bit pairs, or as one uint32 per
// vertex where quarters split a subset's pairs (shared-memory atomicMin).
__device__ __forceinline__ void merge_pair8(uint4 &a, const uint4 *__restrict__ S4, uint32_t pr)
{
    const uint4 y = S4[(pr & 0xffffu) * 8];
    const uint4 z = S4[(pr >> 16) * 8];
    a.x = addmin16(y.x, z.x, a.x);
    a.y = addmin16(y.y, z.y, a.y);
    a.z = addmin16(y.z, z.z, a.z);
    a.w = addmin16(y.w, z.w, a.w);
}

__device__ __forceinline__ uint32_t pack16(int2 x)
{
    return min((uint32_t)x.x, 0xffffu) | min((uint32_t)x.y, 0xffffu) << 16;
}

__global__ void __launch_bounds__(1024) k_merge_stream16(int32_t *__restrict__ table, int64_t ld, int32_t n,
                                                         const uint32_t *__restrict__ xs_level, int32_t cnt,
                                                         const MergePhase *__restrict__ phases, int32_t nphase,
                                                         const int32_t *__restrict__ terms, int32_t k,
                                                         uint32_t *__restrict__ level_max,
                                                         const uint16_t *__restrict__ shadow, int64_t sld)
{
    extern __shared__ __align__(16) uint32_t sm[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int nq = nw * 4, qid = warp * 4 + (lane >> 3), ql = lane & 7;
    const int parts = cnt >= nq ? 1 : nq / cnt;
    const int acc_words = parts > 1 ? 64 : 32;  // per subset
    uint32_t *acc = sm;
    uint32_t *S = sm + (size_t)cnt * acc_words;
    const int32_t v0 = blockIdx.x * 64, va = v0 + 2 * lane;  // this lane's vertices in staging and epilogue
    const bool full = v0 + 64 <= n;
    __shared__ uint32_t s_max;
    if (threadIdx.x == 0) s_max = 0;
    for (int32_t i = threadIdx.x; i < cnt * acc_words; i += blockDim.x) acc[i] = 0xffffffffu;
    const uint4 *S4 = reinterpret_cast<const uint4 *>(S) + ql;  // staged row r, this lane's 8 vertices: S4[r * 8]
    const uint4 ones4 = make_uint4(0xffffffffu, 0xffffffffu, 0xffffffffu, 0xffffffffu);
    for (int32_t ph = 0; ph < nphase; ph++) {
        const MergePhase P = phases[ph];
        __syncthreads();
        if (shadow) {
            // 16-bit shadow rows (stride sld, a multiple of 64 vertices): eight
            // lanes copy a staged row with 16-byte cp.async, all of a warp's
            // rows in flight; vertices past n are read but never stored
            const int sub = lane >> 3, sl = lane & 7;
            for (int32_t c0 = warp * 32; c0 < P.nrows; c0 += nw * 32) {
                const uint32_t myr = c0 + lane < P.nrows ? __ldg(P.rows + c0 + lane) : 0u;
                const int32_t nr = min(32, P.nrows - c0);
                for (int32_t j0 = 0; j0 < nr; j0 += 4) {
                    const int32_t j = j0 + sub;
                    const uint32_t r = __shfl_sync(FULL, myr, j & 31);
                    if (j < nr) cp_async16(S + (c0 + j) * 32 + sl * 4, shadow + (int64_t)r * sld + v0 + sl * 8);
                }
            }
            cp_async_wait_all();
        } else
        // staging through registers: a warp takes 32 rows at a time, 16 row
        // loads in flight per lane (8: 1.4 % slower merge; 32 spills)
        for (int32_t c0 = warp * 32; c0 < P.nrows; c0 += nw * 32) {
            const uint32_t myr = c0 + lane < P.nrows ? __ldg(P.rows + c0 + lane) : 0u;
            const int32_t nr = min(32, P.nrows - c0);
            for (int32_t j0 = 0; j0 < nr; j0 += 16) {
                int2 x[16];
#pragma unroll
                for (int u = 0; u < 16; u++) {
                    const uint32_t r = __shfl_sync(FULL, myr, j0 + u);
                    const int32_t *row = table + (int64_t)r * ld;
                    x[u] = make_int2(-1, -1);
                    if (j0 + u < nr) {
                        if (full) x[u] = __ldg(reinterpret_cast<const int2 *>(row + v0) + lane);
                        else if (va < n) x[u] = make_int2(__ldg(row + va), va + 1 < n ? __ldg(row + va + 1) : -1);
                    }
                }
#pragma unroll
                for (int u = 0; u < 16; u++)
                    if (j0 + u < nr) S[(c0 + j0 + u) * 32 + lane] = pack16(x[u]);
            }
        }
        if (warp == nw - 1) S[P.nrows * 32 + lane] = 0xffffffffu;
        __syncthreads();
        for (int32_t t = qid; t < cnt * parts; t += nq) {
            const int32_t xi = t / parts, part = t - xi * parts;
            const uint32_t qb = __ldg(P.qoff + xi);
            const int32_t quads = (int32_t)(__ldg(P.qoff + xi + 1) - qb);
            const uint4 *Q = reinterpret_cast<const uint4 *>(P.pairs) + qb;
            uint4 a0 = ones4, a1 = ones4;
            int32_t qi = part;
            const uint4 zq = make_uint4(0, 0, 0, 0);
            uint4 q = qi < quads ? __ldg(Q + qi) : zq;
            uint4 q1 = qi + parts < quads ? __ldg(Q + qi + parts) : zq;
            while (qi < quads) {
                const int32_t q2i = qi + 2 * parts;
                const uint4 q2 = q2i < quads ? __ldg(Q + q2i) : zq;
                merge_pair8(a0, S4, q.x);
                merge_pair8(a1, S4, q.y);
                merge_pair8(a0, S4, q.z);
                merge_pair8(a1, S4, q.w);
                q = q1;
                q1 = q2;
                qi += parts;
            }
            const uint4 r = make_uint4(__vminu2(a0.x, a1.x), __vminu2(a0.y, a1.y), __vminu2(a0.z, a1.z),
                                       __vminu2(a0.w, a1.w));
            if (parts == 1) {
                uint4 *A4 = reinterpret_cast<uint4 *>(acc + xi * 32 + ql * 4);
                const uint4 o = *A4;
                *A4 = make_uint4(__vminu2(o.x, r.x), __vminu2(o.y, r.y), __vminu2(o.z, r.z), __vminu2(o.w, r.w));
            } else {
                uint32_t *A = acc + xi * 64 + ql * 8;
                const uint32_t w[4] = {r.x, r.y, r.z, r.w};
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    atomicMin(A + 2 * i, w[i] & 0xffffu);
                    atomicMin(A + 2 * i + 1, w[i] >> 16);
                }
            }
        }
    }
    __syncthreads();
    bool has_term = false;
    for (int t = 0; t < k; t++) {
        const int32_t tv = __ldg(terms + t);
        has_term |= (tv >= v0 && tv < v0 + 64);
    }
    uint32_t vmax = 0;  // largest value written: the relaxation's record width follows it
    if (va < n)
        for (int32_t xi = warp; xi < cnt; xi += nw) {
            const uint32_t X = __ldg(xs_level + xi);
            uint32_t a0, a1;
            if (parts > 1) {
                a0 = acc[xi * 64 + 2 * lane];
                a1 = acc[xi * 64 + 2 * lane + 1];
            } else {
                const uint32_t wd = acc[xi * 32 + lane];
                a0 = wd & 0xffffu;
                a1 = wd >> 16;
            }
            if (has_term)
                for (uint32_t bits = X; bits; bits &= bits - 1) {
                    const int t = __ffs(bits) - 1;
                    const int32_t tv = __ldg(terms + t);
                    if (tv == va) a0 = (uint32_t)table[(int64_t)(X ^ (1u << t)) * ld + va];
                    if (tv == va + 1) a1 = (uint32_t)table[(int64_t)(X ^ (1u << t)) * ld + va + 1];
                }
            int32_t *dst = table + (int64_t)X * ld + va;
            if (va + 1 < n) {
                *reinterpret_cast<int2 *>(dst) = make_int2((int32_t)a0, (int32_t)a1);
                vmax = max(vmax, max(a0, a1));
            } else {
                *dst = (int32_t)a0;
                vmax = max(vmax, a0);
            }
        }
    vmax = __reduce_max_sync(FULL, vmax);
    if (lane == 0) atomicMax(&s_max, vmax);
    __syncthreads();
    if (threadIdx.x == 0) atomicMax(level_max, s_max);
}

// A sweep that takes every vertex and pulls every arc (sweep 0, and the
// sweeps after one that changed most vertices): the task loop of
// relax_sweeps with the selection fixed at compile time -- no flag or stamp
// reads, every arc of a vertex compacted -- so the compiler keeps none of the
// other paths' state live around the gathers.  Clears this sweep's flags of
// the warp's vertices; with flags_next, marks the neighbours of every changed
// vertex for the next sweep.  Returns whether a record changed; counts the
// changed vertices in *s_chg.
template <int VEC, bool U16, int GROUP, int TASK_V>
__device__ __forceinline__ bool relax_pass_all(const RelaxArgs &a, int32_t vbeg, int32_t vend, int32_t s,
                                               bool flags_next, uint8_t *cur, uint8_t *nxt, int2 *warcs,
                                               unsigned *s_chg)
{
    using V = typename IVec<VEC>::T;
    const int lane = threadIdx.x & 31;
    bool any = false;
    for (int32_t base = vbeg; base < vend; base += TASK_V) {
        const int32_t v = base + lane;
        const bool mine = lane < TASK_V && v < vend;
        unsigned act = __ballot_sync(FULL, mine);
        if (mine) cur[v] = 0;
        const int32_t rp0 = mine ? __ldg(a.row_ptr + v) : 0;
        const int32_t rp1 = mine ? __ldg(a.row_ptr + v + 1) : 0;
        int j = __ffs(act) - 1;
        act &= act - 1;
        int32_t beg = __shfl_sync(FULL, rp0, j), end = __shfl_sync(FULL, rp1, j);
        int2 arc = beg + lane < end ? __ldg(a.adj + beg + lane) : make_int2(0, 0);
        for (;;) {
            const int32_t vv = base + j;
            const V old = rec_ld<VEC>(a.scratch, vv, lane);
            V acc = old;
            for (int32_t e0 = beg;;) {
                const int cnt = min(32, end - e0);
                // the arcs in this warp's slots (U16: clamped weight in both halves)
                if (lane < cnt)
                    warcs[lane] = U16 ? make_int2(arc.x, (int32_t)(min((uint32_t)arc.y, 32768u) * 0x10001u)) : arc;
                __syncwarp();
                for (int i = 0; i < cnt; i += GROUP) {
                    V val[GROUP];
                    int32_t wt[GROUP];
#pragma unroll
                    for (int g = 0; g < GROUP; g++) {
                        const bool ok = i + g < cnt;
                        const int2 aw = warcs[(i + g) & 31];  // slots past cnt hold stale arcs: not used
                        wt[g] = ok ? aw.y : 0;
                        val[g] = ok ? rec_ld<VEC>(a.scratch, aw.x, lane) : vsplat<V>(U16 ? -1 : INF);
                    }
#pragma unroll
                    for (int g = 0; g < GROUP; g++)
                        acc = U16 ? vaddmin16(val[g], wt[g], acc) : vmin(acc, vadd(val[g], wt[g]));
                }
                __syncwarp();
                e0 += 32;
                if (e0 >= end) break;
                arc = e0 + lane < end ? __ldg(a.adj + e0 + lane) : make_int2(0, 0);  // high degree: next 32 arcs
            }
            // the next vertex of the task before finishing this one
            const int32_t cbeg = beg, cend = end;
            const bool more = act != 0;
            if (more) {
                j = __ffs(act) - 1;
                act &= act - 1;
                beg = __shfl_sync(FULL, rp0, j);
                end = __shfl_sync(FULL, rp1, j);
                arc = beg + lane < end ? __ldg(a.adj + beg + lane) : make_int2(0, 0);
            }
            const bool dec = U16 ? vne(acc, old) : vlt(acc, old);
            if (dec) rec_st<VEC>(a.scratch, vv, lane, acc);
            if (__ballot_sync(FULL, dec)) {
                any = true;
                if (lane == 0) {
                    __stcg(a.stamp + vv, s);
                    atomicAdd(s_chg, 1u);
                }
                if (flags_next)
                    for (int32_t e = cbeg + lane; e < cend; e += 32) nxt[__ldg(&a.adj[e].x)] = 1;
            }
            if (!more) break;
        }
    }
    return any;
}

// The other sweeps: flags (or, in a dense sweep, every vertex) select the
// vertices, stamps the arcs (unless pull_all).  A vertex is taken when its
// flag in `flags` is set; with clear the flag is cleared first.  Returns
// whether a record changed; counts changed vertices in *s_chg.
template <int VEC, bool U16, int GROUP, int TASK_V>
__device__ __forceinline__ bool relax_pass_sel(const RelaxArgs &a, int32_t vbeg, int32_t vend, int32_t s, bool dense,
                                               bool dense_next, bool pull_all, uint8_t *flags, bool clear,
                                               uint8_t *nxt, int2 *warcs, unsigned *s_chg)
{
    using V = typename IVec<VEC>::T;
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1;
    bool any = false;
    for (int32_t base = vbeg; base < vend; base += TASK_V) {
        const int32_t v = base + lane;
        const bool mine = lane < TASK_V && v < vend;
        const bool f = mine && (dense || __ldcg(flags + v) != 0);
        unsigned act = __ballot_sync(FULL, f);
        if (!act) continue;
        if (f && clear) flags[v] = 0;
        const int32_t rp0 = mine ? __ldg(a.row_ptr + v) : 0;
        const int32_t rp1 = mine ? __ldg(a.row_ptr + v + 1) : 0;
        // first active vertex: bounds, first 32 arcs and their selection
        int j = __ffs(act) - 1;
        act &= act - 1;
        int32_t beg = __shfl_sync(FULL, rp0, j), end = __shfl_sync(FULL, rp1, j);
        int2 arc = make_int2(0, 0);
        bool pull = false;
        if (beg + lane < end) {
            arc = __ldg(a.adj + beg + lane);
            pull = pull_all || __ldcg(a.stamp + arc.x) >= s - 1;
        }
        for (;;) {
            const int32_t vv = base + j;
            const V old = rec_ld<VEC>(a.scratch, vv, lane);
            V acc = old;
            for (int32_t e0 = beg;;) {
                const unsigned sel = __ballot_sync(FULL, pull);
                const int cnt = __popc(sel);
                // selected arcs compacted in this warp's slots (U16: clamped weight in both halves)
                if (pull)
                    warcs[__popc(sel & lt)] =
                        U16 ? make_int2(arc.x, (int32_t)(min((uint32_t)arc.y, 32768u) * 0x10001u)) : arc;
                __syncwarp();
                for (int i = 0; i < cnt; i += GROUP) {
                    V val[GROUP];
                    int32_t wt[GROUP];
#pragma unroll
                    for (int g = 0; g < GROUP; g++) {
                        const bool ok = i + g < cnt;
                        const int2 aw = warcs[(i + g) & 31];  // slots past cnt hold stale arcs: not used
                        wt[g] = ok ? aw.y : 0;
                        val[g] = ok ? rec_ld<VEC>(a.scratch, aw.x, lane) : vsplat<V>(U16 ? -1 : INF);
                    }
#pragma unroll
                    for (int g = 0; g < GROUP; g++)
                        acc = U16 ? vaddmin16(val[g], wt[g], acc) : vmin(acc, vadd(val[g], wt[g]));
                }
                __syncwarp();
                e0 += 32;
                if (e0 >= end) break;
                pull = false;  // high-degree vertex: next 32 arcs
                if (e0 + lane < end) {
                    arc = __ldg(a.adj + e0 + lane);
                    pull = pull_all || __ldcg(a.stamp + arc.x) >= s - 1;
                }
            }
            // prefetch the next active vertex before finishing this one
            const int32_t cbeg = beg, cend = end;
            const bool more = act != 0;
            if (more) {
                j = __ffs(act) - 1;
                act &= act - 1;
                beg = __shfl_sync(FULL, rp0, j);
                end = __shfl_sync(FULL, rp1, j);
                pull = false;
                arc = make_int2(0, 0);
                if (beg + lane < end) {
                    arc = __ldg(a.adj + beg + lane);
                    pull = pull_all || __ldcg(a.stamp + arc.x) >= s - 1;
                }
            }
            const bool dec = U16 ? vne(acc, old) : vlt(acc, old);
            if (dec) rec_st<VEC>(a.scratch, vv, lane, acc);
            if (__ballot_sync(FULL, dec)) {
                any = true;
                if (lane == 0) {
                    __stcg(a.stamp + vv, s);
                    atomicAdd(s_chg, 1u);
                }
                if (!dense_next)
                    for (int32_t e = cbeg + lane; e < cend; e += 32) nxt[__ldg(&a.adj[e].x)] = 1;
            }
            if (!more) break;
        }
    }
    return any;
}

// Frontier sweeps over one chunk (phase B of k_relax).  A warp owns a
// contiguous range of n / W vertices (W warps in the grid, so the shares
// differ by one vertex at most) and takes them TASK_V at a time: it
// reads their active flags and CSR bounds with one load each, and
// for every active vertex pulls min over its arcs (u, w) of rec[u] + w with
// coalesced 128*VEC-byte gathers -- only from heads stamped as changed in the
// previous sweep (a head that last changed earlier was already pulled when
// that change marked this vertex active).  The selected arcs of a window are
// compacted into the warp's shared-memory slots, so the gather loop reads one
// (head, weight) pair per arc instead of searching the selection mask.  The
// arcs and stamps of the next active vertex are requested before the current
// one's record is stored.  Sweeps that take every vertex and pull every arc
// run relax_pass_all, the others relax_pass_sel.  Only the owner writes a
// record and values only decrease, so no atomics are needed.  Returns the
// number of sweeps, or -1 after an error (recorded).
//
// U16: 16-bit records, two rows per int32 word (64*VEC rows a record).  The
// host takes them only when every value of the chunk's rows is at most
// 32767; the arc weight is then clamped to 32768, so a value plus a weight
// stays below 2^16, and a clamped sum (at least 32768) never beats a value.
template <int VEC, bool U16>
__device__ int32_t relax_sweeps(const RelaxArgs &a, int *s_ok)
{
    constexpr int GROUP = VEC == 8 ? 2 : VEC >= 4 ? 4 : 8;  // gathers in flight per group
    constexpr int TASK_V = 8;
    const int32_t n = a.n;
    const int32_t gw = (int32_t)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int32_t nwg = (int32_t)((gridDim.x * blockDim.x) >> 5);
    // each warp owns a contiguous range of n / (warps) vertices, scanned TASK_V at a time
    const int32_t vbeg = (int32_t)((int64_t)n * gw / nwg), vend = (int32_t)((int64_t)n * (gw + 1) / nwg);
    volatile uint32_t *vctrl = a.ctrl;
    __shared__ int2 s_arcs[RELAX_THREADS / 32][32];
    int2 *warcs = s_arcs[threadIdx.x >> 5];
    __shared__ unsigned s_chg;
    // read by thread 0 after each sweep's barrier: [0] the sweep changed a
    // record, [1] its changed count, [2] the count of the sweep before
    __shared__ uint32_t s_ctl[3];
    if (threadIdx.x == 0) {
        s_chg = 0;
        s_ctl[1] = s_ctl[2] = (uint32_t)n;
    }
    __syncthreads();
    // Dense sweeps take every vertex (a vertex with no changed neighbour then
    // selects no arc) and so need no neighbour flags from the sweep before.
    // Sweep s decides whether sweep s + 1 is dense before its own count of
    // changed vertices is known: it predicts that count from the last two
    // (their ratio continued while the counts fall) and makes sweep s + 1
    // dense when the prediction exceeds dense_min.  A wrong guess costs time
    // only: a sparse sweep's flags are written whenever the next one is sparse.
    // Changed counts live in a ring of four words (sweep s: C_CNT0 + s % 4).
    bool dense = true;  // sweep 0: every vertex is active
    int32_t s = 0;
    for (; s < a.max_sweeps; s++) {
        uint8_t *cur = (s & 1) ? a.act1 : a.act0;
        uint8_t *nxt = (s & 1) ? a.act0 : a.act1;
        const uint32_t prev_chg = s_ctl[1];   // n before sweep 0
        const uint32_t prev2_chg = s_ctl[2];  // n before sweeps 0 and 1
        const uint32_t pred_chg = prev_chg < prev2_chg
                                      ? (uint32_t)((uint64_t)prev_chg * prev_chg / prev2_chg)
                                      : prev_chg;
        const bool dense_next = pred_chg > (uint32_t)a.dense_min;
        // after a sweep that changed most vertices, pull every arc without reading stamps
        const bool pull_all = prev_chg >= (uint32_t)a.pull_all_min;
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            vctrl[C_SLOT0 + (s + 1) % 3] = 0;
            vctrl[C_CNT0 + (s + 1) % 4] = 0;
        }
        bool any = false;
        if (dense && pull_all)
            any = relax_pass_all<VEC, U16, GROUP, TASK_V>(a, vbeg, vend, s, !dense_next, cur, nxt, warcs, &s_chg);
        else
            any = relax_pass_sel<VEC, U16, GROUP, TASK_V>(a, vbeg, vend, s, dense, dense_next, pull_all, cur, true,
                                                          nxt, warcs, &s_chg);
        // A sparse sweep whose successor is sparse also takes, once, the vertices
        // already marked for the next sweep (marked by changes earlier in this
        // sweep), so a change travels two arcs per sweep in the frontier's tail.
        // Their marks stay: the next sweep takes them again, after the barrier
        // has made every change of this sweep visible, so a change this early
        // pass missed is still pulled there.
        if (!dense && !dense_next)
            any |= relax_pass_sel<VEC, U16, GROUP, TASK_V>(a, vbeg, vend, s, false, dense_next, pull_all, nxt, false,
                                                           nxt, warcs, &s_chg);
        any = __syncthreads_or(any);
        if (threadIdx.x == 0) {
            if (any) vctrl[C_SLOT0 + s % 3] = 1;
            if (s_chg) atomicAdd(a.ctrl + C_CNT0 + s % 4, s_chg);
            s_chg = 0;
        }
        const bool ok = grid_barrier(a.ctrl, s_ok, [&] {
            s_ctl[0] = vctrl[C_SLOT0 + s % 3];
            s_ctl[2] = s_ctl[1];
            s_ctl[1] = vctrl[C_CNT0 + s % 4];
        });
        if (!ok) {
            if (threadIdx.x == 0) atomicOr(&a.stat->err, a.ctrl[C_ERR]);
            return -1;
        }
        if (s_ctl[0] == 0) return s + 1;
        dense = dense_next;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(&a.stat->err, (uint32_t)EMV_DEV_SWEEP_LIMIT);
    return -1;
}

// Phase A of a relaxation chunk: rows -> vertex-major records (vertex v owns
// 32*VEC int32 words, word e = row e; U16: word e = rows e | (e + 32*VEC) << 16);
// in level-1 mode the rows are the k single-source initialisations.  A tile
// is 32 vertices by all 32*VEC words, so a warp has all its row loads in
// flight before one barrier.  Rows past the chunk's are INF (U16: 0, which
// no sweep lowers).  Also resets the active flags and stamps.
template <int VEC, bool U16>
__device__ __forceinline__ int32_t relax_load_value(const RelaxArgs &a, int32_t row, int32_t v)
{
    if (row >= a.nrows || v >= a.n) return U16 ? 0 : INF;
    if (a.level1) return (v == __ldg(a.terms + row)) ? 0 : INF;
    return __ldcg(a.table + (int64_t)__ldg(a.rows + row) * a.ld + v);
}

template <int VEC, bool U16>
__device__ void relax_load_records(const RelaxArgs &a, int32_t (*tile)[33])
{
    constexpr int R = 32 * VEC, NW = RELAX_THREADS / 32, PER = R / NW;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int32_t n = a.n, ntiles = (n + 31) >> 5;
    // software pipeline: the next tile's row loads are in flight while this
    // tile's records are written
    int32_t x[PER], xh[U16 ? PER : 1];
    auto fetch = [&](int32_t t) {
        const int32_t v = t * 32 + lane;
#pragma unroll
        for (int q = 0; q < PER; q++) {
            x[q] = relax_load_value<VEC, U16>(a, warp + q * NW, v);
            if (U16) xh[q] = relax_load_value<VEC, U16>(a, warp + q * NW + R, v);
        }
    };
    if (blockIdx.x < ntiles) fetch(blockIdx.x);
    for (int32_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
#pragma unroll
        for (int q = 0; q < PER; q++)
            tile[warp + q * NW][lane] =
                U16 ? (int32_t)(min((uint32_t)x[q], 0xffffu) | min((uint32_t)xh[U16 ? q : 0], 0xffffu) << 16) : x[q];
        __syncthreads();
        if (t + (int32_t)gridDim.x < ntiles) fetch(t + gridDim.x);
        for (int vv = warp; vv < 32; vv += NW) {
            const int32_t v2 = t * 32 + vv;
            if (v2 < n)
#pragma unroll
                for (int g = 0; g < VEC; g++) __stcg(a.scratch + (int64_t)v2 * R + g * 32 + lane, tile[g * 32 + lane][vv]);
        }
        __syncthreads();
    }
    for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        a.act0[v] = 1;
        a.act1[v] = 0;
        a.stamp[v] = -1;
    }
}

// Phase C: vertex-major records -> table rows, a whole 32-vertex tile at a
// time; with a.vmax set, the largest value written goes to *a.vmax.
template <int VEC, bool U16>
__device__ void relax_store_records(const RelaxArgs &a, int32_t (*tile)[33])
{
    constexpr int R = 32 * VEC, NW = RELAX_THREADS / 32, PER = R / NW;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int32_t n = a.n, ntiles = (n + 31) >> 5, nrows = a.nrows;
    uint32_t vmax = 0;
    // software pipeline: the next tile's record loads are in flight while
    // this tile's rows are written
    constexpr int VPW = 32 / NW;  // vertices of a tile per warp
    int32_t y[VPW][VEC];
    auto fetch = [&](int32_t t) {
#pragma unroll
        for (int i = 0; i < VPW; i++) {
            const int32_t v2 = t * 32 + warp + i * NW;
#pragma unroll
            for (int g = 0; g < VEC; g++) y[i][g] = (v2 < n) ? __ldcg(a.scratch + (int64_t)v2 * R + g * 32 + lane) : INF;
        }
    };
    if (blockIdx.x < ntiles) fetch(blockIdx.x);
    for (int32_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
#pragma unroll
        for (int i = 0; i < VPW; i++)
#pragma unroll
            for (int g = 0; g < VEC; g++) tile[g * 32 + lane][warp + i * NW] = y[i][g];
        __syncthreads();
        if (t + (int32_t)gridDim.x < ntiles) fetch(t + gridDim.x);
        const int32_t v = t * 32 + lane;
        if (v < n)
#pragma unroll
            for (int q = 0; q < PER; q++) {
                const int32_t row = warp + q * NW;
                const uint32_t word = (uint32_t)tile[row][lane];
                if (U16) {
                    const uint32_t lo = word & 0xffffu, hi = word >> 16;
                    const int32_t xlo = lo == 0xffffu ? INF : (int32_t)lo, xhi = hi == 0xffffu ? INF : (int32_t)hi;
                    if (row < nrows) {
                        const int64_t X = __ldg(a.rows + row);
                        a.table[X * a.ld + v] = xlo;
                        if (a.shadow) a.shadow[X * a.shadow_ld + v] = (uint16_t)lo;
                    }
                    if (row + R < nrows) {
                        const int64_t X = __ldg(a.rows + row + R);
                        a.table[X * a.ld + v] = xhi;
                        if (a.shadow) a.shadow[X * a.shadow_ld + v] = (uint16_t)hi;
                    }
                } else if (row < nrows) {
                    const int64_t X = __ldg(a.rows + row);
                    a.table[X * a.ld + v] = (int32_t)word;
                    if (a.shadow) a.shadow[X * a.shadow_ld + v] = (uint16_t)min(word, 0xffffu);
                    vmax = max(vmax, word);
                }
            }
        __syncthreads();
    }
    if (a.vmax) {
        vmax = __reduce_max_sync(FULL, vmax);
        if (lane == 0) atomicMax(a.vmax, vmax);
    }
}

// Multi-source shortest-path closure of up to 32*VEC rows (R:2109-2130): for
// every row X of the chunk, d[X][v] = min over u of init[u] + dist(u, v).
// One cooperative persistent launch: A. rows -> vertex-major records;
// B. frontier sweeps (relax_sweeps), bounded by n + 1 (the Bellman-Ford
// bound), ending after a sweep that changes nothing; C. records -> rows.
// Records and stamps are read with ld.global.cg (L2), never through a stale
// L1 line.
template <int VEC, bool U16 = false>
__global__ void __launch_bounds__(RELAX_THREADS, 2) k_relax(RelaxArgs a)
{
    __shared__ int32_t tile[32 * VEC][33];  // 32 vertices by all words of the chunk's records
    __shared__ int s_ok;
    relax_load_records<VEC, U16>(a, tile);
    if (!grid_barrier(a.ctrl, &s_ok)) {
        if (threadIdx.x == 0) atomicOr(&a.stat->err, a.ctrl[C_ERR]);
        return;
    }
    const int32_t s = relax_sweeps<VEC, U16>(a, &s_ok);
    if (s < 0) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&a.stat->sweeps, (unsigned long long)s);
    relax_store_records<VEC, U16>(a, tile);
}

// ------------------------------------------------------------- traceback

__device__ __forceinline__ uint32_t deposit_bits(uint32_t p, uint32_t mask)
{
    uint32_t r = 0;
    for (uint32_t b = 1; mask; b <<= 1) {
        const uint32_t lowbit = mask & (0u - mask);
        if (p & b) r |= lowbit;
        mask ^= lowbit;
    }
    return r;
}

struct TbArgs {
    const int32_t *table;
    int64_t ld;
    int32_t n;
    int32_t k;
    const int32_t *row_ptr;
    const int2 *adj;
    const int32_t *terms;
    int32_t *edges;     // 3 * cap
    int32_t cap;
    int32_t *out;       // [0] edge count, [1] status
    int32_t *queue;     // n
    int32_t *parent;    // n
    int32_t *stamp;     // n, -1 on entry
    int32_t max_steps;
};

// Witness of d[X][v] (warp-collective, all lanes return the same):
// 0 leaf (X = {i}, v = t_i); 1 split d[Y][v] + d[X\Y][v] = D (the lowest
// pair index); 2 arc (u, v) of positive weight with d[X][u] + w = D;
// 3 none of those (a zero-weight predecessor must exist).
__device__ int tb_witness(const TbArgs &a, uint32_t X, int32_t v, int32_t D, uint32_t &Y, int32_t &u, int32_t &wt)
{
    const int lane = threadIdx.x & 31;
    const int pc = __popc(X);
    if (pc == 1 && v == __ldg(a.terms + (__ffs(X) - 1))) return 0;
    if (pc >= 2) {
        const uint32_t low = X & (0u - X), rest = X ^ low;
        const uint32_t npairs = (1u << __popc(rest)) - 1;
        for (uint32_t base = 0; base < npairs; base += 32) {
            const uint32_t p = base + lane;
            bool ok = false;
            uint32_t y = 0;
            if (p < npairs) {
                y = low | deposit_bits(p, rest);
                const int32_t x1 = a.table[(int64_t)y * a.ld + v];
                const int32_t x2 = a.table[(int64_t)(X ^ y) * a.ld + v];
                ok = x1 < INF && x2 < INF && x1 + x2 == D;
            }
            const unsigned bal = __ballot_sync(FULL, ok);
            if (bal) {
                Y = __shfl_sync(FULL, y, __ffs(bal) - 1);
                return 1;
            }
        }
    }
    const int32_t beg = a.row_ptr[v], end = a.row_ptr[v + 1];
    for (int32_t e0 = beg; e0 < end; e0 += 32) {
        const int32_t e = e0 + lane;
        bool ok = false;
        int2 arc = make_int2(0, 0);
        if (e < end) {
            arc = a.adj[e];
            if (arc.y > 0) {
                const int32_t du = a.table[(int64_t)X * a.ld + arc.x];
                ok = du < INF && du + arc.y == D;
            }
        }
        const unsigned bal = __ballot_sync(FULL, ok);
        if (bal) {
            const int src = __ffs(bal) - 1;
            u = __shfl_sync(FULL, arc.x, src);
            wt = __shfl_sync(FULL, arc.y, src);
            return 2;
        }
    }
    return 3;
}

// Tree recovery from the finished table (one warp).  Starts at (C, q) and
// repeatedly explains d[X][v] by a leaf, a split into (Y, v) and (X\Y, v),
// or an arc (v, u) into (X, u) -- the decisions the reference records in b_v
// (R:2081-2084, R:2122-2128) and walks in backtrack() (R:1907-1932), found
// here by recomputation instead of a 2x-table predecessor store.  A run of
// zero-weight arcs is resolved by a breadth-first search inside the set of
// vertices with the same value, so zero-weight cycles cannot loop.
__global__ void __launch_bounds__(32) k_traceback(TbArgs a)
{
    __shared__ uint32_t stX[TB_STACK];
    __shared__ int32_t stV[TB_STACK];
    const int lane = threadIdx.x & 31;
    int sp = 0, cnt = 0, walk = 0, steps = 0;
    uint32_t status = 0;
    if (a.k >= 2) {
        if (lane == 0) {
            stX[0] = (1u << (a.k - 1)) - 1;
            stV[0] = a.terms[a.k - 1];
        }
        sp = 1;
    }
    __syncwarp();
    while (sp > 0) {
        if (++steps > a.max_steps) { status |= EMV_DEV_TB_STEPS; break; }
        const uint32_t X = stX[sp - 1];
        const int32_t v = stV[sp - 1];
        sp--;
        __syncwarp();
        const int32_t D = a.table[(int64_t)X * a.ld + v];
        uint32_t Y = 0;
        int32_t u = 0, wt = 0;
        const int kind = tb_witness(a, X, v, D, Y, u, wt);
        if (kind == 0) continue;
        if (kind == 1) {
            if (sp + 2 > TB_STACK) { status |= EMV_DEV_TB_OVERFLOW; break; }
            if (lane == 0) {
                stX[sp] = Y; stV[sp] = v;
                stX[sp + 1] = X ^ Y; stV[sp + 1] = v;
            }
            sp += 2;
            __syncwarp();
            continue;
        }
        if (kind == 2) {
            if (cnt >= a.cap || sp + 1 > TB_STACK) { status |= EMV_DEV_TB_OVERFLOW; break; }
            if (lane == 0) {
                a.edges[3 * cnt] = v; a.edges[3 * cnt + 1] = u; a.edges[3 * cnt + 2] = wt;
                stX[sp] = X; stV[sp] = u;
            }
            cnt++;
            sp++;
            __syncwarp();
            continue;
        }
        // Zero-weight run: BFS over arcs of weight 0 between vertices of value D.
        walk++;
        if (lane == 0) {
            a.queue[0] = v;
            a.parent[v] = -1;
            a.stamp[v] = walk;
        }
        __syncwarp();
        int32_t head = 0, tail = 1, target = -1;
        while (head < tail) {
            const int32_t x = *(volatile int32_t *)(a.queue + head);
            head++;
            if (x != v) {
                uint32_t Y2;
                int32_t u2, w2;
                if (tb_witness(a, X, x, D, Y2, u2, w2) != 3) { target = x; break; }
            }
            const int32_t beg = a.row_ptr[x], end = a.row_ptr[x + 1];
            for (int32_t e0 = beg; e0 < end; e0 += 32) {
                const int32_t e = e0 + lane;
                bool add = false;
                int32_t y = 0;
                if (e < end) {
                    const int2 arc = a.adj[e];
                    y = arc.x;
                    if (arc.y == 0 && a.table[(int64_t)X * a.ld + y] == D)
                        add = atomicExch(a.stamp + y, walk) != walk;
                }
                const unsigned bal = __ballot_sync(FULL, add);
                if (add) {
                    const int pos = tail + __popc(bal & ((1u << lane) - 1));
                    a.queue[pos] = y;
                    a.parent[y] = x;
                }
                tail += __popc(bal);
                __syncwarp();
            }
        }
        if (target < 0) { status |= EMV_DEV_TB_NO_WITNESS; break; }
        int32_t z = target, emitted = 0;
        bool ovf = false;
        if (lane == 0) {
            while (z != v) {
                const int32_t p = *(volatile int32_t *)(a.parent + z);
                if (cnt + emitted >= a.cap) { ovf = true; break; }
                a.edges[3 * (cnt + emitted)] = z;
                a.edges[3 * (cnt + emitted) + 1] = p;
                a.edges[3 * (cnt + emitted) + 2] = 0;
                emitted++;
                z = p;
            }
        }
        emitted = __shfl_sync(FULL, emitted, 0);
        ovf = __shfl_sync(FULL, (int)ovf, 0) != 0;
        cnt += emitted;
        if (ovf || sp + 1 > TB_STACK) { status |= EMV_DEV_TB_OVERFLOW; break; }
        if (lane == 0) { stX[sp] = X; stV[sp] = target; }
        sp++;
        __syncwarp();
    }
    if (lane == 0) {
        a.out[0] = cnt;
        a.out[1] = (int32_t)status;
    }
}

}  // namespace emv
