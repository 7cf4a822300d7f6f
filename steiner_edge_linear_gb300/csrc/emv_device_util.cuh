// emv_device_util.cuh -- device helpers shared by the kernel files: the
// bounded grid barrier of the cooperative launches and the int32-vector
// arithmetic of the relaxation records.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "emv_common.cuh"

namespace emv {

// Grid-wide barrier for a cooperative launch.  Bounded: a block that waits
// longer than SPIN_LIMIT iterations, or sees another block's error, records
// the error and returns false; every block then leaves the kernel.  after()
// runs on thread 0 once the barrier is passed, before the block's threads
// are released: a block reads the control words it needs there, once, into
// shared memory, instead of every thread loading the same L2 line.
template <typename F>
__device__ __forceinline__ bool grid_barrier(uint32_t *ctrl, int *s_ok, F &&after)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile uint32_t *vc = ctrl;
        const uint32_t gen = vc[C_BAR_GEN];
        __threadfence();
        const uint32_t arrived = atomicAdd(ctrl + C_BAR_COUNT, 1u);
        if (arrived == gridDim.x - 1) {
            atomicExch(ctrl + C_BAR_COUNT, 0u);
            __threadfence();
            atomicAdd(ctrl + C_BAR_GEN, 1u);
        } else {
            uint32_t spins = 0;
            while (vc[C_BAR_GEN] == gen) {
                // another block's error is seen within 64 polls
                if ((++spins & 63) == 0 && vc[C_ERR] != 0) break;
                if (spins > SPIN_LIMIT) {
                    atomicOr(ctrl + C_ERR, (uint32_t)EMV_DEV_BARRIER_TIMEOUT);
                    break;
                }
                __nanosleep(256);
            }
        }
        __threadfence();
        *s_ok = (vc[C_ERR] == 0);
        after();
    }
    __syncthreads();
    return *s_ok != 0;
}
__device__ __forceinline__ bool grid_barrier(uint32_t *ctrl, int *s_ok)
{
    return grid_barrier(ctrl, s_ok, [] {});
}

// One thread's share of the device CSR check (grid-stride over arcs and
// row_ptr), reduced per warp into *scan: heads in [0, n), weights in
// [0, 2^30), row_ptr from 0 to arcs and non-decreasing, the largest weight
// and the weight sum.  Every lane of the warp must call it.  With adj set,
// the arcs are also packed as int2 (col, w).
__device__ __forceinline__ void scan_csr(const int32_t *__restrict__ row_ptr, int32_t n,
                                         const int32_t *__restrict__ col, const int32_t *__restrict__ w,
                                         int2 *__restrict__ adj, int64_t arcs, GraphScan *__restrict__ scan)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    uint32_t bad = 0, mx = 0;
    unsigned long long sum = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < arcs; i += stride) {
        const int32_t c = col[i], x = w[i];
        if (adj) adj[i] = make_int2(c, x);
        if (c < 0 || c >= n) bad |= SCAN_BAD_HEAD;
        if (x < 0) bad |= SCAN_BAD_WEIGHT;
        else {
            if (x >= INF) bad |= SCAN_BIG_WEIGHT;
            mx = max(mx, (uint32_t)x);
            sum += (unsigned long long)x;
        }
    }
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= n; i += stride) {
        const int32_t r = row_ptr[i];
        if (r < 0 || (int64_t)r > arcs || (i == 0 && r != 0) || (i == n && (int64_t)r != arcs) ||
            (i < n && row_ptr[i + 1] < r))
            bad |= SCAN_BAD_ROWS;
    }
    bad = __reduce_or_sync(FULL, bad);
    mx = __reduce_max_sync(FULL, mx);
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(FULL, sum, o);
    if ((threadIdx.x & 31) == 0) {
        if (bad) atomicOr(&scan->bad, bad);
        if (mx) atomicMax(&scan->maxw, mx);
        if (sum) atomicAdd(&scan->sumw, sum);
    }
}

// 4-byte asynchronous global -> shared copy (staging without a register round
// trip) and the wait for all of this thread's copies.
__device__ __forceinline__ void cp_async4(void *smem, const void *gmem)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((uint32_t)__cvta_generic_to_shared(smem)), "l"(gmem)
                 : "memory");
}
// 16-byte variant (both addresses 16-byte aligned; L2 only).
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(smem)), "l"(gmem)
                 : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Vector of VEC int32 (one lane's share of a vertex record).
template <int VEC> struct IVec;
template <> struct IVec<1> {
    using T = int32_t;
};
template <> struct IVec<2> {
    using T = int2;
};
template <> struct IVec<4> {
    using T = int4;
};
struct int5v {  // 5 int32 words: a lane's share of a 640-byte record
    int4 a;
    int32_t b;
};
template <> struct IVec<5> {
    using T = int5v;
};
struct int8v {  // 8 int32 words: a lane's share of a 1 KB record
    int4 a, b;
};
template <> struct IVec<8> {
    using T = int8v;
};

__device__ __forceinline__ int32_t vmin(int32_t a, int32_t b) { return min(a, b); }
__device__ __forceinline__ int2 vmin(int2 a, int2 b) { return make_int2(min(a.x, b.x), min(a.y, b.y)); }
__device__ __forceinline__ int4 vmin(int4 a, int4 b)
{
    return make_int4(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z), min(a.w, b.w));
}
__device__ __forceinline__ int32_t vadd(int32_t a, int32_t w) { return a + w; }
__device__ __forceinline__ int2 vadd(int2 a, int32_t w) { return make_int2(a.x + w, a.y + w); }
__device__ __forceinline__ int4 vadd(int4 a, int32_t w) { return make_int4(a.x + w, a.y + w, a.z + w, a.w + w); }
__device__ __forceinline__ bool vlt(int32_t a, int32_t b) { return a < b; }
__device__ __forceinline__ bool vlt(int2 a, int2 b) { return a.x < b.x || a.y < b.y; }
__device__ __forceinline__ bool vlt(int4 a, int4 b) { return a.x < b.x || a.y < b.y || a.z < b.z || a.w < b.w; }
__device__ __forceinline__ int8v vmin(int8v x, int8v y) { return {vmin(x.a, y.a), vmin(x.b, y.b)}; }
__device__ __forceinline__ int8v vadd(int8v x, int32_t w) { return {vadd(x.a, w), vadd(x.b, w)}; }
__device__ __forceinline__ bool vlt(int8v x, int8v y) { return vlt(x.a, y.a) || vlt(x.b, y.b); }
__device__ __forceinline__ int5v vmin(int5v x, int5v y) { return {vmin(x.a, y.a), min(x.b, y.b)}; }
__device__ __forceinline__ int5v vadd(int5v x, int32_t w) { return {vadd(x.a, w), x.b + w}; }
__device__ __forceinline__ bool vlt(int5v x, int5v y) { return vlt(x.a, y.a) || x.b < y.b; }
// L2-only loads and stores of a lane's share (L1 may hold stale lines of records other SMs write)
template <typename T> __device__ __forceinline__ T ldcg_v(const T *p) { return __ldcg(p); }
template <> __device__ __forceinline__ int8v ldcg_v<int8v>(const int8v *p)
{
    const int4 *q = reinterpret_cast<const int4 *>(p);
    return {__ldcg(q), __ldcg(q + 1)};
}
template <typename T> __device__ __forceinline__ void stcg_v(T *p, T v) { __stcg(p, v); }
template <> __device__ __forceinline__ void stcg_v<int8v>(int8v *p, int8v v)
{
    int4 *q = reinterpret_cast<int4 *>(p);
    __stcg(q, v.a);
    __stcg(q + 1, v.b);
}
template <typename T> __device__ __forceinline__ T vsplat(int32_t x);
template <> __device__ __forceinline__ int32_t vsplat<int32_t>(int32_t x) { return x; }
template <> __device__ __forceinline__ int2 vsplat<int2>(int32_t x) { return make_int2(x, x); }
template <> __device__ __forceinline__ int4 vsplat<int4>(int32_t x) { return make_int4(x, x, x, x); }
template <> __device__ __forceinline__ int8v vsplat<int8v>(int32_t x) { return {vsplat<int4>(x), vsplat<int4>(x)}; }
template <> __device__ __forceinline__ int5v vsplat<int5v>(int32_t x) { return {vsplat<int4>(x), x}; }
template <typename T> __device__ __forceinline__ T vinf() { return vsplat<T>(INF); }

// min(a + b, c) per halfword of two packed 16-bit pairs (callers keep every
// halfword sum below 2^16).  Measured faster than a 32-bit add followed by
// __vminu2.
__device__ __forceinline__ uint32_t addmin16(uint32_t a, uint32_t b, uint32_t c)
{
    return __viaddmin_u16x2(a, b, c);
}

// 16-bit records: every int32 word holds two rows.  min(a + w2, c) per
// halfword, w2 the arc weight in both halves (the caller keeps a + w2 below
// 2^16), and "some halfword differs".
__device__ __forceinline__ int32_t vaddmin16(int32_t a, int32_t w2, int32_t c)
{
    return (int32_t)addmin16((uint32_t)a, (uint32_t)w2, (uint32_t)c);
}
__device__ __forceinline__ int2 vaddmin16(int2 a, int32_t w2, int2 c)
{
    return make_int2(vaddmin16(a.x, w2, c.x), vaddmin16(a.y, w2, c.y));
}
__device__ __forceinline__ int4 vaddmin16(int4 a, int32_t w2, int4 c)
{
    return make_int4(vaddmin16(a.x, w2, c.x), vaddmin16(a.y, w2, c.y), vaddmin16(a.z, w2, c.z),
                     vaddmin16(a.w, w2, c.w));
}
__device__ __forceinline__ int8v vaddmin16(int8v a, int32_t w2, int8v c)
{
    return {vaddmin16(a.a, w2, c.a), vaddmin16(a.b, w2, c.b)};
}
__device__ __forceinline__ int5v vaddmin16(int5v a, int32_t w2, int5v c)
{
    return {vaddmin16(a.a, w2, c.a), vaddmin16(a.b, w2, c.b)};
}
__device__ __forceinline__ bool vne(int32_t a, int32_t b) { return a != b; }
__device__ __forceinline__ bool vne(int2 a, int2 b) { return a.x != b.x || a.y != b.y; }
__device__ __forceinline__ bool vne(int4 a, int4 b) { return a.x != b.x || a.y != b.y || a.z != b.z || a.w != b.w; }
__device__ __forceinline__ bool vne(int8v x, int8v y) { return vne(x.a, y.a) || vne(x.b, y.b); }
__device__ __forceinline__ bool vne(int5v x, int5v y) { return vne(x.a, y.a) || x.b != y.b; }

// A lane's share of vertex v's record of 32 * VEC words (L2-only access).
// VEC = 1, 2, 4, 8: words VEC * lane .. VEC * lane + VEC - 1; VEC = 5: words
// 4 * lane .. 4 * lane + 3 and 128 + lane, so that both loads are aligned.
template <int VEC>
__device__ __forceinline__ typename IVec<VEC>::T rec_ld(const int32_t *scratch, int64_t v, int lane)
{
    return ldcg_v(reinterpret_cast<const typename IVec<VEC>::T *>(scratch + v * 32 * VEC) + lane);
}
template <> __device__ __forceinline__ int5v rec_ld<5>(const int32_t *scratch, int64_t v, int lane)
{
    const int32_t *r = scratch + v * 160;
    return {__ldcg(reinterpret_cast<const int4 *>(r) + lane), __ldcg(r + 128 + lane)};
}
template <int VEC>
__device__ __forceinline__ void rec_st(int32_t *scratch, int64_t v, int lane, typename IVec<VEC>::T x)
{
    stcg_v(reinterpret_cast<typename IVec<VEC>::T *>(scratch + v * 32 * VEC) + lane, x);
}
template <> __device__ __forceinline__ void rec_st<5>(int32_t *scratch, int64_t v, int lane, int5v x)
{
    int32_t *r = scratch + v * 160;
    __stcg(reinterpret_cast<int4 *>(r) + lane, x.a);
    __stcg(r + 128 + lane, x.b);
}

}  // namespace emv
