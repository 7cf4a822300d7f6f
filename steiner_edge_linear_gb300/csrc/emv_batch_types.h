// emv_batch_types.h -- descriptors of the CTA-resident batched solver (host and device).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace emv {

constexpr int BATCH_THREADS = 1024;
constexpr int BATCH_KMAX = 12;
constexpr int32_t BATCH_SMEM_BYTES = 200 * 1024;
constexpr int32_t BATCH_RCAP_MAX = 128;  // most rows per relaxation chunk (a lane holds 4 of them)
constexpr int32_t BATCH_MW_MAX = 8;      // widest merge vertex block: 8 columns of 32 vertices
// Shared-memory stride of a vertex in a relaxation chunk of R rows: R + 1
// (conflict-free single-row lanes) or, for R >= 4, R + 4 (16-byte aligned
// 4-row lane shares).
__host__ __device__ constexpr int32_t batch_stride(int32_t R) { return R >= 4 ? R + 4 : R + 1; }

struct BatchInst {
    const int32_t *row_ptr;  // n + 1 entries, arcs of this instance from 0
    const int2 *adj;         // packed (col, w) arcs
    const int32_t *terms;    // k terminals
    int32_t *table;          // 2^k x n int32, row-major (ld = n)
    int32_t n;
    int32_t k;
    int32_t rcap;            // relaxation rows per chunk (autotuned, power of two <= 32)
    int32_t mw;              // merge vertex block of 32 * mw vertices (autotuned, 1, 2, 4 or 8)
    int32_t orig;            // slot of the cost in BatchArgs::costs
    int32_t lo;              // first level to run (1..k)
    int32_t hi;              // last level to run (lo..k)
};

struct BatchArgs {
    const BatchInst *inst;
    int32_t count;
    const uint32_t *xs;      // subsets by level for k = 1..BATCH_KMAX, concatenated
    const int32_t *xs_off;   // xs_off[k * (BATCH_KMAX + 2) + m]: start of level m of k
    int64_t *costs;          // by orig; written when hi == k
    uint32_t *queue;         // [0] next work item
    uint32_t *err;
};

}  // namespace emv
