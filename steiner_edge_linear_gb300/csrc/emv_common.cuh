// emv_common.cuh -- constants and status words shared by every kernel file.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "emv_internal.h"

namespace emv {

constexpr int32_t INF = EMV_INF32;
constexpr unsigned FULL = 0xffffffffu;
constexpr int RELAX_THREADS = 512;       // 16 warps; a warp takes 8 vertices at a time
constexpr int CHUNK_ROWS = 256;          // most int32 rows per relaxation chunk (1 KB records: 32 lanes x 8 words)
constexpr uint32_t SPIN_LIMIT = 1u << 22;  // grid-barrier spin iterations (~1 s with nanosleep)
constexpr int TB_STACK = 64;

// ctrl words of one cooperative relaxation launch (zeroed before the launch),
// each kind on its own 128-byte line: the barrier's arrival count, the
// generation every block polls, the error word, the sweeps' changed flags
// and their changed counts.  On one shared line the polls, arrivals and
// per-sweep atomics queue behind each other at one L2 slice (a pull-all
// sweep at n = 10^5 took 75 us instead of 58 us).
enum : int { C_BAR_COUNT = 0, C_BAR_GEN = 32, C_ERR = 64, C_SLOT0 = 96, C_CNT0 = 128, C_WORDS = 160 };
static_assert(C_BAR_GEN - C_BAR_COUNT >= 32 && C_ERR - C_BAR_GEN >= 32 && C_SLOT0 - C_ERR >= 32 &&
                  C_CNT0 - C_SLOT0 >= 32 && C_WORDS - C_CNT0 >= 32,
              "each kind of control word on its own 128-byte line");

// Result of the device check of a CSR (k_pack_scan), zeroed before it runs.
enum : uint32_t { SCAN_BAD_HEAD = 1, SCAN_BAD_WEIGHT = 2, SCAN_BIG_WEIGHT = 4, SCAN_BAD_ROWS = 8 };
struct GraphScan {
    uint32_t bad;             // SCAN_* bits
    uint32_t maxw;            // largest arc weight
    unsigned long long sumw;  // sum of the arc weights (both arcs of every edge)
};

// Persistent device status of one solve (zeroed at solve start).
struct DevStat {
    uint32_t err;
    uint32_t pad;
    unsigned long long sweeps;
};

}  // namespace emv
