// emv_plan.h -- host-side planning of the DP (no CUDA types): the subsets of
// every level and the streamed merge's groups and phases.  Shared by the
// library and the plan checks of the test suite.
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

// All non-empty subsets of {0..k-1} grouped by size, increasing within a
// size -- the order Gosper's hack gives each level (R:2041-2046).  Level m
// occupies xs[off[m], off[m + 1]).
void subset_levels(int32_t k, std::vector<uint32_t> &xs, std::vector<int64_t> &off);

namespace emv {

// Value widths of level m from the level maxima M[1..m-1] (M[j] = the largest
// value level j's merge wrote, level 1: its relaxation; all ones = unknown).
// 16-bit merge staging when every M[j] + M[m-j] <= 65533, so that no sum of
// two staged values leaves 16 bits and a pad pair (>= 0xfffe) never wins;
// 16-bit relaxation records when M[m-1] + M[1] <= 32767, which bounds every
// merged, hence every relaxed, value of level m (split {X \ t, t}).
bool merge16_allowed(const uint32_t *M, int32_t m);
bool relax16_allowed(const uint32_t *M, int32_t m);

// Rows per relaxation chunk of an n-vertex graph: 512-byte vertex records
// while they fit in three quarters of L2 (the sweeps' gathers are then L2
// hits and larger records only add bytes per sweep), else 1 KB ones, which
// halve the sweeps of graphs whose records stream from HBM anyway; 16-bit
// records hold twice the rows.
int32_t relax_rows_per_chunk(int64_t n, int64_t l2_bytes, bool u16);
// Rows per chunk for a level of cnt subsets.  A launch costs about the same
// whatever its record width, so where 640-byte records (5/4 of the rows of
// 512-byte ones) still fit three quarters of L2 and cut the level's launch
// count, the level is cut into that many equal chunks.
int32_t relax_rows_per_level_chunk(int64_t n, int64_t l2_bytes, bool u16, int64_t cnt);

// One phase of a group: offsets (in 32-bit words of the plan data) of its
// staged rows, per-subset quad offsets and pair quads (posY | posZ << 16,
// padded with (pad, pad), pad = nrows), and its staged row count (the pad
// row is staged after them).
struct HostPhase {
    size_t rows_at, qoff_at, pairs_at;
    int32_t nrows;
};
// One launch: subsets [x0, x0 + cnt) of a level, its shared memory and phases.
struct HostGroup {
    int64_t x0, cnt, smem;
    std::vector<HostPhase> phases;
};

// Accumulator space of a group of g subsets, in 128-byte rows.
int64_t stream_acc_rows(int64_t g);

// Plans every level 2..k into data (all offsets relative to its start, blocks
// read as uint4 16-byte aligned); plan[m] is empty for a level that cannot
// be streamed within smem_bytes of shared memory.
void plan_stream_levels(int32_t k, const std::vector<uint32_t> &xs, const std::vector<int64_t> &off,
                        int64_t smem_bytes, std::vector<uint32_t> &data, std::vector<std::vector<HostGroup>> &plan);

}  // namespace emv
