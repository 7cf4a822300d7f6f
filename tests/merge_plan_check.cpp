// merge_plan_check.cpp -- checks the streamed merge plan of emv_plan.cpp for
// one k (host only, built by tests/test_merge_plan.py with g++):
//   * the per-subset pair lists cover every unordered pair {Y, X \ Y} of
//     every subset exactly once, with both halves staged in the phase (the
//     pad slot only in (pad, pad) quad padding);
//   * staged rows of phase j have sizes j or m - j and are distinct;
//   * shared memory fits the budget; blocks read as uint4 are 16-byte aligned.
// Prints one summary line and exits non-zero on the first violation.
#include "emv_plan.h"

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <set>
#include <utility>

using namespace emv;

static int fail(const char *what, int k, int m)
{
    std::printf("FAIL k=%d m=%d: %s\n", k, m, what);
    return 1;
}

int main(int argc, char **argv)
{
    if (argc < 3) return 2;
    const int k = std::atoi(argv[1]);
    const int64_t smem = std::atoll(argv[2]);
    std::vector<uint32_t> xs, data;
    std::vector<int64_t> off;
    std::vector<std::vector<HostGroup>> plan;
    subset_levels(k, xs, off);
    plan_stream_levels(k, xs, off, smem, data, plan);
    int64_t pairs_total = 0, streamed = 0;
    for (int m = 2; m <= k; m++) {
        if (plan[(size_t)m].empty()) continue;
        streamed++;
        int64_t covered = 0;
        for (const HostGroup &G : plan[(size_t)m]) {
            const int64_t g = G.cnt;
            // pairs seen per subset
            std::vector<std::map<std::pair<uint32_t, uint32_t>, int>> by_pairs((size_t)g);
            int64_t max_rows = 0;
            for (const HostPhase &P : G.phases) {
                if (P.pairs_at % 4) return fail("pair block not aligned", k, m);
                const uint32_t nr = (uint32_t)P.nrows;
                max_rows = std::max<int64_t>(max_rows, nr);
                std::set<uint32_t> rows;
                int jsize = -1;
                for (uint32_t r = 0; r < nr; r++) {
                    const uint32_t R = data[P.rows_at + r];
                    if (!rows.insert(R).second) return fail("row staged twice in a phase", k, m);
                    const int sz = __builtin_popcount(R), j = std::min(sz, m - sz);
                    if (jsize < 0) jsize = j;
                    if (j != jsize) return fail("phase mixes row sizes of different j", k, m);
                }
                auto row = [&](uint32_t slot) { return data[P.rows_at + slot]; };
                for (int64_t x = 0; x < g; x++) {
                    const uint32_t q0 = data[P.qoff_at + (size_t)x], q1 = data[P.qoff_at + (size_t)x + 1];
                    for (uint32_t i = 4 * q0; i < 4 * q1; i++) {
                        const uint32_t w = data[P.pairs_at + i], a = w & 0xffffu, b = w >> 16;
                        if (a > nr || b > nr) return fail("pair slot out of range", k, m);
                        if (a == nr && b == nr) continue;  // quad padding
                        if (a == nr || b == nr) return fail("pair with one pad half", k, m);
                        const uint32_t Y = row(a), Z = row(b);
                        by_pairs[(size_t)x][{std::min(Y, Z), std::max(Y, Z)}]++;
                    }
                }
            }
            if ((stream_acc_rows(g) + max_rows + 1) * 128 != G.smem || G.smem > smem)
                return fail("shared memory of the group", k, m);
            for (int64_t x = 0; x < g; x++) {
                const uint32_t X = xs[(size_t)(off[(size_t)m] + G.x0 + x)];
                std::map<std::pair<uint32_t, uint32_t>, int> want;
                for (uint32_t Y = (X - 1) & X; Y; Y = (Y - 1) & X) {
                    const uint32_t Z = X ^ Y;
                    want[{std::min(Y, Z), std::max(Y, Z)}] = 1;
                }
                if (by_pairs[(size_t)x] != want) return fail("pair lists do not cover the pairs once", k, m);
                pairs_total += (int64_t)want.size();
                covered++;
            }
        }
        if (covered != off[(size_t)m + 1] - off[(size_t)m]) return fail("level not fully covered", k, m);
    }
    std::printf("ok k=%d streamed_levels=%lld pairs=%lld\n", k, (long long)streamed, (long long)pairs_total);
    return 0;
}
