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
#include <string>
#include <utility>

using namespace emv;

static int fail(const char *what, int k, int m)
{
    std::printf("FAIL k=%d m=%d: %s\n", k, m, what);
    return 1;
}

// The relaxation chunk rule: chunks never exceed the kernels' record widths
// (160 words with L2-resident records, 256 otherwise), cover a level in the
// fewest launches the rule allows, and match worked cases.
static int check_chunks()
{
    const int64_t l2 = 126ll << 20;
    auto expect = [&](int64_t n, bool u16, int64_t cnt, int32_t rows) {
        const int32_t got = relax_rows_per_level_chunk(n, l2, u16, cnt);
        if (got != rows) std::printf("FAIL chunks n=%lld u16=%d cnt=%lld: %d rows, want %d\n", (long long)n, (int)u16,
                                     (long long)cnt, got, rows);
        return got == rows;
    };
    bool ok = expect(100000, true, 792, 264) && expect(100000, true, 924, 308) && expect(100000, true, 495, 256) &&
              expect(100000, true, 220, 256) && expect(100000, false, 924, 154) && expect(100000, false, 792, 159) &&
              expect(100000, false, 495, 128) && expect(1 << 20, true, 3432, 512) && expect(1 << 20, false, 3432, 256) &&
              expect(160000, true, 792, 256);
    for (int64_t n : {64ll, 1000ll, 100000ll, 150000ll, 200000ll, 1ll << 20})
        for (int u = 0; u < 2 && ok; u++)
            for (int64_t cnt = 1; cnt <= 3432 && ok; cnt++) {
                const int32_t rows = relax_rows_per_level_chunk(n, l2, u != 0, cnt);
                const int64_t words = u ? (rows + 1) / 2 : rows;
                const bool resident = n * 512 <= l2 * 3 / 4;
                const int64_t base = relax_rows_per_chunk(n, l2, u != 0);
                if (rows < 1 || words > (resident ? 160 : 256) || (cnt + rows - 1) / rows > (cnt + base - 1) / base) {
                    std::printf("FAIL chunks n=%lld u16=%d cnt=%lld: %d rows\n", (long long)n, u, (long long)cnt, rows);
                    ok = false;
                }
            }
    if (ok) std::printf("ok chunks\n");
    return ok ? 0 : 1;
}

// The value-width rules at their edges: exact thresholds, unknown maxima
// (all ones) and sums that would overflow 32 bits.
static int check_widths()
{
    bool ok = true;
    auto want = [&](bool got, bool exp, const char *what) {
        if (got != exp) {
            std::printf("FAIL widths: %s\n", what);
            ok = false;
        }
    };
    uint32_t M[8] = {0, 16000, 16767, 30000, 0, 0, 0, 0};
    want(relax16_allowed(M, 2), true, "2 * 16000 <= 32767");
    want(relax16_allowed(M, 3), true, "16767 + 16000 = 32767");
    M[2] = 16768;
    want(relax16_allowed(M, 3), false, "16768 + 16000 > 32767");
    want(merge16_allowed(M, 3), true, "16000 + 16768 <= 65533");
    M[3] = 49533;
    want(merge16_allowed(M, 4), true, "max(16000 + 49533, 2 * 16768) = 65533");
    M[3] = 49534;
    want(merge16_allowed(M, 4), false, "16000 + 49534 = 65534");
    M[3] = 0xffffffffu;  // level 3 not recorded
    want(merge16_allowed(M, 4), false, "unknown maximum");
    want(relax16_allowed(M, 4), false, "unknown maximum, no 32-bit wrap");
    M[1] = 0x80000000u;
    want(relax16_allowed(M, 2), false, "2^31 + 2^31 must not wrap to 0");
    if (ok) std::printf("ok widths\n");
    return ok ? 0 : 1;
}

int main(int argc, char **argv)
{
    if (argc == 2 && std::string(argv[1]) == "chunks") return check_chunks();
    if (argc == 2 && std::string(argv[1]) == "widths") return check_widths();
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
