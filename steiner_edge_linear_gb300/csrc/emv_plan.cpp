// emv_plan.cpp -- host-side planning of the DP: subset levels and the
// streamed merge plan (see emv_plan.h).
#include "emv_plan.h"

#include <algorithm>

void subset_levels(int32_t k, std::vector<uint32_t> &xs, std::vector<int64_t> &off)
{
    const uint32_t rows = 1u << k;
    off.assign((size_t)k + 2, 0);
    for (uint32_t X = 1; X < rows; X++) off[(size_t)__builtin_popcount(X) + 1]++;
    for (int32_t m = 1; m <= k; m++) off[(size_t)m + 1] += off[(size_t)m];
    xs.resize(rows - 1);
    std::vector<int64_t> fill(off.begin(), off.end());
    for (uint32_t X = 1; X < rows; X++) xs[(size_t)fill[(size_t)__builtin_popcount(X)]++] = X;
}


namespace emv {

bool merge16_allowed(const uint32_t *M, int32_t m)
{
    uint64_t worst = 0;
    for (int32_t j = 1; 2 * j <= m; j++) worst = std::max<uint64_t>(worst, (uint64_t)M[j] + M[m - j]);
    return m >= 2 && worst <= 65533;
}

bool relax16_allowed(const uint32_t *M, int32_t m) { return m >= 2 && (uint64_t)M[m - 1] + M[1] <= 32767; }

int32_t relax_rows_per_chunk(int64_t n, int64_t l2_bytes, bool u16)
{
    // 256 int32 words a vertex is the relaxation scratch's capacity (CHUNK_ROWS)
    const int32_t rows = n * 512 <= l2_bytes * 3 / 4 ? 128 : 256;
    return u16 ? 2 * rows : rows;
}

int32_t relax_rows_per_level_chunk(int64_t n, int64_t l2_bytes, bool u16, int64_t cnt)
{
    const int32_t rows = relax_rows_per_chunk(n, l2_bytes, u16);
    const int64_t rows5 = (int64_t)rows * 5 / 4;
    if (n * 512 > l2_bytes * 3 / 4 || n * 640 > l2_bytes * 3 / 4) return rows;
    const int64_t nch = (cnt + rows - 1) / rows, nch5 = (cnt + rows5 - 1) / rows5;
    if (nch5 >= nch) return rows;
    return (int32_t)((cnt + nch5 - 1) / nch5);
}

// Accumulator space of a streamed-merge group of g subsets, in 128-byte rows:
// one per subset, two where the 16-bit kernel keeps one uint32 per vertex
// (g <= 64: its 128 quarter-warps then split each subset's pairs).
int64_t stream_acc_rows(int64_t g) { return g <= 64 ? 2 * g : g; }

// Plan of the streamed merge (k_merge_stream) for every level of k.  The
// subsets of level m are cut into groups whose accumulators (128 bytes per
// subset and 32 vertices) leave room for staged rows; for each group and each
// j = 1..m/2 the pairs {Y, X\Y} with |Y| = j are cut into phases whose rows
// fit the rest of the shared memory, taking the Y's in level order, each with
// all the X\Y it pairs with in the group.  Several group sizes are planned
// and the one staging the fewest rows is kept; up to k = 12 that is the whole
// level in one group with one phase per j.  A level with no workable plan
// keeps the staged-all-lower-rows kernel.
namespace {

// Plans level m with groups of at most gx subsets into `data` (offsets
// relative to its start); returns false when a group cannot hold one pair.
bool plan_level(const std::vector<uint32_t> &xs, const std::vector<int64_t> &off, const std::vector<uint32_t> &rank,
                std::vector<int32_t> &pos, int32_t m, int64_t gx, int64_t smem_bytes, std::vector<uint32_t> &data,
                std::vector<HostGroup> &groups, int64_t &cost)
{
    const int64_t lvl = off[(size_t)m], cnt = off[(size_t)m + 1] - lvl;
    const int64_t cap = smem_bytes / 128 - stream_acc_rows(gx) - 1;  // staged rows besides the INF pad row
    if (cap < 2) return false;
    data.clear();
    groups.clear();
    cost = 0;
    struct Entry {
        uint32_t ry, xi, y, z;
    };
    std::vector<Entry> ent;
    std::vector<std::vector<uint32_t>> per_x;
    std::vector<uint32_t> rows;
    for (int64_t x0 = 0; x0 < cnt; x0 += gx) {
        const int64_t g = std::min(gx, cnt - x0);
        HostGroup G{x0, g, 0, {}};
        per_x.assign((size_t)g, {});
        int64_t max_rows = 0;
        auto emit = [&]() {
            if (rows.empty()) return;
            HostPhase hp;
            hp.nrows = (int32_t)rows.size();
            hp.rows_at = data.size();
            data.insert(data.end(), rows.begin(), rows.end());
            hp.qoff_at = data.size();
            uint32_t q = 0;
            for (int64_t x = 0; x < g; x++) {
                data.push_back(q);
                q += (uint32_t)((per_x[(size_t)x].size() + 3) / 4);
            }
            data.push_back(q);
            while (data.size() % 4) data.push_back(0);  // pairs are read as uint4: 16-byte aligned
            hp.pairs_at = data.size();
            const uint32_t pad = (uint32_t)hp.nrows | ((uint32_t)hp.nrows << 16);
            for (int64_t x = 0; x < g; x++) {
                std::vector<uint32_t> &l = per_x[(size_t)x];
                while (l.size() % 4) l.push_back(pad);
                data.insert(data.end(), l.begin(), l.end());
                cost += (int64_t)l.size() / 4;  // padded pair quads
                l.clear();
            }
            for (uint32_t r : rows) pos[r] = -1;
            max_rows = std::max<int64_t>(max_rows, hp.nrows);
            cost += hp.nrows + 32;
            rows.clear();
            G.phases.push_back(hp);
        };
        for (int32_t j = 1; 2 * j <= m; j++) {
            const bool same = (j == m - j);
            ent.clear();
            for (int64_t x = 0; x < g; x++) {
                const uint32_t X = xs[(size_t)(lvl + x0 + x)];
                const uint32_t low = X & (0u - X);
                for (uint32_t Y = (X - 1) & X; Y; Y = (Y - 1) & X) {
                    if (__builtin_popcount(Y) != j || (same && !(Y & low))) continue;
                    ent.push_back({rank[Y], (uint32_t)x, Y, X ^ Y});
                }
            }
            std::stable_sort(ent.begin(), ent.end(), [](const Entry &a, const Entry &b) { return a.ry < b.ry; });
            for (const Entry &e : ent) {
                const int64_t need = (pos[e.y] < 0) + (pos[e.z] < 0 && e.z != e.y);
                if ((int64_t)rows.size() + need > cap) emit();
                if (pos[e.y] < 0) {
                    pos[e.y] = (int32_t)rows.size();
                    rows.push_back(e.y);
                }
                if (pos[e.z] < 0) {
                    pos[e.z] = (int32_t)rows.size();
                    rows.push_back(e.z);
                }
                per_x[e.xi].push_back((uint32_t)pos[e.y] | ((uint32_t)pos[e.z] << 16));
            }
            emit();
        }
        G.smem = (stream_acc_rows(g) + max_rows + 1) * 128;
        cost += 64;
        groups.push_back(std::move(G));
    }
    return true;
}

}  // namespace

void plan_stream_levels(int32_t k, const std::vector<uint32_t> &xs, const std::vector<int64_t> &off,
                        int64_t smem_bytes, std::vector<uint32_t> &data, std::vector<std::vector<HostGroup>> &plan)
{
    std::vector<uint32_t> rank((size_t)1 << k, 0);  // position within its level
    for (int32_t m = 1; m <= k; m++)
        for (int64_t i = off[(size_t)m]; i < off[(size_t)m + 1]; i++) rank[xs[(size_t)i]] = (uint32_t)(i - off[(size_t)m]);
    std::vector<int32_t> pos((size_t)1 << k, -1);
    std::vector<uint32_t> tmp, best_data;
    std::vector<HostGroup> tmp_groups, best_groups;
    data.clear();
    plan.assign((size_t)k + 2, {});
    for (int32_t m = 2; m <= k; m++) {
        const int64_t cnt = off[(size_t)m + 1] - off[(size_t)m];
        int64_t best_cost = -1;
        for (int64_t gx : {cnt, (int64_t)1024, (int64_t)768, (int64_t)512, (int64_t)384, (int64_t)256, (int64_t)128}) {
            if (gx != cnt && gx >= cnt) continue;
            int64_t cost;
            if (!plan_level(xs, off, rank, pos, m, gx, smem_bytes, tmp, tmp_groups, cost)) continue;
            if (best_cost < 0 || cost < best_cost) {
                best_cost = cost;
                best_data.swap(tmp);
                best_groups.swap(tmp_groups);
            }
        }
        if (best_cost < 0) continue;  // not streamed
        while (data.size() % 4) data.push_back(0);
        const size_t rel = data.size();
        data.insert(data.end(), best_data.begin(), best_data.end());
        for (HostGroup &G : best_groups)
            for (HostPhase &hp : G.phases) {
                hp.rows_at += rel;
                hp.qoff_at += rel;
                hp.pairs_at += rel;
            }
        plan[(size_t)m] = best_groups;
    }
}

}  // namespace emv
