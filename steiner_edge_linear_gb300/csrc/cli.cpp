// cli.cpp -- reader-el-gpu: the reference's command surface over the GPU solver.
//
// Same flags as reader-el's main() (reader/reader-el.c:2368-2412):
//   -in <file> (else stdin), -el / -erickson, -list, -seed <n>, -dijkstra, -h / -help
// plus -bin (the input is an EMVBIN01 container, see emv_bin_open; the
// reference's report.py passes -bin but its reader has no binary format) and
// -index <i> (which instance of the container, default 0)
// and the same stdout lines (R:2414-2437, R:603-614, R:735-896, R:2445,
// R:2298-2340, R:1891-1903, R:2500-2528), so the reference's scripts parse
// them unchanged.  As in the reference, a "cost" line in the input that
// differs from the computed cost ends the program with an ERROR (R:2489-2491).
// Memory fields report the solver's device allocations.  One extra line,
// "gpu: ...", gives the per-phase device times and rates.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <sys/utsname.h>
#include <vector>

#include "emv.h"
#include "emv_internal.h"

namespace {

double now_ms()
{
    using namespace std::chrono;
    return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

double gib(int64_t b) { return (double)b / (double)(1 << 30); }

[[noreturn]] void die(const char *func, const char *fmt, const char *arg)
{
    std::fprintf(stderr, "ERROR [file = %s, line = %d] %s: ", __FILE__, __LINE__, func);
    std::fprintf(stderr, fmt, arg);
    std::fprintf(stderr, "\n");
    std::exit(1);
}

[[noreturn]] void die_status(const char *func, int st)
{
    std::fprintf(stderr, "ERROR [file = %s, line = %d] %s: %s: %s\n", __FILE__, __LINE__, func,
                 emv_status_str(st), emv_last_error());
    std::exit(1);
}

}  // namespace

int main(int argc, char **argv)
{
    const double t_main = now_ms();
    long seed = 123456789;
    bool have_seed = false, list_soln = false, file_input = false, bin_input = false;
    long bin_index = 0;
    int cmd = 0;  // 0 nop, 1 dijkstra, 2 edge-linear
    const char *filename = nullptr;
    for (int f = 1; f < argc; f++) {
        if (argv[f][0] != '-') continue;
        if (!std::strcmp(argv[f], "-dijkstra")) cmd = 1;
        if (!std::strcmp(argv[f], "-el") || !std::strcmp(argv[f], "-erickson")) cmd = 2;
        if (!std::strcmp(argv[f], "-list")) list_soln = true;
        if (!std::strcmp(argv[f], "-bin")) bin_input = true;
        if (!std::strcmp(argv[f], "-index")) {
            if (f == argc - 1) die("main", "%s", "instance index missing from command line");
            bin_index = std::atol(argv[++f]);
        }
        if (!std::strcmp(argv[f], "-in")) {
            if (f == argc - 1) die("main", "%s", "file name missing from command line");
            filename = argv[++f];
            file_input = true;
        }
        if (!std::strcmp(argv[f], "-seed")) {
            if (f == argc - 1) die("main", "%s", "random seed missing from command line");
            seed = std::atol(argv[++f]);
            have_seed = true;
        }
        if (!std::strcmp(argv[f], "-h") || !std::strcmp(argv[f], "-help")) {
            std::printf("usage: %s -in <input graph> <arguments>\n\narguments :\n"
                        "\t-seed : seed value\n\t-el : Erickson-Monma-Veinott algorithm\n"
                        "\t-dijkstra : Dijkstra single source shortest path\n"
                        "\t-list : Output Steiner tree\n"
                        "\t-bin : input is an EMVBIN01 container (-index <i> selects the instance)\n\n",
                        argv[0]);
            return 0;
        }
    }
    std::printf("invoked as:");
    for (int f = 0; f < argc; f++) std::printf(" %s", argv[f]);
    std::printf("\n");
    if (!file_input) std::printf("no input file specified, defaulting to stdin\n");
    if (!have_seed) std::printf("no random seed given, defaulting to %ld\n", seed);
    std::printf("random seed = %ld\n", seed);
    std::fflush(stdout);

    // graph_load (R:473-618), or a container record read as arrays
    double t0 = now_ms();
    emv_stp *g = nullptr;
    emv_bin *bin = nullptr;
    emv_instance binst{};
    int64_t n = 0, m = 0, k = 0, stp_cost = -1;
    int st;
    if (bin_input) {
        if (!file_input) die("main", "%s", "-bin needs -in <file>");
        st = emv_bin_open(filename, &bin);
        if (!st) st = emv_bin_instance(bin, (int32_t)bin_index, &binst, &stp_cost);
        if (st) die_status("graph_load", st);
        n = binst.g.n;
        m = binst.g.arcs / 2;
        k = binst.k;
    } else {
        st = emv_stp_load(file_input ? filename : nullptr, &g);
        if (st) die_status("graph_load", st);
        n = g->n;
        m = g->m;
        k = g->k;
        stp_cost = g->cost;
    }
    std::printf("input: n = %lld, m = %lld, k = %lld, cost = %lld [%.2lf ms] {peak: %.2lfGiB} {curr: %.2lfGiB}\n",
                (long long)n, (long long)m, (long long)k, (long long)stp_cost, now_ms() - t0, 0.0, 0.0);
    std::printf("terminals:");
    for (int64_t i = 0; i < k; i++)
        std::printf(" %lld", (long long)(bin ? binst.terminals[i] : g->terminals[i]) + 1);
    std::printf("\n");
    std::fflush(stdout);

    // root_build (R:706-899): CSR and the terminal index (a container holds the CSR already).
    const double t_rb = now_ms();
    std::printf("root build: ");
    double t1 = now_ms();
    std::vector<int32_t> row, col, w;
    if (!bin) {
        row.resize((size_t)n + 1);
        col.resize((size_t)(2 * m));
        w.resize((size_t)(2 * m));
    }
    std::printf("[zero: %.2lf ms] ", now_ms() - t1);
    double pos_ms = 0, adj_ms = 0;  // a container holds the CSR already: both phases take no time
    if (!bin) {
        st = emv_csr_build_timed(n, m, g->edges, row.data(), col.data(), w.data(), &pos_ms, &adj_ms);
        if (st) die_status("root_build", st);
    }
    std::printf("[pos: %.2lf ms] [adj: %.2lf ms] ", pos_ms, adj_ms);
    t1 = now_ms();
    std::vector<int32_t> kk((size_t)k);
    for (int64_t i = 0; i < k; i++) kk[(size_t)i] = bin ? binst.terminals[i] : (int32_t)g->terminals[i];
    std::printf("[term: %.2lf ms] ", now_ms() - t1);
    const int64_t host_bytes = (4 * (n + 1) + 16 * m);
    std::printf("done. [%.2lf ms] {peak: %.2lfGiB} {curr: %.2lfGiB}\n", now_ms() - t_rb, gib(host_bytes),
                gib(host_bytes));
    emv_graph graph = bin ? binst.g : emv_graph{(int32_t)n, 2 * m, row.data(), col.data(), w.data()};

    static const char *legend[] = {"no operation", "Dijkstra Single-Source-Shortest-Path", "Erickson-Monma-Veinott"};
    std::printf("command: %s\n", legend[cmd]);
    std::fflush(stdout);
    const double t_cmd = now_ms();
    emv_ctx *ctx = nullptr;
    int64_t dev_peak = 0;
    if (cmd == 1) {
        // R:2454-2484: random source from srand(seed); rand() % n.
        std::srand((unsigned)seed);
        const int32_t s = (int32_t)(std::rand() % n);
        st = emv_create(&ctx, 0);
        if (st) die_status("emv_create", st);
        std::vector<int64_t> dist((size_t)n);
        float ms = 0;
        st = emv_sssp(ctx, &graph, s, dist.data(), &ms, nullptr);
        if (st) die_status("dijkstra", st);
        int64_t reach = 0, far = 0;
        for (int64_t v = 0; v < n; v++)
            if (dist[(size_t)v] != INT64_MAX) { reach++; if (dist[(size_t)v] > far) far = dist[(size_t)v]; }
        std::printf("dijkstra: [source: %d] [total: %.2lf ms %.2lfGiB/s] [reached: %lld] [max: %lld]\n", s + 1,
                    (double)ms, (double)(12 * n + 16 * m + 4 * (n + 1)) / (ms / 1000.0) / (1 << 30),
                    (long long)reach, (long long)far);
    } else if (cmd == 2) {
        st = emv_create(&ctx, 0);
        if (st) die_status("emv_create", st);
        emv_result res;
        std::memset(&res, 0, sizeof(res));
        std::vector<int32_t> tree;
        if (list_soln) {
            tree.resize((size_t)(3 * (n + 1)));
            res.tree = tree.data();
            res.tree_cap = n + 1;
        }
        const double t_el = now_ms();
        st = emv_solve(ctx, &graph, kk.data(), (int32_t)k, list_soln ? EMV_SOLVE_TREE : 0, &res, nullptr);
        if (st) die_status("erickson_monma_veinott", st);
        const double el_ms = now_ms() - t_el;
        const emv_timing &tm = res.timing;
        const int64_t table_bytes = (int64_t)4 * ((n + 31) / 32 * 32) << k;
        dev_peak = table_bytes + 4 * (n + 1) + 24 * m + 128 * ((n + 31) / 32 * 32);
        // Bytes of the reference's own accounting (R:2294): 3^(k+1) n words plus
        // 2^k graph sweeps, here in int32 words.
        const double merge_bytes = 12.0 * (double)n * (std::pow(3.0, (double)k) - std::pow(2.0, (double)k + 1) + 1);
        const double relax_bytes = (std::pow(2.0, (double)k) - 1) * (12.0 * n + 16.0 * m + 4.0 * (n + 1));
        const double kernel_gib = (merge_bytes + relax_bytes) / (tm.kernel_ms / 1000.0) / (1 << 30);
        if (k == 2) {
            std::printf("erickson: [kernel: %.2lf ms %.2lfGiB/s] ", (double)tm.kernel_ms, kernel_gib);
        } else {
            std::printf("erickson: [zero: %.2lf ms] [kernel: %.2lf ms %.2lfGiB/s] ", (double)tm.zero_ms,
                        (double)tm.kernel_ms, kernel_gib);
        }
        if (list_soln && k != 2) std::printf("[traceback: %.2lf ms] ", (double)tm.traceback_ms);
        std::printf("done. [%.2lf ms] [cost: %lld] {peak: %.2lfGiB} {curr: %.2lfGiB}\n", el_ms,
                    (long long)res.cost, gib(dev_peak), gib(dev_peak));
        if (list_soln) {
            std::printf("solution: [");
            for (int64_t i = 0; i < res.tree_count; i++)
                std::printf("%s\"%d %d\"", i ? ", " : "", tree[(size_t)(3 * i)] + 1, tree[(size_t)(3 * i + 1)] + 1);
            std::printf("]\n");
        }
        std::printf("gpu: [level1: %.3f ms] [merge: %.3f ms %.1f GB/s] [relax: %.3f ms %.1f GB/s %lld sweeps] "
                    "[%.3f Gcell/s] [launches: %lld]\n",
                    (double)tm.level1_ms, (double)tm.merge_ms, merge_bytes / (tm.merge_ms * 1e6),
                    (double)tm.relax_ms, relax_bytes / ((tm.relax_ms + tm.level1_ms) * 1e6),
                    (long long)tm.relax_sweeps, (double)(n << k) / (tm.kernel_ms * 1e6), (long long)tm.launches);
        std::fflush(stdout);
        if (stp_cost != -1 && stp_cost != res.cost) {
            std::fprintf(stderr, "ERROR [file = %s, line = %d] main: min_cost != cost: minimum cost = %lld, cost = %lld\n",
                         __FILE__, __LINE__, (long long)stp_cost, (long long)res.cost);
            std::exit(1);
        }
    }
    if (ctx) emv_destroy(ctx);
    emv_stp_free(g);
    emv_bin_close(bin);
    std::printf("command done [%.2lf ms]\n", now_ms() - t_cmd);
    std::printf("grand total [%.2lf ms] {peak: %.2lfGiB}\n", now_ms() - t_main, gib(dev_peak + host_bytes));
    struct utsname un;
    uname(&un);
    std::printf("host: %s\n", un.nodename);
    std::printf("build: %s, %s, %s\n", "edge-linear kernel", "gb300 cuda sm_103a", "frontier relaxation");
    std::printf("list solution: %s\n", list_soln ? "true" : "false");
    std::printf("num threads: %d\n", 1);
    std::printf("compiler: gcc %d.%d.%d\n", __GNUC__, __GNUC_MINOR__, __GNUC_PATCHLEVEL__);
    std::fflush(stdout);
    return 0;
}
