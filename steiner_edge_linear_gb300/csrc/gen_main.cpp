// gen_main.cpp -- emv-gen: writes a generated instance as STP text.
//
// A stand-alone executable built from the host sources of the library
// (emv_host.cpp) without CUDA and without libemv.so, so that programs which
// must not load the solver -- the timed reference runs, which read the same
// instance from a file -- still get bit-identical instances.  Counterpart of
// the reference's generator command (graph-gen/gen-unique.c:480-571).
//
//   emv-gen regular <n> <degree> <wmin> <wmax> <k> <seed> <out.stp>
//   emv-gen mixed <base_seed> <index> <out.stp>
//   emv-gen powlaw <n> <degree> <alpha> <classes> <wmin> <wmax> <k> <seed> <out.stp>
//   emv-gen clique <n> <wmin> <wmax> <k> <seed> <out.stp>
#include "emv.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>

static int usage()
{
    std::fprintf(stderr,
                 "usage: emv-gen regular <n> <degree> <wmin> <wmax> <k> <seed> <out.stp>\n"
                 "       emv-gen mixed <base_seed> <index> <out.stp>\n"
                 "       emv-gen powlaw <n> <degree> <alpha> <classes> <wmin> <wmax> <k> <seed> <out.stp>\n"
                 "       emv-gen clique <n> <wmin> <wmax> <k> <seed> <out.stp>\n");
    return 2;
}

static long long num(const char *s) { return std::strtoll(s, nullptr, 10); }

int main(int argc, char **argv)
{
    if (argc < 2) return usage();
    emv_stp *g = nullptr;
    int st = EMV_ERR_BAD_INPUT;
    const char *out = argv[argc - 1];
    if (!std::strcmp(argv[1], "regular") && argc == 9)
        st = emv_gen_regular(num(argv[2]), (int32_t)num(argv[3]), (int32_t)num(argv[4]), (int32_t)num(argv[5]),
                             (int32_t)num(argv[6]), std::strtoull(argv[7], nullptr, 10), &g);
    else if (!std::strcmp(argv[1], "mixed") && argc == 5)
        st = emv_gen_mixed(std::strtoull(argv[2], nullptr, 10), num(argv[3]), 64, 4096, 4, 10, 10, &g);
    else if (!std::strcmp(argv[1], "powlaw") && argc == 11)
        st = emv_gen_powlaw(num(argv[2]), (int32_t)num(argv[3]), std::strtod(argv[4], nullptr), (int32_t)num(argv[5]),
                            (int32_t)num(argv[6]), (int32_t)num(argv[7]), (int32_t)num(argv[8]),
                            std::strtoull(argv[9], nullptr, 10), &g);
    else if (!std::strcmp(argv[1], "clique") && argc == 7)
        st = emv_gen_clique(num(argv[2]), (int32_t)num(argv[3]), (int32_t)num(argv[4]), (int32_t)num(argv[5]),
                            std::strtoull(argv[6], nullptr, 10), &g);
    else
        return usage();
    if (st == EMV_OK) st = emv_stp_write(g, out);
    if (st != EMV_OK) {
        std::fprintf(stderr, "emv-gen: %s: %s\n", emv_status_str(st), emv_last_error());
        emv_stp_free(g);
        return 1;
    }
    std::printf("n=%lld m=%lld k=%lld\n", (long long)g->n, (long long)g->m, (long long)g->k);
    emv_stp_free(g);
    return 0;
}
