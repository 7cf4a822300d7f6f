// emv_solver.h -- the solver context and the host-side helpers of the GPU DP.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "emv_internal.h"
#include "emv_plan.h"

#define CUDA_TRY(x)                                                                                        \
    do {                                                                                                   \
        cudaError_t e_ = (x);                                                                              \
        if (e_ != cudaSuccess) {                                                                           \
            cudaGetLastError();                                                                            \
            return emv_fail(EMV_ERR_CUDA, "%s: %s (%s:%d)", #x, cudaGetErrorString(e_), __FILE__, __LINE__); \
        }                                                                                                  \
    } while (0)

// A device allocation that only grows (freed on context destruction).
struct DevBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
};

int dev_reserve(DevBuf &b, size_t bytes);
void dev_release(DevBuf &b);

constexpr int MAX_EVENTS = 64;
constexpr int RELAX_VARIANTS = 10;  // relaxation kernels by record width (relax_fns)
constexpr int BATCH_CLASSES = 12;  // (n bucket 0..3) x (k bucket 0..2)

// One launch of the streamed merge: subsets [x0, x0 + cnt) of a level, its
// phases and its dynamic shared memory.
struct StreamGroup {
    int64_t x0, cnt, phase_off, nphase, smem;
};

// Everything the DP needs per k, built once per k and context: the subsets by
// level, the pair and override slots of the staged-all-rows merge and the
// streamed merge's groups and phases.
struct KPlan {
    std::vector<uint32_t> xs_host;
    std::vector<int64_t> xs_off;   // level m occupies xs[off[m], off[m+1])
    DevBuf xs;                     // subsets by level
    DevBuf mpairs, movr;           // merge pair slots and override slots, all levels
    std::vector<int64_t> mpair_base, movr_base;  // per level
    DevBuf mstream_data, mstream_phases;
    std::vector<std::vector<StreamGroup>> mstream_groups;  // per level (none = not streamed)
};

struct emv_ctx {
    int device = 0;
    int sms = 0;
    int relax_blocks_max[RELAX_VARIANTS] = {};  // cooperative grid of each relaxation kernel
    int relax_sm_cap = 0;          // > 0: relaxation grids sized for this many SMs (the server's large solves)
    int64_t l2_bytes = 0;
    int64_t sweep_limit = 0;       // relaxation sweeps per chunk, 0 = n + 1
    int32_t value_bits = 0;        // 0: 16-bit merge staging / relaxation records where bounded, 32: never
    bool merge16_last = false;     // the last launch_merge took the 16-bit kernel
    int64_t relax_arcs = 0;       // arcs of the graph being relaxed (dense-sweep threshold)
    DevBuf ctrl, stat;             // relaxation barrier words, solve status
    DevBuf lvlmax;                 // per level: largest value its merge (level 1: relaxation) wrote
    DevBuf shadow;                 // 16-bit copy of the relaxed rows (the 16-bit merge's staging source)
    cudaEvent_t evmax[EMV_MAX_K + 1] = {};  // level m's maximum has reached the pinned buffer
    DevBuf scratch, act;           // vertex-major chunk buffer, active flags
    DevBuf stamp;                  // per vertex: last sweep in which it changed
    DevBuf adj;                    // packed (col, w) arcs
    DevBuf gscan;                  // GraphScan of the last packed graph (device admission check)
    DevBuf terms;                  // terminals
    DevBuf g_row, g_col, g_w;      // device copy of a host CSR
    DevBuf table;                  // DP table of emv_solve
    DevBuf tb_edges, tb_out, tb_work;
    void *pinned = nullptr;        // small pinned host buffer for scalar reads
    cudaEvent_t ev[MAX_EVENTS] = {};
    int32_t xs_k = -1;             // k of the current plan
    KPlan *kp = nullptr;           // plan of xs_k
    KPlan *kplans[EMV_MAX_K + 1] = {};  // plans of every k used so far
    bool merge_attr = false;
    int64_t launches = 0;
    // batched launch
    DevBuf bxs, bxs_off;           // subset lists of every k <= BATCH_KMAX
    bool bxs_ready = false;
    int batch_blocks = 0;
    DevBuf b_row, b_adj, b_term, b_desc, b_table, b_costs, b_ctrl;
    void *bstage = nullptr;        // pinned staging of the packed batch
    size_t bstage_bytes = 0;
    cudaGraphExec_t bgraph_exec = nullptr;
    char bgraph_args[160] = {};    // BatchArgs of the captured graph
    int32_t tune_rcap[BATCH_CLASSES] = {};
    int32_t tune_mw[BATCH_CLASSES] = {};  // merge vertex-block width per class (0: default 1)
};

int prepare_subsets(emv_ctx *c, int32_t k, cudaStream_t st);
int reserve_relax(emv_ctx *c, int32_t n);
int32_t relax_chunk_rows(const emv_ctx *c, int32_t n, bool u16);
int32_t relax_chunk_rows_level(const emv_ctx *c, int32_t n, bool u16, int64_t cnt);
