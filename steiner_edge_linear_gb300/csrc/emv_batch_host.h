// emv_batch_host.h -- host helpers of the batched launch, shared with the server.
#pragma once

#include <chrono>
#include <vector>

#include "emv_batch_types.h"
#include "emv_solver.h"

struct BatchPack {
    std::vector<emv::BatchInst> desc;  // in launch order
    std::vector<int64_t> row_off, arc_off, term_off, table_off;  // into the packed device buffers
    int64_t rows = 0, arcs = 0, terms = 0, table_words = 0;
    int32_t count = 0;
    int32_t rcap_used = 0;
    int64_t cost_slots = 0;            // entries the device cost array needs (max orig + 1)
    int32_t *h_row = nullptr;          // views into the pinned staging buffer
    int2 *h_adj = nullptr;
    int32_t *h_term = nullptr;
    emv::BatchInst *h_desc = nullptr;
    std::chrono::steady_clock::time_point t_upload_end;
};

int32_t batch_class_of(int32_t n, int32_t k);
int32_t batch_rcap_max(int32_t n);
int32_t batch_rcap_for(const emv_ctx *c, int32_t n, int32_t k);
int32_t batch_mw_max(int32_t n, int32_t k);
int32_t batch_mw_for(const emv_ctx *c, int32_t n, int32_t k);
bool batch_fits(int32_t n, int32_t k);
double batch_work(int32_t n, int32_t k, int64_t arcs);
int prepare_batch_subsets(emv_ctx *c, cudaStream_t st);
int batch_kernel_setup(emv_ctx *c);
int batch_pack(emv_ctx *c, const emv_instance *inst, const std::vector<int32_t> &order, int32_t lo, int32_t hi,
               BatchPack &pk);
int batch_upload(emv_ctx *c, BatchPack &pk, cudaStream_t st);
emv::BatchArgs batch_args(emv_ctx *c, const BatchPack &pk);
// max_blocks > 0 caps the persistent grid (the autotuner's samples).
int launch_batch(emv_ctx *c, const emv::BatchArgs &a, int32_t count, cudaStream_t st, int32_t max_blocks = 0);
int batch_graph_launch(emv_ctx *c, const emv::BatchArgs &a, int32_t count, cudaStream_t st);
