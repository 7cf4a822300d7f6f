// emv_internal.h -- declarations shared by the host and device translation units.
#pragma once

#include "emv.h"

#include <cstdint>

int emv_fail(int status, const char *fmt, ...);
int emv_graph_validate(const emv_graph *g);
// emv_csr_build with the host time of its two phases: degree count and
// prefix sum ("pos", R:750-792) and the arc fill ("adj", R:794-826).
int emv_csr_build_timed(int64_t n, int64_t m, const int64_t *edges, int32_t *row_ptr, int32_t *col, int32_t *w,
                        double *pos_ms, double *adj_ms);

// Device status words written by bounded device loops (never a trap).
enum emv_dev_status : uint32_t {
    EMV_DEV_OK = 0,
    EMV_DEV_BARRIER_TIMEOUT = 1u << 0,   // a grid barrier spin ran out
    EMV_DEV_SWEEP_LIMIT = 1u << 1,       // relaxation exceeded n+1 sweeps
    EMV_DEV_TB_NO_WITNESS = 1u << 2,     // traceback found no split or predecessor
    EMV_DEV_TB_OVERFLOW = 1u << 3,       // traceback output or stack full
    EMV_DEV_TB_STEPS = 1u << 4,          // traceback step limit
    EMV_DEV_QUEUE_TIMEOUT = 1u << 5,     // batched work-queue wait ran out
    EMV_DEV_OVERFLOW = 1u << 6,          // a finite value plus a weight reached EMV_INF32
    EMV_DEV_BAD_VALUE = 1u << 7,         // an input value above EMV_INF32
};

int emv_dev_status_to_emv(uint32_t s);
