// emv_internal.h -- declarations shared by the host and device translation units.
#pragma once

#include "emv.h"

#include <cstdint>

int emv_fail(int status, const char *fmt, ...);
int emv_graph_validate(const emv_graph *g);

// Device status words written by bounded device loops (never a trap).
enum emv_dev_status : uint32_t {
    EMV_DEV_OK = 0,
    EMV_DEV_BARRIER_TIMEOUT = 1u << 0,   // a grid barrier spin ran out
    EMV_DEV_SWEEP_LIMIT = 1u << 1,       // relaxation exceeded n+1 sweeps
    EMV_DEV_TB_NO_WITNESS = 1u << 2,     // traceback found no split or predecessor
    EMV_DEV_TB_OVERFLOW = 1u << 3,       // traceback output or stack full
    EMV_DEV_TB_STEPS = 1u << 4,          // traceback step limit
    EMV_DEV_QUEUE_TIMEOUT = 1u << 5,     // batched work-queue wait ran out
};

int emv_dev_status_to_emv(uint32_t s);
