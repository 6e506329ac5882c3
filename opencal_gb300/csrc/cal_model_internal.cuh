/*
 * cal_model_internal.cuh -- library-private device state hung off the public
 * CALModel2D / CALModel3D structs (their `gpu` field).
 */
#pragma once

#include "cal_core.cuh"
#include "opencal/cal2D.h"
#include "opencal/cal3D.h"

struct CALGpuModel2D {
    cal::CalGrid g;
    struct CALCell2D* d_X = nullptr; /* device copy of the neighbourhood table */
    int d_X_len = 0;                 /* entries uploaded; -1 forces an upload */
    CALLaunchFunc2D launch[CAL_MAX_ELEMENTARY_PROCESSES];
    bool pure[CAL_MAX_ELEMENTARY_PROCESSES] = {}; /* calSetElementaryProcessPure2D */
    /* calSetElementaryProcessReads2D: the substates (type, slot) each
     * process reads, staged into shared memory by TMA */
    /* calSetElementaryProcessGuard2Dr: CAL_GUARD_* and the real slot / value */
    int guard_op[CAL_MAX_ELEMENTARY_PROCESSES] = {};
    int guard_slot[CAL_MAX_ELEMENTARY_PROCESSES] = {};
    double guard_value[CAL_MAX_ELEMENTARY_PROCESSES] = {};
    int nreads[CAL_MAX_ELEMENTARY_PROCESSES] = {};
    int read_t[CAL_MAX_ELEMENTARY_PROCESSES][CAL_MAX_STAGED] = {};
    int read_s[CAL_MAX_ELEMENTARY_PROCESSES][CAL_MAX_STAGED] = {};
    int* d_stage_err = nullptr; /* a staged box that did not arrive in time */
};

struct CALGpuModel3D {
    cal::CalGrid g;
    struct CALCell3D* d_X = nullptr;
    int d_X_len = 0;
    CALLaunchFunc3D launch[CAL_MAX_ELEMENTARY_PROCESSES];
};
