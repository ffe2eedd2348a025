// Interface of the SSPRK stage kernel (amr_ssprk.cu, compiled without
// multiply-add contraction).
#pragma once

#include <algorithm>

#include "amr_device.cuh"

namespace amr_gb300 {

// One stage over every cell of P padded patches (FP64).  mode: 0 = first
// stage (u + R dt), 2 = SSPRK2 second stage, 31 / 32 = SSPRK3 second / third
// stage.  vel: per instance, 3 each; step_dt: per instance, the step in use.
struct SsprkStage {
    const double*   in;
    const double*   un;
    double*         out;
    const uint64_t* keys;
    int             P;
    Geo             g;
    const double*   vel;
    const double*   step_dt;
    int             mode;
    cudaStream_t    stream;
};

cudaError_t ssprk_stage(const SsprkStage& s);

} // namespace amr_gb300
