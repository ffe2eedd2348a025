// Interface of the Euler solver kernels (amr_euler.cu) for the tree.  The
// translation unit is compiled without multiply-add contraction so every
// operation rounds as in the reference's CPU code.
#pragma once

#include "amr_device.cuh"

namespace amr_gb300 {

// Device buffers of one Euler advance.  State fields (rho, rho u_d, E) and
// the one-side flux terms of each direction d (|u_d| + a, m_k u_d + [k = d]
// p, u_d (E + p): rank * (rank + 2) quantities) are each fstride elements
// apart; state[b] and prim[b] belong together (buffer b).  Side terms are
// kept for interior and face-ghost cells.
struct EulerBufs {
    Geo                  g;
    int                  P;
    size_t               fstride;
    const int32_t*       levels;
    const amr_halo_meta* meta;
    double*              state[2];
    double*              prim[2];
    unsigned long long*  min_slot; // two alternating minima of dx / (|u_d| + a), as bit patterns
    double*              step_dt;  // [0] the step in use
    int32_t*             ctl;      // [0] the step runs, [1] the advance has stopped
    double*              acc;      // simulated time of the advance
    double*              rem;      // time still allowed
    uint32_t*            cnt;      // executed steps
    cudaStream_t         stream;
};

// Starts an advance on state[cur] (face ghosts current): resets the time
// bookkeeping to `remaining`, computes the side terms of state[cur] into
// prim[cur] and the minimum for the first step into slot 0.
// Adds the kernels launched to *launches.
cudaError_t euler_begin(const EulerBufs& b, int cur, double gamma, double remaining, uint64_t* launches);

// One step from state[cur] into state[1 - cur]: the step size from slot
// `slot` (clamped to the remaining time), the Rusanov update of every field,
// the side terms and the next step's minimum (slot 1 - slot), then the face
// halo of every field with the ghosts' side terms.
// ev0 / ev1 (optional) are recorded on the stream right before and after the
// update kernel.
cudaError_t euler_step(const EulerBufs& b, int cur, int slot, double gamma, double cfl, uint64_t* launches,
                       cudaEvent_t ev0 = nullptr, cudaEvent_t ev1 = nullptr);

// Threads and shared memory of the update kernel for a patch shape; false
// when no tile of the patch fits in shared memory.
bool euler_supported(const Geo& g);

} // namespace amr_gb300
