// Strong-stability-preserving Runge-Kutta steps (SSPRK2, SSPRK3) of the FV
// advection operator on the device tree: the reference's integrators
// (include/dg_helpers/time_integration/time.hpp:83-272, driven per patch with
// a halo exchange before every stage as include/dg_helpers/solver.hpp:159-232
// does) applied to the residual
//     R = -sum_d (F_R - F_L) / dx_d
// with the Rusanov flux of AdvectionPhysics (include/solver/
// AdvectionPhysics.hpp:45-66).  Built with -fmad=false: every operation
// rounds as in the reference's C++, so states are bit-identical to it.
//
// One stage is one launch over every cell of every padded patch (the
// reference combines whole patch containers): interior cells take the
// residual of the halo-exchanged input, ghost cells a zero residual.
//     stage 0          u* = u + R dt
//     SSPRK2 stage 1   u' = ((u^n + u*) + R dt) * 0.5
//     SSPRK3 stage 1   u2 = u^n * 0.75 + (u1 + R dt) * 0.25
//     SSPRK3 stage 2   u' = u^n * (1/3) + (u2 + R dt) * (2/3)
#include "amr_ssprk.cuh"

namespace amr_gb300 {
namespace {

template <int R>
__global__ void __launch_bounds__(256)
k_ssprk_stage(const double* __restrict__ in, const double* __restrict__ un, double* __restrict__ out,
              const uint64_t* __restrict__ keys, long long total, Geo g, const double* __restrict__ vel,
              const double* __restrict__ step_dt, int mode)
{
    for (long long t = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; t < total;
         t += static_cast<long long>(gridDim.x) * blockDim.x) {
        const long long p  = t / g.flat;
        const int       li = static_cast<int>(t - p * g.flat);
        const uint64_t  key  = keys[p];
        const int       inst = g.inst_shift >= 64 ? 0 : static_cast<int>(key >> g.inst_shift);
        const int       lev  = key_level(key);
        const double    dt   = step_dt[inst];
        const double*   a    = in + p * g.flat;
        int             r = li, interior = 1;
#pragma unroll
        for (int L = R - 1; L >= 0; --L) {
            const int c = r % g.P1;
            r /= g.P1;
            if (c < g.h || c >= g.n + g.h) interior = 0;
        }
        const double uc = a[li];
        double       Rs = 0.0;
        if (interior) {
#pragma unroll
            for (int d = 0; d < R; ++d) {
                const int    st = g.s[R - 1 - d]; // Morton axis d
                const double v  = vel[3 * inst + d];
                const double uL = a[li - st];
                const double uR = a[li + st];
                const double sp = fabs(v);
                const double fL = 0.5 * (uL * v + uc * v) - 0.5 * sp * (uc - uL);
                const double fR = 0.5 * (uc * v + uR * v) - 0.5 * sp * (uR - uc);
                Rs -= (fR - fL) / cell_size(g, d, lev);
            }
        }
        const double Rdt = Rs * dt;
        const double b   = un[p * g.flat + li];
        double       res;
        if (!(dt > 0.0)) res = mode == 0 ? uc : b; // a step past the time limit leaves the state as it is
        else if (mode == 0) res = uc + Rdt;
        else if (mode == 2) res = (b + uc + Rdt) * 0.5;
        else if (mode == 31) res = b * 0.75 + (uc + Rdt) * 0.25;
        else res = b * (1.0 / 3.0) + (uc + Rdt) * (2.0 / 3.0);
        out[p * g.flat + li] = res;
    }
}

} // namespace

cudaError_t ssprk_stage(const SsprkStage& s)
{
    const long long total = static_cast<long long>(s.P) * s.g.flat;
    if (total <= 0) return cudaSuccess;
    const unsigned grid = static_cast<unsigned>(std::min<long long>((total + 255) / 256, 152LL * 64));
    if (s.g.rank == 2)
        k_ssprk_stage<2><<<grid, 256, 0, s.stream>>>(s.in, s.un, s.out, s.keys, total, s.g, s.vel, s.step_dt, s.mode);
    else
        k_ssprk_stage<3><<<grid, 256, 0, s.stream>>>(s.in, s.un, s.out, s.keys, total, s.g, s.vel, s.step_dt, s.mode);
    return cudaGetLastError();
}

} // namespace amr_gb300
