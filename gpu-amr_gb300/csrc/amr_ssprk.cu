// Strong-stability-preserving Runge-Kutta steps (SSPRK2, SSPRK3) of the FV
// advection operator on the device tree: the reference's integrators
// (include/dg_helpers/time_integration/time.hpp:83-272, driven per patch with
// a halo exchange before every stage as include/dg_helpers/solver.hpp:162-244
// does) applied to the residual
//     R = -sum_d (F_R - F_L) / dx_d
// with the Rusanov flux of AdvectionPhysics (include/solver/
// AdvectionPhysics.hpp:45-66).  Built with -fmad=false: every operation
// rounds as in the reference's C++, so states are bit-identical to it.
//
// One stage is one launch over every cell of every padded patch (the
// reference combines whole patch containers): interior cells take the
// residual of the halo-exchanged input, ghost cells a zero residual.  2D
// patches of 8x8 or 16x16 cells with one ghost layer evaluate each face flux
// once (k_ssprk_stage2d), other shapes per cell (k_ssprk_stage).
//     stage 0          u* = u + R dt
//     SSPRK2 stage 1   u' = ((u^n + u*) + R dt) * 0.5
//     SSPRK3 stage 1   u2 = u^n * 0.75 + (u1 + R dt) * 0.25
//     SSPRK3 stage 2   u' = u^n * (1/3) + (u2 + R dt) * (2/3)
#include <cmath>

#include "amr_ssprk.cuh"

namespace amr_gb300 {
namespace {

// x / dx for a cell size of level `lev`: dx = dx_root / 2^lev exactly (a
// power-of-two scaling).  When dx_root is itself a power of two, dx is one
// and x * (1 / dx) equals x / dx bit for bit (the reciprocal is exact), so
// the division becomes a multiplication; otherwise the division stays.
struct InvDx {
    double dx, inv;
    bool   pow2;
};

__device__ __forceinline__ double div_dx(double x, const InvDx& c) { return c.pow2 ? x * c.inv : x / c.dx; }

// One block per patch (grid-stride over patches), threads over the padded
// cells of the patch.
template <int R>
__global__ void __launch_bounds__(256)
k_ssprk_stage(const double* __restrict__ in, const double* __restrict__ un, double* __restrict__ out,
              const uint64_t* __restrict__ keys, int P, Geo g, const double* __restrict__ vel,
              const double* __restrict__ step_dt, int mode, unsigned pow2_mask)
{
    for (int p = blockIdx.x; p < P; p += gridDim.x) {
        const uint64_t key  = keys[p];
        const int      inst = g.inst_shift >= 64 ? 0 : static_cast<int>(key >> g.inst_shift);
        const int      lev  = key_level(key);
        const double   dt   = step_dt[inst];
        InvDx          cdx[R];
        double         v[R];
#pragma unroll
        for (int d = 0; d < R; ++d) {
            cdx[d].dx   = cell_size(g, d, lev);
            cdx[d].pow2 = (pow2_mask >> d) & 1u;
            cdx[d].inv  = 1.0 / cdx[d].dx;
            v[d]        = vel[3 * inst + d];
        }
        const size_t  pb = static_cast<size_t>(p) * g.flat;
        const double* a  = in + pb;
        for (int li = threadIdx.x; li < g.flat; li += blockDim.x) {
            int r = li, interior = 1;
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
                    const double uL = a[li - st];
                    const double uR = a[li + st];
                    const double sp = fabs(v[d]);
                    const double fL = 0.5 * (uL * v[d] + uc * v[d]) - 0.5 * sp * (uc - uL);
                    const double fR = 0.5 * (uc * v[d] + uR * v[d]) - 0.5 * sp * (uR - uc);
                    Rs -= div_dx(fR - fL, cdx[d]);
                }
            }
            const double Rdt = Rs * dt;
            const double b   = un[pb + li];
            double       res;
            if (!(dt > 0.0)) res = mode == 0 ? uc : b; // a step past the time limit leaves the state as it is
            else if (mode == 0) res = uc + Rdt;
            else if (mode == 2) res = (b + uc + Rdt) * 0.5;
            else if (mode == 31) res = b * 0.75 + (uc + Rdt) * 0.25;
            else res = b * (1.0 / 3.0) + (uc + Rdt) * (2.0 / 3.0);
            out[pb + li] = res;
        }
    }
}

// 2D patches of N x N cells and one ghost layer: the same stage with each
// face flux evaluated once.  A face flux depends only on its two cells and
// the reference evaluates it the same way from either side (f(a, b) =
// 0.5 (a v + b v) - (0.5 |v|) (b - a) with a the cell on the minus side), so
// sharing it between the two cells changes no rounding.  One block per patch:
// the padded patch and the fluxes of its (N + 1) N faces per axis in shared
// memory, then every padded cell as above.
template <int N>
__global__ void __launch_bounds__(256)
k_ssprk_stage2d(const double* __restrict__ in, const double* __restrict__ un, double* __restrict__ out,
                const uint64_t* __restrict__ keys, int P, Geo g, const double* __restrict__ vel,
                const double* __restrict__ step_dt, int mode, unsigned pow2_mask)
{
    constexpr int P1 = N + 2, FLAT = P1 * P1;
    __shared__ double tile[FLAT];
    __shared__ double fx[N][N + 1]; // x faces of interior row r: face j between padded columns j and j + 1
    __shared__ double fy[N + 1][N]; // y faces of interior column c: face i between padded rows i and i + 1
    for (int p = blockIdx.x; p < P; p += gridDim.x) {
        const uint64_t key  = keys[p];
        const int      inst = g.inst_shift >= 64 ? 0 : static_cast<int>(key >> g.inst_shift);
        const int      lev  = key_level(key);
        const double   dt   = step_dt[inst];
        InvDx          cdx[2];
        double         v[2], hsp[2];
#pragma unroll
        for (int d = 0; d < 2; ++d) {
            cdx[d].dx   = cell_size(g, d, lev);
            cdx[d].pow2 = (pow2_mask >> d) & 1u;
            cdx[d].inv  = 1.0 / cdx[d].dx;
            v[d]        = vel[3 * inst + d];
            hsp[d]      = 0.5 * fabs(v[d]); // the reference's 0.5 * sp * (...), left to right
        }
        const size_t  pb = static_cast<size_t>(p) * FLAT;
        const double* a  = in + pb;
        for (int li = threadIdx.x; li < FLAT; li += blockDim.x) tile[li] = a[li];
        __syncthreads();
        for (int k = threadIdx.x; k < N * (N + 1); k += blockDim.x) {
            {
                const int    r = k / (N + 1), j = k % (N + 1);
                const double uL = tile[(r + 1) * P1 + j], uR = tile[(r + 1) * P1 + j + 1];
                fx[r][j] = 0.5 * (uL * v[0] + uR * v[0]) - hsp[0] * (uR - uL);
            }
            {
                const int    i = k / N, c = k % N;
                const double uL = tile[i * P1 + c + 1], uR = tile[(i + 1) * P1 + c + 1];
                fy[i][c] = 0.5 * (uL * v[1] + uR * v[1]) - hsp[1] * (uR - uL);
            }
        }
        __syncthreads();
        for (int li = threadIdx.x; li < FLAT; li += blockDim.x) {
            const int    r = li / P1, c = li % P1;
            const double uc = tile[li];
            double       Rs = 0.0;
            if (r >= 1 && r <= N && c >= 1 && c <= N) {
                Rs -= div_dx(fx[r - 1][c] - fx[r - 1][c - 1], cdx[0]);
                Rs -= div_dx(fy[r][c - 1] - fy[r - 1][c - 1], cdx[1]);
            }
            const double Rdt = Rs * dt;
            const double b   = un[pb + li];
            double       res;
            if (!(dt > 0.0)) res = mode == 0 ? uc : b;
            else if (mode == 0) res = uc + Rdt;
            else if (mode == 2) res = (b + uc + Rdt) * 0.5;
            else if (mode == 31) res = b * 0.75 + (uc + Rdt) * 0.25;
            else res = b * (1.0 / 3.0) + (uc + Rdt) * (2.0 / 3.0);
            out[pb + li] = res;
        }
        __syncthreads(); // the tile and fluxes are refilled for the next patch
    }
}

} // namespace

cudaError_t ssprk_stage(const SsprkStage& s)
{
    if (s.P <= 0) return cudaSuccess;
    // axes whose root cell size is a power of two
    unsigned mask = 0;
    for (int d = 0; d < s.g.rank; ++d) {
        int e = 0;
        if (std::frexp(s.g.dx_root[d], &e) == 0.5) mask |= 1u << d;
    }
    const unsigned grid    = static_cast<unsigned>(std::min(s.P, 152 * 32));
    const int      threads = s.g.flat >= 256 ? 256 : ((s.g.flat + 31) / 32) * 32;
    if (s.g.rank == 2 && s.g.h == 1 && s.g.n == 16)
        k_ssprk_stage2d<16><<<grid, 256, 0, s.stream>>>(s.in, s.un, s.out, s.keys, s.P, s.g, s.vel, s.step_dt,
                                                         s.mode, mask);
    else if (s.g.rank == 2 && s.g.h == 1 && s.g.n == 8)
        k_ssprk_stage2d<8><<<grid, 128, 0, s.stream>>>(s.in, s.un, s.out, s.keys, s.P, s.g, s.vel, s.step_dt,
                                                       s.mode, mask);
    else if (s.g.rank == 2)
        k_ssprk_stage<2><<<grid, threads, 0, s.stream>>>(s.in, s.un, s.out, s.keys, s.P, s.g, s.vel, s.step_dt,
                                                         s.mode, mask);
    else
        k_ssprk_stage<3><<<grid, threads, 0, s.stream>>>(s.in, s.un, s.out, s.keys, s.P, s.g, s.vel, s.step_dt,
                                                         s.mode, mask);
    return cudaGetLastError();
}

} // namespace amr_gb300
