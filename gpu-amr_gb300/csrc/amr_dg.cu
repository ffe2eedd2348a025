// Nodal discontinuous-Galerkin patch solver on the device tree: the
// reference's DG residual (include/dg_helpers/rhs.hpp:117-255, volume.hpp:
// 24-44, surface.hpp:36-113) for its generated configuration (order 2, 2D,
// four advected variables, velocity 1), combined into SSPRK2 stages
// (include/dg_helpers/time_integration/time.hpp:134-168).  Built with
// -fmad=false and evaluated in the reference's order and grouping, so every
// interior value is the reference's bit for bit.
//
// Per cell and variable, with U[ix][iy] the 2 x 2 nodal values:
//   volume   G = U * (w (x) w);  du = (0 + s C_x) + s C_y,  s = (1/edge) *
//            edge^2, C_x[i][j] = (0 + d[i][0] G[0][j]) + d[i][1] G[1][j],
//            C_y[i][j] = (0 + d[j][0] G[i][0]) + d[j][1] G[i][1]
//   faces    in the reference's direction order (y-, y+, x-, x+): the cell
//            and its neighbour projected onto the shared face with the face
//            kernels, the Rusanov flux (sign (f + f_n) 0.5 + (u - u_n) 0.5)
//            times the face area, the surface weights, lifted back with the
//            face kernel and subtracted
//   mass     du * (4 / edge^2)
#include <cmath>

#include "amr_dg.cuh"

namespace amr_gb300 {

DgTables dg_tables()
{
    // Gauss-Legendre points and the Lagrange values as the reference forms
    // them (gauss_legendre.hpp:16-35, lagrange.hpp:37-67)
    const double pre[2] = { -0.5773502691896257, 0.5773502691896257 };
    const double half = (1.0 - 0.0) / 2.0, mid = (0.0 + 1.0) / 2.0;
    double       p[2];
    for (int i = 0; i < 2; ++i) p[i] = mid + half * pre[i];
    auto lag = [&](int i, double x) {
        double num = 1.0, den = 1.0;
        for (int k = 0; k < 2; ++k) {
            if (k == i) continue;
            num *= (x - p[k]);
            den *= (p[i] - p[k]);
        }
        return num / den;
    };
    auto dlag = [&](int i, double x) {
        double res = 0.0;
        for (int j = 0; j < 2; ++j) {
            if (j == i) continue;
            double term = 1.0 / (p[i] - p[j]);
            for (int k = 0; k < 2; ++k) {
                if (k == i || k == j) continue;
                term *= (x - p[k]) / (p[i] - p[k]);
            }
            res += term;
        }
        return res;
    };
    DgTables t{};
    for (int i = 0; i < 2; ++i) {
        t.k[0][i] = lag(i, 0.0);
        t.k[1][i] = lag(i, 1.0);
        for (int j = 0; j < 2; ++j) t.d[i][j] = dlag(i, p[j]);
    }
    return t;
}

namespace {

__device__ __forceinline__ void dg_face_project(const double (&U)[2][2], const double (&k)[2], int adim, double (&f)[2])
{
#pragma unroll
    for (int r = 0; r < 2; ++r)
        f[r] = adim == 0 ? U[0][r] * k[0] + U[1][r] * k[1] : U[r][0] * k[0] + U[r][1] * k[1];
}

// Combination of one ghost cell (zero residual) for every field.
__device__ __forceinline__ void dg_ghost(const double* __restrict__ in, const double* un, double* out, size_t fstride,
                                         size_t at, double dt, int mode)
{
#pragma unroll 4
    for (int f = 0; f < kDgFields; ++f) {
        const size_t i   = f * fstride + at;
        const double u   = in[i];
        const double rdt = 0.0 * dt;
        out[i]           = mode == 0 ? u + rdt : ((un[i] + u) + rdt) * 0.5;
    }
}

// Sixteen threads per patch, one per interior cell (two patches per warp, so
// the FP64 residual runs on full warps), grid-stride over patches; the same
// threads combine the patch's twenty ghost cells.  The four variables one
// after another.
__global__ void __launch_bounds__(256)
k_dg_stage(const double* __restrict__ in, const double* un, double* out, const uint64_t* __restrict__ keys, int P,
           Geo g, size_t fstride, DgTables tb, double dt, int mode)
{
    constexpr int   P1    = kDgPatch + 2, FLAT = P1 * P1, CELLS = kDgPatch * kDgPatch;
    const long long total = static_cast<long long>(P) * CELLS;
    for (long long c = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; c < total;
         c += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int    p = static_cast<int>(c >> 4), k = static_cast<int>(c & 15);
        const int    li   = ((k >> 2) + 1) * P1 + (k & 3) + 1;
        const size_t base = static_cast<size_t>(p) * FLAT + li;
        const int    lev  = key_level(keys[p]);
        const double edge = (1.0 / static_cast<double>(1u << lev)) / static_cast<double>(kDgPatch);
        const double vol  = (1.0 * edge) * edge;
        const double area = 1.0 * edge;
        const double s    = (1.0 / edge) * vol;
        const double im   = 4.0 / vol; // inverse mass (1/w)(1/w) = 4 over the volume
#pragma unroll 1
        for (int v = 0; v < kDgVars; ++v) {
            double U[2][2];
#pragma unroll
            for (int ix = 0; ix < 2; ++ix)
#pragma unroll
                for (int iy = 0; iy < 2; ++iy) U[ix][iy] = in[((ix * 2 + iy) * kDgVars + v) * fstride + base];
            double G[2][2];
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int j = 0; j < 2; ++j) G[i][j] = (1.0 * U[i][j]) * 0.25; // flux v u, volume mass w (x) w
            double du[2][2];
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int j = 0; j < 2; ++j) {
                    const double cx = (0.0 + tb.d[i][0] * G[0][j]) + tb.d[i][1] * G[1][j];
                    du[i][j]        = 0.0 + s * cx;
                }
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int j = 0; j < 2; ++j) {
                    const double cy = (0.0 + tb.d[j][0] * G[i][0]) + tb.d[j][1] * G[i][1];
                    du[i][j]        = du[i][j] + s * cy;
                }
#pragma unroll
            for (int f = 0; f < 4; ++f) {
                const int pdim = f >> 1, sign = (f & 1) ? 1 : -1, sidx = (f & 1);
                const int adim = 1 - pdim;
                const int off  = (pdim == 0 ? P1 : 1) * sign;
                double    Un[2][2];
#pragma unroll
                for (int ix = 0; ix < 2; ++ix)
#pragma unroll
                    for (int iy = 0; iy < 2; ++iy)
                        Un[ix][iy] = in[((ix * 2 + iy) * kDgVars + v) * fstride + base + off];
                double uf[2], un2[2];
                dg_face_project(U, tb.k[sidx], adim, uf);       // the flux v u projects to the same values
                dg_face_project(Un, tb.k[1 - sidx], adim, un2); // (v = 1)
                double wf[2];
#pragma unroll
                for (int rr = 0; rr < 2; ++rr) {
                    const double nf = (static_cast<double>(sign) * (uf[rr] + un2[rr]) * 0.5 +
                                       (uf[rr] - un2[rr]) * (0.5 * 1.0)) *
                                      area;
                    wf[rr] = nf * 0.5; // surface weights
                }
#pragma unroll
                for (int ix = 0; ix < 2; ++ix)
#pragma unroll
                    for (int iy = 0; iy < 2; ++iy) {
                        const double face = adim == 1 ? wf[ix] * tb.k[sidx][iy] : tb.k[sidx][ix] * wf[iy];
                        du[ix][iy]        = du[ix][iy] - face;
                    }
            }
#pragma unroll
            for (int ix = 0; ix < 2; ++ix)
#pragma unroll
                for (int iy = 0; iy < 2; ++iy) {
                    const size_t at  = ((ix * 2 + iy) * kDgVars + v) * fstride + base;
                    const double u   = U[ix][iy];
                    const double rdt = (du[ix][iy] * im) * dt;
                    out[at]          = mode == 0 ? u + rdt : ((un[at] + u) + rdt) * 0.5;
                }
        }
        // ghost cells: rows 0 and P1-1 (6 each), then columns 0 and P1-1 of
        // the interior rows (4 each)
        for (int gi = k; gi < 2 * P1 + 2 * kDgPatch; gi += CELLS) {
            int gr, gc;
            if (gi < P1) gr = 0, gc = gi;
            else if (gi < 2 * P1) gr = P1 - 1, gc = gi - P1;
            else if (gi < 2 * P1 + kDgPatch) gr = gi - 2 * P1 + 1, gc = 0;
            else gr = gi - 2 * P1 - kDgPatch + 1, gc = P1 - 1;
            dg_ghost(in, un, out, fstride, static_cast<size_t>(p) * FLAT + gr * P1 + gc, dt, mode);
        }
    }
}

} // namespace

cudaError_t dg_stage(const DgStage& s)
{
    if (s.P <= 0) return cudaSuccess;
    const DgTables  tb    = dg_tables();
    if (s.g.n != kDgPatch || s.g.h != 1) return cudaErrorInvalidValue;
    const long long total = static_cast<long long>(s.P) * kDgPatch * kDgPatch;
    const unsigned  grid  = static_cast<unsigned>(std::min<long long>((total + 255) / 256, 152LL * 16));
    k_dg_stage<<<grid, 256, 0, s.stream>>>(s.in, s.un, s.out, s.keys, s.P, s.g, s.fstride, tb, s.dt, s.mode);
    return cudaGetLastError();
}

} // namespace amr_gb300
