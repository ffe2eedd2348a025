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
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <string>

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
__global__ void __launch_bounds__(64)
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

// ------------------------------------------------ DG Euler
constexpr double kDgGamma = 1.4;

// compute_pressure and compute_velocity (euler.hpp:69-113) of one node;
// max_eigenvalue (euler.hpp:165-181) is |m_n / rho| + sqrt(gamma p / rho)
// at a cell's first node
__device__ __forceinline__ void dg_euler_node(double mx, double my, double rho, double E, double& p, double& u,
                                              double& v)
{
    double kin = 0.0;
    kin += 0.5 * mx * mx / rho;
    kin += 0.5 * my * my / rho;
    p = (kDgGamma - 1.0) * (E - kin);
    u = mx / rho;
    v = my / rho;
}

__device__ __forceinline__ double dg_max(double a, double b) { return a < b ? b : a; } // std::max(a, b)

// p, u, v per node, then the cell's eigenvalues in x and y (max_eigenvalue
// from the first node: |m_d / rho| is that node's velocity component, the
// same division), of every padded cell the stage reads: the interior and
// the face ghosts (the four corner ghosts are never read and are skipped)
__global__ void __launch_bounds__(256)
k_dg_euler_prims(const double* __restrict__ in, double* __restrict__ prims, long long total, size_t fstride)
{
    constexpr int P1 = kDgPatch + 2, FLAT = P1 * P1;
    for (long long c = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; c < total;
         c += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int li = static_cast<int>(c % FLAT);
        if (li == 0 || li == P1 - 1 || li == FLAT - P1 || li == FLAT - 1) continue;
        double p0 = 0.0, u0 = 0.0, v0 = 0.0, rho0 = 1.0;
#pragma unroll
        for (int node = 0; node < 4; ++node) {
            const double* U = in + node * kDgVars * fstride + c;
            double        p, u, v;
            const double  rho = U[2 * fstride];
            dg_euler_node(U[0], U[fstride], rho, U[3 * fstride], p, u, v);
            prims[(node * 3 + 0) * fstride + c] = p;
            prims[(node * 3 + 1) * fstride + c] = u;
            prims[(node * 3 + 2) * fstride + c] = v;
            if (node == 0) p0 = p, u0 = u, v0 = v, rho0 = rho;
        }
        const double a = sqrt(kDgGamma * p0 / rho0);
        prims[12 * fstride + c] = fabs(u0) + a;
        prims[13 * fstride + c] = fabs(v0) + a;
    }
}

// flux component adim (0: x, 1: y) of variable var at one node (evaluate_flux,
// euler.hpp:120-160): rho u_i u_d (+ p if i = d), rho u_d, (E + p) u_d
__device__ __forceinline__ double dg_euler_flux(const double* U, const double* pr, size_t fstride, int node, int var,
                                                int adim)
{
    const double ud = pr[(node * 3 + 1 + adim) * fstride];
    const double q  = U[(node * kDgVars + var) * fstride];
    if (var < 2) {
        const double f = q * ud;
        return var == adim ? f + pr[(node * 3) * fstride] : f;
    }
    if (var == 2) return q * ud;
    return (q + pr[(node * 3) * fstride]) * ud;
}

// Sixteen threads per patch as k_dg_stage; the face speeds are formed first
// and the patch's running maximum is a prefix maximum over its 16 cells
// (the reference visits the cells row-major and each cell's faces in order).
__global__ void __launch_bounds__(64)
k_dg_euler_stage(const double* __restrict__ in, const double* un, double* out, const double* __restrict__ prims,
                 const uint64_t* __restrict__ keys, int P, Geo g, size_t fstride, DgTables tb,
                 const double* __restrict__ dtp, unsigned long long* dt_min, int mode)
{
    constexpr int   P1    = kDgPatch + 2, FLAT = P1 * P1, CELLS = kDgPatch * kDgPatch;
    const long long total = static_cast<long long>(P) * CELLS;
    const double    dt    = dtp[0];
    const int       lane  = threadIdx.x & 31;
    for (long long c = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; c - lane < total;
         c += static_cast<long long>(gridDim.x) * blockDim.x) {
        const bool   valid = c < total;
        const int    p = valid ? static_cast<int>(c >> 4) : 0, k = static_cast<int>(c & 15);
        const int    li   = ((k >> 2) + 1) * P1 + (k & 3) + 1;
        const size_t base = static_cast<size_t>(p) * FLAT + li;
        const int    lev  = key_level(keys[p]);
        const double edge = (1.0 / static_cast<double>(1u << lev)) / static_cast<double>(kDgPatch);
        const double vol  = (1.0 * edge) * edge;
        const double area = 1.0 * edge;
        const double s    = (1.0 / edge) * vol;
        const double im   = 4.0 / vol;
        const double* U   = in + base;
        const double* pr  = prims + base;
        // face speeds: max(eig(cell), eig(neighbour)) per face, the cell's
        // running maximum over its faces, then the prefix over the patch
        double lam[4];
        {
            const double eig_cell[2] = { pr[12 * fstride], pr[13 * fstride] };
            double       run         = -INFINITY;
#pragma unroll
            for (int f = 0; f < 4; ++f) {
                const int    pdim = f >> 1, sign = (f & 1) ? 1 : -1, adim = 1 - pdim;
                const int    off  = (pdim == 0 ? P1 : 1) * sign;
                const double en   = pr[(12 + adim) * fstride + off];
                run               = dg_max(run, dg_max(eig_cell[adim], en));
                lam[f]             = run;
            }
            if (!valid) run = -INFINITY;
            // exclusive prefix maximum of the cells' maxima over the 16 lanes
            // of this patch (lanes 0-15 or 16-31 of the warp)
            double x = run;
#pragma unroll
            for (int o = 1; o < 16; o <<= 1) {
                const double y = __shfl_up_sync(0xffffffffu, x, o, 16);
                if ((lane & 15) >= o) x = dg_max(y, x);
            }
            double before = __shfl_up_sync(0xffffffffu, x, 1, 16);
            if ((lane & 15) == 0) before = -INFINITY;
#pragma unroll
            for (int f = 0; f < 4; ++f) lam[f] = dg_max(before, lam[f]);
        }
        if (valid) {
#pragma unroll 1
            for (int v = 0; v < kDgVars; ++v) {
                double Uv[2][2], du[2][2];
#pragma unroll
                for (int ix = 0; ix < 2; ++ix)
#pragma unroll
                    for (int iy = 0; iy < 2; ++iy) Uv[ix][iy] = U[((ix * 2 + iy) * kDgVars + v) * fstride];
                // volume: d/dx of F_x and d/dy of F_y against the mass
                {
                    double G[2][2];
#pragma unroll
                    for (int i = 0; i < 2; ++i)
#pragma unroll
                        for (int j = 0; j < 2; ++j) G[i][j] = dg_euler_flux(U, pr, fstride, i * 2 + j, v, 0) * 0.25;
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
                        for (int j = 0; j < 2; ++j) G[i][j] = dg_euler_flux(U, pr, fstride, i * 2 + j, v, 1) * 0.25;
#pragma unroll
                    for (int i = 0; i < 2; ++i)
#pragma unroll
                        for (int j = 0; j < 2; ++j) {
                            const double cy = (0.0 + tb.d[j][0] * G[i][0]) + tb.d[j][1] * G[i][1];
                            du[i][j]        = du[i][j] + s * cy;
                        }
                }
#pragma unroll
                for (int f = 0; f < 4; ++f) {
                    const int     pdim = f >> 1, sign = (f & 1) ? 1 : -1, sidx = (f & 1);
                    const int     adim = 1 - pdim;
                    const int     off  = (pdim == 0 ? P1 : 1) * sign;
                    const double* Un   = U + off;
                    const double* prn  = pr + off;
                    double        Vn[2][2], Fc[2][2], Fn[2][2];
#pragma unroll
                    for (int ix = 0; ix < 2; ++ix)
#pragma unroll
                        for (int iy = 0; iy < 2; ++iy) {
                            Vn[ix][iy] = Un[((ix * 2 + iy) * kDgVars + v) * fstride];
                            Fc[ix][iy] = dg_euler_flux(U, pr, fstride, ix * 2 + iy, v, adim);
                            Fn[ix][iy] = dg_euler_flux(Un, prn, fstride, ix * 2 + iy, v, adim);
                        }
                    double uf[2], ff[2], un2[2], fn2[2];
                    dg_face_project(Uv, tb.k[sidx], adim, uf);
                    dg_face_project(Fc, tb.k[sidx], adim, ff);
                    dg_face_project(Vn, tb.k[1 - sidx], adim, un2);
                    dg_face_project(Fn, tb.k[1 - sidx], adim, fn2);
                    double wf[2];
#pragma unroll
                    for (int rr = 0; rr < 2; ++rr) {
                        const double nf = (static_cast<double>(sign) * (ff[rr] + fn2[rr]) * 0.5 +
                                           (uf[rr] - un2[rr]) * (0.5 * lam[f])) *
                                          area;
                        wf[rr] = nf * 0.5;
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
                        const double u   = Uv[ix][iy];
                        const double rdt = (du[ix][iy] * im) * dt;
                        out[at]          = mode == 0 ? u + rdt : ((un[at] + u) + rdt) * 0.5;
                    }
            }
            // the patch's final speed (last cell, last face) sets its CFL step
            if (mode == 1 && k == 15 && lam[3] > 0.0) {
                const double scale = 1.0 / (4.0 + 1.0); // 1 / (order^dim + 1)
                const double h     = scale * 0.5 * edge / lam[3];
                atomicMin(dt_min, static_cast<unsigned long long>(__double_as_longlong(h)));
            }
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
}

__global__ void k_dg_euler_next(double* dt, double* time, unsigned long long* dt_min)
{
    const double h    = dt[0];
    const double m    = __longlong_as_double(static_cast<long long>(*dt_min));
    const double dmin = m < h ? m : h;    // dt_min starts at dt (solver.hpp:127)
    const double next = dmin < h ? dmin : h; // dt = std::min(dt, dt_min)
    dt[0]             = next;
    time[0] += next;                        // time += dt, the updated step (solver.hpp:129, 134)
    *dt_min = 0x7ff0000000000000ull;        // +inf
}

// ------------------------------------------------ DG prolongation / restriction
// The tree's DefaultAMRPolicy (include/dg_helpers/tree_builder.hpp:59-289)
// for the DG tensor: a fine cell's nodal values are the coarse cell's
// polynomial at the fine nodes (interpolation), a coarse cell's nodal values
// the polynomial of the fine cell holding each node (restriction).  Child
// offsets number the fine cells of a coarse cell with bit 0 = x half, bit 1 =
// y half.  Lagrange values and the basis sum follow Lagrange::evaluate
// (lagrange.hpp:37-50) and Basis::evaluate_basis (polynomial.hpp:36-57).
__device__ __forceinline__ double dg_lag(const double (&p)[2], int i, double x)
{
    double num = 1.0, den = 1.0;
    num *= (x - p[1 - i]);
    den *= (p[i] - p[1 - i]);
    return num / den;
}

// polynomial with nodal values C[ix][iy] at reference point (x0, x1)
__device__ __forceinline__ double dg_eval(const double (&C)[2][2], const double (&p)[2], double x0, double x1)
{
    const double lx[2] = { dg_lag(p, 0, x0), dg_lag(p, 1, x0) };
    const double ly[2] = { dg_lag(p, 0, x1), dg_lag(p, 1, x1) };
    double       sum   = 0.0;
#pragma unroll
    for (int i0 = 0; i0 < 2; ++i0)
#pragma unroll
        for (int i1 = 0; i1 < 2; ++i1) {
            double prod = 1.0;
            prod *= lx[i0];
            prod *= ly[i1];
            sum = sum + C[i0][i1] * prod;
        }
    return sum;
}

// fine cell `co` of coarse cell (field base pointers fields apart): all 16
// nodal values into dst (fields apart)
__device__ __forceinline__ void dg_interp(const double* src, double* dst, size_t fstride, int co,
                                          const double (&p)[2])
{
    const double o0 = (co & 1) ? 0.5 : 0.0, o1 = (co & 2) ? 0.5 : 0.0;
#pragma unroll 1
    for (int v = 0; v < kDgVars; ++v) {
        double C[2][2];
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int b = 0; b < 2; ++b) C[a][b] = src[((a * 2 + b) * kDgVars + v) * fstride];
#pragma unroll
        for (int ix = 0; ix < 2; ++ix)
#pragma unroll
            for (int iy = 0; iy < 2; ++iy)
                dst[((ix * 2 + iy) * kDgVars + v) * fstride] = dg_eval(C, p, 0.5 * p[ix] + o0, 0.5 * p[iy] + o1);
    }
}

// coarse cell from its four fine cells (child offset order), all 16 values
__device__ __forceinline__ void dg_restrict(const double* const (&child)[4], double* dst, size_t fstride,
                                            const double (&p)[2])
{
#pragma unroll 1
    for (int v = 0; v < kDgVars; ++v)
#pragma unroll
        for (int ix = 0; ix < 2; ++ix)
#pragma unroll
            for (int iy = 0; iy < 2; ++iy) {
                const double pp0 = p[ix], pp1 = p[iy];
                const int    co  = (pp0 >= 0.5 ? 1 : 0) | (pp1 >= 0.5 ? 2 : 0);
                const double o0 = (co & 1) ? 0.5 : 0.0, o1 = (co & 2) ? 0.5 : 0.0;
                const double c0 = 2.0 * pp0 - (o0 > 0.0 ? 1.0 : 0.0);
                const double c1 = 2.0 * pp1 - (o1 > 0.0 ? 1.0 : 0.0);
                double       C[2][2];
#pragma unroll
                for (int a = 0; a < 2; ++a)
#pragma unroll
                    for (int b = 0; b < 2; ++b) C[a][b] = child[co][((a * 2 + b) * kDgVars + v) * fstride];
                dst[((ix * 2 + iy) * kDgVars + v) * fstride] = dg_eval(C, p, c0, c1);
            }
}

// Halo of a DG tree: same-level faces copy, a ghost facing finer leaves is
// the restriction of the 2 x 2 fine cells behind the face (patch_utils.hpp:
// 334-386), a ghost facing a coarser leaf the interpolation of the coarse
// cell at the ghost's position (patch_utils.hpp:388-441).  One thread per
// ghost cell of a face, all 16 fields.
__global__ void __launch_bounds__(256)
k_dg_halo(double* buf, const amr_halo_meta* __restrict__ meta, long long total, Geo g, size_t fstride, double p0,
          double p1)
{
    const double p[2] = { p0, p1 };
    const int    n = g.n, h = g.h, half = n / 2;
    for (long long t = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; t < total;
         t += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int  pidx = static_cast<int>(t / (4 * n));
        const int  r    = static_cast<int>(t % (4 * n));
        const int  d = r / n, f = r % n;
        const int  L = d / 2, pos = d % 2;
        int        G0 = L == 0 ? (pos ? n + h : h - 1) : f + h;
        int        G1 = L == 1 ? (pos ? n + h : h - 1) : f + h;
        const amr_halo_meta m = meta[static_cast<size_t>(pidx) * 4 + d];
        if (m.relation == REL_NONE) continue;
        double*    dst = buf + static_cast<size_t>(pidx) * g.flat + G0 * g.s[0] + G1;
        const int  sh  = pos ? -n : n;
        int        f0 = G0 + (L == 0 ? sh : 0), f1 = G1 + (L == 1 ? sh : 0);
        if (m.relation == REL_SAME) {
            const double* src = buf + static_cast<size_t>(m.neighbor) * g.flat + f0 * g.s[0] + f1;
#pragma unroll 4
            for (int k = 0; k < kDgFields; ++k) dst[k * fstride] = src[k * fstride];
        } else if (m.relation == REL_COARSER) {
            const int cy = L == 0 ? (pos ? 0 : 1) : (G0 - h) % 2;
            const int cx = L == 1 ? (pos ? 0 : 1) : (G1 - h) % 2;
            f0           = h + m.quadrant[0] * half + (f0 - h) / 2;
            f1           = h + m.quadrant[1] * half + (f1 - h) / 2;
            dg_interp(buf + static_cast<size_t>(m.neighbor) * g.flat + f0 * g.s[0] + f1, dst, fstride, cy * 2 + cx,
                      p);
        } else if (m.relation == REL_FINER) {
            f0            = ((f0 - h) * 2) % n + h;
            f1            = ((f1 - h) * 2) % n + h;
            const int fpi = L == 0 ? (G1 - h) / half : (G0 - h) / half;
            const int id  = fpi == 0 ? m.finer_ids[0] : m.finer_ids[1];
            const double* fp = buf + static_cast<size_t>(id) * g.flat + f0 * g.s[0] + f1;
            const double* const ch[4] = { fp, fp + 1, fp + g.s[0], fp + g.s[0] + 1 };
            dg_restrict(ch, dst, fstride, p);
        }
    }
}

// Re-mesh of a DG state: one block per new leaf; kept leaves move whole,
// refined children interpolate their parent's cells, coarsened parents
// restrict their children's cells (ndtree.hpp:1499-1555 with the policy).
__global__ void __launch_bounds__(64)
k_dg_remap(const double* __restrict__ old_state, double* __restrict__ new_state, const int32_t* __restrict__ src,
           const int8_t* __restrict__ skind, int P, Geo g, size_t fstride, double p0, double p1)
{
    const double p[2] = { p0, p1 };
    const int    j    = blockIdx.x;
    if (j >= P) return;
    const int kind = skind[j];
    const int n = g.n, h = g.h, half = n / 2;
    if (kind == 0) {
        for (int e = threadIdx.x; e < kDgFields * g.flat; e += blockDim.x) {
            const int k = e / g.flat, li = e % g.flat;
            new_state[k * fstride + static_cast<size_t>(j) * g.flat + li] =
                old_state[k * fstride + static_cast<size_t>(src[j]) * g.flat + li];
        }
        return;
    }
    for (int c = threadIdx.x; c < n * n; c += blockDim.x) {
        const int y = c / n + h, x = c % n + h; // padded coordinates
        double*   dst = new_state + static_cast<size_t>(j) * g.flat + y * g.s[0] + x;
        if (kind > 0) {
            const int off = kind - 1;
            const int py  = h + child_coord(g, off, 0) * half + (y - h) / 2;
            const int px  = h + child_coord(g, off, 1) * half + (x - h) / 2;
            const int co  = ((y - h) % 2) * 2 + (x - h) % 2;
            dg_interp(old_state + static_cast<size_t>(src[j]) * g.flat + py * g.s[0] + px, dst, fstride, co, p);
        } else {
            const int child = ((y - h) / half) * 2 + (x - h) / half;
            const int by = ((y - h) % half) * 2 + h, bx = ((x - h) % half) * 2 + h;
            const double* fp = old_state + static_cast<size_t>(src[j] + child) * g.flat + by * g.s[0] + bx;
            const double* const ch[4] = { fp, fp + 1, fp + g.s[0], fp + g.s[0] + 1 };
            dg_restrict(ch, dst, fstride, p);
        }
    }
}

// Re-mesh decisions of GradientAMRIndicator::compute_patch_decisions
// (include/dg_helpers/globals/amr_indicators.hpp:86-225): per interior cell
// the largest nodal range of the variables 0..dim-1 over |mean of variable
// dim| + 1e-10; refine if some cell exceeds rthr, coarsen if every cell is
// below cthr.  Sixteen threads per patch.
__global__ void __launch_bounds__(256)
k_dg_flags(const double* __restrict__ in, int P, Geo g, size_t fstride, double rthr, double cthr,
           int8_t* __restrict__ flags)
{
    const int       n = g.n, h = g.h;
    const long long total = static_cast<long long>(P) * 16;
    const int       lane  = threadIdx.x & 31;
    // whole warps iterate together (two patches per warp); lanes past the
    // last patch take part in the votes without a cell
    for (long long c = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; c - lane < total;
         c += static_cast<long long>(gridDim.x) * blockDim.x) {
        const bool valid = c < total;
        const int  p = static_cast<int>(c >> 4), k = static_cast<int>(c & 15);
        double     ind = 0.0;
        if (valid) {
            const size_t base    = static_cast<size_t>(p) * g.flat + (k / n + h) * g.s[0] + (k % n + h);
            double       vmin[2] = { 1.7976931348623157e308, 1.7976931348623157e308 };
            double       vmax[2] = { -1.7976931348623157e308, -1.7976931348623157e308 };
            double       rho_sum = 0.0;
#pragma unroll
            for (int node = 0; node < 4; ++node) {
#pragma unroll
                for (int d = 0; d < 2; ++d) {
                    const double val = in[(node * kDgVars + d) * fstride + base];
                    vmin[d]          = val < vmin[d] ? val : vmin[d]; // std::min(vmin, val)
                    vmax[d]          = vmax[d] < val ? val : vmax[d]; // std::max(vmax, val)
                }
                rho_sum += in[(node * kDgVars + 2) * fstride + base];
            }
            const double mean_rho = rho_sum / 4.0;
            const double inv_rho  = 1.0 / (fabs(mean_rho) + 1.0e-10);
#pragma unroll
            for (int d = 0; d < 2; ++d) {
                const double r = (vmax[d] - vmin[d]) * inv_rho;
                ind            = ind < r ? r : ind; // std::max(indicator, r)
            }
        }
        const unsigned grp = 0xffffu << (lane & 16);
        const unsigned up  = __ballot_sync(0xffffffffu, valid && ind > rthr);
        const unsigned lo  = __ballot_sync(0xffffffffu, !valid || !(ind >= cthr));
        if (valid && k == 0) flags[p] = (up & grp) ? FLAG_REFINE : ((lo & grp) == grp ? FLAG_COARSEN : FLAG_STABLE);
    }
}

} // namespace

cudaError_t dg_halo(double* buf, const amr_halo_meta* meta, int P, const Geo& g, size_t fstride, cudaStream_t s)
{
    if (P <= 0) return cudaSuccess;
    const double    p0 = 0.5 + 0.5 * -0.5773502691896257, p1 = 0.5 + 0.5 * 0.5773502691896257;
    const long long total = static_cast<long long>(P) * 4 * g.n;
    const unsigned  grid  = static_cast<unsigned>(std::min<long long>((total + 255) / 256, 152LL * 16));
    k_dg_halo<<<grid, 256, 0, s>>>(buf, meta, total, g, fstride, p0, p1);
    return cudaGetLastError();
}

cudaError_t dg_remap(const double* old_state, double* new_state, const int32_t* src, const int8_t* skind, int P,
                     const Geo& g, size_t fstride, cudaStream_t s)
{
    if (P <= 0) return cudaSuccess;
    const double p0 = 0.5 + 0.5 * -0.5773502691896257, p1 = 0.5 + 0.5 * 0.5773502691896257;
    k_dg_remap<<<P, 64, 0, s>>>(old_state, new_state, src, skind, P, g, fstride, p0, p1);
    return cudaGetLastError();
}

cudaError_t dg_flags(const double* in, int P, const Geo& g, size_t fstride, double rthr, double cthr, int8_t* flags,
                     cudaStream_t s)
{
    if (P <= 0) return cudaSuccess;
    const long long total = static_cast<long long>(P) * 16;
    const unsigned  grid  = static_cast<unsigned>(std::min<long long>((total + 255) / 256, 152LL * 16));
    k_dg_flags<<<grid, 256, 0, s>>>(in, P, g, fstride, rthr, cthr, flags);
    return cudaGetLastError();
}

cudaError_t dg_euler_prims(const double* in, double* prims, int P, const Geo& g, size_t fstride, cudaStream_t s)
{
    if (P <= 0) return cudaSuccess;
    const long long total = static_cast<long long>(P) * g.flat;
    const unsigned  grid  = static_cast<unsigned>(std::min<long long>((total + 255) / 256, 152LL * 16));
    k_dg_euler_prims<<<grid, 256, 0, s>>>(in, prims, total, fstride);
    return cudaGetLastError();
}

cudaError_t dg_euler_stage(const DgEulerStage& s)
{
    if (s.P <= 0) return cudaSuccess;
    if (s.g.n != kDgPatch || s.g.h != 1) return cudaErrorInvalidValue;
    const DgTables  tb    = dg_tables();
    const long long total = static_cast<long long>(s.P) * kDgPatch * kDgPatch;
    const unsigned  grid  = static_cast<unsigned>(std::min<long long>((total + 63) / 64, 152LL * 32));
    k_dg_euler_stage<<<grid, 64, 0, s.stream>>>(s.in, s.un, s.out, s.prims, s.keys, s.P, s.g, s.fstride, tb, s.dt,
                                                s.dt_min, s.mode);
    return cudaGetLastError();
}

cudaError_t dg_euler_next(double* dt, double* time, unsigned long long* dt_min, cudaStream_t s)
{
    k_dg_euler_next<<<1, 1, 0, s>>>(dt, time, dt_min);
    return cudaGetLastError();
}

cudaError_t dg_stage(const DgStage& s)
{
    if (s.P <= 0) return cudaSuccess;
    const DgTables  tb    = dg_tables();
    if (s.g.n != kDgPatch || s.g.h != 1) return cudaErrorInvalidValue;
    // 64-thread blocks: a small tree (the reference's level 5 has 16384
    // cells) still spreads over every SM
    const long long total = static_cast<long long>(s.P) * kDgPatch * kDgPatch;
    const unsigned  grid  = static_cast<unsigned>(std::min<long long>((total + 63) / 64, 152LL * 32));
    k_dg_stage<<<grid, 64, 0, s.stream>>>(s.in, s.un, s.out, s.keys, s.P, s.g, s.fstride, tb, s.dt, s.mode);
    return cudaGetLastError();
}

// ------------------------------------------------ DG printer
// dg_tree_printer_2d (include/ndtree/print_dg_tree_v2.hpp:145-370): every
// interior cell is a VTK Lagrange quadrilateral whose (order + 1)^2 = 9
// points (xi, eta in {0, 1/2, 1}, eta slowest) carry the cell's polynomial
// evaluated there.  One thread per cell and section, big-endian output.
namespace {

__device__ __forceinline__ void dgv_be32(unsigned char* d, uint32_t v)
{
    *reinterpret_cast<uint32_t*>(d) = __byte_perm(v, 0, 0x0123);
}
__device__ __forceinline__ void dgv_be64(unsigned char* d, double v)
{
    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(v));
    dgv_be32(d, static_cast<uint32_t>(b >> 32));
    dgv_be32(d + 4, static_cast<uint32_t>(b));
}

// centre and edge of interior cell `cell` on the unit square (the printer's
// finest-grid arithmetic: the patch origin in finest cells, cell size
// 2^(depth - level) / 4, divided by 2^depth)
__device__ __forceinline__ void dgv_cell(const uint64_t* keys, const Geo& g, long long cell, int& p, int& lx, int& ly,
                                         double& cx, double& cy, double& h)
{
    p  = static_cast<int>(cell >> 4);
    lx = static_cast<int>(cell & 3);
    ly = static_cast<int>((cell >> 2) & 3);
    uint32_t c[3];
    key_decode(g, keys[p], c);
    const int    lev  = key_level(keys[p]);
    const double csg  = static_cast<double>(1u << (g.depth - lev)) / static_cast<double>(kDgPatch);
    const double norm = static_cast<double>(1u << g.depth);
    cx                = (static_cast<double>(c[0]) + (static_cast<double>(lx) + 0.5) * csg) / norm;
    cy                = (static_cast<double>(c[1]) + (static_cast<double>(ly) + 0.5) * csg) / norm;
    h                 = csg / norm;
}

// POINTS: 9 x (x, y, 0) per cell
__global__ void k_dgvtk_points(const uint64_t* __restrict__ keys, Geo g, long long first, long long count,
                               unsigned char* __restrict__ out)
{
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < count;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        int    p, lx, ly;
        double cx, cy, h;
        dgv_cell(keys, g, first + i, p, lx, ly, cx, cy, h);
        unsigned char* d = out + i * 9 * 24;
        for (int jj = 0; jj < 3; ++jj)
            for (int ii = 0; ii < 3; ++ii) {
                const double xi = static_cast<double>(ii) / 2.0, eta = static_cast<double>(jj) / 2.0;
                const double x  = cx + (2.0 * xi - 1.0) * (0.5 * h);
                const double y  = cy + (2.0 * eta - 1.0) * (0.5 * h);
                unsigned char* q = d + (jj * 3 + ii) * 24;
                dgv_be64(q, x);
                dgv_be64(q + 8, y);
                dgv_be64(q + 16, 0.0);
            }
    }
}

// CELLS: 9, then the cell's point ids in VTK Lagrange-quad order (corners,
// edges, face; point_idx_lagrange_quad, print_dg_tree_v2.hpp:61-97): the
// point (ii, jj) of cell c is 9 c + 3 jj + ii
__global__ void k_dgvtk_cells(long long first, long long count, unsigned char* __restrict__ out)
{
    constexpr int order[9] = { 0, 2, 8, 6, 1, 5, 7, 3, 4 };
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < count;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        unsigned char*  d    = out + i * 40;
        const long long base = (first + i) * 9;
        dgv_be32(d, 9u);
        for (int v = 0; v < 9; ++v) dgv_be32(d + 4 * (v + 1), static_cast<uint32_t>(static_cast<int>(base + order[v])));
    }
}

__global__ void k_dgvtk_types(long long count, unsigned char* __restrict__ out)
{
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < count;
         i += static_cast<long long>(gridDim.x) * blockDim.x)
        dgv_be32(out + 4 * i, 70u); // VTK_LAGRANGE_QUADRILATERAL
}

// POINT_DATA component `var`: Basis::evaluate_basis (polynomial.hpp:36-55)
// at the 9 points, sum over the nodes in tensor order of value x (1 x L_i0(xi)
// x L_i1(eta))
__global__ void k_dgvtk_values(const double* __restrict__ state, Geo g, size_t fstride, int var, double p0, double p1, long long first, long long count,
                               unsigned char* __restrict__ out)
{
    const double pts[2] = { p0, p1 };
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < count;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const long long cell = first + i;
        const int       p = static_cast<int>(cell >> 4), lx = static_cast<int>(cell & 3);
        const int       ly = static_cast<int>((cell >> 2) & 3);
        const size_t    at = static_cast<size_t>(p) * g.flat + (ly + 1) * (kDgPatch + 2) + lx + 1;
        double          C[2][2];
        for (int i0 = 0; i0 < 2; ++i0)
            for (int i1 = 0; i1 < 2; ++i1) C[i0][i1] = state[((i0 * 2 + i1) * kDgVars + var) * fstride + at];
        unsigned char* d = out + i * 9 * 8;
        for (int jj = 0; jj < 3; ++jj)
            for (int ii = 0; ii < 3; ++ii) {
                const double xi = static_cast<double>(ii) / 2.0, eta = static_cast<double>(jj) / 2.0;
                dgv_be64(d + (jj * 3 + ii) * 8, dg_eval(C, pts, xi, eta));
            }
    }
}

} // namespace

amr_status dg_write_vtk(const uint64_t* keys, const double* state, size_t size, const Geo& g, size_t fstride,
                        cudaStream_t s, const char* path, std::string& err, uint64_t& launches)
{
    const long long cells = static_cast<long long>(size) * kDgPatch * kDgPatch;
    FILE*           f     = std::fopen(path, "wb");
    if (!f) {
        err = std::string("cannot open ") + path;
        return AMR_ERR_INVALID;
    }
    // staging: at most 2^18 cells of the widest section (points, 216 B a cell)
    const long long chunk     = std::min<long long>(std::max<long long>(cells, 1), 1LL << 18);
    const size_t    max_bytes = static_cast<size_t>(chunk) * 9 * 24;
    unsigned char*  dbuf      = nullptr;
    unsigned char*  hbuf      = nullptr;
    cudaError_t     e         = cudaMalloc(&dbuf, max_bytes);
    if (e == cudaSuccess) e = cudaMallocHost(&hbuf, max_bytes);
    bool io_ok   = true;
    auto section = [&](size_t per_cell, auto&& launch) {
        for (long long first = 0; first < cells && e == cudaSuccess && io_ok; first += chunk) {
            const long long n    = std::min(chunk, cells - first);
            const unsigned  grid = static_cast<unsigned>(std::min<long long>((n + 255) / 256, 152LL * 32));
            launch(first, n, grid);
            ++launches;
            if (e == cudaSuccess) e = cudaGetLastError();
            if (e == cudaSuccess) e = cudaMemcpyAsync(hbuf, dbuf, n * per_cell, cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            if (e == cudaSuccess && std::fwrite(hbuf, 1, n * per_cell, f) != static_cast<size_t>(n * per_cell))
                io_ok = false;
        }
    };
    const double p0 = 0.5 + 0.5 * -0.5773502691896257, p1 = 0.5 + 0.5 * 0.5773502691896257;
    if (e == cudaSuccess) {
        std::fprintf(f, "# vtk DataFile Version 3.0\nDG 2D Printer (Order=%d)\nBINARY\nDATASET UNSTRUCTURED_GRID\n",
                     kDgOrder);
        std::fprintf(f, "POINTS %lld double\n", cells * 9);
        section(9 * 24, [&](long long first, long long n, unsigned grid) {
            k_dgvtk_points<<<grid, 256, 0, s>>>(keys, g, first, n, dbuf);
        });
        std::fprintf(f, "CELLS %lld %lld\n", cells, cells * 10);
        section(40, [&](long long first, long long n, unsigned grid) {
            k_dgvtk_cells<<<grid, 256, 0, s>>>(first, n, dbuf);
        });
        std::fprintf(f, "CELL_TYPES %lld\n", cells);
        section(4, [&](long long, long long n, unsigned grid) { k_dgvtk_types<<<grid, 256, 0, s>>>(n, dbuf); });
        if (cells > 0) std::fprintf(f, "POINT_DATA %lld\n", cells * 9);
        for (int var = 0; cells > 0 && var < kDgVars; ++var) {
            std::fprintf(f, "SCALARS dof_component_%d double 1\nLOOKUP_TABLE default\n", var);
            section(9 * 8, [&](long long first, long long n, unsigned grid) {
                k_dgvtk_values<<<grid, 256, 0, s>>>(state, g, fstride, var, p0, p1, first, n, dbuf);
            });
        }
    }
    if (dbuf) cudaFree(dbuf);
    if (hbuf) cudaFreeHost(hbuf);
    const bool closed = std::fclose(f) == 0;
    if (e != cudaSuccess) {
        err = std::string("DG printer: ") + cudaGetErrorString(e);
        return AMR_ERR_CUDA;
    }
    if (!io_ok || !closed) {
        err = "DG printer: write failed";
        return AMR_ERR_INVALID;
    }
    return AMR_OK;
}

} // namespace amr_gb300
