// The discrete adjoint of the frozen-mesh advection step (transposed
// update, gather per cell).
#pragma once

#include "amr_kernels.cuh"

namespace amr_gb300 {

// ------------------------------------------------------------- adjoint
// Transpose of one fused step (step_cell with ghosts on the fly) on a frozen
// mesh, gathered per interior cell j of patch p: lout_j = c0 lin_j plus, for
// every axis a with upwind offset up_a, the cells whose update reads j:
//   * the downwind cell j - up_a inside p (weight c_a of p's level);
//   * on the downwind face (relation from p's own neighbour record):
//       same    -> the adjacent cell of the neighbour (its c_a),
//       finer   -> the 2^(rank-1) fine cells whose coarse ghost injects j
//                  (ghost_value's coarser rule inverted, each with c_a of
//                  the fine level),
//   * in the two layers next to the downwind face, when that neighbour is
//     coarser: the coarse cell whose ghost is the mean of the 2^rank fine
//     cells containing j (weight c_a(coarse) / 2^rank).
// FP32 uses the difference form of the forward (u + c (u_up - u)), whose
// transpose is lin_j + sum_a (contributions - c_a(p) lin_j), with the
// coefficient rows rounded to FP32 once (coef32: (c_x, c_y) float2 entries
// for 2D trees, (c_x, c_y, c_z, c0) float4 entries for 3D trees, the values
// the FP64 rows round to).  Upwind sides per instance come from the packed
// integer codes (upcode), or from the launch.  Ghost cells of lout are not
// written (the caller keeps them zero).
template <typename T>
__device__ __forceinline__ T adjoint_coef(const Coef* coef, const float2* coef32, const Geo& g, int row, int a)
{
    if constexpr (sizeof(T) == 4) {
        if (g.rank == 3) {
            const float4 c = reinterpret_cast<const float4*>(coef32)[row];
            return a == 0 ? c.x : (a == 1 ? c.y : c.z);
        }
        const float2 c = coef32[row];
        return a == 0 ? c.x : c.y;
    } else {
        return coef[row].c[a];
    }
}

template <typename T>
__device__ inline void adjoint_cell(const T* lin, T* lout, const amr_halo_meta* meta, const uint64_t* keys,
                                    const Geo& g, const Coef* coef, const float2* coef32, const int* up_launch,
                                    const int32_t* upcode, int p, int c)
{
    constexpr bool F32 = sizeof(T) == 4;
    int            idx[3];
    interior_coords(g, c, idx);
    const int      nl   = g.depth + 1;
    const uint64_t kp   = keys[p];
    const int      inst = g.inst_shift >= 64 ? 0 : static_cast<int>(kp >> g.inst_shift);
    int            up[3] = { up_launch[0], up_launch[1], up_launch[2] };
    if (upcode) {
        const int32_t code = upcode[inst];
        for (int a = 0; a < 3; ++a) up[a] = a < g.rank ? unpack_upwind(code, a) : 0;
    }
    const int    rowp = inst * nl + key_level(kp);
    const size_t base = static_cast<size_t>(p) * g.flat;
    const int    li   = padded_index(g, idx);
    const T      lj   = lin[base + li];
    T            acc  = lj;
    if constexpr (!F32) acc = coef[rowp].c0 * lj;
    const int    half = g.n / 2;
    for (int a = 0; a < g.rank; ++a) {
        if (up[a] == 0) continue;
        const int L = g.rank - 1 - a, d = -up[a], pos_d = d > 0 ? 1 : 0;
        const int dist = pos_d ? (g.n + g.h - 1 - idx[L]) : (idx[L] - g.h); // cells to the downwind face
        const T   ca   = adjoint_coef<T>(coef, coef32, g, rowp, a);
        if (dist > 0) {
            const T ld = lin[base + li + d * g.s[L]];
            acc        = F32 ? fma(ca, static_cast<T>(ld - lj), acc) : fma(ca, ld, acc);
        } else if (F32) {
            acc = fma(-ca, lj, acc);
        }
        if (dist > 1) continue;
        const amr_halo_meta& m = meta[static_cast<size_t>(p) * g.ndir + 2 * L + pos_d];
        const int            face = pos_d ? g.h : g.n + g.h - 1; // the neighbour's layer next to the face
        if (m.relation == REL_COARSER) {
            int ci[3] = { idx[0], idx[1], idx[2] };
            for (int k = 0; k < g.rank; ++k)
                if (k != L) ci[k] = g.h + m.quadrant[k] * half + (idx[k] - g.h) / 2;
            ci[L]           = face;
            const T    cq   = adjoint_coef<T>(coef, coef32, g, inst * nl + key_level(keys[m.neighbor]), a);
            const T    w    = static_cast<T>(cq / static_cast<T>(1 << g.rank));
            acc             = fma(w, lin[static_cast<size_t>(m.neighbor) * g.flat + padded_index(g, ci)], acc);
        } else if (dist == 0 && m.relation == REL_SAME) {
            int ci[3] = { idx[0], idx[1], idx[2] };
            ci[L]     = face;
            acc = fma(ca, lin[static_cast<size_t>(m.neighbor) * g.flat + padded_index(g, ci)], acc);
        } else if (dist == 0 && m.relation == REL_FINER) {
            // section of j across the tangential dims (dim 0 fastest)
            int fpi = 0, st = 1, sec[3] = { 0, 0, 0 };
            for (int k = 0; k < g.rank; ++k) {
                if (k == L) continue;
                sec[k] = (idx[k] - g.h) / half;
                fpi += sec[k] * st;
                st *= 2;
            }
            const int   f   = fpi == 0 ? m.finer_ids[0] : fpi == 1 ? m.finer_ids[1] : fpi == 2 ? m.finer_ids[2] : m.finer_ids[3];
            const T     cfa = adjoint_coef<T>(coef, coef32, g, inst * nl + key_level(keys[f]), a);
            const T*    fp  = lin + static_cast<size_t>(f) * g.flat;
            int         fi[3];
            fi[L]           = face;
            int t0 = -1, t1 = -1; // tangential dims
            for (int k = 0; k < g.rank; ++k)
                if (k != L) {
                    fi[k] = g.h + 2 * ((idx[k] - g.h) - sec[k] * half);
                    if (t0 < 0) t0 = k;
                    else t1 = k;
                }
            if (g.rank == 2) {
                fi[2] = 0;
                T s   = fp[padded_index(g, fi)];
                fi[t0] += 1;
                s += fp[padded_index(g, fi)];
                acc = fma(cfa, s, acc);
            } else {
                T s = T(0);
                for (int b0 = 0; b0 < 2; ++b0)
                    for (int b1 = 0; b1 < 2; ++b1) {
                        int q[3] = { fi[0], fi[1], fi[2] };
                        q[t0] += b0;
                        q[t1] += b1;
                        s += fp[padded_index(g, q)];
                    }
                acc = fma(cfa, s, acc);
            }
        }
    }
    lout[base + li] = acc;
}

template <typename T>
__global__ void __launch_bounds__(256)
k_adjoint(const T* __restrict__ lin, T* __restrict__ lout, const amr_halo_meta* __restrict__ meta,
          const uint64_t* __restrict__ keys, int P, Geo g, const Coef* __restrict__ coef,
          const float2* __restrict__ coef32, int up0, int up1, int up2, const int32_t* __restrict__ upcode, int ppb)
{
    const int up[3] = { up0, up1, up2 };
    const int p0    = blockIdx.x * ppb;
    for (int t = threadIdx.x; t < ppb * g.cells; t += blockDim.x) {
        const int p = p0 + t / g.cells;
        if (p >= P) break;
        adjoint_cell<T>(lin, lout, meta, keys, g, coef, coef32, up, upcode, p, t - (p - p0) * g.cells);
    }
}

// Ghost cells of every patch set to zero (interior untouched).
template <typename T>
__global__ void k_zero_ghosts(T* __restrict__ buf, long long total, Geo g)
{
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < total;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        long long r      = i % g.flat;
        bool      inside = true;
        for (int k = g.rank - 1; k >= 0; --k) {
            const int c = static_cast<int>(r % g.P1);
            r /= g.P1;
            inside = inside && c >= g.h && c < g.n + g.h;
        }
        if (!inside) buf[i] = T(0);
    }
}

// Coefficient rows (step s, instance i) of `steps` steps from recorded step
// sizes dts[s * ninst + i] (the fill of k_batch_begin, without the clamp).
static __global__ void k_coef_from_dt(const double* __restrict__ dts, Geo g, const double* __restrict__ vel, int steps,
                               int ninst, Coef* __restrict__ coef, float2* __restrict__ coef32)
{
    const int nl    = g.depth + 1;
    const int total = steps * ninst * nl;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
        const int    l = e % nl, si = e / nl, inst = si % ninst;
        const double v[3] = { vel[3 * inst], vel[3 * inst + 1], vel[3 * inst + 2] };
        const Coef   c    = make_coef(g, dts[si], v, l);
        coef[e]           = c;
        if (g.rank == 3) // the FP32 rows, laid out as k_batch_begin writes them
            reinterpret_cast<float4*>(coef32)[e] = make_float4(static_cast<float>(c.c[0]), static_cast<float>(c.c[1]),
                                                               static_cast<float>(c.c[2]), static_cast<float>(c.c0));
        else
            coef32[e] = make_float2(static_cast<float>(c.c[0]), static_cast<float>(c.c[1]));
    }
}

} // namespace amr_gb300
