// Device-side building blocks shared by every kernel of the GB300 AMR path.
//
// Geometry contract (the reference's patch_layout / padded_layout): a patch is
// (n+2h)^rank cells, row-major, layout dim 0 slowest; Morton axis m (x=0,
// y=1, z=2) is layout dim rank-1-m.  Direction index = 2*dim + positive
// (include/ndtree/neighbor.hpp:103-255).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "amr_gb300.h"

namespace amr_gb300 {

struct Geo {
    int    rank, n, h, P1, flat, cells, depth, nd, nf, ndir;
    int    s[3];          // layout strides, s[rank-1] == 1
    int    inst_shift;    // bit position of the instance prefix in a key; 64 = none
    double dx_root[3];    // cell size at level 0 per Morton axis (L_axis / n)
    uint64_t morton_mask; // bits of the interleaved coordinate field
};

enum : int8_t { REL_NONE = 0, REL_SAME = 1, REL_FINER = 2, REL_COARSER = 3 };
enum : int8_t { FLAG_STABLE = 0, FLAG_REFINE = 1, FLAG_COARSEN = 2 };

// ------------------------------------------------------------------ Morton
// Bit interleave, coordinate k of a rank-r point at bit r*b + k (x lowest);
// the layout of libmorton's 64-bit encoders used by morton_id
// (include/morton/morton_id.hpp:118-140, 334-359), by binary magic numbers.
__host__ __device__ inline uint64_t spread2(uint64_t v)
{
    v &= 0xFFFFFFFFull;
    v = (v | (v << 16)) & 0x0000FFFF0000FFFFull;
    v = (v | (v << 8)) & 0x00FF00FF00FF00FFull;
    v = (v | (v << 4)) & 0x0F0F0F0F0F0F0F0Full;
    v = (v | (v << 2)) & 0x3333333333333333ull;
    v = (v | (v << 1)) & 0x5555555555555555ull;
    return v;
}
__host__ __device__ inline uint32_t compact2(uint64_t v)
{
    v &= 0x5555555555555555ull;
    v = (v | (v >> 1)) & 0x3333333333333333ull;
    v = (v | (v >> 2)) & 0x0F0F0F0F0F0F0F0Full;
    v = (v | (v >> 4)) & 0x00FF00FF00FF00FFull;
    v = (v | (v >> 8)) & 0x0000FFFF0000FFFFull;
    v = (v | (v >> 16)) & 0x00000000FFFFFFFFull;
    return static_cast<uint32_t>(v);
}
__host__ __device__ inline uint64_t spread3(uint64_t v)
{
    v &= 0x1FFFFFull;
    v = (v | (v << 32)) & 0x001F00000000FFFFull;
    v = (v | (v << 16)) & 0x001F0000FF0000FFull;
    v = (v | (v << 8)) & 0x100F00F00F00F00Full;
    v = (v | (v << 4)) & 0x10C30C30C30C30C3ull;
    v = (v | (v << 2)) & 0x1249249249249249ull;
    return v;
}
__host__ __device__ inline uint32_t compact3(uint64_t v)
{
    v &= 0x1249249249249249ull;
    v = (v | (v >> 2)) & 0x10C30C30C30C30C3ull;
    v = (v | (v >> 4)) & 0x100F00F00F00F00Full;
    v = (v | (v >> 8)) & 0x001F0000FF0000FFull;
    v = (v | (v >> 16)) & 0x001F00000000FFFFull;
    v = (v | (v >> 32)) & 0x00000000001FFFFFull;
    return static_cast<uint32_t>(v);
}

__host__ __device__ inline int key_level(uint64_t k) { return static_cast<int>(k & 0x3F); }

__host__ __device__ inline uint64_t key_prefix(const Geo& g, uint64_t k)
{
    return g.inst_shift >= 64 ? 0ull : (k >> g.inst_shift) << g.inst_shift;
}

__host__ __device__ inline void key_decode(const Geo& g, uint64_t k, uint32_t* c)
{
    const uint64_t m = (k >> 6) & g.morton_mask;
    if (g.rank == 2) {
        c[0] = compact2(m);
        c[1] = compact2(m >> 1);
        c[2] = 0;
    } else {
        c[0] = compact3(m);
        c[1] = compact3(m >> 1);
        c[2] = compact3(m >> 2);
    }
}

__host__ __device__ inline uint64_t key_encode(const Geo& g, uint64_t prefix, const uint32_t* c, int level)
{
    const uint64_t m = g.rank == 2 ? (spread2(c[0]) | (spread2(c[1]) << 1))
                                   : (spread3(c[0]) | (spread3(c[1]) << 1) | (spread3(c[2]) << 2));
    return prefix | (m << 6) | static_cast<uint64_t>(level & 0x3F);
}

// morton_id::child_of(p, off) = offset(p.id()+1, off), offset i = x + 2y (+4z)
// (include/morton/morton_id.hpp:64-83, 142-148).
__host__ __device__ inline uint64_t key_child(const Geo& g, uint64_t k, int off)
{
    uint32_t c[3];
    key_decode(g, k, c);
    const int      level = key_level(k) + 1;
    const uint32_t delta = 1u << (g.depth - level);
    c[0] += static_cast<uint32_t>(off & 1) * delta;
    c[1] += static_cast<uint32_t>((off >> 1) & 1) * delta;
    c[2] += static_cast<uint32_t>((off >> 2) & 1) * delta;
    return key_encode(g, key_prefix(g, k), c, level);
}

// morton_id::parent_of (include/morton/morton_id.hpp:103-116).
__host__ __device__ inline uint64_t key_parent(const Geo& g, uint64_t k)
{
    uint32_t c[3];
    key_decode(g, k, c);
    const int      level = key_level(k);
    const uint32_t off   = 1u << (g.depth - level);
    c[0] &= ~off;
    c[1] &= ~off;
    c[2] &= ~off;
    return key_encode(g, key_prefix(g, k), c, level - 1);
}

// Offset of a key within its parent (morton_id::offset_of, :55-62).
__host__ __device__ inline int key_offset(const Geo& g, uint64_t k)
{
    uint32_t c[3];
    key_decode(g, k, c);
    const int      level = key_level(k);
    const uint32_t bit   = 1u << (g.depth - level);
    return ((c[0] & bit) ? 1 : 0) | ((c[1] & bit) ? 2 : 0) | ((c[2] & bit) ? 4 : 0);
}

// Child offset -> hypercube coordinate in layout dim L (row-major, dim 0 slowest).
__host__ __device__ inline int child_coord(const Geo& g, int off, int L) { return (off >> (g.rank - 1 - L)) & 1; }

// --------------------------------------------------------------- geometry
__host__ __device__ inline double cell_size(const Geo& g, int axis, int level)
{
    // physics_system::cell_sizes (physics_system.hpp:75-85): L*2^(D-l)/2^D/n,
    // equal to (L/n)*2^-l because scaling by a power of two is exact.
    return g.dx_root[axis] / static_cast<double>(1ull << level);
}

__host__ __device__ inline int padded_index(const Geo& g, const int* idx)
{
    int li = 0;
    for (int L = 0; L < g.rank; ++L) li += idx[L] * g.s[L];
    return li;
}

// ------------------------------------------------------------- halo cell
// Value the reference's halo exchange writes into ghost cell G (padded layout
// coordinates) of a patch whose neighbour across direction (L, pos) is `m`:
//   same    -> copy of the neighbour interior cell shifted by n
//              (include/ndtree/patch_utils.hpp:315-332)
//   finer   -> mean of the 2^rank fine cells, summed row-major with dim 0
//              slowest, divided by 2^rank (patch_utils.hpp:334-386,
//              intergrid_operator.hpp:92-107)
//   coarser -> injection of the coarse cell picked by the contact quadrant
//              (patch_utils.hpp:388-441)
//   none    -> the ghost keeps its current value (:303-313).
// The mean is formed in double for every state type.
template <typename T>
__device__ inline double ghost_value(const T* __restrict__ buf, size_t pstride, const amr_halo_meta& m,
                                     const int* G, int L, int pos, const Geo& g, const T* __restrict__ self)
{
    int from[3] = { G[0], G[1], G[2] };
    from[L] += pos ? -g.n : g.n;
    if (m.relation == REL_SAME) {
        return static_cast<double>(buf[static_cast<size_t>(m.neighbor) * pstride + padded_index(g, from)]);
    }
    if (m.relation == REL_COARSER) {
        for (int k = 0; k < g.rank; ++k) from[k] = g.h + m.quadrant[k] * (g.n / 2) + (from[k] - g.h) / 2;
        return static_cast<double>(buf[static_cast<size_t>(m.neighbor) * pstride + padded_index(g, from)]);
    }
    if (m.relation == REL_FINER) {
        int fpi = 0, stride = 1;
        for (int k = 0; k < g.rank; ++k) {
            // the reference reduces every coordinate modulo the normal
            // dimension's size (patch_utils.hpp:357-359); patches are cubic.
            from[k] = ((from[k] - g.h) * 2) % g.n + g.h;
            if (k != L) {
                fpi += ((G[k] - g.h) / (g.n / 2)) * stride;
                stride *= 2;
            }
        }
        const T* fp = buf + static_cast<size_t>(m.finer_ids[fpi]) * pstride + padded_index(g, from);
        double   sum = 0.0;
        if (g.rank == 2) {
            sum += static_cast<double>(fp[0]);
            sum += static_cast<double>(fp[1]);
            sum += static_cast<double>(fp[g.s[0]]);
            sum += static_cast<double>(fp[g.s[0] + 1]);
            return sum / 4.0;
        }
        for (int a = 0; a < 2; ++a)
            for (int b = 0; b < 2; ++b)
                for (int c = 0; c < 2; ++c) sum += static_cast<double>(fp[a * g.s[0] + b * g.s[1] + c]);
        return sum / 8.0;
    }
    return static_cast<double>(self[padded_index(g, G)]);
}

} // namespace amr_gb300
