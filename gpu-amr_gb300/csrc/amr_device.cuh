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
#include "morton/morton_bits.hpp"

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
using amr::morton_bits::compact2;
using amr::morton_bits::compact3;
using amr::morton_bits::spread2;
using amr::morton_bits::spread3;

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

// ------------------------------------------------- bulk async copy (TMA)
// 1D bulk copies global -> shared completed on an mbarrier (cp.async.bulk,
// sm_90+), and a wait on the mbarrier with an iteration cap: a copy that
// never lands sets an error flag instead of spinning forever.
__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async_smem()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(smem_u32(bar)), "r"(parity)
                 : "memory");
    return ok != 0;
}
// 1D bulk copy shared -> global in a bulk async-group of the issuing
// thread, and that thread's waits: until the sources of all but the newest
// `Pending` groups have been read (the shared memory may be reused), or
// until every group has completed (the global writes are done).
__device__ __forceinline__ void bulk_copy_s2g(void* dst, const void* src, uint32_t bytes)
{
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(smem_u32(src)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
template <int Pending>
__device__ __forceinline__ void bulk_wait_read()
{
    asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(Pending) : "memory");
}
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

constexpr int kWaitLimit = 1 << 22;
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, int limit = kWaitLimit)
{
    for (int it = 0; it < limit; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// --------------------------------------------------------------- geometry
__host__ __device__ inline double cell_size(const Geo& g, int axis, int level)
{
    // physics_system::cell_sizes (physics_system.hpp:75-85): L*2^(D-l)/2^D/n,
    // equal to (L/n)*2^-l because scaling by a power of two is exact.
    return g.dx_root[axis] / static_cast<double>(1ull << level);
}

__host__ __device__ __forceinline__ int padded_index(const Geo& g, const int* idx)
{
    // s[2] == 0 and idx[2] == 0 in 2D
    return idx[0] * g.s[0] + idx[1] * g.s[1] + idx[2] * g.s[2];
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
// The mean is formed in double for every state type.  Coordinates are held
// in scalars (no runtime-indexed arrays) so the function stays in registers.
// R = T returns the value rounded to the state type: a copied or injected
// value as stored (a round trip through double is the identity), the mean
// rounded once; R = double returns the value before that rounding.
template <typename T, typename R = double>
__device__ __forceinline__ R ghost_value(const T* buf, size_t pstride, const amr_halo_meta& m, const int* G, int L,
                                         int pos, const Geo& g, const T* self)
{
    const int sh = pos ? -g.n : g.n;
    int       f0 = G[0] + (L == 0 ? sh : 0);
    int       f1 = G[1] + (L == 1 ? sh : 0);
    int       f2 = G[2] + (L == 2 ? sh : 0);
    const int rel = m.relation;
    if (rel == REL_SAME)
        return static_cast<R>(buf[static_cast<size_t>(m.neighbor) * pstride + f0 * g.s[0] + f1 * g.s[1] + f2 * g.s[2]]);
    const int half = g.n / 2;
    if (rel == REL_COARSER) {
        f0 = g.h + m.quadrant[0] * half + (f0 - g.h) / 2;
        f1 = g.h + m.quadrant[1] * half + (f1 - g.h) / 2;
        if (g.rank == 3) f2 = g.h + m.quadrant[2] * half + (f2 - g.h) / 2;
        return static_cast<R>(buf[static_cast<size_t>(m.neighbor) * pstride + f0 * g.s[0] + f1 * g.s[1] + f2 * g.s[2]]);
    }
    if (rel == REL_FINER) {
        // the reference reduces every coordinate modulo the normal
        // dimension's size (patch_utils.hpp:357-359); patches are cubic.
        f0 = ((f0 - g.h) * 2) % g.n + g.h;
        f1 = ((f1 - g.h) * 2) % g.n + g.h;
        if (g.rank == 3) f2 = ((f2 - g.h) * 2) % g.n + g.h;
        // section index over the tangential dims, dim 0 fastest
        int fpi = 0, st = 1;
        if (L != 0) {
            fpi += ((G[0] - g.h) / half) * st;
            st *= 2;
        }
        if (L != 1) {
            fpi += ((G[1] - g.h) / half) * st;
            st *= 2;
        }
        if (g.rank == 3 && L != 2) fpi += ((G[2] - g.h) / half) * st;
        const int id = fpi == 0 ? m.finer_ids[0] : fpi == 1 ? m.finer_ids[1] : fpi == 2 ? m.finer_ids[2] : m.finer_ids[3];
        const T*  fp = buf + static_cast<size_t>(id) * pstride + f0 * g.s[0] + f1 * g.s[1] + f2 * g.s[2];
        double    sum = 0.0;
        if (g.rank == 2) {
            sum += static_cast<double>(fp[0]);
            sum += static_cast<double>(fp[1]);
            sum += static_cast<double>(fp[g.s[0]]);
            sum += static_cast<double>(fp[g.s[0] + 1]);
            return static_cast<R>(sum / 4.0);
        }
        sum += static_cast<double>(fp[0]);
        sum += static_cast<double>(fp[1]);
        sum += static_cast<double>(fp[g.s[1]]);
        sum += static_cast<double>(fp[g.s[1] + 1]);
        sum += static_cast<double>(fp[g.s[0]]);
        sum += static_cast<double>(fp[g.s[0] + 1]);
        sum += static_cast<double>(fp[g.s[0] + g.s[1]]);
        sum += static_cast<double>(fp[g.s[0] + g.s[1] + 1]);
        return static_cast<R>(sum / 8.0);
    }
    return static_cast<R>(self[G[0] * g.s[0] + G[1] * g.s[1] + G[2] * g.s[2]]);
}

} // namespace amr_gb300
