// Fused re-mesh interval of the 2D FP32 forest: D update steps and the
// gradient flags of the interval's end state in one pass over memory.
//
// Applies to trees whose every neighbour relation is "same level" (each
// instance uniform at its own level L >= 2, as the batched forests are) with
// 16x16 patches and one ghost layer.  In Morton order the 16 leaves
// 16b .. 16b+15 of such a tree are one aligned 4x4 block of patches of one
// instance (64x64 cells), so block b is found from the key of leaf 16b alone;
// its neighbour patches follow from the block's position and the instance's
// level (periodic wrap), with no neighbour records.
//
// One CTA per block (grid-stride over blocks), in upwind-normalized
// coordinates (an axis whose upwind side is + is mirrored, so a cell's upwind
// neighbours are at row - 1 and column - 1).  The region computed is
// [-(D+1), 65) x [-(D+1), 65): D upwind lines, whose valid part shrinks by
// one per step, so that after D steps the block and the ring of cells around
// it (the ghosts its flags read) are exact.
//  1. bulk copies (cp.async.bulk, one mbarrier) bring the padded rows the
//     region needs of the block's 6x6 patch neighbourhood into shared memory
//     (packed: each patch row keeps only the rows the region uses); the copies
//     of the next block are issued as soon as the threads hold the current
//     one in registers, so they land during its steps;
//  2. thread (tx, ty) holds rows ty*RY - (D+1) .. + RY-1 of four columns as
//     two FP32 pairs: p1 = (c, c + HW) and p2 = (c + 1, c + 1 + HW), c =
//     2tx - (D+1), HW half the region width.  The x-neighbour of p2 is p1, of
//     p1 the left thread's p2; the y-neighbour of a row is the row above;
//  3. D steps in registers: per step each thread publishes its p2 column and
//     its last row into double-buffered shared arrays, one CTA barrier, and
//     updates its cells in place from the last row up, p2 before p1.  The
//     update is two packed FP32 subtractions and two packed FMAs per pair
//     (sub.rn.f32x2 / fma.rn.f32x2: per component the rounding of upd2d_core,
//     acc = fma(c_y, yn - u, fma(c_x, xn - u, u))), so every cell is
//     bit-identical to D one-step launches;
//  4. flags: each thread evaluates the gradient rule of flags2d_uniform_body
//     (FP32 squared gradient with packed operations, the proven band, FP64
//     inside it) on its cells of the block, with the ring cells as the ghosts
//     a halo exchange would store; per patch "any refine" / "all coarsen"
//     through shared-memory atomics; one thread per patch writes the decision;
//  5. the block's padded rows 1..16 (ghost columns included, written with the
//     current neighbour cells, the values a halo exchange would store) are
//     staged in shared memory and go to memory by one bulk store per patch
//     plus four single floats at the 16-byte-misaligned ends of each span.
//
// The kernel checks that each block is one aligned 4x4 block of one instance
// at a level >= 2 and that its neighbourhood holds the expected keys before
// any copy is issued.
#pragma once

#include "amr_graph.cuh"

namespace amr_gb300 {

constexpr int32_t kRetryFused = 101;

template <int D>
struct IntervalShape {
    static constexpr int N = 16, P1 = 18, FLAT = P1 * P1;
    static constexpr int HALO = D + 1;          // upwind lines of the region
    static constexpr int RW   = 64 + HALO + 1;  // region width (columns and rows)
    static constexpr int HW   = RW / 2;         // half width: the two columns of a pair are HW apart
    static constexpr int TX   = HW / 2;         // threads per row group (two pairs each)
    static constexpr int TY   = 8;              // row groups
    static constexpr int RY   = 10;             // rows per thread
    static constexpr int THREADS = TX * TY;
    static constexpr int XS   = TY * RY + 2;    // X column pitch in pairs: an odd multiple of 16 bytes
    static constexpr int TILES = 6 * (800 + 4 * 1168 + 80); // packed tile rows (bytes), either mirroring
    static constexpr int STAGE = 292;           // floats per staged patch: padded indices 16 .. 307
    static_assert(RW % 4 == 0, "region width is a multiple of four columns");
    static_assert(TY * RY >= RW, "row groups cover the region");
    static_assert((XS * 8) % 32 == 16, "X pitch spreads 16-byte stores over the banks");
    static_assert(D == 10, "tile packing sized for ten steps");
    // shared memory: tiles | X (2 buffers x (TX + 1) columns x XS pairs; the
    // output stage once the flags are done) | Y (2 buffers x (TY + 1) rows x
    // TX double pairs) | patch bases, flags, slot table, coefficients, barrier
    static constexpr size_t x_bytes = 2 * (TX + 1) * XS * 8;
    static constexpr size_t y_bytes = 2 * (TY + 1) * TX * 16;
    static constexpr size_t smem    = TILES + x_bytes + y_bytes + 16 * 4 * 3 + 24 * 4 + D * 16 + 16;
    static_assert(16 * STAGE * 4 <= x_bytes, "the output stage fits in the X buffers");
};

// Padded rows of an actual patch row py (-1 .. 4) that the region needs:
// interior rows [a, b] (0-based), from the region's actual row range.
template <int D>
__device__ __forceinline__ void interval_rows(int py, bool mirrored, int& a, int& b)
{
    constexpr int H = IntervalShape<D>::HALO;
    // normalized rows [-H, 64] -> actual rows [-H, 64] or [-1, 63 + H]
    const int ylo = mirrored ? -1 : -H, yhi = mirrored ? 63 + H : 64;
    a = max(ylo - 16 * py, 0);
    b = min(yhi - 16 * py, 15);
}

// Byte span [lo, hi) of a padded patch covering interior rows a..b (all 18
// columns), rounded out to 16 bytes; within [64, 1232).
__device__ __forceinline__ void interval_span(int a, int b, uint32_t& lo, uint32_t& hi)
{
    lo = static_cast<uint32_t>((a + 1) * 18 * 4) & ~15u;
    hi = (static_cast<uint32_t>((b + 2) * 18 * 4) + 15u) & ~15u;
}

// Packed tile rows: patch row py (-1 .. 4) keeps the byte span [lo, lo +
// size) of each of its six patches, one patch row after another from `start`.
template <int D>
__device__ __forceinline__ void interval_slot_row(int py, bool sy, uint32_t& lo, uint32_t& size, uint32_t& start)
{
    start = 0;
#pragma unroll
    for (int q = -1; q <= 4; ++q) {
        int a, b;
        interval_rows<D>(q, sy, a, b);
        uint32_t l, h;
        interval_span(a, b, l, h);
        if (q == py) {
            lo   = l;
            size = h - l;
            return;
        }
        start += 6 * (h - l);
    }
}

// Packed FP32 pairs (bit patterns of two floats, low word first).
__device__ __forceinline__ uint64_t pk(float lo, float hi)
{
    return static_cast<uint64_t>(__float_as_uint(lo)) | (static_cast<uint64_t>(__float_as_uint(hi)) << 32);
}
__device__ __forceinline__ float    pk_lo(uint64_t v) { return __uint_as_float(static_cast<uint32_t>(v)); }
__device__ __forceinline__ float    pk_hi(uint64_t v) { return __uint_as_float(static_cast<uint32_t>(v >> 32)); }
__device__ __forceinline__ uint32_t pk_lo_bits(uint64_t v) { return static_cast<uint32_t>(v); }
__device__ __forceinline__ uint32_t pk_hi_bits(uint64_t v) { return static_cast<uint32_t>(v >> 32); }

// One cell update of upd2d_core (FP32 difference form) on a pair of cells.
template <bool XU, bool YU>
__device__ __forceinline__ uint64_t upd_pair(uint64_t u, uint64_t xn, uint64_t yn, uint64_t cx, uint64_t cy)
{
    uint64_t acc = u;
    if constexpr (XU) {
        uint64_t d;
        asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(xn), "l"(u));
        asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(acc) : "l"(cx), "l"(d), "l"(acc));
    }
    if constexpr (YU) {
        uint64_t d;
        asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(yn), "l"(u));
        asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(acc) : "l"(cy), "l"(d), "l"(acc));
    }
    return acc;
}

// grad_sq_f32_2 on a pair of cells: fma(gy, gy, fma(gx, gx, 0)) with
// gx = 0.5 (xh - xl), gy = 0.5 (yh - yl); fma(g, g, 0) is the rounded square.
__device__ __forceinline__ uint64_t grad_pair(uint64_t xl, uint64_t xh, uint64_t yl, uint64_t yh)
{
    const uint64_t half = pk(0.5f, 0.5f);
    uint64_t       dx, dy, gx, gy, s;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(dx) : "l"(xh), "l"(xl));
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(dy) : "l"(yh), "l"(yl));
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(gx) : "l"(half), "l"(dx));
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(gy) : "l"(half), "l"(dy));
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(s) : "l"(gx), "l"(gx));
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(s) : "l"(gy), "l"(gy), "l"(s));
    return s;
}

// Guard of an interval captured with the fused kernel (after
// k_run_require_uniform, before any kernel changes state or time): every
// 16 leaves from 16b must be one aligned 4x4 block of one instance at a level
// >= 2, else kRetryFused stops the replay and the host re-runs the interval
// with the per-leaf kernels.
static __global__ void __launch_bounds__(256) k_run_require_blocks(RunBufs B, RunCtl* ctl, Geo g)
{
    if (ctl->err) return;
    const int P = ctl->P;
    if (P % 16 != 0) {
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicCAS(&ctl->err, 0, kRetryFused);
        return;
    }
    const uint64_t* keys = B.keys[ctl->tb];
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < P / 16; b += gridDim.x * blockDim.x) {
        const uint64_t k0 = keys[16 * b], k15 = keys[16 * b + 15];
        const int      L  = key_level(k0);
        const uint32_t m0 = static_cast<uint32_t>(((k0 >> 6) & g.morton_mask) >> (2 * (g.depth - L)));
        if (L < 2 || key_level(k15) != L || key_prefix(g, k15) != key_prefix(g, k0) || (m0 & 15u) != 0u)
            atomicCAS(&ctl->err, 0, kRetryFused);
    }
}

// What a CTA knows about one block.
struct IntervalBlock {
    int      base;     // leaf index of the instance's first patch
    int      L, inst;  // level, instance
    int      bx0, by0; // block origin (patch coordinates)
    int      ux, uy;   // upwind offsets
    uint64_t pre;      // instance key prefix
};

template <int D, bool FLAGS>
__global__ void __launch_bounds__(IntervalShape<D>::THREADS, 3)
k_run_interval2d(RunBufs B, RunCtl* ctl, Geo g, const float2* __restrict__ coef32, size_t cstride, int nl,
                 GradRule rule, int min_level, int max_level, int upx0, int upy0, int parity)
{
    using S                = IntervalShape<D>;
    constexpr int TX       = S::TX, TY = S::TY, RY = S::RY, XS = S::XS, HALO = S::HALO, HW = S::HW;
    constexpr int FLAT     = S::FLAT, STAGE = S::STAGE;
    if (ctl->err) return;
    extern __shared__ __align__(128) unsigned char smem[];
    unsigned char* tiles = smem;
    uint64_t*      Xb    = reinterpret_cast<uint64_t*>(smem + S::TILES);
    float*         stage = reinterpret_cast<float*>(smem + S::TILES); // aliases X after the flags
    ulonglong2*    Yb    = reinterpret_cast<ulonglong2*>(smem + S::TILES + S::x_bytes);
    int*           pbase = reinterpret_cast<int*>(smem + S::TILES + S::x_bytes + S::y_bytes);
    int*           pany  = pbase + 16;
    int*           pall  = pany + 16;
    int*           slot  = pall + 16; // per patch row of the tiles: lo, size, start (6 x 3, padded)
    ulonglong2*    cf    = reinterpret_cast<ulonglong2*>(slot + 24); // (c_x, c_x), (c_y, c_y) per step
    uint64_t*      bar   = reinterpret_cast<uint64_t*>(cf + D);

    const int tid = threadIdx.x;
    const int tx = tid % TX, ty = tid / TX;
    const int P = ctl->P, tb = ctl->tb, s = ctl->sb ^ parity;
    const float* __restrict__ in   = static_cast<const float*>(B.state[s]);
    float* __restrict__       out  = static_cast<float*>(B.state[s ^ 1]);
    const uint64_t* __restrict__ keys = B.keys[tb];
    const int nblk = P / 16;
    if (P % 16 != 0) {
        if (tid == 0) atomicCAS(&ctl->err, 0, kRetryFused);
        return;
    }
    if (tid == 0) {
        mbar_init(bar, 1);
        mbar_init_fence();
    }
    // rows above the region in the Y buffers are never written: zero once
    for (int i = tid; i < 2 * TX; i += blockDim.x) Yb[(i / TX) * (TY + 1) * TX + (i % TX)] = make_ulonglong2(0, 0);
    __syncthreads();

    // the block's description from its first key
    auto describe = [&](int blk, IntervalBlock& b) -> bool {
        const uint64_t k0  = __ldg(keys + 16 * blk);
        const uint64_t k15 = __ldg(keys + 16 * blk + 15);
        b.L                = key_level(k0);
        b.pre              = key_prefix(g, k0);
        const uint32_t m0  = static_cast<uint32_t>(((k0 >> 6) & g.morton_mask) >> (2 * (g.depth - b.L)));
        b.inst             = g.inst_shift >= 64 ? 0 : static_cast<int>(k0 >> g.inst_shift);
        b.base             = 16 * blk - static_cast<int>(m0);
        b.bx0              = static_cast<int>(compact2(m0));
        b.by0              = static_cast<int>(compact2(m0 >> 1));
        b.ux               = upx0;
        b.uy               = upy0;
        if (B.upcode) {
            const int32_t code = __ldg(B.upcode + b.inst);
            b.ux               = unpack_upwind(code, 0);
            b.uy               = unpack_upwind(code, 1);
        }
        return !(b.L < 2 || key_level(k15) != b.L || key_prefix(g, k15) != b.pre || (m0 & 15u) != 0u);
    };
    // leaf of actual block-relative patch offsets (px, py), periodic
    auto leaf_at = [&](const IntervalBlock& b, int px, int py) -> int {
        const int      Wm = (1 << b.L) - 1;
        const uint32_t x = static_cast<uint32_t>((b.bx0 + px) & Wm), y = static_cast<uint32_t>((b.by0 + py) & Wm);
        return b.base + static_cast<int>(spread2(x) | (spread2(y) << 1));
    };
    // validate the block and its neighbourhood (every slot's leaf holds the
    // key of that position at level L), write its slot table, issue the
    // copies; false when the block is not valid (nothing issued: the CTA
    // leaves).  Its barriers also order every earlier read of the tiles and
    // of the slot table before the copies and the new table.
    auto issue = [&](int blk, IntervalBlock& b) -> bool {
        int bad = describe(blk, b) ? 0 : 1;
        if (!bad && tid < 36) {
            const int      py = tid / 6 - 1, px = tid % 6 - 1;
            const int      Wm = (1 << b.L) - 1;
            const uint32_t x = static_cast<uint32_t>((b.bx0 + px) & Wm), y = static_cast<uint32_t>((b.by0 + py) & Wm);
            const int      q = b.base + static_cast<int>(spread2(x) | (spread2(y) << 1));
            const uint64_t m = (spread2(x) | (spread2(y) << 1)) << (2 * (g.depth - b.L));
            bad = q < 0 || q >= P || __ldg(keys + q) != (b.pre | (m << 6) | static_cast<uint64_t>(b.L));
        }
        if (__syncthreads_or(bad)) {
            if (tid == 0) atomicCAS(&ctl->err, 0, static_cast<int32_t>(AMR_ERR_UNBALANCED));
            return false;
        }
        const bool sy = b.uy > 0;
        if (tid == 0) mbar_expect_tx(bar, S::TILES); // either mirroring packs to TILES bytes
        if (tid >= 64 && tid < 70) {
            uint32_t lo, size, start;
            interval_slot_row<D>(tid - 65, sy, lo, size, start);
            slot[3 * (tid - 64)]     = static_cast<int>(lo);
            slot[3 * (tid - 64) + 1] = static_cast<int>(size);
            slot[3 * (tid - 64) + 2] = static_cast<int>(start);
        }
        fence_proxy_async_smem();
        __syncthreads();
        if (tid < 36) {
            const int py = tid / 6 - 1, px = tid % 6 - 1;
            uint32_t  lo, size, start;
            interval_slot_row<D>(py, sy, lo, size, start);
            const char* src = reinterpret_cast<const char*>(in + static_cast<size_t>(leaf_at(b, px, py)) * FLAT);
            bulk_copy_g2s(tiles + start + (px + 1) * size, src + lo, size, bar);
        }
        return true;
    };

    IntervalBlock cur{}, nxt{};
    uint32_t      phase = 0;
    int           blk   = blockIdx.x;
    if (blk >= nblk || !issue(blk, cur)) return;

    while (true) {
        // ---- 1. the copies of this block
        if (__syncthreads_or(mbar_wait_bounded(bar, phase) ? 0 : 1)) {
            if (tid == 0) atomicExch(&ctl->err, static_cast<int32_t>(AMR_ERR_TIMEOUT));
            mbar_wait_bounded(bar, phase); // copies still in flight land before the CTA goes
            if (tid < 16) bulk_wait_all();
            return;
        }
        phase ^= 1u;
        const bool sx = cur.ux > 0, sy = cur.uy > 0;
        if (tid < D) {
            const float2 c = __ldg(coef32 + tid * cstride + static_cast<size_t>(cur.inst) * nl + cur.L);
            cf[tid]        = make_ulonglong2(pk(c.x, c.x), pk(c.y, c.y));
        }
        if (tid < 16) {
            const int px = tid & 3, py = tid >> 2; // actual block patch
            pbase[tid]   = leaf_at(cur, px, py) * FLAT;
            pany[tid]    = 0;
            pall[tid]    = 1;
        }

        // ---- 2. the thread's cells into registers
        // column k of the thread: 0 -> p1.lo, 1 -> p2.lo, 2 -> p1.hi, 3 -> p2.hi
        const int c0 = 2 * tx - HALO;
        int       colX[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int c = c0 + (k & 1) + (k >> 1) * HW;
            colX[k]     = sx ? 63 - c : c;
        }
        const int r0 = ty * RY - HALO;
        uint64_t  v1[RY], v2[RY];
#pragma unroll
        for (int i = 0; i < RY; ++i) {
            const int r    = r0 + i;
            float     e[4] = { 0.0f, 0.0f, 0.0f, 0.0f };
            if (r <= 64) {
                const int      Y  = sy ? 63 - r : r;
                const int      q  = (Y >> 4) + 1;
                const int      lo = slot[3 * q], size = slot[3 * q + 1], start = slot[3 * q + 2];
                const unsigned char* rowp = tiles + start + ((Y & 15) + 1) * 72 + 4 - lo;
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const int X = colX[k];
                    e[k]        = *reinterpret_cast<const float*>(rowp + ((X >> 4) + 1) * size + (X & 15) * 4);
                }
            }
            v1[i] = pk(e[0], e[2]);
            v2[i] = pk(e[1], e[3]);
        }
        // ---- the next block's copies land during this block's steps
        const int  nb   = blk + static_cast<int>(gridDim.x);
        const bool more = nb < nblk;
        if (more) {
            if (!issue(nb, nxt)) {
                if (tid < 16) bulk_wait_all();
                return;
            }
        } else {
            __syncthreads(); // pbase, cf and the flags' zeroing are visible
        }

        // ---- 3. D steps
        auto steps = [&]<bool XU, bool YU>() {
#pragma unroll 1
            for (int m = 0; m < D; ++m) {
                uint64_t* const   X = Xb + (m & 1) * (TX + 1) * XS;
                ulonglong2* const Y = Yb + (m & 1) * (TY + 1) * TX;
                {
                    uint64_t* xo = X + (tx + 1) * XS + ty * RY;
#pragma unroll
                    for (int i = 0; i < RY; i += 2)
                        *reinterpret_cast<ulonglong2*>(xo + i) = make_ulonglong2(v2[i], v2[i + 1]);
                    if (tx == TX - 1) { // the left neighbour of the second half's first column
                        uint64_t* x0 = X + ty * RY;
#pragma unroll
                        for (int i = 0; i < RY; i += 2) {
                            const float a = pk_lo(v2[i]), b = pk_lo(v2[i + 1]);
                            *reinterpret_cast<ulonglong2*>(x0 + i) = make_ulonglong2(pk(a, a), pk(b, b));
                        }
                    }
                    Y[(ty + 1) * TX + tx] = make_ulonglong2(v1[RY - 1], v2[RY - 1]);
                }
                __syncthreads();
                const ulonglong2 c   = cf[m];
                const ulonglong2 yin = Y[ty * TX + tx];
                const uint64_t*  xi  = X + tx * XS + ty * RY;
#pragma unroll
                for (int i = RY - 2; i >= 0; i -= 2) {
                    const ulonglong2 xw = *reinterpret_cast<const ulonglong2*>(xi + i);
                    // row i + 1, then row i: p2 first (its x-neighbour is p1)
                    v2[i + 1] = upd_pair<XU, YU>(v2[i + 1], v1[i + 1], v2[i], c.x, c.y);
                    v1[i + 1] = upd_pair<XU, YU>(v1[i + 1], xw.y, v1[i], c.x, c.y);
                    v2[i]     = upd_pair<XU, YU>(v2[i], v1[i], i > 0 ? v2[i - 1] : yin.y, c.x, c.y);
                    v1[i]     = upd_pair<XU, YU>(v1[i], xw.x, i > 0 ? v1[i - 1] : yin.x, c.x, c.y);
                }
            }
        };
        if (cur.ux != 0 && cur.uy != 0) steps.template operator()<true, true>();
        else if (cur.ux != 0) steps.template operator()<true, false>();
        else if (cur.uy != 0) steps.template operator()<false, true>();
        else steps.template operator()<false, false>();
        // the step loop's last reads of X and Y finish here
        __syncthreads();

        // ---- 4. flags of the block's 16 patches
        if constexpr (FLAGS) {
            // exchange: p2 to the right neighbour (X buffer 0), p1 to the left
            // (X buffer 1), last row down (Y buffer 0), first row up (Y buffer 1)
            uint64_t* const   XL = Xb;
            uint64_t* const   XR = Xb + (TX + 1) * XS;
            ulonglong2* const YD = Yb;
            ulonglong2* const YU = Yb + (TY + 1) * TX;
            {
                uint64_t* a = XL + (tx + 1) * XS + ty * RY;
                uint64_t* b = XR + tx * XS + ty * RY;
#pragma unroll
                for (int i = 0; i < RY; i += 2) {
                    *reinterpret_cast<ulonglong2*>(a + i) = make_ulonglong2(v2[i], v2[i + 1]);
                    *reinterpret_cast<ulonglong2*>(b + i) = make_ulonglong2(v1[i], v1[i + 1]);
                }
                if (tx == TX - 1) {
                    uint64_t* x0 = XL + ty * RY;
#pragma unroll
                    for (int i = 0; i < RY; i += 2) {
                        const float p = pk_lo(v2[i]), q = pk_lo(v2[i + 1]);
                        *reinterpret_cast<ulonglong2*>(x0 + i) = make_ulonglong2(pk(p, p), pk(q, q));
                    }
                }
                if (tx == 0) { // the right neighbour of the first half's last column
                    uint64_t* xe = XR + TX * XS + ty * RY;
#pragma unroll
                    for (int i = 0; i < RY; i += 2) {
                        const float p = pk_hi(v1[i]), q = pk_hi(v1[i + 1]);
                        *reinterpret_cast<ulonglong2*>(xe + i) = make_ulonglong2(pk(p, p), pk(q, q));
                    }
                }
                YD[(ty + 1) * TX + tx] = make_ulonglong2(v1[RY - 1], v2[RY - 1]);
                YU[ty * TX + tx]       = make_ulonglong2(v1[0], v2[0]);
            }
            __syncthreads();
            const ulonglong2 ya = YD[ty * TX + tx];       // the row above row 0
            const ulonglong2 yb = YU[(ty + 1) * TX + tx]; // the row below row RY - 1
            const uint64_t*  xl = XL + tx * XS + ty * RY;
            const uint64_t*  xr = XR + (tx + 1) * XS + ty * RY;
            // per column k and patch-row part (the thread's rows cross at most
            // one patch boundary): the largest FP32 squared gradient as a bit
            // pattern (s >= +0 or NaN, so unsigned order is value order and
            // a pattern >= that of +inf means some value is not finite)
            const int ra = max(r0, 0), rb = min(r0 + RY - 1, 63);
            const int split = ((ra >> 4) + 1) * 16; // first row of the second part
            uint32_t  m0[4] = { 0u, 0u, 0u, 0u }, m1[4] = { 0u, 0u, 0u, 0u };
#pragma unroll
            for (int i = 0; i < RY; ++i) {
                const int r = r0 + i;
                if (r < ra || r > rb) continue;
                const uint64_t up1 = i > 0 ? v1[i - 1] : ya.x, dn1 = i < RY - 1 ? v1[i + 1] : yb.x;
                const uint64_t up2 = i > 0 ? v2[i - 1] : ya.y, dn2 = i < RY - 1 ? v2[i + 1] : yb.y;
                const uint64_t s1  = grad_pair(xl[i], v2[i], up1, dn1);
                const uint64_t s2  = grad_pair(v1[i], xr[i], up2, dn2);
                const uint32_t e[4] = { pk_lo_bits(s1), pk_lo_bits(s2), pk_hi_bits(s1), pk_hi_bits(s2) };
                if (r >= split) {
#pragma unroll
                    for (int k = 0; k < 4; ++k) m1[k] = max(m1[k], e[k]);
                } else {
#pragma unroll
                    for (int k = 0; k < 4; ++k) m0[k] = max(m0[k], e[k]);
                }
            }
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int c = c0 + (k & 1) + (k >> 1) * HW;
                if (c < 0 || c > 63 || ra > rb) continue;
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int lo = h ? split : ra, hi = h ? rb : min(rb, split - 1);
                    if (lo > hi) continue;
                    const uint32_t mb  = h ? m1[k] : m0[k];
                    const float    sm  = __uint_as_float(mb);
                    const bool     bad = mb >= 0x7f800000u;
                    int            any = 0, all = 1;
                    const bool known = rule.fast && !bad && (sm >= rule.r_hi || sm < rule.r_lo) &&
                                       (sm < rule.c_lo || sm >= rule.c_hi);
                    if (known) {
                        any = sm >= rule.r_hi ? 1 : 0;
                        all = sm < rule.c_lo ? 1 : 0;
                    } else {
                        // the exact rule on this column's cells of the part
                        for (int i = 0; i < RY; ++i) {
                            const int r = r0 + i;
                            if (r < lo || r > hi) continue;
                            uint64_t up, dn, wl, wh;
                            if (k & 1) {
                                up = i > 0 ? v2[i - 1] : ya.y;
                                dn = i < RY - 1 ? v2[i + 1] : yb.y;
                                wl = v1[i];
                                wh = xr[i];
                            } else {
                                up = i > 0 ? v1[i - 1] : ya.x;
                                dn = i < RY - 1 ? v1[i + 1] : yb.x;
                                wl = xl[i];
                                wh = v2[i];
                            }
                            const bool   hh = (k >> 1) != 0;
                            const double e  = grad_sq_exact2<float>(hh ? pk_hi(wl) : pk_lo(wl), hh ? pk_hi(wh) : pk_lo(wh),
                                                                    hh ? pk_hi(up) : pk_lo(up), hh ? pk_hi(dn) : pk_lo(dn));
                            if (e >= rule.rsq) any = 1;
                            if (!(e < rule.csq)) all = 0;
                        }
                    }
                    const int pb = (lo >> 4) * 4 + (c >> 4); // normalized patch
                    if (any) atomicOr(&pany[pb], 1);
                    if (!all) atomicAnd(&pall[pb], 0);
                }
            }
            __syncthreads(); // the exchange reads end before the stage overwrites X
        }

        // ---- 5. the block's padded rows 1..16 into the stage (patch p =
        // px + 4 py keeps padded indices 16 .. 307 at p * STAGE); column X of
        // a patch's row also serves as the ghost column of its neighbour in
        // the block (X & 15 == 15: the next patch's column 0; X & 15 == 0:
        // the previous patch's column 17)
#pragma unroll
        for (int i = 0; i < RY; ++i) {
            const int r = r0 + i;
            if (r < 0 || r > 63) continue;
            const int   Y    = sy ? 63 - r : r;
            float*      srow = stage + (Y >> 4) * 4 * STAGE + ((Y & 15) + 1) * 18 - 16;
            const float e[4] = { pk_lo(v1[i]), pk_lo(v2[i]), pk_hi(v1[i]), pk_hi(v2[i]) };
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int X = colX[k];
                if (X >= 0 && X <= 63) srow[(X >> 4) * STAGE + (X & 15) + 1] = e[k];
                if ((X & 15) == 15 && X + 1 >= 0 && X + 1 <= 63) srow[((X + 1) >> 4) * STAGE] = e[k];
                if ((X & 15) == 0 && X - 1 >= 0 && X - 1 <= 63) srow[((X - 1) >> 4) * STAGE + 17] = e[k];
            }
        }
        fence_proxy_async_smem(); // the stage writes before the async proxy reads them
        __syncthreads();
        if (tid < 16) { // padded bytes [80, 1216): rows 1..16 but for two floats at each end
            bulk_copy_s2g(reinterpret_cast<char*>(out + pbase[tid]) + 80,
                          reinterpret_cast<const char*>(stage + tid * STAGE + 4), 1136u);
            bulk_commit();
        } else if (tid >= 32 && tid < 96) { // the four floats outside the 16-byte span
            const int p = (tid - 32) >> 2, w = (tid - 32) & 3;
            const int j = w < 2 ? 18 + w : 302 + w; // row 1 columns 0, 1; row 16 columns 16, 17
            out[pbase[p] + j] = stage[p * STAGE + j - 16];
        }

        if constexpr (FLAGS) {
            if (tid >= 128 && tid < 144) {
                const int t   = tid - 128;
                const int bpx = t & 3, bpy = t >> 2; // normalized block patch
                const int px = sx ? 3 - bpx : bpx, py = sy ? 3 - bpy : bpy;
                int       lo = min_level, hi = max_level;
                if (B.bounds) {
                    lo = __ldg(B.bounds + 2 * cur.inst);
                    hi = __ldg(B.bounds + 2 * cur.inst + 1);
                }
                const int8_t f = gradient_decision(pany[t], pall[t], cur.L, lo, hi);
                B.flags[pbase[py * 4 + px] / FLAT] = f;
                if (f != FLAG_STABLE) ctl->flagged = 1;
            }
        }
        // the stores have read the stage before the next steps write X, and
        // pbase, pany, pall and cf are free for the next block
        if (tid < 16) bulk_wait_read<0>();
        __syncthreads();
        if (!more) break;
        blk = nb;
        cur = nxt;
    }
    if (tid < 16) bulk_wait_all();
}

} // namespace amr_gb300
