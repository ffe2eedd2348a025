// Fused re-mesh interval of the 2D FP32 forest: D update steps and the
// gradient flags of the interval's end state in one pass over memory.
//
// Applies to trees whose every neighbour relation is "same level" (each
// instance uniform at its own level L >= 2, as the batched forests are) with
// 16x16 patches and one ghost layer.  In Morton order the 16 leaves
// 16b .. 16b+15 of such a tree are one aligned 4x4 block of patches of one
// instance (64x64 cells), described by the key of leaf 16b alone; its
// neighbour patches follow from the block's position and the instance's
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
// The guard kernel k_run_require_blocks checks that each block is one aligned
// 4x4 block of one instance at a level >= 2 and writes its descriptor; the
// fused kernel checks that every leaf of a block's neighbourhood lies in the
// tree before it issues a copy.
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
    static constexpr int XS   = TY * RY + 1;    // X column pitch in pairs (odd: 64-bit accesses hit distinct banks)
    static constexpr int TILES = 6 * (800 + 4 * 1168 + 80); // packed tile rows (bytes), either mirroring
    static constexpr int STAGE = 292;           // floats per staged patch: padded indices 16 .. 307
    static_assert(RW % 4 == 0, "region width is a multiple of four columns");
    static_assert(TY * RY >= RW, "row groups cover the region");
    static_assert(XS % 2 == 1, "odd X pitch");
    static_assert(D == 10, "tile packing sized for ten steps");
    // shared memory: tiles | X (2 buffers x (TX + 1) columns x XS pairs; the
    // output stage once the flags are done) | Y (2 buffers x 2 pairs x (TY +
    // 1) rows x TX) | patch bases, flags, slot table, coefficients, barrier
    static constexpr size_t x_bytes = 2 * (TX + 1) * XS * 8;
    static constexpr int    YB      = (TY + 1) * TX; // pairs of one Y array
    static constexpr size_t y_bytes = 2 * 2 * YB * 8;
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
// with the per-leaf kernels.  For each block it writes the descriptor the
// fused kernel reads (blocks[b], see IntervalBlock), so that kernel needs no
// dependent loads of keys and upwind codes.
static __global__ void __launch_bounds__(256) k_run_require_blocks(RunBufs B, RunCtl* ctl, Geo g, int upx0, int upy0)
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
        if (L < 2 || key_level(k15) != L || key_prefix(g, k15) != key_prefix(g, k0) || (m0 & 15u) != 0u) {
            atomicCAS(&ctl->err, 0, kRetryFused);
            continue;
        }
        const int inst = g.inst_shift >= 64 ? 0 : static_cast<int>(k0 >> g.inst_shift);
        int       ux = upx0, uy = upy0;
        if (B.upcode) {
            const int32_t code = B.upcode[inst];
            ux                 = unpack_upwind(code, 0);
            uy                 = unpack_upwind(code, 1);
        }
        B.frec[b] = make_int4(16 * b - static_cast<int>(m0), L | (inst << 8),
                              static_cast<int>(compact2(m0)) | (static_cast<int>(compact2(m0 >> 1)) << 16),
                              (ux + 1) | ((uy + 1) << 2));
    }
}

// What a CTA knows about one block, decoded from its descriptor
// (k_run_require_blocks): x = leaf index of the instance's first patch,
// y = level | instance << 8, z = block origin x | y << 16 (patch
// coordinates), w = (upwind x + 1) | (upwind y + 1) << 2.
struct IntervalBlock {
    int base, L, inst, bx0, by0, ux, uy;
};
__device__ __forceinline__ IntervalBlock interval_block(int4 d)
{
    IntervalBlock b;
    b.base = d.x;
    b.L    = d.y & 255;
    b.inst = d.y >> 8;
    b.bx0  = d.z & 0xFFFF;
    b.by0  = d.z >> 16;
    b.ux   = (d.w & 3) - 1;
    b.uy   = ((d.w >> 2) & 3) - 1;
    return b;
}

template <int D, bool FLAGS>
__global__ void __launch_bounds__(IntervalShape<D>::THREADS, 3)
k_run_interval2d(RunBufs B, RunCtl* ctl, Geo g, const float2* __restrict__ coef32, size_t cstride, int nl,
                 GradRule rule, int min_level, int max_level, int parity)
{
    using S                = IntervalShape<D>;
    constexpr int TX       = S::TX, RY = S::RY, XS = S::XS, HALO = S::HALO, HW = S::HW, YB = S::YB;
    constexpr int FLAT     = S::FLAT, STAGE = S::STAGE;
    if (ctl->err) return;
    extern __shared__ __align__(128) unsigned char smem[];
    unsigned char* tiles = smem;
    uint64_t*      Xb    = reinterpret_cast<uint64_t*>(smem + S::TILES);
    float*         stage = reinterpret_cast<float*>(smem + S::TILES); // aliases X after the flags
    uint64_t*      Yb    = reinterpret_cast<uint64_t*>(smem + S::TILES + S::x_bytes);
    int*           pbase = reinterpret_cast<int*>(smem + S::TILES + S::x_bytes + S::y_bytes);
    int*           pany  = pbase + 16;
    int*           pall  = pany + 16;
    int*           slot  = pall + 16; // per patch row of the tiles: lo, size, start (6 x 3, padded)
    ulonglong2*    cf    = reinterpret_cast<ulonglong2*>(slot + 24); // (c_x, c_x), (c_y, c_y) per step
    uint64_t*      bar   = reinterpret_cast<uint64_t*>(cf + D);

    const int tid = threadIdx.x;
    const int tx = tid % TX, ty = tid / TX;
    const int P = ctl->P, s = ctl->sb ^ parity;
    const float* __restrict__ in   = static_cast<const float*>(B.state[s]);
    float* __restrict__       out  = static_cast<float*>(B.state[s ^ 1]);
    const int4* __restrict__  desc = B.frec; // block descriptors (k_run_require_blocks)
    const int nblk = P / 16;
    if (tid == 0) {
        mbar_init(bar, 1);
        mbar_init_fence();
    }
    // rows above the region in the Y arrays are never written: zero once
    for (int i = tid; i < 4 * TX; i += blockDim.x) Yb[(i / TX) * YB + (i % TX)] = 0ull;
    __syncthreads();

    // leaf of actual block-relative patch offsets (px, py), periodic
    auto leaf_at = [&](const IntervalBlock& b, int px, int py) -> int {
        const int      Wm = (1 << b.L) - 1;
        const uint32_t x = static_cast<uint32_t>((b.bx0 + px) & Wm), y = static_cast<uint32_t>((b.by0 + py) & Wm);
        return b.base + static_cast<int>(spread2(x) | (spread2(y) << 1));
    };
    // every leaf of the block's 6x6 neighbourhood inside the tree (checked
    // before any copy is issued: the neighbourhood lies in the instance's
    // leaf range [base, base + 4^L), the same for every thread), its copies
    // and slot table; false when that range leaves the tree (nothing issued:
    // the CTA leaves).  The barrier orders every earlier read of the tiles
    // and of the slot table before the copies and the new table; the next
    // block's wait barrier orders the new table before its reads.
    auto issue = [&](const IntervalBlock& b) -> bool {
        if (b.L < 2 || b.base < 0 || static_cast<long long>(b.base) + (1ll << (2 * b.L)) > P) {
            if (tid == 0) atomicCAS(&ctl->err, 0, static_cast<int32_t>(AMR_ERR_UNBALANCED));
            return false;
        }
        const bool sy = b.uy > 0;
        if (tid == 0) mbar_expect_tx(bar, S::TILES); // either mirroring packs to TILES bytes
        __syncthreads(); // the tiles and the slot table were only read since their last copies
        if (tid >= 64 && tid < 70) {
            uint32_t lo, size, start;
            interval_slot_row<D>(tid - 65, sy, lo, size, start);
            slot[3 * (tid - 64)]     = static_cast<int>(lo);
            slot[3 * (tid - 64) + 1] = static_cast<int>(size);
            slot[3 * (tid - 64) + 2] = static_cast<int>(start);
        }
        if (tid < 36) {
            const int py = tid / 6 - 1, px = tid % 6 - 1;
            uint32_t  lo, size, start;
            interval_slot_row<D>(py, sy, lo, size, start);
            const char* src = reinterpret_cast<const char*>(in + static_cast<size_t>(leaf_at(b, px, py)) * FLAT);
            bulk_copy_g2s(tiles + start + (px + 1) * size, src + lo, size, bar);
        }
        return true;
    };

    // per block, loaded one block ahead so that no global load sits on the
    // path between two barriers: threads < D its coefficient row of step tid,
    // threads 128 .. 143 its instance's level bounds
    auto coef_of = [&](const IntervalBlock& b) -> float2 {
        return tid < D ? __ldg(coef32 + tid * cstride + static_cast<size_t>(b.inst) * nl + b.L) : float2{};
    };
    auto bounds_of = [&](const IntervalBlock& b) -> int2 {
        if (!FLAGS || tid < 128 || tid >= 144) return make_int2(min_level, max_level);
        return B.bounds ? make_int2(__ldg(B.bounds + 2 * b.inst), __ldg(B.bounds + 2 * b.inst + 1))
                        : make_int2(min_level, max_level);
    };
    uint32_t      phase = 0;
    int           blk   = blockIdx.x;
    if (blk >= nblk) return;
    IntervalBlock cur    = interval_block(__ldg(desc + blk));
    float2        ccoef  = coef_of(cur);
    int2          cbound = bounds_of(cur);
    if (!issue(cur)) return;

    while (true) {
        // the next block's descriptor, needed after this block's register load
        const int  nb   = blk + static_cast<int>(gridDim.x);
        const bool more = nb < nblk;
        const int4 dn   = more ? __ldg(desc + nb) : make_int4(0, 0, 0, 0);
        // ---- 1. the copies of this block
        if (__syncthreads_or(mbar_wait_bounded(bar, phase) ? 0 : 1)) {
            if (tid == 0) atomicExch(&ctl->err, static_cast<int32_t>(AMR_ERR_TIMEOUT));
            mbar_wait_bounded(bar, phase); // copies still in flight land before the CTA goes
            if (tid < 16) bulk_wait_all();
            return;
        }
        phase ^= 1u;
        const bool sx = cur.ux > 0, sy = cur.uy > 0;
        if (tid < D) cf[tid] = make_ulonglong2(pk(ccoef.x, ccoef.x), pk(ccoef.y, ccoef.y));
        if (tid < 16) {
            const int px = tid & 3, py = tid >> 2; // actual block patch
            pbase[tid]   = leaf_at(cur, px, py) * FLAT;
            pany[tid]    = 0;
            pall[tid]    = 1;
        }

        // ---- 2. the thread's cells into registers
        // column k of the thread: 0 -> p1.lo, 1 -> p2.lo, 2 -> p1.hi, 3 -> p2.hi;
        // its actual block column X, slot column and byte offset in the row
        const int c0 = 2 * tx - HALO;
        int       colX[4], cslot[4], cbyte[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int c = c0 + (k & 1) + (k >> 1) * HW;
            colX[k]     = sx ? 63 - c : c;
            cslot[k]    = (colX[k] >> 4) + 1;
            cbyte[k]    = ((colX[k] & 15) + 1) * 4;
        }
        const int r0 = ty * RY - HALO;
        uint64_t  v1[RY], v2[RY];
        // the thread's rows cross at most one patch-row boundary: the slot
        // entries of the first row's patch row (A) and of the next one (B),
        // and per column the byte offset of row 0 in each
        const int YA  = sy ? 63 - r0 : r0;
        const int pyA = YA >> 4;
        const int pyB = max(-1, min(4, sy ? pyA - 1 : pyA + 1));
        int       offA[4], offB[4];
        {
            const int* sa = slot + 3 * (pyA + 1);
            const int* sb = slot + 3 * (pyB + 1);
            const int  a0 = sa[0], a1 = sa[1], a2 = sa[2], b0 = sb[0], b1 = sb[1], b2 = sb[2];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                offA[k] = a2 - a0 + cslot[k] * a1 + cbyte[k];
                offB[k] = b2 - b0 + cslot[k] * b1 + cbyte[k];
            }
        }
#pragma unroll
        for (int i = 0; i < RY; ++i) {
            const int r    = r0 + i;
            float     e[4] = { 0.0f, 0.0f, 0.0f, 0.0f };
            if (r <= 64) {
                const int  Y   = sy ? 63 - r : r;
                const bool inA = (Y >> 4) == pyA;
                const int  ro  = ((Y & 15) + 1) * 72;
#pragma unroll
                for (int k = 0; k < 4; ++k)
                    e[k] = *reinterpret_cast<const float*>(tiles + (inA ? offA[k] : offB[k]) + ro);
            }
            v1[i] = pk(e[0], e[2]);
            v2[i] = pk(e[1], e[3]);
        }
        // ---- the next block's copies land during this block's steps
        IntervalBlock nxt{};
        float2        ncoef{};
        int2          nbound{};
        if (more) {
            nxt    = interval_block(dn);
            ncoef  = coef_of(nxt);
            nbound = bounds_of(nxt);
            if (!issue(nxt)) {
                if (tid < 16) bulk_wait_all();
                return;
            }
        } else {
            __syncthreads(); // pbase, cf and the flags' zeroing are visible
        }

        // ---- 3. D steps; X column tx + 1 holds thread tx's p2, read by thread
        // tx + 1 as the x-neighbour of its p1.  The last thread's column is
        // read only by thread 0, whose second half's x-neighbour is the first
        // half's last column (that thread's p2 low word): the last thread
        // publishes its low word in both words, every other thread its p2,
        // and thread 0 reads column TX instead of column 0
        const bool      last = tx == TX - 1;
        const int       xsrc = tx == 0 ? TX : tx;
        auto            pub  = [&](uint64_t v) { return last ? pk(pk_lo(v), pk_lo(v)) : v; };
        auto steps = [&]<bool XU, bool YU>() {
#pragma unroll
            for (int m = 0; m < D; ++m) {
                uint64_t* const X  = Xb + (m & 1) * (TX + 1) * XS;
                uint64_t* const Y1 = Yb + (m & 1) * 2 * YB;
                uint64_t* const Y2 = Y1 + YB;
                {
                    uint64_t* xo = X + (tx + 1) * XS + ty * RY;
#pragma unroll
                    for (int i = 0; i < RY; ++i) xo[i] = pub(v2[i]);
                    Y1[(ty + 1) * TX + tx] = v1[RY - 1];
                    Y2[(ty + 1) * TX + tx] = v2[RY - 1];
                }
                __syncthreads();
                const ulonglong2 c  = cf[m];
                const uint64_t   y1 = Y1[ty * TX + tx], y2 = Y2[ty * TX + tx];
                const uint64_t*  xi = X + xsrc * XS + ty * RY;
#pragma unroll
                for (int i = RY - 1; i >= 0; --i) {
                    // p2 first: its x-neighbour is p1
                    v2[i] = upd_pair<XU, YU>(v2[i], v1[i], i > 0 ? v2[i - 1] : y2, c.x, c.y);
                    v1[i] = upd_pair<XU, YU>(v1[i], xi[i], i > 0 ? v1[i - 1] : y1, c.x, c.y);
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
            // (X buffer 1), last row down, first row up (Y buffer 0)
            uint64_t* const XL  = Xb;
            uint64_t* const XR  = Xb + (TX + 1) * XS;
            uint64_t* const YD1 = Yb;
            uint64_t* const YD2 = Yb + YB;
            uint64_t* const YU1 = Yb + 2 * YB;
            uint64_t* const YU2 = Yb + 3 * YB;
            {
                // XR column tx holds thread tx's p1, read by thread tx - 1 as
                // the right neighbour of its p2; thread 0's column is read only
                // by the last thread, whose first half's last column has the
                // second half's first column (thread 0's p1 high word) to its
                // right: thread 0 publishes that word in both words
                uint64_t* a = XL + (tx + 1) * XS + ty * RY;
                uint64_t* b = XR + tx * XS + ty * RY;
#pragma unroll
                for (int i = 0; i < RY; ++i) {
                    a[i] = pub(v2[i]);
                    b[i] = tx == 0 ? pk(pk_hi(v1[i]), pk_hi(v1[i])) : v1[i];
                }
                YD1[(ty + 1) * TX + tx] = v1[RY - 1];
                YD2[(ty + 1) * TX + tx] = v2[RY - 1];
                YU1[ty * TX + tx]       = v1[0];
                YU2[ty * TX + tx]       = v2[0];
            }
            __syncthreads();
            const uint64_t ya1 = YD1[ty * TX + tx], ya2 = YD2[ty * TX + tx];             // the row above row 0
            const uint64_t yb1 = YU1[(ty + 1) * TX + tx], yb2 = YU2[(ty + 1) * TX + tx]; // below row RY - 1
            const uint64_t* xl = XL + xsrc * XS + ty * RY;
            const uint64_t* xr = XR + (last ? 0 : tx + 1) * XS + ty * RY;
            // per column k and patch-row part (the thread's rows cross at most
            // one patch boundary): the largest FP32 squared gradient as a bit
            // pattern (s >= +0 or NaN, so unsigned order is value order and
            // a pattern >= that of +inf means some value is not finite)
            const int ra = max(r0, 0), rb = min(r0 + RY - 1, 63);
            const int split = ((ra >> 4) + 1) * 16; // first row of the second part
            uint32_t  m0[4] = { 0u, 0u, 0u, 0u }, m1[4] = { 0u, 0u, 0u, 0u };
#pragma unroll
            for (int i = 0; i < RY; ++i) {
                const int      r   = r0 + i;
                const uint64_t up1 = i > 0 ? v1[i - 1] : ya1, dn1 = i < RY - 1 ? v1[i + 1] : yb1;
                const uint64_t up2 = i > 0 ? v2[i - 1] : ya2, dn2 = i < RY - 1 ? v2[i + 1] : yb2;
                const uint64_t s1  = grad_pair(xl[i], v2[i], up1, dn1);
                const uint64_t s2  = grad_pair(v1[i], xr[i], up2, dn2);
                const uint32_t e[4] = { pk_lo_bits(s1), pk_lo_bits(s2), pk_hi_bits(s1), pk_hi_bits(s2) };
                const bool     inr = r >= ra && r <= rb, hi = r >= split;
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const uint32_t v = inr ? e[k] : 0u;
                    m0[k]            = max(m0[k], hi ? 0u : v);
                    m1[k]            = max(m1[k], hi ? v : 0u);
                }
            }
            // per (column k, part h), bit 4h + k: decided by the FP32 maximum
            // unless it lies in a band or some value is not finite; those take
            // the exact rule
            uint32_t kn = 0, an = 0, al = 0;
#pragma unroll
            for (int b = 0; b < 8; ++b) {
                const uint32_t mb = b < 4 ? m0[b] : m1[b - 4];
                const float    sm = __uint_as_float(mb);
                const bool     k1 = rule.fast && mb < 0x7f800000u && (sm >= rule.r_hi || sm < rule.r_lo) &&
                                (sm < rule.c_lo || sm >= rule.c_hi);
                kn |= (k1 ? 1u : 0u) << b;
                an |= (k1 && sm >= rule.r_hi ? 1u : 0u) << b;
                al |= (!k1 || sm < rule.c_lo ? 1u : 0u) << b;
            }
            if (kn != 0xFFu) { // the exact FP64 rule on every cell of the undecided parts
#pragma unroll
                for (int i = 0; i < RY; ++i) {
                    const int r = r0 + i;
                    if (r < ra || r > rb) continue;
                    const int      sh  = r >= split ? 4 : 0;
                    const uint64_t up1 = i > 0 ? v1[i - 1] : ya1, dn1 = i < RY - 1 ? v1[i + 1] : yb1;
                    const uint64_t up2 = i > 0 ? v2[i - 1] : ya2, dn2 = i < RY - 1 ? v2[i + 1] : yb2;
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        if ((kn >> (sh + k)) & 1u) continue;
                        const uint64_t up = k & 1 ? up2 : up1, dn = k & 1 ? dn2 : dn1;
                        const uint64_t wl = k & 1 ? v1[i] : xl[i], wh = k & 1 ? xr[i] : v2[i];
                        const bool     hh = (k >> 1) != 0;
                        const double   e  = grad_sq_exact2<float>(hh ? pk_hi(wl) : pk_lo(wl), hh ? pk_hi(wh) : pk_lo(wh),
                                                                  hh ? pk_hi(up) : pk_lo(up), hh ? pk_hi(dn) : pk_lo(dn));
                        if (e >= rule.rsq) an |= 1u << (sh + k);
                        if (!(e < rule.csq)) al &= ~(1u << (sh + k));
                    }
                }
            }
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int c = c0 + (k & 1) + (k >> 1) * HW;
                if (c < 0 || c > 63 || ra > rb) continue;
                const int pc = c >> 4;
                if (ra <= min(rb, split - 1)) { // part 0
                    const int pb = (ra >> 4) * 4 + pc;
                    if ((an >> k) & 1u) atomicOr(&pany[pb], 1);
                    if (!((al >> k) & 1u)) atomicAnd(&pall[pb], 0);
                }
                if (split <= rb) { // part 1
                    const int pb = (split >> 4) * 4 + pc;
                    if ((an >> (4 + k)) & 1u) atomicOr(&pany[pb], 1);
                    if (!((al >> (4 + k)) & 1u)) atomicAnd(&pall[pb], 0);
                }
            }
            __syncthreads(); // the exchange reads end before the stage overwrites X
        }

        // ---- 5. the block's padded rows 1..16 into the stage (patch p =
        // px + 4 py keeps padded indices 16 .. 307 at p * STAGE); column X of
        // a patch's row also serves as the ghost column of its neighbour in
        // the block (X & 15 == 15: the next patch's column 0; X & 15 == 0:
        // the previous patch's column 17).  Offsets per column k, -1 = none.
        {
            int oi[4], og[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int X = colX[k];
                oi[k]       = (X >= 0 && X <= 63) ? (X >> 4) * STAGE + (X & 15) + 1 : -1;
                og[k]       = ((X & 15) == 15 && X + 1 >= 0 && X + 1 <= 63)  ? ((X + 1) >> 4) * STAGE
                              : ((X & 15) == 0 && X - 1 >= 0 && X - 1 <= 63) ? ((X - 1) >> 4) * STAGE + 17
                                                                             : -1;
            }
#pragma unroll
            for (int i = 0; i < RY; ++i) {
                const int r = r0 + i;
                if (r >= 0 && r <= 63) {
                    const int   Y    = sy ? 63 - r : r;
                    float*      srow = stage + (Y >> 4) * 4 * STAGE + ((Y & 15) + 1) * 18 - 16;
                    const float e[4] = { pk_lo(v1[i]), pk_lo(v2[i]), pk_hi(v1[i]), pk_hi(v2[i]) };
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        if (oi[k] >= 0) srow[oi[k]] = e[k];
                        if (og[k] >= 0) srow[og[k]] = e[k];
                    }
                }
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
                const int8_t f = gradient_decision(pany[t], pall[t], cur.L, cbound.x, cbound.y);
                B.flags[pbase[py * 4 + px] / FLAT] = f;
                if (f != FLAG_STABLE) ctl->flagged = 1;
            }
        }
        // the stores have read the stage before the next steps write X, and
        // pbase, pany, pall and cf are free for the next block
        if (tid < 16) bulk_wait_read<0>();
        __syncthreads();
        if (!more) break;
        blk    = nb;
        cur    = nxt;
        ccoef  = ncoef;
        cbound = nbound;
    }
    if (tid < 16) bulk_wait_all();
}

} // namespace amr_gb300
