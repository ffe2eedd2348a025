// Gradient flags of 2D 16x16 and 8x8 patches (bulk-copied tiles, all four
// ghost faces by the lanes, the FP32 band rule with FP64 inside the band),
// and the same flags on same-level trees from face records.
#pragma once

#include "amr_step2d.cuh"

namespace amr_gb300 {

// ------------------------------------------------ 2D gradient flags, sized at compile time
// One warp per patch (grid-stride).  The patch's interior rows move into a
// per-warp shared-memory tile by bulk async copy (double-buffered); the
// lanes fill all four ghost faces (lanes 0..N-1 the two ghost columns at row
// tg, lanes N..2N-1 the two ghost rows at column tg) by the halo rules, the
// values a halo exchange would store; FromBuffer copies the whole padded
// patch and takes the buffer's ghosts instead.  Each lane then applies the
// gradient rule (FP32 sum with the proven band, FP64 inside it, the same
// arithmetic as gradient_sq_cell) to N*N/32 cells and the warp votes.
template <typename T, int N, int H, bool FromBuffer>
struct Flags2dShape {
    static constexpr int      P1    = N + 2 * H;
    static constexpr int      FLAT  = P1 * P1;
    static constexpr uint32_t LO    = FromBuffer ? 0u : ((H * P1 * sizeof(T)) & ~15u);
    static constexpr uint32_t HI    = FromBuffer ? FLAT * sizeof(T) : (((N + H) * P1 * sizeof(T) + 15u) & ~15u);
    static constexpr uint32_t BYTES = HI - LO;
    static constexpr int      SEG   = N * N / 32;
    static constexpr size_t   TILE  = FLAT * sizeof(T);
    static_assert(TILE % 16 == 0 && HI <= TILE, "patch is not a whole number of 16-byte words");
    static_assert(32 % N == 0 && (32 / N) * SEG == N, "a lane's cells must form one column segment");
    static constexpr size_t smem(int W) { return static_cast<size_t>(W) * 2 * (TILE + 8); }
};

// FP64 squared gradient of a 2D cell from its four neighbour values, in
// gradient_sq_cell's order (Morton x, then y) and rounding.
template <typename T>
__device__ __forceinline__ double grad_sq_exact2(T xl, T xh, T yl, T yh)
{
    const double gx = __dmul_rn(0.5, __dsub_rn(static_cast<double>(xh), static_cast<double>(xl)));
    double       s  = __dadd_rn(0.0, __dmul_rn(gx, gx));
    const double gy = __dmul_rn(0.5, __dsub_rn(static_cast<double>(yh), static_cast<double>(yl)));
    return __dadd_rn(s, __dmul_rn(gy, gy));
}

template <typename T>
__device__ __forceinline__ float grad_sq_f32_2(T xl, T xh, T yl, T yh)
{
    float dx, dy;
    if constexpr (sizeof(T) == 4) {
        dx = xh - xl;
        dy = yh - yl;
    } else {
        dx = static_cast<float>(xh - xl);
        dy = static_cast<float>(yh - yl);
    }
    const float gx = 0.5f * dx, gy = 0.5f * dy;
    return fmaf(gy, gy, fmaf(gx, gx, 0.0f));
}

template <typename T, int N, int H, bool FromBuffer>
__device__ __forceinline__ void flags2d_body(const T* __restrict__ in, const amr_halo_meta* __restrict__ meta,
                                             const uint64_t* __restrict__ keys, int P, const Geo& g,
                                             const GradRule& rule, int min_level, int max_level,
                                             const int32_t* __restrict__ bounds, int8_t* __restrict__ flags,
                                             int32_t* err, T* tiles, uint64_t* bars, int p, int nwarp,
                                             int32_t* flagged = nullptr)
{
    using Sh                = Flags2dShape<T, N, H, FromBuffer>;
    constexpr int      P1   = Sh::P1;
    constexpr int      FLAT = Sh::FLAT;
    constexpr uint32_t LO = Sh::LO, BYTES = Sh::BYTES;
    constexpr int      SEG  = Sh::SEG;
    constexpr int      HALF = N / 2;
    const int          lane = threadIdx.x & 31;
    if (lane == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        mbar_init_fence();
    }
    __syncwarp();
    const char* in_bytes = reinterpret_cast<const char*>(in);
    auto        request  = [&](int q, int slot) {
        fence_proxy_async_smem();
        mbar_expect_tx(&bars[slot], BYTES);
        bulk_copy_g2s(reinterpret_cast<char*>(tiles + static_cast<size_t>(slot) * FLAT) + LO,
                      in_bytes + static_cast<size_t>(q) * FLAT * sizeof(T) + LO, BYTES, &bars[slot]);
    };
    if (p < P && lane == 0) request(p, 0);
    uint32_t   phase = 0;
    // column-segment mapping (conflict-free shared memory, see Step2dShape)
    const int  cl = lane % N + H, r0 = (lane / N) * SEG + H;
    // ghost jobs: lanes 0..N-1 column faces (normal layout dim 1) at row tg,
    // lanes N..2N-1 row faces (dim 0) at column tg; pos 0 and 1
    const bool col  = lane < N;
    const bool job  = !FromBuffer && lane < 2 * N;
    const int  L    = col ? 1 : 0;
    const int  tg   = (col ? lane : lane - N) + H;
    const int  fsel = (tg - H) / HALF;
    struct Rec {
        int rel, nb, fid, q0, q1;
    };
    auto rec_of = [&](int q, int pos, Rec& m) {
        m.rel = REL_NONE;
        if (!job) return;
        const amr_halo_meta* rp = meta + static_cast<size_t>(q) * 4 + 2 * L + pos;
        m.rel                   = rp->relation;
        m.nb                    = rp->neighbor;
        m.fid                   = rp->finer_ids[fsel];
        m.q0                    = rp->quadrant[0];
        m.q1                    = rp->quadrant[1];
    };
    // ghost cell (G0, G1) of face pos from record m: the halo rules of
    // ghost_value, rounded to T
    auto ghost = [&](int q, int pos, const Rec& m, int& G0, int& G1) -> T {
        const int gc = pos ? N + H : H - 1;
        G0           = col ? tg : gc;
        G1           = col ? gc : tg;
        const int sh = pos ? -N : N;
        int       f0 = G0 + (L == 0 ? sh : 0), f1 = G1 + (L == 1 ? sh : 0);
        if (m.rel == REL_SAME) return in[static_cast<size_t>(m.nb) * FLAT + f0 * P1 + f1];
        if (m.rel == REL_COARSER) {
            f0 = H + m.q0 * HALF + (f0 - H) / 2;
            f1 = H + m.q1 * HALF + (f1 - H) / 2;
            return in[static_cast<size_t>(m.nb) * FLAT + f0 * P1 + f1];
        }
        if (m.rel == REL_FINER) {
            f0           = ((f0 - H) * 2) % N + H;
            f1           = ((f1 - H) * 2) % N + H;
            const T* fp  = in + static_cast<size_t>(m.fid) * FLAT + f0 * P1 + f1;
            double   sum = static_cast<double>(fp[0]);
            sum += static_cast<double>(fp[1]);
            sum += static_cast<double>(fp[P1]);
            sum += static_cast<double>(fp[P1 + 1]);
            return static_cast<T>(sum / 4.0);
        }
        return in[static_cast<size_t>(q) * FLAT + G0 * P1 + G1];
    };
    Rec mn0{}, mn1{};
    if (p < P) {
        rec_of(p, 0, mn0);
        rec_of(p, 1, mn1);
    }
    for (int it = 0; p < P; ++it, p += nwarp) {
        const int b  = it & 1;
        const int pn = p + nwarp;
        if (pn < P && lane == 0) request(pn, b ^ 1);
        const uint64_t key = keys[p];
        const Rec      m0 = mn0, m1 = mn1;
        if (pn < P) {
            rec_of(pn, 0, mn0);
            rec_of(pn, 1, mn1);
        }
        T   gv0 = T(0), gv1 = T(0);
        int a0 = 0, a1 = 0, b0 = 0, b1 = 0;
        if (job) {
            gv0 = ghost(p, 0, m0, a0, a1);
            gv1 = ghost(p, 1, m1, b0, b1);
        }
        if (!mbar_wait_bounded(&bars[b], (phase >> b) & 1u)) {
            if (lane == 0) atomicExch(err, static_cast<int32_t>(AMR_ERR_TIMEOUT));
            phase ^= 1u << b;
            if (pn < P) mbar_wait_bounded(&bars[b ^ 1], (phase >> (b ^ 1)) & 1u);
            return;
        }
        phase ^= 1u << b;
        T* tile = tiles + static_cast<size_t>(b) * FLAT;
        if (job) {
            tile[a0 * P1 + a1] = gv0;
            tile[b0 * P1 + b1] = gv1;
        }
        __syncwarp();
        // Both decisions depend on the lane's largest squared gradient only
        // (refine: some cell at or above the threshold; coarsen: every cell
        // below it), so the FP32 maximum decides them when it lies outside
        // both bands and every FP32 value is finite; otherwise each cell is
        // evaluated exactly.  Same outcome as a per-cell decision.
        int   any = 0, all = 1;
        T     colv[SEG + 2];
        float smax = 0.0f;
        bool  bad  = false;
#pragma unroll
        for (int k = 0; k < SEG + 2; ++k) colv[k] = tile[(r0 - 1 + k) * P1 + cl];
#pragma unroll
        for (int k = 0; k < SEG; ++k) {
            const int   idx = (r0 + k) * P1 + cl;
            const float s   = grad_sq_f32_2<T>(tile[idx - 1], tile[idx + 1], colv[k], colv[k + 2]);
            smax            = fmaxf(smax, s);
            bad |= !(fabsf(s) < INFINITY);
        }
        const bool known = rule.fast && !bad && (smax >= rule.r_hi || smax < rule.r_lo) &&
                           (smax < rule.c_lo || smax >= rule.c_hi);
        if (known) {
            any = smax >= rule.r_hi ? 1 : 0;
            all = smax < rule.c_lo ? 1 : 0;
        } else {
#pragma unroll
            for (int k = 0; k < SEG; ++k) {
                const int    idx = (r0 + k) * P1 + cl;
                const double s   = grad_sq_exact2<T>(tile[idx - 1], tile[idx + 1], colv[k], colv[k + 2]);
                if (s >= rule.rsq) any = 1;
                if (!(s < rule.csq)) all = 0;
            }
        }
        any = __any_sync(0xffffffffu, any);
        all = __all_sync(0xffffffffu, all);
        if (lane == 0) {
            int lo = min_level, hi = max_level;
            if (bounds) {
                const int inst = g.inst_shift >= 64 ? 0 : static_cast<int>(key >> g.inst_shift);
                lo             = bounds[2 * inst];
                hi             = bounds[2 * inst + 1];
            }
            const int8_t f = gradient_decision(any, all, key_level(key), lo, hi);
            flags[p]       = f;
            if (flagged && f != FLAG_STABLE) *flagged = 1; // some leaf will change: the re-mesh runs
        }
        __syncwarp();
    }
}

// Gradient flags of a tree whose every relation is same-level (the graph
// intervals that run multi-step passes).  A ghost face is then a copy of the
// neighbour's edge line, so each lane fetches its two ghost values (lanes
// 0..N-1 the low and high ghost column at row tg, lanes N..2N-1 the low and
// high ghost row at column tg) one patch ahead, from the face record (all
// four neighbours) read two patches ahead; instance and level come from the
// pass record.  The cells, the gradient arithmetic and the decision are
// flags2d_body's, so the flags are identical.
template <typename T, int N, int H>
__device__ __forceinline__ void flags2d_uniform_body(const T* __restrict__ in, const int4* __restrict__ prec,
                                                     const int4* __restrict__ frec, int P, const GradRule& rule,
                                                     int min_level, int max_level, const int32_t* __restrict__ bounds,
                                                     int8_t* __restrict__ flags, int32_t* err, T* tiles,
                                                     uint64_t* bars, int p, int nwarp, int32_t* flagged)
{
    using Sh                = Flags2dShape<T, N, H, false>;
    constexpr int      P1   = Sh::P1;
    constexpr int      FLAT = Sh::FLAT;
    constexpr uint32_t LO = Sh::LO, BYTES = Sh::BYTES;
    constexpr int      SEG  = Sh::SEG;
    const int          lane = threadIdx.x & 31;
    if (lane == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        mbar_init_fence();
    }
    __syncwarp();
    const char* in_bytes = reinterpret_cast<const char*>(in);
    auto        request  = [&](int q, int slot) {
        fence_proxy_async_smem();
        mbar_expect_tx(&bars[slot], BYTES);
        bulk_copy_g2s(reinterpret_cast<char*>(tiles + static_cast<size_t>(slot) * FLAT) + LO,
                      in_bytes + static_cast<size_t>(q) * FLAT * sizeof(T) + LO, BYTES, &bars[slot]);
    };
    if (p < P && lane == 0) request(p, 0);
    uint32_t   phase = 0;
    const int  cl = lane % N + H, r0 = (lane / N) * SEG + H;
    const bool col = lane < N;
    const bool job = lane < 2 * N;
    const int  tg  = (col ? lane : lane - N) + H;
    // the lane's ghost cells in the tile and their sources in the low / high
    // neighbour (the neighbour's last / first interior line)
    const int  g0 = col ? tg * P1 + (H - 1) : (H - 1) * P1 + tg;
    const int  g1 = col ? tg * P1 + (N + H) : (N + H) * P1 + tg;
    const int  s0 = col ? tg * P1 + (N + H - 1) : (N + H - 1) * P1 + tg;
    const int  s1 = col ? tg * P1 + H : H * P1 + tg;
    auto       fetch = [&](const int4& f, T& a, T& b) {
        a = b = T(0);
        if (!job) return;
        a = in[static_cast<size_t>(col ? f.x : f.z) * FLAT + s0];
        b = in[static_cast<size_t>(col ? f.y : f.w) * FLAT + s1];
    };
    // face records two patches ahead, ghost values one ahead
    int4 f0{}, f1{}, f2{};
    int  c0 = 0, c1 = 0, c2 = 0;
    T    ga = T(0), gb = T(0), na = T(0), nb = T(0);
    if (p < P) {
        f0 = __ldg(frec + p);
        c0 = __ldg(&prec[p].w);
        fetch(f0, ga, gb);
    }
    if (p + nwarp < P) {
        f1 = __ldg(frec + p + nwarp);
        c1 = __ldg(&prec[p + nwarp].w);
    }
    for (int it = 0; p < P; ++it, p += nwarp) {
        const int b  = it & 1;
        const int pn = p + nwarp, pm = p + 2 * nwarp;
        if (pn < P && lane == 0) request(pn, b ^ 1);
        if (pm < P) {
            f2 = __ldg(frec + pm);
            c2 = __ldg(&prec[pm].w);
        }
        if (pn < P) fetch(f1, na, nb);
        if (!mbar_wait_bounded(&bars[b], (phase >> b) & 1u)) {
            if (lane == 0) atomicExch(err, static_cast<int32_t>(AMR_ERR_TIMEOUT));
            phase ^= 1u << b;
            if (pn < P) mbar_wait_bounded(&bars[b ^ 1], (phase >> (b ^ 1)) & 1u);
            return;
        }
        phase ^= 1u << b;
        T* tile = tiles + static_cast<size_t>(b) * FLAT;
        if (job) {
            tile[g0] = ga;
            tile[g1] = gb;
        }
        __syncwarp();
        // the decision rule of flags2d_body: the lane's FP32 maximum decides
        // unless it lies in a band or some value is not finite
        int   any = 0, all = 1;
        T     colv[SEG + 2];
        float smax = 0.0f;
        bool  bad  = false;
#pragma unroll
        for (int k = 0; k < SEG + 2; ++k) colv[k] = tile[(r0 - 1 + k) * P1 + cl];
#pragma unroll
        for (int k = 0; k < SEG; ++k) {
            const int   idx = (r0 + k) * P1 + cl;
            const float s   = grad_sq_f32_2<T>(tile[idx - 1], tile[idx + 1], colv[k], colv[k + 2]);
            smax            = fmaxf(smax, s);
            bad |= !(fabsf(s) < INFINITY);
        }
        const bool known = rule.fast && !bad && (smax >= rule.r_hi || smax < rule.r_lo) &&
                           (smax < rule.c_lo || smax >= rule.c_hi);
        if (known) {
            any = smax >= rule.r_hi ? 1 : 0;
            all = smax < rule.c_lo ? 1 : 0;
        } else {
#pragma unroll
            for (int k = 0; k < SEG; ++k) {
                const int    idx = (r0 + k) * P1 + cl;
                const double s   = grad_sq_exact2<T>(tile[idx - 1], tile[idx + 1], colv[k], colv[k + 2]);
                if (s >= rule.rsq) any = 1;
                if (!(s < rule.csq)) all = 0;
            }
        }
        any = __any_sync(0xffffffffu, any);
        all = __all_sync(0xffffffffu, all);
        if (lane == 0) {
            int lo = min_level, hi = max_level;
            if (bounds) {
                const int inst = pass_inst(c0);
                lo             = bounds[2 * inst];
                hi             = bounds[2 * inst + 1];
            }
            const int8_t f = gradient_decision(any, all, pass_level(c0), lo, hi);
            flags[p]       = f;
            if (f != FLAG_STABLE) *flagged = 1; // some leaf will change: the re-mesh runs
        }
        __syncwarp();
        f0 = f1;
        f1 = f2;
        c0 = c1;
        c1 = c2;
        ga = na;
        gb = nb;
    }
}

template <typename T, int N, int H, bool FromBuffer>
__device__ __forceinline__ void flags2d_smem(unsigned char* smem, int W, T*& tiles, uint64_t*& bars)
{
    using Sh      = Flags2dShape<T, N, H, FromBuffer>;
    const int wib = threadIdx.x >> 5;
    tiles         = reinterpret_cast<T*>(smem) + static_cast<size_t>(wib) * 2 * Sh::FLAT;
    bars          = reinterpret_cast<uint64_t*>(smem + static_cast<size_t>(W) * 2 * Sh::TILE) + wib * 2;
}

template <typename T, int N, int H, bool FromBuffer>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 4 : 3)
k_flags2d(const T* __restrict__ in, const amr_halo_meta* __restrict__ meta, const uint64_t* __restrict__ keys, int P,
          Geo g, GradRule rule, int min_level, int max_level, const int32_t* __restrict__ bounds,
          int8_t* __restrict__ flags, int32_t* err)
{
    extern __shared__ __align__(128) unsigned char smem[];
    T*        tiles;
    uint64_t* bars;
    flags2d_smem<T, N, H, FromBuffer>(smem, blockDim.x >> 5, tiles, bars);
    const int nwarp = (gridDim.x * blockDim.x) >> 5;
    const int p     = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    flags2d_body<T, N, H, FromBuffer>(in, meta, keys, P, g, rule, min_level, max_level, bounds, flags, err, tiles, bars,
                                      p, nwarp);
}

} // namespace amr_gb300
