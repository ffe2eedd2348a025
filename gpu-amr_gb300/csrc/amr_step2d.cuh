// 2D forward-Euler updates of 16x16 and 8x8 patches: the one-step kernel (one
// warp per patch, bulk-copied tiles), the pass records and the multi-step
// pass for same-level trees.
#pragma once

#include "amr_kernels.cuh"

namespace amr_gb300 {

// ------------------------------------------------ 2D update, sized at compile time
// One warp per patch (grid-stride over patches: the Morton-ordered leaf array
// of every instance is the work list).  The whole padded patch is contiguous,
// so it moves into a per-warp shared-memory tile with one bulk async copy
// (cp.async.bulk, completed on an mbarrier).  Each warp owns S tiles in a
// ring and keeps S-1 copies in flight ahead of the patch it works on (S = 1:
// load, then compute).  Lanes write the upwind ghost column and ghost row
// into the tile (halo rules, ghost_value), each lane updates a contiguous run
// of N*N/32 interior cells, the results go back into the tile, and the tile
// is stored to the output patch whole in 16-byte words (ghost cells pass
// through), so every HBM access is a full aligned sector.  A copy that does
// not land within the wait cap sets *err = AMR_ERR_TIMEOUT; the warp then
// drains its other copies (also capped) and stops.
template <typename T, int N, int H>
struct Step2dShape {
    static constexpr int P1   = N + 2 * H;
    static constexpr int FLAT = P1 * P1;
    // Only the interior rows are read and written: the 16-byte-aligned byte
    // span [LO, HI) covering rows H .. N+H-1 (ghost columns included).  The
    // upwind ghost row and column are evaluated on the fly, the other ghost
    // cells are never read.
    static constexpr uint32_t LO    = (H * P1 * sizeof(T)) & ~15u;
    static constexpr uint32_t HI    = ((N + H) * P1 * sizeof(T) + 15u) & ~15u;
    static constexpr uint32_t BYTES = HI - LO;
    static constexpr int      WORDS = BYTES / 16;
    // Each lane updates a column segment: column (lane % N), rows
    // (lane / N) * SEG .. + SEG - 1 (interior coordinates).  For a fixed row
    // offset the warp reads whole rows, so shared-memory accesses are free of
    // bank conflicts, and the y-neighbours of a lane's cells are its own
    // registers.
    static constexpr int      RG    = 32 / N;      // row groups
    static constexpr int      SEG   = N * N / 32;  // interior cells per lane
    static constexpr size_t   TILE  = FLAT * sizeof(T);
    static_assert(TILE % 16 == 0 && HI <= TILE, "patch is not a whole number of 16-byte words");
    static_assert(32 % N == 0 && RG * SEG == N, "a lane's cells must form one column segment");
    // dynamic shared memory of a block of W warps with S tiles each
    static constexpr size_t smem(int W, int S) { return static_cast<size_t>(W) * S * (TILE + 8); }
};

// Coefficients of one (step, instance, level) row as the 2D kernel reads
// them: FP32 needs only (c_x, c_y) (difference form), FP64 (c0, c_x, c_y).
template <typename T>
struct Coef2 {
    double c0, cx, cy;
};
template <>
struct Coef2<float> {
    float cx, cy;
};

// One cell update of the 2D kernels from the cell u, its upwind x neighbour
// xn and upwind y neighbour yn.  FP32: u + c (u_up - u), exact for a constant
// state, so the rounding of the coefficients does not bias the solution;
// FP64: c0 u + c_x u_x + c_y u_y.  Every 2D update goes through this one
// function, so fused and separate steps round alike.
template <typename T>
__device__ __forceinline__ T upd2d_core(T u, T xn, T yn, const Coef2<T>& cf, bool xu, bool yu)
{
    if constexpr (sizeof(T) == 4) {
        float acc = u;
        if (xu) acc = fmaf(cf.cx, xn - u, acc);
        if (yu) acc = fmaf(cf.cy, yn - u, acc);
        return acc;
    } else {
        T acc = static_cast<T>(cf.c0) * u;
        if (xu) acc = fma(static_cast<T>(cf.cx), xn, acc);
        if (yu) acc = fma(static_cast<T>(cf.cy), yn, acc);
        return acc;
    }
}
template <typename T>
__device__ __forceinline__ T upd2d(T u, T xn, T yn, const Coef2<T>& cf, int ux, int uy)
{
    return upd2d_core<T>(u, xn, yn, cf, ux != 0, uy != 0);
}
// The same update with the upwind axes known at compile time (the multi-step
// pass branches once per patch on them).
template <typename T, bool XU, bool YU>
__device__ __forceinline__ T upd2d_fixed(T u, T xn, T yn, const Coef2<T>& cf)
{
    return upd2d_core<T>(u, xn, yn, cf, XU, YU);
}

// coef: the full rows (FP64 path); coef32: (c_x, c_y) rows (FP32 path);
// upcode: per-instance packed upwind offsets, or nullptr for upx0/upy0.
template <typename T, int N, int H, int S>
__device__ __forceinline__ void step2d_body(const T* __restrict__ in, T* __restrict__ out,
                                            const amr_halo_meta* __restrict__ meta, int P, const Geo& g,
                                            const Coef* __restrict__ coef, const float2* __restrict__ coef32,
                                            int upx0, int upy0, int32_t* err, const uint64_t* __restrict__ keys,
                                            const int32_t* __restrict__ upcode, T* tiles, uint64_t* bars, int p,
                                            int nwarp)
{
    using Sh                = Step2dShape<T, N, H>;
    constexpr int      P1   = Sh::P1;
    constexpr int      FLAT = Sh::FLAT;
    constexpr uint32_t LO = Sh::LO, BYTES = Sh::BYTES;
    constexpr int      SEG  = Sh::SEG;
    constexpr int      HALF = N / 2;
    const int          lane = threadIdx.x & 31;
    if (lane == 0) {
        for (int b = 0; b < S; ++b) mbar_init(&bars[b], 1);
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
    // prologue: copies for the first S-1 patches of this warp
    if (lane == 0)
        for (int j = 0; j < S - 1; ++j)
            if (p + j * nwarp < P) request(p + j * nwarp, j);
    uint32_t  phase = 0; // bit b: parity of slot b's next completion
    const int cl = lane % N + H, r0 = (lane / N) * SEG + H; // this lane's column and first row
    const int nl = g.depth + 1;

    // Ghost job of this lane: lanes 0..N-1 the upwind ghost column (normal
    // layout dim 1), lanes N..2N-1 the upwind ghost row (dim 0); tg is the
    // tangential padded coordinate, fsel the finer-neighbour section it lies in.
    const bool col  = lane < N;
    const bool job  = lane < 2 * N;
    const int  L    = col ? 1 : 0;
    const int  tg   = (col ? lane : lane - N) + H;
    const int  fsel = (tg - H) / HALF;

    // Per-patch metadata, software-pipelined so that no load is consumed in
    // the iteration that issues it: the key three patches ahead, the upwind
    // sides, coefficient row and this lane's neighbour record two ahead, the
    // raw ghost source values one ahead.  The instance comes from the key;
    // the upwind sides from its velocity (vel != nullptr) or upx0/upy0.
    struct Side {
        int      ux, uy;
        Coef2<T> cf;
    };
    struct Rec {
        int rel, nb, fid, q0, q1;
    };
    struct Raw {
        T   v[4];
        int kind; // 0 none, 1 one value, 4 mean of four
    };
    auto side_of = [&](uint64_t key, Side& sd) {
        const int inst = g.inst_shift >= 64 ? 0 : static_cast<int>(key >> g.inst_shift);
        sd.ux          = upx0;
        sd.uy          = upy0;
        if (upcode) {
            const int32_t code = upcode[inst];
            sd.ux              = unpack_upwind(code, 0);
            sd.uy              = unpack_upwind(code, 1);
        }
        const int row = inst * nl + key_level(key);
        if constexpr (sizeof(T) == 4) {
            const float2 c = coef32[row];
            sd.cf.cx       = c.x;
            sd.cf.cy       = c.y;
        } else {
            const Coef& c = coef[row];
            sd.cf.c0      = c.c0;
            sd.cf.cx      = c.c[0];
            sd.cf.cy      = c.c[1];
        }
    };
    auto has_job = [&](const Side& sd) { return job && (col ? sd.ux != 0 : sd.uy != 0); };
    auto pos_of  = [&](const Side& sd) { return col ? (sd.ux > 0 ? 1 : 0) : (sd.uy > 0 ? 1 : 0); };
    auto rec_of  = [&](int q, const Side& sd, Rec& m) {
        m.rel = REL_NONE;
        if (!has_job(sd)) return;
        const amr_halo_meta* rp = meta + static_cast<size_t>(q) * 4 + 2 * L + pos_of(sd);
        m.rel                   = rp->relation;
        m.nb                    = rp->neighbor;
        m.fid                   = rp->finer_ids[fsel];
        m.q0                    = rp->quadrant[0];
        m.q1                    = rp->quadrant[1];
    };
    // The halo rules of ghost_value for one 2D face ghost cell, split into
    // issuing the source loads and combining them.
    // (the source address is formed with selects so lanes with different
    // relations do not diverge; only the three extra loads of the mean are
    // predicated)
    auto fetch = [&](int q, const Side& sd, const Rec& m, Raw& raw) {
        raw.kind = 0;
        if (!has_job(sd)) return;
        const int  pos = pos_of(sd);
        const int  gc  = pos ? N + H : H - 1;
        const int  G0 = col ? tg : gc, G1 = col ? gc : tg;
        const int  sh = pos ? -N : N;
        const int  s0 = G0 + (L == 0 ? sh : 0), s1 = G1 + (L == 1 ? sh : 0); // same-level source
        const bool same = m.rel == REL_SAME, coarser = m.rel == REL_COARSER, finer = m.rel == REL_FINER;
        const int  c0 = H + m.q0 * HALF + (s0 - H) / 2, c1 = H + m.q1 * HALF + (s1 - H) / 2;
        const int  d0 = ((s0 - H) * 2) % N + H, d1 = ((s1 - H) * 2) % N + H;
        const int  f0 = same ? s0 : coarser ? c0 : finer ? d0 : G0;
        const int  f1 = same ? s1 : coarser ? c1 : finer ? d1 : G1;
        const int  src = (same || coarser) ? m.nb : finer ? m.fid : q;
        const T*   fp  = in + static_cast<size_t>(src) * FLAT + f0 * P1 + f1;
        raw.v[0]       = fp[0];
        raw.kind       = finer ? 4 : 1;
        if (finer) {
            raw.v[1] = fp[1];
            raw.v[2] = fp[P1];
            raw.v[3] = fp[P1 + 1];
        }
    };
    auto combine = [&](const Raw& raw) -> T {
        if (raw.kind == 4) {
            double sum = static_cast<double>(raw.v[0]);
            sum += static_cast<double>(raw.v[1]);
            sum += static_cast<double>(raw.v[2]);
            sum += static_cast<double>(raw.v[3]);
            return static_cast<T>(sum / 4.0);
        }
        return raw.v[0];
    };

    // pipeline prologue
    const int q1 = p + nwarp, q2 = p + 2 * nwarp;
    Side      sd0{}, sd1{}, sd2{};
    Rec       m1{}, m2{};
    Raw       g0{}, g1{};
    uint64_t  k2 = 0;
    if (p < P) {
        side_of(keys[p], sd0);
        Rec m0;
        rec_of(p, sd0, m0);
        fetch(p, sd0, m0, g0);
    }
    if (q1 < P) {
        side_of(keys[q1], sd1);
        rec_of(q1, sd1, m1);
    }
    if (q2 < P) k2 = keys[q2];

    for (int it = 0; p < P; ++it, p += nwarp) {
        const int b  = it % S;
        const int pf = p + (S - 1) * nwarp; // patch whose copy is issued now
        if (pf < P && lane == 0) request(pf, (it + S - 1) % S);
        // advance the metadata pipeline
        const int pa = p + nwarp, pb = p + 2 * nwarp, pc = p + 3 * nwarp;
        uint64_t  k3 = 0;
        if (pc < P) k3 = keys[pc];
        if (pb < P) {
            side_of(k2, sd2);
            rec_of(pb, sd2, m2);
        }
        if (pa < P) fetch(pa, sd1, m1, g1);
        // this patch
        const bool has = has_job(sd0);
        const int  pos = pos_of(sd0);
        const int  gc  = pos ? N + H : H - 1;
        const int  G0 = col ? tg : gc, G1 = col ? gc : tg;
        const T    gv  = combine(g0);
        if (!mbar_wait_bounded(&bars[b], (phase >> b) & 1u)) {
            if (lane == 0) atomicExch(err, static_cast<int32_t>(AMR_ERR_TIMEOUT));
            phase ^= 1u << b;
            for (int j = 1; j < S; ++j) // drain the copies still in flight
                if (p + j * nwarp < P) {
                    const int sl = (it + j) % S;
                    mbar_wait_bounded(&bars[sl], (phase >> sl) & 1u);
                    phase ^= 1u << sl;
                }
            return;
        }
        phase ^= 1u << b;
        T* tile = tiles + static_cast<size_t>(b) * FLAT;
        if (has) tile[G0 * P1 + G1] = gv;
        __syncwarp();
        const int ux = sd0.ux, uy = sd0.uy;
        // the lane's column, rows r0-1 .. r0+SEG (the end rows are the
        // neighbouring segments' cells or the upwind ghost row)
        T colv[SEG + 2];
#pragma unroll
        for (int k = 0; k < SEG + 2; ++k) colv[k] = tile[(r0 - 1 + k) * P1 + cl];
        T res[SEG];
#pragma unroll
        for (int k = 0; k < SEG; ++k)
            res[k] = upd2d<T>(colv[k + 1], tile[(r0 + k) * P1 + cl + ux], uy < 0 ? colv[k] : colv[k + 2], sd0.cf, ux, uy);
        __syncwarp();
#pragma unroll
        for (int k = 0; k < SEG; ++k) tile[(r0 + k) * P1 + cl] = res[k];
        __syncwarp();
        const uint4* t4  = reinterpret_cast<const uint4*>(reinterpret_cast<const char*>(tile) + LO);
        uint4*       dst = reinterpret_cast<uint4*>(reinterpret_cast<char*>(out + static_cast<size_t>(p) * FLAT) + LO);
        for (int w = lane; w < Sh::WORDS; w += 32) dst[w] = t4[w];
        __syncwarp();
        // rotate the pipeline
        sd0 = sd1;
        g0  = g1;
        sd1 = sd2;
        m1  = m2;
        k2  = k3;
    }
}

// ------------------------------------------------ pass records
// One 16-byte record per leaf for the multi-step pass: the same-level
// neighbours across the upwind x face (x) and y face (y), the x-neighbour's
// y-neighbour (z: the diagonal whose corner reaches the patch within a
// pass), and the instance, level and upwind offsets packed into w.  A zero
// velocity component names the patch itself.  Optionally a second record
// per leaf holds all four face neighbours (x low, x high, y low, y high) for
// the gradient flags of the same tree.  The records are built once per mesh
// and velocity field, so the kernels read one record per patch instead of a
// chain of dependent face-record loads.  A face that is not same-level sets
// AMR_ERR_UNBALANCED (passes run only where every relation is same-level).
__host__ __device__ __forceinline__ int pass_code(int ux, int uy, int inst, int level)
{
    return (inst << 10) | (level << 4) | ((ux + 1) << 2) | (uy + 1);
}
__host__ __device__ __forceinline__ int pass_ux(int code) { return ((code >> 2) & 3) - 1; }
__host__ __device__ __forceinline__ int pass_uy(int code) { return (code & 3) - 1; }
__host__ __device__ __forceinline__ int pass_level(int code) { return (code >> 4) & 63; }
__host__ __device__ __forceinline__ int pass_inst(int code) { return code >> 10; }

__device__ __forceinline__ void pass_record(const amr_halo_meta* __restrict__ meta, const uint64_t* __restrict__ keys,
                                            const int32_t* __restrict__ upcode, int upx0, int upy0, const Geo& g,
                                            int q, int4* __restrict__ rec, int4* __restrict__ frec, int32_t* err)
{
    const uint64_t key  = keys[q];
    const int      inst = g.inst_shift >= 64 ? 0 : static_cast<int>(key >> g.inst_shift);
    int            ux = upx0, uy = upy0;
    if (upcode) {
        const int32_t code = upcode[inst];
        ux                 = unpack_upwind(code, 0);
        uy                 = unpack_upwind(code, 1);
    }
    auto same = [&](const amr_halo_meta& m, int self) {
        if (m.relation != REL_SAME) {
            atomicExch(err, static_cast<int32_t>(AMR_ERR_UNBALANCED));
            return self;
        }
        return m.neighbor;
    };
    int4 r;
    r.x    = ux != 0 ? same(meta[static_cast<size_t>(q) * 4 + 2 + (ux > 0 ? 1 : 0)], q) : q;
    r.y    = uy != 0 ? same(meta[static_cast<size_t>(q) * 4 + (uy > 0 ? 1 : 0)], q) : q;
    r.z    = ux != 0 && uy != 0 ? same(meta[static_cast<size_t>(r.x) * 4 + (uy > 0 ? 1 : 0)], r.x) : q;
    r.w    = pass_code(ux, uy, inst, key_level(key));
    rec[q] = r;
    if (frec) {
        const amr_halo_meta* m = meta + static_cast<size_t>(q) * 4;
        frec[q]                = make_int4(same(m[2], q), same(m[3], q), same(m[0], q), same(m[1], q));
    }
}

// Host-driven build: P leaves, upwind offsets per instance (upcode) or
// launch-wide (upx0, upy0).
static __global__ void __launch_bounds__(256)
k_pass_records(const amr_halo_meta* __restrict__ meta, const uint64_t* __restrict__ keys,
               const int32_t* __restrict__ upcode, int upx0, int upy0, int P, Geo g, int4* __restrict__ rec,
               int32_t* err)
{
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < P; q += gridDim.x * blockDim.x)
        pass_record(meta, keys, upcode, upx0, upy0, g, q, rec, nullptr, err);
}

// ------------------------------------------------ 2D update, D steps per pass
// D consecutive steps of a tree whose every neighbour relation is "same
// level" (each instance uniform, as in the batched forests), in one pass over
// memory: the patch is read once and written once per D steps.  Step m needs
// the upwind ghost column and row of u^{m-1}, which are the neighbours' edge
// cells after m-1 steps.  The warp recomputes them with upd2d from u^n: the
// neighbours' D outermost columns / rows (the strips) and the D(D-1)/2 cells
// of the diagonal neighbour's corner that reach the patch within D steps
// (upwind distance a in y and b in x, a, b >= 1, a + b <= D).  Each value is
// formed by the same operation on the same inputs as in D separate steps (the
// halo exchange of a same-level neighbour is a copy), so the result is
// bit-identical.
//
// Between the tile load and the write-back the cells stay in registers, in
// upwind-normalized coordinates: on an axis whose upwind side is + the
// normalized index i' is N-1-i (i the interior index), otherwise i, so a
// cell's upwind neighbours are always at i'-1 and j'-1.  Lane (r, c) =
// (lane / 8, lane % 8) owns the BR x BC block of normalized rows r*BR..,
// columns c*BC..  Per step only block edges cross lanes, through two small
// shared buffers per warp: X[c][i'] holds, for normalized row i', the cell
// left of block column c (normalized column c*BC-1, the distance-1 ghost for
// c = 0); Y[r][j'] the cell above block row r.  Each lane stores its last
// column and its last row (one vector store each) and loads its block's
// upwind edges (one vector load each); the buffers alternate between steps,
// so one warp barrier per step orders them.
//
// Strips: lanes 0..N-1 hold the ghost column of normalized row lane, lanes
// N..2N-1 the ghost row of normalized column lane-N; each holds s[1..D]
// (s[d] = the ghost cell at upwind distance d) and stores s[1] into X[0] /
// Y[0] every step.  Lanes 0 and N hold the corner triangle.  After step m
// the strips and the corner advance one step on the distances still needed
// (d <= D-m).  Per patch the warp reads its pass record two patches ahead,
// its strips one ahead and the corner before the tile wait; the steps branch
// once on which velocity components are non-zero, and each step's
// coefficient row is read one step ahead.
template <int D>
__host__ __device__ constexpr int corner_index(int a, int b)
{
    int base = 0;
    for (int r = 1; r < a; ++r) base += D - r;
    return base + (b - 1);
}

// Warp layout and shared memory of the multi-step pass.
template <typename T, int N, int H>
struct PassShape {
    using Sh                = Step2dShape<T, N, H>;
    static constexpr int RB = 4, CB = 8;           // block rows and block columns of the warp
    static constexpr int BR = N / RB, BC = N / CB; // cells of a lane's block
    // X rows are padded by 16 bytes: the lanes of one block row store and
    // load X rows c = 0..7 at the same offset, and the padding spreads them
    // over distinct banks (Y rows are contiguous across lanes already)
    static constexpr int XN = N + 16 / static_cast<int>(sizeof(T));
    static constexpr int XS = (CB + 1) * XN;       // X[c][i'], c = 0..CB
    static constexpr int YS = (RB + 1) * N;        // Y[r][j'], r = 0..RB
    static constexpr int XY = 2 * (XS + YS);       // elements per warp: two of each
    static_assert(BR * RB == N && BC * CB == N, "patch edge must be a multiple of 8");
    static_assert((XS * sizeof(T)) % 16 == 0 && (YS * sizeof(T)) % 16 == 0, "exchange buffers stay 16-byte aligned");
    // dynamic shared memory of a block of W warps with S tiles each: the
    // tiles, the exchange buffers, the barriers
    static constexpr size_t smem(int W, int S)
    {
        return static_cast<size_t>(W) * (S * (Sh::TILE + 8) + XY * sizeof(T));
    }
};

// K consecutive shared-memory elements moved as the widest aligned vectors
// (callers' offsets are multiples of K elements).
template <typename T, int K>
__device__ __forceinline__ void lds_vec(const T* p, T (&v)[K])
{
    if constexpr ((K * sizeof(T)) % 16 == 0) {
#pragma unroll
        for (int i = 0; i < static_cast<int>(K * sizeof(T) / 16); ++i) {
            if constexpr (sizeof(T) == 4) {
                const float4 w = reinterpret_cast<const float4*>(p)[i];
                v[4 * i]       = w.x;
                v[4 * i + 1]   = w.y;
                v[4 * i + 2]   = w.z;
                v[4 * i + 3]   = w.w;
            } else {
                const double2 w = reinterpret_cast<const double2*>(p)[i];
                v[2 * i]        = w.x;
                v[2 * i + 1]    = w.y;
            }
        }
    } else if constexpr (sizeof(T) == 4 && K == 2) {
        const float2 w = *reinterpret_cast<const float2*>(p);
        v[0]           = w.x;
        v[1]           = w.y;
    } else {
#pragma unroll
        for (int i = 0; i < K; ++i) v[i] = p[i];
    }
}
template <typename T, int K>
__device__ __forceinline__ void sts_vec(T* p, const T (&v)[K])
{
    if constexpr ((K * sizeof(T)) % 16 == 0) {
#pragma unroll
        for (int i = 0; i < static_cast<int>(K * sizeof(T) / 16); ++i) {
            if constexpr (sizeof(T) == 4)
                reinterpret_cast<float4*>(p)[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
            else
                reinterpret_cast<double2*>(p)[i] = make_double2(v[2 * i], v[2 * i + 1]);
        }
    } else if constexpr (sizeof(T) == 4 && K == 2) {
        *reinterpret_cast<float2*>(p) = make_float2(v[0], v[1]);
    } else {
#pragma unroll
        for (int i = 0; i < K; ++i) p[i] = v[i];
    }
}

template <typename T, int N, int H, int S, int D>
__device__ __forceinline__ void step2d_pass_body(const T* __restrict__ in, T* __restrict__ out,
                                                                                                  const int4* __restrict__ rec, int P, int nl,
                                                 const Coef* __restrict__ coef, const float2* __restrict__ coef32,
                                                 size_t cstride, int32_t* err, T* tiles, T* xy, uint64_t* bars, int p,
                                                 int nwarp)
{
    static_assert(D >= 2 && D <= 6, "two to six steps per pass");
    using Sh                = Step2dShape<T, N, H>;
    using Ps                = PassShape<T, N, H>;
    constexpr int      P1   = Sh::P1;
    constexpr int      FLAT = Sh::FLAT;
    constexpr uint32_t LO = Sh::LO, BYTES = Sh::BYTES;
    constexpr int      BR = Ps::BR, BC = Ps::BC, XN = Ps::XN, XS = Ps::XS, YS = Ps::YS;
    constexpr int      NC   = D * (D - 1) / 2; // corner cells
    const int          lane = threadIdx.x & 31;
    if (lane == 0) {
        for (int b = 0; b < S; ++b) mbar_init(&bars[b], 1);
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
    // A tiles are in flight ahead of the current one; a slot is refilled only
    // once the bulk store of its previous patch has read it, and at most
    // PEND stores (the newest) may still be reading when a slot is refilled
    constexpr int A    = S >= 2 ? S - 2 : 0;
    constexpr int PEND = S - 1 - A;
    if (lane == 0)
        for (int j = 0; j < A; ++j)
            if (p + j * nwarp < P) request(p + j * nwarp, j);
    uint32_t   phase = 0;
    const int  rb = lane >> 3, cb = lane & 7; // the lane's block
    const bool col  = lane < N;              // ghost-column strip of normalized row `lane`
    const bool job  = lane < 2 * N;
    const int  sl   = col ? lane : lane - N; // normalized tangential index of the lane's strip
    const bool inr  = sl > 0;                // tangential upwind neighbour: the previous strip lane, else the corner
    const int  src  = inr ? lane - 1 : lane;
    const bool hold = lane == 0 || lane == N; // corner holders

    auto coef_of = [&](int step, int row, Coef2<T>& c) {
        if constexpr (sizeof(T) == 4) {
            const float2 v = coef32[step * cstride + row];
            c.cx           = v.x;
            c.cy           = v.y;
        } else {
            const Coef& v = coef[step * cstride + row];
            c.c0          = v.c0;
            c.cx          = v.c[0];
            c.cy          = v.c[1];
        }
    };
    auto has_job = [&](int ux, int uy) { return job && (col ? ux != 0 : uy != 0); };
    // one patch ahead: the lane's strip (u^n at distances 1..D, at the actual
    // tangential coordinate of its normalized index)
    auto fetch = [&](const int4& r, T* v) {
#pragma unroll
        for (int d = 1; d <= D; ++d) v[d] = T(0);
        const int ux = pass_ux(r.w), uy = pass_uy(r.w);
        if (!has_job(ux, uy)) return;
        const int pos = col ? (ux > 0 ? 1 : 0) : (uy > 0 ? 1 : 0);
        const int tg  = ((col ? uy : ux) > 0 ? N - 1 - sl : sl) + H;
        const T*  nbp = in + static_cast<size_t>(col ? r.x : r.y) * FLAT;
#pragma unroll
        for (int d = 1; d <= D; ++d) {
            const int line = pos ? H + d - 1 : N + H - d; // the neighbour's line at distance d
            v[d]           = nbp[col ? tg * P1 + line : line * P1 + tg];
        }
    };

    // records two patches ahead, strips one ahead
    const int q1 = p + nwarp;
    int4      r0{}, r1{}, r2{};
    T         sa[D + 1], sb[D + 1]; // strips of this patch and the next
#pragma unroll
    for (int d = 0; d <= D; ++d) sa[d] = sb[d] = T(0);
    if (p < P) {
        r0 = __ldg(rec + p);
        fetch(r0, sa);
    }
    if (q1 < P) r1 = __ldg(rec + q1);
    // the strip's distance-1 ghost in X[0] / Y[0] of the first buffer
    T* const gx = xy + (col ? sl : XS + sl);

    for (int it = 0; p < P; ++it, p += nwarp) {
        const int b  = it % S;
        const int pf = p + A * nwarp;
        if (pf < P && lane == 0) {
            bulk_wait_read<PEND>(); // the slot's last store has read it
            request(pf, (it + A) % S);
        }
        const int pa = p + nwarp, pb = p + 2 * nwarp;
        if (pb < P) r2 = __ldg(rec + pb);
        if (pa < P) fetch(r1, sb);
        // this patch
        const int ux = pass_ux(r0.w), uy = pass_uy(r0.w), row = pass_inst(r0.w) * nl + pass_level(r0.w);
        T         cn[NC > 0 ? NC : 1];
#pragma unroll
        for (int c = 0; c < (NC > 0 ? NC : 1); ++c) cn[c] = T(0);
        if (hold && ux != 0 && uy != 0) {
            const T* dg = in + static_cast<size_t>(r0.z) * FLAT;
#pragma unroll
            for (int a = 1; a < D; ++a)
#pragma unroll
                for (int bb = 1; a + bb <= D; ++bb)
                    cn[corner_index<D>(a, bb)] = dg[(uy > 0 ? H + a - 1 : N + H - a) * P1 + (ux > 0 ? H + bb - 1 : N + H - bb)];
        }
        if (!mbar_wait_bounded(&bars[b], (phase >> b) & 1u)) {
            if (lane == 0) atomicExch(err, static_cast<int32_t>(AMR_ERR_TIMEOUT));
            phase ^= 1u << b;
            for (int j = 1; j <= A; ++j)
                if (p + j * nwarp < P) {
                    const int sl2 = (it + j) % S;
                    mbar_wait_bounded(&bars[sl2], (phase >> sl2) & 1u);
                    phase ^= 1u << sl2;
                }
            if (lane == 0) bulk_wait_all();
            return;
        }
        phase ^= 1u << b;
        T*         tile = tiles + static_cast<size_t>(b) * FLAT;
        const bool has  = has_job(ux, uy);
        // the lane's block: normalized cell (rb*BR + a, cb*BC + e) is the
        // tile cell cell[a * sr + e * sc]
        const int sr = uy > 0 ? -P1 : P1, sc = ux > 0 ? -1 : 1;
        T*        cell = tile + (H + (uy > 0 ? N - 1 - rb * BR : rb * BR)) * P1 + H + (ux > 0 ? N - 1 - cb * BC : cb * BC);
        T         v[BR][BC];
#pragma unroll
        for (int a = 0; a < BR; ++a)
#pragma unroll
            for (int e = 0; e < BC; ++e) v[a][e] = cell[a * sr + e * sc];
        // the D steps, compiled once per combination of upwind axes
        auto steps = [&]<bool XU, bool YU>() {
            Coef2<T> cf, cfn;
            coef_of(0, row, cf);
#pragma unroll
            for (int m = 1; m <= D; ++m) {
                if (m < D) coef_of(m, row, cfn); // the next step's row, one step ahead
                T* const X = xy + (m & 1) * (XS + YS);
                T* const Y = X + XS;
                {
                    T last[BR];
#pragma unroll
                    for (int a = 0; a < BR; ++a) last[a] = v[a][BC - 1];
                    sts_vec<T, BR>(X + (cb + 1) * XN + rb * BR, last);
                }
                sts_vec<T, BC>(Y + (rb + 1) * N + cb * BC, v[BR - 1]);
                if (has) gx[(m & 1) * (XS + YS)] = sa[1]; // u^{m-1} ghosts
                __syncwarp();
                T xin[BR], yin[BC];
                lds_vec<T, BR>(X + cb * XN + rb * BR, xin);
                lds_vec<T, BC>(Y + rb * N + cb * BC, yin);
                // in place, last row and column first: a cell's upwind
                // neighbours are still u^{m-1} when it is updated
#pragma unroll
                for (int a = BR - 1; a >= 0; --a)
#pragma unroll
                    for (int e = BC - 1; e >= 0; --e)
                        v[a][e] = upd2d_fixed<T, XU, YU>(v[a][e], e == 0 ? xin[a] : v[a][e - 1],
                                                         a == 0 ? yin[e] : v[a - 1][e], cf);
                if (m < D) {
                    // strips to u^m on the distances still needed, ascending:
                    // a lane's distance d+1 and its neighbours' distance d
                    // are still u^{m-1} when distance d is updated (the
                    // shuffles of distance d precede every lane's update)
#pragma unroll
                    for (int d = 1; d <= D - m; ++d) {
                        const T tnb  = __shfl_sync(0xffffffffu, sa[d], src);
                        const T tang = inr ? tnb : (col ? cn[corner_index<D>(1, d)] : cn[corner_index<D>(d, 1)]);
                        const T nrm  = sa[d + 1];
                        sa[d]        = upd2d_fixed<T, XU, YU>(sa[d], col ? nrm : tang, col ? tang : nrm, cf);
                    }
                    // the corner in place, by increasing distance a + b: a
                    // cell reads the cells at distance + 1, still u^{m-1}
                    if (NC > 0 && XU && YU) {
#pragma unroll
                        for (int sum = 2; sum <= D - m; ++sum)
#pragma unroll
                            for (int a = 1; a < sum; ++a)
                                cn[corner_index<D>(a, sum - a)] = upd2d_fixed<T, XU, YU>(
                                    cn[corner_index<D>(a, sum - a)], cn[corner_index<D>(a, sum - a + 1)],
                                    cn[corner_index<D>(a + 1, sum - a)], cf);
                    }
                    cf = cfn;
                }
            }
        };
        if (ux != 0 && uy != 0) steps.template operator()<true, true>();
        else if (ux != 0) steps.template operator()<true, false>();
        else if (uy != 0) steps.template operator()<false, true>();
        else steps.template operator()<false, false>();
        // back into the tile in its own orientation, then the interior rows
        // out by one bulk store (the async proxy sees every lane's writes)
#pragma unroll
        for (int a = 0; a < BR; ++a)
#pragma unroll
            for (int e = 0; e < BC; ++e) cell[a * sr + e * sc] = v[a][e];
        fence_proxy_async_smem();
        __syncwarp();
        if (lane == 0) {
            bulk_copy_s2g(reinterpret_cast<char*>(out + static_cast<size_t>(p) * FLAT) + LO,
                          reinterpret_cast<const char*>(tile) + LO, BYTES);
            bulk_commit();
        }
        r0 = r1;
        r1 = r2;
#pragma unroll
        for (int d = 1; d <= D; ++d) sa[d] = sb[d];
    }
    if (lane == 0) bulk_wait_all(); // the last stores complete before the block's shared memory goes
}

// Warp w of the block: its S tiles, its exchange buffers and its S barriers
// in dynamic shared memory (multi-step pass).
template <typename T, int N, int H, int W, int S>
__device__ __forceinline__ void pass2d_smem(unsigned char* smem, T*& tiles, T*& xy, uint64_t*& bars)
{
    using Sh      = Step2dShape<T, N, H>;
    using Ps      = PassShape<T, N, H>;
    const int wib = threadIdx.x >> 5;
    tiles         = reinterpret_cast<T*>(smem) + static_cast<size_t>(wib) * S * Sh::FLAT;
    xy            = reinterpret_cast<T*>(smem + static_cast<size_t>(W) * S * Sh::TILE) + static_cast<size_t>(wib) * Ps::XY;
    bars          = reinterpret_cast<uint64_t*>(smem + static_cast<size_t>(W) * (S * Sh::TILE + Ps::XY * sizeof(T))) +
           wib * S;
}

// Warp w of the block: its S tiles and S barriers in dynamic shared memory.
template <typename T, int N, int H, int W, int S>
__device__ __forceinline__ void step2d_smem(unsigned char* smem, T*& tiles, uint64_t*& bars)
{
    using Sh       = Step2dShape<T, N, H>;
    const int wib  = threadIdx.x >> 5;
    tiles          = reinterpret_cast<T*>(smem) + static_cast<size_t>(wib) * S * Sh::FLAT;
    bars           = reinterpret_cast<uint64_t*>(smem + static_cast<size_t>(W) * S * Sh::TILE) + wib * S;
}

// Register budget: 32 resident warps per SM for FP32, 24 for FP64 (the
// metadata pipeline keeps three patches' records in registers).
template <typename T, int W>
struct Step2dOcc {
    static constexpr int blocks = ((sizeof(T) == 4 ? 40 : 24) / W) > 0 ? ((sizeof(T) == 4 ? 40 : 24) / W) : 1;
};

// Host-driven launch: leaf count and buffers from the arguments.
template <typename T, int N, int H, int W, int S>
__global__ void __launch_bounds__(W * 32, Step2dOcc<T, W>::blocks)
k_step2d(const T* __restrict__ in, T* __restrict__ out, const amr_halo_meta* __restrict__ meta, int P, Geo g,
         const Coef* __restrict__ coef, const float2* __restrict__ coef32, int upx0, int upy0, int32_t* err,
         const uint64_t* __restrict__ keys, const int32_t* __restrict__ upcode)
{
    extern __shared__ __align__(128) unsigned char smem[];
    T*        tiles;
    uint64_t* bars;
    step2d_smem<T, N, H, W, S>(smem, tiles, bars);
    const int nwarp = (gridDim.x * blockDim.x) >> 5;
    const int p     = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    step2d_body<T, N, H, S>(in, out, meta, P, g, coef, coef32, upx0, upy0, err, keys, upcode, tiles, bars, p, nwarp);
}

// Register budget of the multi-step pass: 24 resident warps per SM (the
// lane's cell block, its strips and the corner stay in registers for the
// whole pass; two tiles in flight per warp keep the memory system busy).
template <typename T, int W>
struct Pass2dOcc {
    static constexpr int blocks = (24 / W) > 0 ? (24 / W) : 1;
};

// Host-driven launch of D steps per pass: coefficient rows of step m at
// coef / coef32 + m * cstride.
template <typename T, int N, int H, int W, int S, int D>
__global__ void __launch_bounds__(W * 32, Pass2dOcc<T, W>::blocks)
k_step2d_pass(const T* __restrict__ in, T* __restrict__ out, const int4* __restrict__ rec, int P, int nl,
              const Coef* __restrict__ coef, const float2* __restrict__ coef32, size_t cstride, int32_t* err)
{
    extern __shared__ __align__(128) unsigned char smem[];
    T*        tiles;
    T*        xy;
    uint64_t* bars;
    pass2d_smem<T, N, H, W, S>(smem, tiles, xy, bars);
    const int nwarp = (gridDim.x * blockDim.x) >> 5;
    const int p     = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    step2d_pass_body<T, N, H, S, D>(in, out, rec, P, nl, coef, coef32, cstride, err, tiles, xy, bars, p, nwarp);
}

} // namespace amr_gb300
