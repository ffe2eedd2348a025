// Device-resident re-mesh interval.  Every kernel here reads the leaf count
// and the buffer selection (which tree buffer and which state buffer are
// current) from a control block in device memory and walks its work with a
// fixed grid, so one interval (step coefficients, k update steps, halo fill,
// flags, 2:1 closure, counts, scan, emit, remap, neighbour rebuild, commit) is
// a fixed launch sequence: it is captured once in a CUDA graph and replayed
// with no host round trip.  The arithmetic of every leaf and cell is the
// device functions the host-driven kernels use, so results are identical.
// Once a kernel records an error in the control block, every later kernel
// returns at once, leaving the tree as it was when the error was found.
#pragma once

#include "amr_flags2d.cuh"
#include "amr_step2d.cuh"
#include "amr_step3d.cuh"

namespace amr_gb300 {

struct RunCtl {
    int32_t P;          // current leaves
    int32_t tb;         // tree buffer (keys/levels/meta) of the current tree
    int32_t sb;         // state buffer of the current state
    int32_t err;        // first error (amr_status), 0 = none
    int32_t changed;    // the pending re-mesh changes the tree
    int32_t NP;         // leaves after the pending re-mesh
    int32_t max_level;  // finest level over all instances
    int32_t nerr;       // neighbour rebuild error of the pending re-mesh
    int32_t leaves_min; // over interval starts
    int32_t leaves_max;
    int32_t uniform;    // every neighbour relation of the current tree is "same level"
    int32_t flagged;    // some leaf of the pending re-mesh is flagged (zeroed at each commit)
    int32_t recs;       // the pass and face records describe the current tree (zero at a run's start)
    unsigned long long cell_updates, leaves_sum, intervals, remeshes, remeshes_changed;
};

struct RunBufs {
    void*          state[2];
    uint64_t*      keys[2];
    int32_t*       levels[2];
    amr_halo_meta* meta[2];
    int8_t*        flags;
    uint8_t*       rmark;
    uint8_t*       chead;
    uint32_t*      cnt;
    uint32_t*      pos;
    int32_t*       src;
    int8_t*        skind;
    int32_t*       maxlev;     // per instance, read by the step prologue
    int32_t*       maxlev_new; // per instance, filled by emit, zero between re-meshes
    const double*  vel;        // per instance x3, or null (launch-wide upwind sides)
    const int32_t* upcode;     // per instance packed upwind offsets (with vel), or null
    const int32_t* bounds;     // per instance (min, max) level bounds, or null
    int4*          prec;       // pass records of the current tree (multi-step passes)
    int4*          frec;       // face records of the current tree (flags of a same-level tree)
    uint32_t*      tile_sums;  // scan partials, one per tile
    unsigned long long cap;
    int            ninst;
};

constexpr int kScanThreads = 512;
constexpr int kScanPer     = 8;
constexpr int kScanTile    = kScanThreads * kScanPer;

// ---------------------------------------------------------------- steps
template <typename T, int N, int H, int W, int S>
__global__ void __launch_bounds__(W * 32, Step2dOcc<T, W>::blocks)
k_run_step2d(RunBufs B, RunCtl* ctl, Geo g, const Coef* __restrict__ coef, const float2* __restrict__ coef32,
             int parity, int upx0, int upy0)
{
    if (ctl->err) return;
    extern __shared__ __align__(128) unsigned char smem[];
    T*        tiles;
    uint64_t* bars;
    step2d_smem<T, N, H, W, S>(smem, tiles, bars);
    const int P = ctl->P, tb = ctl->tb, s = ctl->sb ^ parity;
    const int nwarp = (gridDim.x * blockDim.x) >> 5;
    const int p     = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    step2d_body<T, N, H, S>(static_cast<const T*>(B.state[s]), static_cast<T*>(B.state[s ^ 1]), B.meta[tb], P, g,
                            coef, coef32, upx0, upy0, &ctl->err, B.keys[tb], B.upcode, tiles, bars, p, nwarp);
}

// Pass records of the current tree (first kernel of an interval run with
// multi-step passes, after the guard).
static __global__ void __launch_bounds__(256) k_run_pass_records(RunBufs B, RunCtl* ctl, Geo g, int upx0, int upy0)
{
    if (ctl->err || ctl->recs) return; // still valid: the last interval left the tree as it was
    const int P = ctl->P, tb = ctl->tb;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < P; q += gridDim.x * blockDim.x)
        pass_record(B.meta[tb], B.keys[tb], B.upcode, upx0, upy0, g, q, B.prec, B.frec, &ctl->err);
}

// D steps per pass (trees of same-level relations only; the interval's
// guard has checked ctl->uniform and k_run_pass_records has built the
// records).  parity selects the buffers of this pass.
template <typename T, int N, int H, int W, int S, int D>
__global__ void __launch_bounds__(W * 32, Pass2dOcc<T, W>::blocks)
k_run_step2d_pass(RunBufs B, RunCtl* ctl, int nl, const Coef* __restrict__ coef, const float2* __restrict__ coef32,
                  size_t cstride, int parity)
{
    if (ctl->err) return;
    extern __shared__ __align__(128) unsigned char smem[];
    T*        tiles;
    T*        xy;
    uint64_t* bars;
    pass2d_smem<T, N, H, W, S>(smem, tiles, xy, bars);
    const int P = ctl->P, s = ctl->sb ^ parity;
    const int nwarp = (gridDim.x * blockDim.x) >> 5;
    const int p     = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    step2d_pass_body<T, N, H, S, D>(static_cast<const T*>(B.state[s]), static_cast<T*>(B.state[s ^ 1]), B.prec, P, nl,
                                    coef, coef32, cstride, &ctl->err, tiles, xy, bars, p, nwarp);
}

// First kernel of an interval captured with multi-step passes: when a re-mesh
// has made the tree non-uniform, the interval must not run; kRetryUniform
// stops every later kernel of the replay, and the host re-runs the interval
// with one-step launches.
constexpr int32_t kRetryUniform = 100;
static __global__ void k_run_require_uniform(RunCtl* ctl)
{
    if (threadIdx.x == 0 && ctl->err == 0 && !ctl->uniform) ctl->err = kRetryUniform;
}

// 3D patches of N^3 cells and one ghost layer, one warp per patch
// (step3d_body); parity selects the buffers of this step.
template <typename T, int N, int W, int S>
__global__ void __launch_bounds__(W * 32)
k_run_step3d(RunBufs B, RunCtl* ctl, Geo g, const Coef* __restrict__ coef, const float4* __restrict__ coef4,
             int parity, int up0, int up1, int up2)
{
    if (ctl->err) return;
    extern __shared__ __align__(128) unsigned char smem3d[];
    T*        tiles;
    uint64_t* bars;
    step3d_smem<T, N, W, S>(smem3d, tiles, bars);
    const int P = ctl->P, tb = ctl->tb, s = ctl->sb ^ parity;
    const int nwarp = (gridDim.x * blockDim.x) >> 5;
    const int p     = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    step3d_body<T, N, S>(static_cast<const T*>(B.state[s]), static_cast<T*>(B.state[s ^ 1]), B.meta[tb],
                         B.levels[tb], B.keys[tb], P, g, coef, coef4, up0, up1, up2, B.upcode,
                         &ctl->err, tiles, bars, p, nwarp);
}

// Any geometry: ppb patches per block per round, grid-stride over rounds.
template <typename T>
__global__ void __launch_bounds__(256)
k_run_step(RunBufs B, RunCtl* ctl, Geo g, const Coef* __restrict__ coef, int parity, int up0, int up1, int up2,
           int ppb)
{
    if (ctl->err) return;
    const int P = ctl->P, tb = ctl->tb, s = ctl->sb ^ parity;
    const T*  in     = static_cast<const T*>(B.state[s]);
    T*        out    = static_cast<T*>(B.state[s ^ 1]);
    const int cells  = g.cells;
    const int nl     = g.depth + 1;
    int       up[3]  = { up0, up1, up2 };
    for (int p0 = blockIdx.x * ppb; p0 < P; p0 += gridDim.x * ppb) {
        for (int t = threadIdx.x; t < ppb * cells; t += blockDim.x) {
            const int p = p0 + t / cells;
            if (p >= P) break;
            const int inst = instance_of(g, B.keys[tb], p);
            if (B.vel)
                for (int a = 0; a < 3; ++a) up[a] = a < g.rank ? upwind(B.vel[3 * inst + a]) : 0;
            step_cell<T, true>(in, out, B.meta[tb], g, coef[inst * nl + B.levels[tb][p]], up, p, t - (p - p0) * cells);
        }
    }
}

// --------------------------------------------------------- halo + flags
// sp: the current state is state[sb ^ sp] (sp = parity of the steps run so
// far in the interval).
template <typename T>
__global__ void __launch_bounds__(256) k_run_halo(RunBufs B, RunCtl* ctl, Geo g, int sp)
{
    if (ctl->err) return;
    const long long total = static_cast<long long>(ctl->P) * g.ndir * g.h * (g.cells / g.n);
    T*              buf   = static_cast<T*>(B.state[ctl->sb ^ sp]);
    const amr_halo_meta* meta = B.meta[ctl->tb];
    for (long long t = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; t < total;
         t += static_cast<long long>(gridDim.x) * blockDim.x)
        halo_cell<T>(buf, meta, g, t);
}

// Gradient flags, one warp per patch, ghosts from the neighbours on the fly
// (the values a halo exchange would store), so no halo pass runs.
template <typename T, int R>
__global__ void __launch_bounds__(256)
k_run_flags_grad(RunBufs B, RunCtl* ctl, Geo g, GradRule rule, int min_level, int max_level, int sp)
{
    if (ctl->err) return;
    const int            P    = ctl->P, tb = ctl->tb;
    const T*             buf  = static_cast<const T*>(B.state[ctl->sb ^ sp]);
    const amr_halo_meta* meta = B.meta[tb];
    const int            lane = threadIdx.x & 31;
    for (int p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; p < P; p += (gridDim.x * blockDim.x) >> 5) {
        int any = 0, all = 1;
        for (int c = lane; c < g.cells; c += 32) gradient_rule_cell<T, true, R>(buf, meta, g, rule, p, c, any, all);
        any = __any_sync(0xffffffffu, any);
        all = __all_sync(0xffffffffu, all);
        if (lane == 0) {
            int lo = min_level, hi = max_level;
            if (B.bounds) {
                const int inst = instance_of(g, B.keys[tb], p);
                lo             = B.bounds[2 * inst];
                hi             = B.bounds[2 * inst + 1];
            }
            const int8_t f = gradient_decision(any, all, B.levels[tb][p], lo, hi);
            B.flags[p]     = f;
            if (f != FLAG_STABLE) ctl->flagged = 1;
        }
    }
}

// 2D gradient flags of the sized kernel (flags2d_body), ghosts on the fly.
template <typename T, int N, int H>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 4 : 3)
k_run_flags2d(RunBufs B, RunCtl* ctl, Geo g, GradRule rule, int min_level, int max_level, int sp)
{
    if (ctl->err) return;
    extern __shared__ __align__(128) unsigned char smem[];
    T*        tiles;
    uint64_t* bars;
    flags2d_smem<T, N, H, false>(smem, blockDim.x >> 5, tiles, bars);
    const int tb    = ctl->tb;
    const int nwarp = (gridDim.x * blockDim.x) >> 5;
    const int p     = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    flags2d_body<T, N, H, false>(static_cast<const T*>(B.state[ctl->sb ^ sp]), B.meta[tb], B.keys[tb], ctl->P, g, rule,
                                 min_level, max_level, B.bounds, B.flags, &ctl->err, tiles, bars, p, nwarp,
                                 &ctl->flagged);
}

// The same flags on a tree whose every relation is same-level, from the pass
// and face records k_run_pass_records built at the start of the interval.
template <typename T, int N, int H>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 4 : 3)
k_run_flags2d_uniform(RunBufs B, RunCtl* ctl, GradRule rule, int min_level, int max_level, int sp)
{
    if (ctl->err) return;
    extern __shared__ __align__(128) unsigned char smem[];
    T*        tiles;
    uint64_t* bars;
    flags2d_smem<T, N, H, false>(smem, blockDim.x >> 5, tiles, bars);
    const int nwarp = (gridDim.x * blockDim.x) >> 5;
    const int p     = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    flags2d_uniform_body<T, N, H>(static_cast<const T*>(B.state[ctl->sb ^ sp]), B.prec, B.frec, ctl->P, rule,
                                  min_level, max_level, B.bounds, B.flags, &ctl->err, tiles, bars, p, nwarp,
                                  &ctl->flagged);
}

// Max-value flags (k_flags_max's rule over the exchanged ghosts), one block
// per patch, grid-stride.
template <typename T>
__global__ void __launch_bounds__(128)
k_run_flags_max(RunBufs B, RunCtl* ctl, Geo g, double rthr, double cthr, int min_level, int max_level, int sp)
{
    if (ctl->err) return;
    const int P = ctl->P, tb = ctl->tb;
    const T*  buf = static_cast<const T*>(B.state[ctl->sb ^ sp]);
    __shared__ double red[128];
    for (int p = blockIdx.x; p < P; p += gridDim.x) {
        int lo = min_level, hi = max_level;
        if (B.bounds) {
            const int inst = instance_of(g, B.keys[tb], p);
            lo             = B.bounds[2 * inst];
            hi             = B.bounds[2 * inst + 1];
        }
        const T* u = buf + static_cast<size_t>(p) * g.flat;
        double   m = 0.0;
        for (int c = threadIdx.x; c < g.flat; c += blockDim.x)
            if (face_or_interior(g, c)) m = fmax(m, static_cast<double>(u[c]));
        red[threadIdx.x] = m;
        __syncthreads();
        for (int w = 64; w > 0; w >>= 1) {
            if (threadIdx.x < w) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + w]);
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            const int8_t f = max_decision(red[0], B.levels[tb][p], rthr, cthr, lo, hi);
            B.flags[p]     = f;
            if (f != FLAG_STABLE) ctl->flagged = 1;
        }
        __syncthreads();
    }
}

// --------------------------------------------------------------- re-mesh
#define AMR_RUN_LEAVES(P)                                                                              \
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < (P); i += gridDim.x * blockDim.x)

// The flag kernels set ctl->flagged when they flag some leaf; without one
// the re-mesh changes nothing (reconstruction_is_noop, ndtree.hpp:1242-1246)
// and the marks are not needed.
static __global__ void k_run_mark(RunBufs B, RunCtl* ctl, Geo g)
{
    if (ctl->err) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) ctl->changed = 0;
    if (!ctl->flagged) return;
    const int P = ctl->P, tb = ctl->tb;
    AMR_RUN_LEAVES(P)
    mark_leaf(B.keys[tb], B.flags, P, g, B.rmark, B.chead, i);
}

// With no leaf flagged the re-mesh changes nothing (reconstruction_is_noop,
// ndtree.hpp:1242-1246): closure, veto, count and scan return at once.
static __global__ void k_run_closure(RunBufs B, RunCtl* ctl, Geo g)
{
    if (ctl->err || !ctl->flagged) return;
    const int P = ctl->P, tb = ctl->tb;
    AMR_RUN_LEAVES(P) closure_leaf(B.meta[tb], g, B.rmark, i);
}

static __global__ void k_run_veto(RunBufs B, RunCtl* ctl, Geo g)
{
    if (ctl->err || !ctl->flagged) return;
    const int P = ctl->P, tb = ctl->tb;
    AMR_RUN_LEAVES(P) veto_leaf(B.meta[tb], g, B.rmark, B.chead, i);
}

static __global__ void k_run_count(RunBufs B, RunCtl* ctl, Geo g)
{
    if (ctl->err || !ctl->flagged) return;
    const int P = ctl->P, tb = ctl->tb;
    AMR_RUN_LEAVES(P) count_leaf(B.keys[tb], B.rmark, B.chead, g, B.cnt, &ctl->changed, i);
}

// Block-wide exclusive scan of one value per thread; returns the exclusive
// prefix, *total = block sum.  blockDim.x == kScanThreads.
__device__ inline uint32_t scan_block_exclusive(uint32_t v, uint32_t* warp_sums, uint32_t* total)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t  x    = v;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[w] = x;
    __syncthreads();
    if (w == 0) {
        uint32_t s = lane < kScanThreads / 32 ? warp_sums[lane] : 0u;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < kScanThreads / 32) warp_sums[lane] = s; // inclusive
    }
    __syncthreads();
    const uint32_t before = (w > 0 ? warp_sums[w - 1] : 0u) + x - v;
    *total                = warp_sums[kScanThreads / 32 - 1];
    __syncthreads();
    return before;
}

// Scan, pass 1: sum of the counts of each tile of kScanTile leaves.
static __global__ void __launch_bounds__(kScanThreads) k_run_scan_tiles(RunBufs B, RunCtl* ctl)
{
    if (ctl->err || !ctl->flagged) return;
    const int P = ctl->P;
    __shared__ uint32_t ws[kScanThreads / 32];
    for (int tile = blockIdx.x; tile * kScanTile < P; tile += gridDim.x) {
        const int base = tile * kScanTile + threadIdx.x * kScanPer;
        uint32_t  s    = 0;
#pragma unroll
        for (int k = 0; k < kScanPer; ++k)
            if (base + k < P) s += B.cnt[base + k];
        uint32_t tot;
        scan_block_exclusive(s, ws, &tot);
        if (threadIdx.x == 0) B.tile_sums[tile] = tot;
    }
}

// Scan, pass 2: each tile adds the sums of the tiles before it and writes
// its exclusive positions; the last tile writes pos[P] and the new size and
// flags AMR_ERR_CAPACITY when it exceeds the capacity.
static __global__ void __launch_bounds__(kScanThreads) k_run_scan_apply(RunBufs B, RunCtl* ctl)
{
    if (ctl->err || !ctl->flagged) return;
    const int P      = ctl->P;
    const int ntiles = (P + kScanTile - 1) / kScanTile;
    __shared__ uint32_t ws[kScanThreads / 32];
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        uint32_t before = 0;
        for (int j = threadIdx.x; j < tile; j += blockDim.x) before += B.tile_sums[j];
        uint32_t prior;
        scan_block_exclusive(before, ws, &prior);
        const int base = tile * kScanTile + threadIdx.x * kScanPer;
        uint32_t  v[kScanPer];
        uint32_t  s = 0;
#pragma unroll
        for (int k = 0; k < kScanPer; ++k) {
            v[k] = base + k < P ? B.cnt[base + k] : 0u;
            s += v[k];
        }
        uint32_t tot;
        uint32_t run = prior + scan_block_exclusive(s, ws, &tot);
#pragma unroll
        for (int k = 0; k < kScanPer; ++k)
            if (base + k < P) {
                B.pos[base + k] = run;
                run += v[k];
            }
        if (tile == ntiles - 1 && threadIdx.x == 0) {
            const uint32_t np = prior + tot;
            B.pos[P]          = np;
            ctl->NP           = static_cast<int32_t>(np);
            if (np > B.cap) ctl->err = AMR_ERR_CAPACITY;
        }
    }
}

static __global__ void k_run_emit(RunBufs B, RunCtl* ctl, Geo g)
{
    if (ctl->err || !ctl->changed) return;
    const int P = ctl->P, tb = ctl->tb, nb = tb ^ 1;
    if (blockIdx.x == 0 && threadIdx.x == 0) ctl->uniform = 1; // k_run_neighbors clears it
    AMR_RUN_LEAVES(P)
    emit_leaf(B.keys[tb], B.rmark, B.chead, B.pos, g, B.keys[nb], B.levels[nb], B.src, B.skind, B.maxlev_new, i);
}

// The new state (k_remap's work), one unit per 16-byte word of each new
// leaf, grid-stride over all of them: a kept leaf moves word by word (ghosts
// included), a refined or coarsened leaf is built cell by cell, each unit
// taking the same share of its cells.  Every thread has independent loads in
// flight, instead of one block stepping through the leaves one at a time.
template <typename T>
__global__ void __launch_bounds__(256) k_run_remap(RunBufs B, RunCtl* ctl, Geo g, int sp)
{
    if (ctl->err || !ctl->changed) return;
    const int       NP        = ctl->NP;
    const T*        old_state = static_cast<const T*>(B.state[ctl->sb ^ sp]);
    T*              new_state = static_cast<T*>(B.state[ctl->sb ^ sp ^ 1]);
    const int       words     = g.flat * static_cast<int>(sizeof(T)) / 16; // padded sides are even
    const int       per       = (g.cells + words - 1) / words;
    const long long total     = static_cast<long long>(NP) * words;
    for (long long u = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; u < total;
         u += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int j    = static_cast<int>(u / words);
        const int w    = static_cast<int>(u - static_cast<long long>(j) * words);
        const int kind = B.skind[j];
        if (kind == 0) {
            const uint4* f4 = reinterpret_cast<const uint4*>(old_state + static_cast<size_t>(B.src[j]) * g.flat);
            reinterpret_cast<uint4*>(new_state + static_cast<size_t>(j) * g.flat)[w] = f4[w];
        } else {
            const int c1 = min(g.cells, (w + 1) * per);
            for (int c = w * per; c < c1; ++c) remap_cell<T>(old_state, new_state, g, kind, B.src[j], j, c);
        }
    }
}

static __global__ void k_run_neighbors(RunBufs B, RunCtl* ctl, Geo g)
{
    if (ctl->err || !ctl->changed) return;
    const int NP = ctl->NP, nb = ctl->tb ^ 1;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < NP * g.ndir; t += gridDim.x * blockDim.x) {
        neighbor_entry(B.keys[nb], NP, g, B.meta[nb], &ctl->nerr, t);
        if (B.meta[nb][t].relation != REL_SAME) ctl->uniform = 0;
    }
}

// End of an interval (one block): statistics of the interval just run and
// the state buffer the steps left current, then, when the re-mesh changed the
// tree, the switch to the new buffers and the new per-instance finest levels.
static __global__ void __launch_bounds__(256)
k_run_commit(RunBufs B, RunCtl* ctl, int steps, int cells, int remesh, int sp, int records)
{
    __shared__ int chg;
    __shared__ int red[256 / 32];
    if (threadIdx.x == 0) {
        const int  P  = ctl->P;
        const bool ok = ctl->err == 0;
        chg           = (remesh && ok && ctl->changed) ? 1 : 0;
        ctl->flagged  = 0; // the next interval's flag kernels set it again
        ctl->recs     = records && ok && !chg ? 1 : 0; // this interval's records outlive it if the tree stays
        if (ok) {
            ctl->sb ^= sp;
            ctl->cell_updates += static_cast<unsigned long long>(P) * steps * cells;
            ctl->leaves_sum += static_cast<unsigned long long>(P);
            ctl->intervals += 1;
            ctl->leaves_min = min(ctl->leaves_min, P);
            ctl->leaves_max = max(ctl->leaves_max, P);
            if (remesh) ctl->remeshes += 1;
            if (chg) ctl->remeshes_changed += 1;
        }
    }
    __syncthreads();
    if (!chg) return;
    int m = 0;
    for (int i = threadIdx.x; i < B.ninst; i += blockDim.x) {
        const int v     = B.maxlev_new[i];
        B.maxlev[i]     = v;
        B.maxlev_new[i] = 0;
        m               = max(m, v);
    }
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < static_cast<int>(blockDim.x / 32); ++w) m = max(m, red[w]);
        m              = max(m, red[0]);
        ctl->max_level = m;
        ctl->P         = ctl->NP;
        ctl->tb ^= 1;
        ctl->sb ^= 1;
        if (ctl->nerr) ctl->err = ctl->nerr;
    }
}

// Per-instance time bookkeeping at the start of a graph chunk: an empty
// batch, the remaining time, and the totals carried in from earlier work of
// the run (tot0, ctot0).
static __global__ void k_run_dt_init(DtState d, int ninst, double remaining0, double tot0, uint32_t ctot0)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ninst) return;
    d.acc[i]  = 0.0;
    d.rem[i]  = remaining0;
    d.cnt[i]  = 0u;
    d.tot[i]  = tot0;
    d.ctot[i] = ctot0;
}

// offsets[i] = first leaf of instance i (lower bound of its key prefix).
static __global__ void k_instance_offsets(const uint64_t* __restrict__ keys, int P, Geo g, int ninst,
                                   unsigned long long* __restrict__ offsets)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > ninst) return;
    if (i == ninst) {
        offsets[i] = static_cast<unsigned long long>(P);
        return;
    }
    const uint64_t first = g.inst_shift >= 64 ? 0ull : static_cast<uint64_t>(i) << g.inst_shift;
    int            lo = 0, hi = P;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (keys[mid] < first) lo = mid + 1;
        else hi = mid;
    }
    offsets[i] = static_cast<unsigned long long>(lo);
}

} // namespace amr_gb300
