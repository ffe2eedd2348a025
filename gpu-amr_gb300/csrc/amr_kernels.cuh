// Kernels of the GB300 AMR hot path.
//
// Every per-item body is a __device__ function so the same arithmetic runs in
// the per-launch kernels below and in the persistent cluster kernel
// (amr_cycle.cuh).  Pointers into buffers that a persistent kernel rewrites
// between phases are passed without __restrict__ so no load goes through the
// non-coherent path.
#pragma once

#include "amr_device.cuh"

namespace amr_gb300 {

// Per-(step, level) update coefficients of the upwind form of the reference's
// Rusanov flux for linear advection (AdvectionPhysics.hpp:45-66 inside
// amr_solver::time_step_cpu, amr_solver.hpp:317-346):
//   F(uL,uR) = v+ uL + v- uR  =>  u' = c0 u + sum_a c_a u_upwind(a)
// with c_a = (dt/dx_a) |v_a| and c0 = 1 - sum_a c_a.
struct Coef {
    double c0, c[3];
};

__host__ __device__ inline Coef make_coef(const Geo& g, double dt, const double* v, int level)
{
    Coef   c;
    double tot = 0.0;
    for (int a = 0; a < 3; ++a) {
        c.c[a] = 0.0;
        if (a < g.rank) {
            c.c[a] = (dt / cell_size(g, a, level)) * fabs(v[a]);
            tot += c.c[a];
        }
    }
    c.c0 = 1.0 - tot;
    return c;
}

// Raw CFL step of compute_time_step_cpu (amr_solver.hpp:355-413): the
// advection wave speed is |v| in every cell, so the minimum over cells of
// dx/|v| is attained on the finest level present.
__host__ __device__ inline double raw_dt(const Geo& g, const double* v, int max_level)
{
    double raw = 1.7976931348623157e308;
    for (int a = 0; a < g.rank; ++a) {
        const double sp = fabs(v[a]);
        if (sp > 1e-12) raw = fmin(raw, cell_size(g, a, max_level) / sp);
    }
    return raw;
}

// The clamp of finalize_step_dt_kernel (fvm_time_step.cu:204-233).
__host__ __device__ inline double clamp_step(double raw, double cfl, double rem)
{
    double dt = raw * cfl;
    if (rem <= 0.0) dt = 0.0;
    else if (dt > rem) dt = rem;
    return dt;
}

// Instance of a leaf: the key prefix above the Morton field (0 for a single tree).
__device__ __forceinline__ int instance_of(const Geo& g, const uint64_t* keys, int p)
{
    return g.inst_shift >= 64 ? 0 : static_cast<int>(keys[p] >> g.inst_shift);
}

// Upwind offset per Morton axis from the sign of the velocity: -1 when the
// flow comes from the lower side, +1 from the upper side, 0 at rest.
__host__ __device__ __forceinline__ int upwind(double v) { return v > 0.0 ? -1 : (v < 0.0 ? 1 : 0); }

// The upwind offsets of a velocity packed in one int (2 bits per axis,
// offset + 1), and unpacked.
__host__ __device__ __forceinline__ int32_t pack_upwind(const double* v)
{
    return (upwind(v[0]) + 1) | ((upwind(v[1]) + 1) << 2) | ((upwind(v[2]) + 1) << 4);
}
__host__ __device__ __forceinline__ int unpack_upwind(int32_t code, int axis) { return ((code >> (2 * axis)) & 3) - 1; }

__device__ inline void interior_coords(const Geo& g, int c, int* idx)
{
    idx[2] = 0;
    for (int L = g.rank - 1; L >= 0; --L) {
        idx[L] = c % g.n + g.h;
        c /= g.n;
    }
}

// Coefficients rounded to the state type once per row: the FP32 update
// multiplies by the FP32 roundings of c_a, and a row read as CoefT<float>
// spares each cell the double-to-float conversions (on GB300 they share the
// narrow FP64 pipe).
template <typename T>
struct CoefT {
    T c0, c[3];
};
__host__ __device__ __forceinline__ CoefT<float> coef_f32(const Coef& c)
{
    return CoefT<float>{ static_cast<float>(c.c0),
                         { static_cast<float>(c.c[0]), static_cast<float>(c.c[1]), static_cast<float>(c.c[2]) } };
}

// ------------------------------------------------------------ time step
// Interior cell c of patch p: u' = c0 u + sum_a c_a u_up(a).  Upwind values
// outside the interior come from the neighbour patches through the halo rules
// (GhostsOnTheFly) or from the padded buffer (the caller exchanged halos).
template <typename T, bool GhostsOnTheFly, typename C = Coef>
__device__ inline void step_cell(const T* in, T* out, const amr_halo_meta* meta, const Geo& g, const C& cf,
                                 const int* up, int p, int c)
{
    int idx[3];
    interior_coords(g, c, idx);
    const size_t base = static_cast<size_t>(p) * g.flat;
    const int    li   = padded_index(g, idx);
    const T      u    = in[base + li];
    // FP64: c0 u + sum c_a u_up (the reference's flux term for term); FP32:
    // u + sum c_a (u_up - u), which keeps a constant state exactly
    T            acc  = sizeof(T) == 4 ? u : static_cast<T>(cf.c0) * u;
    for (int a = 0; a < g.rank; ++a) {
        const int dirn = up[a];
        if (dirn == 0) continue;
        const int L    = g.rank - 1 - a;
        const int nidx = idx[L] + dirn;
        T         val;
        if (!GhostsOnTheFly || (nidx >= g.h && nidx < g.n + g.h)) {
            val = in[base + li + dirn * g.s[L]];
        } else {
            int G[3] = { idx[0], idx[1], idx[2] };
            G[L]     = nidx;
            const int pos = dirn > 0 ? 1 : 0;
            val = ghost_value<T, T>(in, g.flat, meta[static_cast<size_t>(p) * g.ndir + 2 * L + pos], G, L, pos, g,
                                    in + base);
        }
        acc = fma(static_cast<T>(cf.c[a]), sizeof(T) == 4 ? static_cast<T>(val - u) : val, acc);
    }
    out[base + li] = acc;
}

// One step over P patches; ppb patches per block.  With CoefFromDt the
// coefficients are formed per patch in shared memory from the device dt
// (drop-in launcher, no per-step table); ppb <= 64.
// With `vel` (per-instance velocities, 3 each) and `keys` the upwind sides and
// the coefficient row (coef + instance * (depth+1)) follow each leaf's
// instance; otherwise up0..up2 and coef[level] apply to every leaf.
template <typename T, bool GhostsOnTheFly, bool CoefFromDt = false>
__global__ void __launch_bounds__(256)
k_step(const T* __restrict__ in, T* __restrict__ out, const int32_t* __restrict__ levels,
       const amr_halo_meta* __restrict__ meta, int P, Geo g, const Coef* __restrict__ coef,
       int up0, int up1, int up2, int ppb, const double* __restrict__ dt_dev = nullptr, double v0 = 0.0,
       double v1 = 0.0, double v2 = 0.0, const uint64_t* __restrict__ keys = nullptr,
       const double* __restrict__ vel = nullptr)
{
    const int cells = g.cells;
    const int p0    = blockIdx.x * ppb;
    int       up[3] = { up0, up1, up2 };
    __shared__ Coef local[CoefFromDt ? 64 : 1];
    if (CoefFromDt) {
        const int q = threadIdx.x;
        if (q < ppb && p0 + q < P) {
            const double v[3] = { v0, v1, v2 };
            local[q]          = make_coef(g, *dt_dev, v, levels[p0 + q]);
        }
        __syncthreads();
    }
    for (int t = threadIdx.x; t < ppb * cells; t += blockDim.x) {
        const int p = p0 + t / cells;
        if (p >= P) break;
        const int inst = keys ? instance_of(g, keys, p) : 0;
        if (vel)
            for (int a = 0; a < 3; ++a) up[a] = a < g.rank ? upwind(vel[3 * inst + a]) : 0;
        const Coef cf = CoefFromDt ? local[p - p0] : coef[inst * (g.depth + 1) + levels[p]];
        step_cell<T, GhostsOnTheFly>(in, out, meta, g, cf, up, p, t - (p - p0) * cells);
    }
}

// --------------------------------------------------------- halo exchange
// Face ghost cell t of the P * 2*rank * h * n^(rank-1) ghost cells.  Only
// interior cells are read, so the in-place update has no read/write overlap.
template <typename T>
__device__ inline void halo_cell(T* buf, const amr_halo_meta* meta, const Geo& g, long long t)
{
    const long long per_dir   = static_cast<long long>(g.h) * (g.cells / g.n);
    const long long per_patch = per_dir * g.ndir;
    const long long p         = t / per_patch;
    const long long r         = t - p * per_patch;
    const int       d         = static_cast<int>(r / per_dir);
    int             f         = static_cast<int>(r - d * per_dir);
    const int       L = d / 2, pos = d % 2;
    int             G[3] = { 0, 0, 0 };
    for (int k = g.rank - 1; k >= 0; --k) { // tangential coordinates, then layer
        if (k == L) continue;
        G[k] = f % g.n + g.h;
        f /= g.n;
    }
    G[L]                  = pos ? g.n + g.h + f : f;
    const amr_halo_meta m = meta[p * g.ndir + d];
    if (m.relation == REL_NONE) return;
    T* self                  = buf + p * g.flat;
    self[padded_index(g, G)] = ghost_value<T, T>(buf, g.flat, m, G, L, pos, g, self);
}

// blockIdx.y = field of a multi-field state (fields fstride elements apart).
// With step_dt (per instance), patches of instances whose step is not taken
// (step size 0: past the time limit) keep their ghosts.
template <typename T>
__global__ void __launch_bounds__(256) k_halo(T* __restrict__ buf, const amr_halo_meta* __restrict__ meta,
                                              long long total, Geo g, size_t fstride = 0,
                                              const uint64_t* __restrict__ keys = nullptr,
                                              const double* __restrict__ step_dt = nullptr)
{
    buf += blockIdx.y * fstride;
    const long long per_patch = static_cast<long long>(g.h) * (g.cells / g.n) * g.ndir;
    for (long long t = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; t < total;
         t += static_cast<long long>(gridDim.x) * blockDim.x) {
        if (step_dt) {
            const int p = static_cast<int>(t / per_patch);
            if (!(step_dt[instance_of(g, keys, p)] > 0.0)) continue;
        }
        halo_cell<T>(buf, meta, g, t);
    }
}

// ------------------------------------------------------------------ flags
// max|grad u|*h at interior cell c of patch p: central differences over face
// ghosts, evaluated in double with explicit rounding (no contraction) so the
// oracle's arithmetic is reproduced bit for bit.  Ghosts come from the buffer
// or, with GhostsOnTheFly, from the neighbours by the halo rules, rounded to
// the state type as a halo exchange would store them.
template <typename T, bool GhostsOnTheFly>
__device__ inline double gradient_cell(const T* buf, const amr_halo_meta* meta, const Geo& g, int p, int c)
{
    int idx[3];
    interior_coords(g, c, idx);
    const T*  u  = buf + static_cast<size_t>(p) * g.flat;
    const int li = padded_index(g, idx);
    double    s  = 0.0;
    for (int a = 0; a < g.rank; ++a) {
        const int L = g.rank - 1 - a;
        double    side[2];
        for (int pos = 0; pos < 2; ++pos) {
            const int nidx = idx[L] + (pos ? 1 : -1);
            if (!GhostsOnTheFly || (nidx >= g.h && nidx < g.n + g.h)) {
                side[pos] = static_cast<double>(u[li + (pos ? g.s[L] : -g.s[L])]);
            } else {
                int G[3] = { idx[0], idx[1], idx[2] };
                G[L]     = nidx;
                side[pos] = static_cast<double>(ghost_value<T, T>(
                    buf, g.flat, meta[static_cast<size_t>(p) * g.ndir + 2 * L + pos], G, L, pos, g, u));
            }
        }
        const double gr = __dmul_rn(0.5, __dsub_rn(side[1], side[0]));
        s               = __dadd_rn(s, __dmul_rn(gr, gr));
    }
    return __dsqrt_rn(s);
}

// Squared form of gradient_cell: the same rounded sum of squares, without the
// square root.  With S_r = min{s : sqrt_rn(s) > rthr} and
// S_c = min{s : sqrt_rn(s) >= cthr} (host-side search, sqrt is correctly
// rounded on both sides), "v > rthr" is "s >= S_r" and "v < cthr" is
// "s < S_c" for every s, NaN and infinity included.
template <typename T, bool GhostsOnTheFly>
__device__ inline double gradient_sq_cell(const T* buf, const amr_halo_meta* meta, const Geo& g, int p, int c)
{
    int idx[3];
    interior_coords(g, c, idx);
    const T*  u  = buf + static_cast<size_t>(p) * g.flat;
    const int li = padded_index(g, idx);
    double    s  = 0.0;
    for (int a = 0; a < g.rank; ++a) {
        const int L = g.rank - 1 - a;
        double    side[2];
        for (int pos = 0; pos < 2; ++pos) {
            const int nidx = idx[L] + (pos ? 1 : -1);
            if (!GhostsOnTheFly || (nidx >= g.h && nidx < g.n + g.h)) {
                side[pos] = static_cast<double>(u[li + (pos ? g.s[L] : -g.s[L])]);
            } else {
                int G[3] = { idx[0], idx[1], idx[2] };
                G[L]     = nidx;
                side[pos] = static_cast<double>(ghost_value<T, T>(
                    buf, g.flat, meta[static_cast<size_t>(p) * g.ndir + 2 * L + pos], G, L, pos, g, u));
            }
        }
        const double gr = __dmul_rn(0.5, __dsub_rn(side[1], side[0]));
        s               = __dadd_rn(s, __dmul_rn(gr, gr));
    }
    return s;
}

// The gradient rule on squared norms with an FP32 pre-filter.  Exact tests:
// refine if s >= rsq, coarsen-eligible if s < csq (sq_threshold makes these
// equal to the reference's sqrt(s) > rthr and sqrt(s) < cthr for every
// double s).  An FP32 evaluation s32 of the same sum (FP32 differences of the
// FP32 state, or FP64 differences rounded once to FP32; FP32 squares and
// sums) is within a relative 1e-6 of it whenever it is finite and the
// thresholds lie in [1e-20, 1e30], so s32 >= r_hi proves s >= rsq and
// s32 < r_lo proves s < rsq (margins of 1e-5, likewise c_lo / c_hi); only
// cells inside a band re-evaluate in FP64.  fast = 0 turns the filter off.
struct GradRule {
    double rsq, csq;
    float  r_lo, r_hi, c_lo, c_hi;
    int    fast;
};

// R: the rank at compile time (2 or 3), so coordinate arrays stay in registers.
template <typename T, bool GhostsOnTheFly, int R>
__device__ inline float gradient_sq_f32(const T* buf, const amr_halo_meta* meta, const Geo& g, int p, int c)
{
    int idx[3];
    idx[2] = 0;
#pragma unroll
    for (int L = R - 1; L >= 0; --L) {
        idx[L] = c % g.n + g.h;
        c /= g.n;
    }
    const T*  u  = buf + static_cast<size_t>(p) * g.flat;
    const int li = padded_index(g, idx);
    float     s  = 0.0f;
#pragma unroll
    for (int a = 0; a < R; ++a) {
        const int L = R - 1 - a;
        T         lo, hi;
        {
            const int nidx = idx[L] - 1;
            if (!GhostsOnTheFly || nidx >= g.h) {
                lo = u[li - g.s[L]];
            } else {
                int G[3] = { idx[0], idx[1], idx[2] };
                G[L]     = nidx;
                lo = ghost_value<T, T>(buf, g.flat, meta[static_cast<size_t>(p) * g.ndir + 2 * L], G, L, 0,
                                                   g, u);
            }
        }
        {
            const int nidx = idx[L] + 1;
            if (!GhostsOnTheFly || nidx < g.n + g.h) {
                hi = u[li + g.s[L]];
            } else {
                int G[3] = { idx[0], idx[1], idx[2] };
                G[L]     = nidx;
                hi = ghost_value<T, T>(buf, g.flat, meta[static_cast<size_t>(p) * g.ndir + 2 * L + 1], G, L,
                                                   1, g, u);
            }
        }
        float d;
        if constexpr (sizeof(T) == 4) d = hi - lo;
        else d = static_cast<float>(hi - lo);
        const float gr = 0.5f * d;
        s              = fmaf(gr, gr, s);
    }
    return s;
}

// Refine (any) / coarsen (all) votes of interior cell c under the rule.
template <typename T, bool GhostsOnTheFly, int R>
__device__ inline void gradient_rule_cell(const T* buf, const amr_halo_meta* meta, const Geo& g, const GradRule& r,
                                          int p, int c, int& any, int& all)
{
    if (r.fast) {
        const float s = gradient_sq_f32<T, GhostsOnTheFly, R>(buf, meta, g, p, c);
        if (isfinite(s)) {
            const bool r_sure = s >= r.r_hi || s < r.r_lo;
            const bool c_sure = s < r.c_lo || s >= r.c_hi;
            if (r_sure && c_sure) {
                if (s >= r.r_hi) any = 1;
                if (s >= r.c_hi) all = 0;
                return;
            }
        }
    }
    const double s = gradient_sq_cell<T, GhostsOnTheFly>(buf, meta, g, p, c);
    if (s >= r.rsq) any = 1;
    if (!(s < r.csq)) all = 0;
}

// Patch decision from the any/all rule of
// dg_helpers/globals/amr_indicators.hpp:186-225 with the level bounds of
// bench_fvm_solver_integration_active_amr.b.cpp:92-102.
__device__ inline int8_t gradient_decision(int any, int all, int level, int min_level, int max_level)
{
    return (level < max_level && any) ? FLAG_REFINE : (level > min_level && all) ? FLAG_COARSEN : FLAG_STABLE;
}

// Gradient flags, one warp per patch (grid-stride).  bounds (optional):
// per-instance (min_level, max_level) pairs, indexed by the leaf's instance;
// they replace min_level/max_level.
template <typename T, bool GhostsOnTheFly, int R>
__global__ void __launch_bounds__(256)
k_flags_grad(const T* __restrict__ buf, const amr_halo_meta* __restrict__ meta, const int32_t* __restrict__ levels,
             int P, Geo g, GradRule rule, int min_level, int max_level, int8_t* __restrict__ flags,
             const uint64_t* __restrict__ keys, const int32_t* __restrict__ bounds)
{
    const int lane = threadIdx.x & 31;
    for (int p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; p < P; p += (gridDim.x * blockDim.x) >> 5) {
        int any = 0, all = 1;
        for (int c = lane; c < g.cells; c += 32)
            gradient_rule_cell<T, GhostsOnTheFly, R>(buf, meta, g, rule, p, c, any, all);
        any = __any_sync(0xffffffffu, any);
        all = __all_sync(0xffffffffu, all);
        if (lane == 0) {
            int lo = min_level, hi = max_level;
            if (bounds) {
                const int inst = instance_of(g, keys, p);
                lo             = bounds[2 * inst];
                hi             = bounds[2 * inst + 1];
            }
            flags[p] = gradient_decision(any, all, levels[p], lo, hi);
        }
    }
}

// Max-value rule (fvm_refinement_criterion.cu:27-67, tests'
// advection_equation_amr.t.cpp:155-170) over interior and face-ghost cells.
__device__ inline bool face_or_interior(const Geo& g, int c)
{
    int outside = 0;
    for (int L = g.rank - 1; L >= 0; --L) {
        const int i = c % g.P1;
        c /= g.P1;
        outside += (i < g.h || i >= g.n + g.h) ? 1 : 0;
    }
    return outside <= 1;
}

__device__ inline int8_t max_decision(double mx, int level, double rthr, double cthr, int min_level, int max_level)
{
    return (mx > rthr && level < max_level) ? FLAG_REFINE : (mx < cthr && level > min_level) ? FLAG_COARSEN : FLAG_STABLE;
}

template <typename T>
__global__ void __launch_bounds__(128)
k_flags_max(const T* __restrict__ buf, const int32_t* __restrict__ levels, int P, Geo g, double rthr,
            double cthr, int min_level, int max_level, int8_t* __restrict__ flags,
            const uint64_t* __restrict__ keys = nullptr, const int32_t* __restrict__ bounds = nullptr)
{
    const int p = blockIdx.x;
    if (p >= P) return;
    if (bounds) {
        const int inst = instance_of(g, keys, p);
        min_level      = bounds[2 * inst];
        max_level      = bounds[2 * inst + 1];
    }
    const T* u = buf + static_cast<size_t>(p) * g.flat;
    double   m = 0.0;
    for (int c = threadIdx.x; c < g.flat; c += blockDim.x)
        if (face_or_interior(g, c)) m = fmax(m, static_cast<double>(u[c]));
    __shared__ double red[128];
    red[threadIdx.x] = m;
    __syncthreads();
    for (int w = 64; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + w]);
        __syncthreads();
    }
    if (threadIdx.x == 0) flags[p] = max_decision(red[0], levels[p], rthr, cthr, min_level, max_level);
}

// ------------------------------------------------------------- time step dt
// Per-batch prologue for one instance (one block): thread 0 walks the step
// sizes of the batch (the clamp is sequential in the remaining time), then
// the block fills the (step, level) coefficient table in parallel.
// Per-instance time bookkeeping: acc/cnt = simulated time and executed steps
// of the current batch, rem = time still to go, tot/ctot = the sums of the
// batches before it in the current run (batch sums are added in order, as
// the reference's host loop adds finish_advance_batch results).
struct DtState {
    double*   acc;
    double*   rem;
    uint32_t* cnt;
    double*   tot;
    uint32_t* ctot;
};

// Batch opening modes of k_batch_begin.
enum : int {
    BATCH_CONTINUE = 0, // same batch (a further chunk of one advance call)
    BATCH_RESET    = 1, // first batch: totals, batch sums and remaining time start over
    BATCH_NEXT     = 2, // next batch of a run: fold the batch into the totals, keep the remaining time
    BATCH_NEXT_REM = 3, // next batch of a run with the remaining time given by the host
};

// Block b handles instance b: its CFL step from its own finest level and
// velocity; coef row (step s, instance b) starts at (s * ninst + b) * (depth+1).
// coef32 holds the rows rounded to FP32 once: (c_x, c_y) float2 entries for
// 2D trees, (c_x, c_y, c_z, c0) float4 entries for 3D trees.
static __global__ void __launch_bounds__(256)
k_batch_begin(const int32_t* __restrict__ max_level, Geo g, const double* __restrict__ vel, double cfl, int steps,
              int mode, double remaining0, DtState d, double* __restrict__ step_dt, Coef* __restrict__ coef,
              float2* __restrict__ coef32 = nullptr, int32_t* __restrict__ upcode = nullptr,
              const int32_t* __restrict__ skip = nullptr)
{
    __shared__ double dts[1024];
    if (skip && *skip) return; // a graph interval that was stopped before it began
    const int         inst  = blockIdx.x;
    const int         ninst = gridDim.x;
    const double      v[3]  = { vel[3 * inst], vel[3 * inst + 1], vel[3 * inst + 2] };
    if (threadIdx.x == 0) {
        const double raw = raw_dt(g, v, max_level[inst]);
        double       rem = d.rem[inst], sum = d.acc[inst];
        uint32_t     cnt = d.cnt[inst];
        if (mode == BATCH_RESET) {
            d.tot[inst]  = 0.0;
            d.ctot[inst] = 0u;
        } else if (mode != BATCH_CONTINUE) {
            d.tot[inst] += sum;
            d.ctot[inst] += cnt;
        }
        if (mode != BATCH_CONTINUE) {
            sum = 0.0;
            cnt = 0u;
        }
        if (mode == BATCH_RESET || mode == BATCH_NEXT_REM) rem = remaining0;
        for (int s = 0; s < steps; ++s) {
            const double dt = clamp_step(raw, cfl, rem);
            sum += dt;
            if (dt > 0.0) {
                rem -= dt;
                ++cnt;
            }
            dts[s]                                         = dt;
            step_dt[static_cast<size_t>(s) * ninst + inst] = dt;
        }
        d.acc[inst] = sum;
        d.rem[inst] = rem;
        d.cnt[inst] = cnt;
    }
    if (threadIdx.x == 0 && upcode) upcode[inst] = pack_upwind(v);
    __syncthreads();
    const int nl = g.depth + 1;
    for (int e = threadIdx.x; e < steps * nl; e += blockDim.x) {
        const int    st = e / nl, l = e % nl;
        const size_t at = (static_cast<size_t>(st) * ninst + inst) * nl + l;
        const Coef   c  = make_coef(g, dts[st], v, l);
        coef[at]        = c;
        if (coef32) {
            if (g.rank == 3) // (c_x, c_y, c_z, c0) rows of the 3D FP32 update
                reinterpret_cast<float4*>(coef32)[at] = make_float4(
                    static_cast<float>(c.c[0]), static_cast<float>(c.c[1]), static_cast<float>(c.c[2]),
                    static_cast<float>(c.c0));
            else
                coef32[at] = make_float2(static_cast<float>(c.c[0]), static_cast<float>(c.c[1]));
        }
    }
}

// Refinement flags that refine every leaf below its instance's target level.
static __global__ void k_flags_to_level(const uint64_t* __restrict__ keys, int P, Geo g, const int32_t* __restrict__ target,
                                 int8_t* __restrict__ flags)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    flags[p] = key_level(keys[p]) < target[instance_of(g, keys, p)] ? FLAG_REFINE : FLAG_STABLE;
}

// Maximum level over a level array.
static __global__ void k_max_level(const int32_t* __restrict__ levels, int P, int32_t* __restrict__ out)
{
    int m = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P; i += gridDim.x * blockDim.x) m = max(m, levels[i]);
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

// ------------------------------------------------------------ re-mesh
// (C1-C9) Every leaf array is in Morton order on entry and on exit.

// Refine eligibility (is_refine_elegible, ndtree.hpp:1888-1896) and coarsen
// candidates: a leaf that is child 0 of its parent, followed by its 2^rank-1
// siblings, all flagged Coarsen (apply_refine_coarsen + is_coarsen_elegible,
// ndtree.hpp:904-940, 1899-1917).
__device__ inline void mark_leaf(const uint64_t* keys, const int8_t* flags, int P, const Geo& g, uint8_t* rmark,
                                 uint8_t* chead, int i)
{
    const uint64_t k     = keys[i];
    const int      level = key_level(k);
    rmark[i]             = (flags[i] == FLAG_REFINE && level < g.depth) ? 1 : 0;
    uint8_t head         = 0;
    if (level > 0 && key_offset(g, k) == 0 && i + g.nd <= P) {
        const uint64_t parent = key_parent(g, k);
        head                  = 1;
        for (int j = 0; j < g.nd && head; ++j)
            if (keys[i + j] != key_child(g, parent, j) || flags[i + j] != FLAG_COARSEN) head = 0;
    }
    chead[i] = head;
}

// One round of the 2:1 refinement closure (balancing, ndtree.hpp:1129-1165):
// a refining leaf marks its coarser face neighbours.  Marks only grow, so as
// many rounds as the deepest level reach the fixed point the reference's
// work list reaches.
__device__ inline void closure_leaf(const amr_halo_meta* meta, const Geo& g, uint8_t* rmark, int i)
{
    if (!rmark[i]) return;
    for (int d = 0; d < g.ndir; ++d) {
        const amr_halo_meta& m = meta[static_cast<size_t>(i) * g.ndir + d];
        if (m.relation == REL_COARSER) rmark[m.neighbor] = 1;
    }
}

// Coarsening veto (balancing, ndtree.hpp:1173-1239): a candidate parent is
// dropped if a boundary child has a finer neighbour across that face, or a
// same-level neighbour that refines.
__device__ inline void veto_leaf(const amr_halo_meta* meta, const Geo& g, const uint8_t* rmark, uint8_t* chead, int i)
{
    if (!chead[i]) return;
    for (int d = 0; d < g.ndir; ++d) {
        const int L = d / 2, pos = d % 2;
        for (int off = 0; off < g.nd; ++off) {
            if (child_coord(g, off, L) != pos) continue; // boundary children of face d
            const amr_halo_meta& m = meta[static_cast<size_t>(i + off) * g.ndir + d];
            if (m.relation == REL_FINER || (m.relation == REL_SAME && rmark[m.neighbor])) {
                chead[i] = 0;
                return;
            }
        }
    }
}

__device__ inline bool in_coarsen_group(const uint64_t* keys, const uint8_t* chead, int i, const Geo& g)
{
    const uint64_t k = keys[i];
    if (key_level(k) == 0) return false;
    const int h = i - key_offset(g, k);
    return h >= 0 && chead[h];
}

// Output count per old leaf: 2^rank for a refined leaf, 1 for the head of a
// coarsened group (the new parent), 0 for the other members, 1 otherwise.
__device__ inline void count_leaf(const uint64_t* keys, const uint8_t* rmark, const uint8_t* chead, const Geo& g,
                                  uint32_t* cnt, int32_t* changed, int i)
{
    uint32_t c = 1;
    if (rmark[i]) {
        c        = g.nd;
        *changed = 1;
    } else if (in_coarsen_group(keys, chead, i, g)) {
        c        = chead[i] ? 1u : 0u;
        *changed = 1;
    }
    cnt[i] = c;
}

// Exclusive scan of cnt[0..P) into pos[0..P] by one block (part has one slot
// per thread); pos[P] = new size; status[2] = new size, status[0] set to
// AMR_ERR_CAPACITY when it exceeds cap.
__device__ inline void block_scan(const uint32_t* cnt, uint32_t* pos, int P, size_t cap, int32_t* status,
                                  uint32_t* part)
{
    const int per = (P + blockDim.x - 1) / blockDim.x;
    const int lo = threadIdx.x * per, hi = min(P, lo + per);
    uint32_t  s  = 0;
    for (int i = lo; i < hi; ++i) s += cnt[i];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int o = 1; o < blockDim.x; o <<= 1) {
        const uint32_t v = threadIdx.x >= o ? part[threadIdx.x - o] : 0;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    uint32_t run = part[threadIdx.x] - s;
    for (int i = lo; i < hi; ++i) {
        pos[i] = run;
        run += cnt[i];
    }
    if (threadIdx.x == blockDim.x - 1) {
        pos[P]    = part[threadIdx.x];
        status[2] = static_cast<int32_t>(part[threadIdx.x]);
        if (part[threadIdx.x] > cap) status[0] = AMR_ERR_CAPACITY;
    }
    __syncthreads();
}

// Source descriptor of a new leaf: kind 0 copy, 1..2^rank child (offset+1)
// of a refined leaf, -1 parent of a coarsened group.
__device__ inline void emit_leaf(const uint64_t* keys, const uint8_t* rmark, const uint8_t* chead, const uint32_t* pos,
                                 const Geo& g, uint64_t* nkeys, int32_t* nlevels, int32_t* src, int8_t* skind,
                                 int32_t* max_level, int i)
{
    const uint64_t k = keys[i];
    const uint32_t q = pos[i];
    const int      l = key_level(k);
    int            lmax;
    if (rmark[i]) {
        for (int j = 0; j < g.nd; ++j) {
            nkeys[q + j]   = key_child(g, k, j);
            nlevels[q + j] = l + 1;
            src[q + j]     = i;
            skind[q + j]   = static_cast<int8_t>(j + 1);
        }
        lmax = l + 1;
    } else if (in_coarsen_group(keys, chead, i, g)) {
        if (!chead[i]) return;
        nkeys[q]   = key_parent(g, k);
        nlevels[q] = l - 1;
        src[q]     = i;
        skind[q]   = -1;
        lmax       = l - 1;
    } else {
        nkeys[q]   = k;
        nlevels[q] = l;
        src[q]     = i;
        skind[q]   = 0;
        lmax       = l;
    }
    const int inst = g.inst_shift >= 64 ? 0 : static_cast<int>(k >> g.inst_shift);
    atomicMax(max_level + inst, lmax);
}

// Interior cell c of new leaf j: copy, piecewise-constant prolongation
// (interpolate_patch, ndtree.hpp:1528-1555) or mean restriction
// (restrict_patches, :1499-1526; sum order of hypercube_offset,
// patch_utils.hpp:203-234).
template <typename T>
__device__ inline void remap_cell(const T* old_state, T* new_state, const Geo& g, int kind, int srcj, int j, int c)
{
    int idx[3];
    interior_coords(g, c, idx);
    const int li   = padded_index(g, idx);
    const T*  from = old_state + static_cast<size_t>(srcj) * g.flat;
    T*        to   = new_state + static_cast<size_t>(j) * g.flat;
    const int half = g.n / 2;
    if (kind == 0) {
        to[li] = from[li];
    } else if (kind > 0) {
        const int off   = kind - 1;
        int       pc[3] = { 0, 0, 0 };
        for (int L = 0; L < g.rank; ++L) pc[L] = g.h + child_coord(g, off, L) * half + (idx[L] - g.h) / 2;
        to[li] = from[padded_index(g, pc)];
    } else {
        int child = 0, base[3] = { 0, 0, 0 };
        for (int L = 0; L < g.rank; ++L) {
            child   = (child << 1) | ((idx[L] - g.h) / half);
            base[L] = ((idx[L] - g.h) % half) * 2 + g.h;
        }
        const T* fp  = from + static_cast<size_t>(child) * g.flat + padded_index(g, base);
        double   sum = 0.0;
        if (g.rank == 2) {
            sum += static_cast<double>(fp[0]);
            sum += static_cast<double>(fp[1]);
            sum += static_cast<double>(fp[g.s[0]]);
            sum += static_cast<double>(fp[g.s[0] + 1]);
            to[li] = static_cast<T>(sum / 4.0);
        } else {
            for (int a = 0; a < 2; ++a)
                for (int b = 0; b < 2; ++b)
                    for (int e = 0; e < 2; ++e) sum += static_cast<double>(fp[a * g.s[0] + b * g.s[1] + e]);
            to[li] = static_cast<T>(sum / 8.0);
        }
    }
}

// One block per new leaf; kept patches move whole (16-byte words, ghosts
// included), new ones are built cell by cell.  blockIdx.y = field of a
// multi-field state (fields fstride elements apart).
template <typename T>
__global__ void __launch_bounds__(256)
k_remap(const T* __restrict__ old_state, T* __restrict__ new_state, const int32_t* __restrict__ src,
        const int8_t* __restrict__ skind, int P, Geo g, size_t fstride = 0)
{
    old_state += blockIdx.y * fstride;
    new_state += blockIdx.y * fstride;
    const int j = blockIdx.x;
    if (j >= P) return;
    const int kind = skind[j];
    if (kind == 0) {
        const size_t bytes = static_cast<size_t>(g.flat) * sizeof(T);
        const uint4* f4    = reinterpret_cast<const uint4*>(old_state + static_cast<size_t>(src[j]) * g.flat);
        uint4*       t4    = reinterpret_cast<uint4*>(new_state + static_cast<size_t>(j) * g.flat);
        for (size_t w = threadIdx.x; w < bytes / 16; w += blockDim.x) t4[w] = f4[w];
        return;
    }
    for (int c = threadIdx.x; c < g.cells; c += blockDim.x) remap_cell<T>(old_state, new_state, g, kind, src[j], j, c);
}

// flag = 1 when some neighbour record is not "same level" (flag zeroed first).
static __global__ void k_any_not_same(const amr_halo_meta* __restrict__ meta, long long n, int32_t* flag)
{
    for (long long t = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; t < n;
         t += static_cast<long long>(gridDim.x) * blockDim.x)
        if (meta[t].relation != REL_SAME) *flag = 1;
}

__device__ inline int upper_bound_u64(const uint64_t* a, int n, uint64_t x)
{
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (a[mid] <= x) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

__device__ inline int find_u64(const uint64_t* a, int n, uint64_t x)
{
    const int u = upper_bound_u64(a, n, x);
    return (u > 0 && a[u - 1] == x) ? u - 1 : -1;
}

// Neighbour record t = (leaf, direction) from geometry.  The reference
// maintains the tables incrementally through fragment/recombine
// (neighbor.hpp:420-572, ndtree.hpp:942-1125); on a 2:1-balanced periodic
// tree its tables equal the geometric relation of each face:
//   same    : the leaf covering the adjacent same-size region,
//   coarser : the covering leaf one level up, with the quadrant of it that
//             touches this leaf (neighbor.hpp:367-379),
//   finer   : the children of the adjacent region on the shared face, in
//             compute_boundary_children order (neighbor.hpp:397-417).
// The domain wraps in every direction (the root is its own neighbour,
// ndtree.hpp:411-421).  A face that is not 2:1 gets relation none (never an
// invalid index) and status[0] = AMR_ERR_UNBALANCED.
__device__ inline void neighbor_entry(const uint64_t* keys, int P, const Geo& g, amr_halo_meta* meta, int32_t* status,
                                      int t)
{
    const int      i = t / g.ndir, d = t % g.ndir;
    const int      L = d / 2, pos = d % 2, axis = g.rank - 1 - L;
    const uint64_t k = keys[i];
    const int      l = key_level(k);
    uint32_t       c[3];
    key_decode(g, k, c);
    const uint32_t s    = 1u << (g.depth - l);
    const uint32_t wrap = (g.depth >= 32) ? 0xFFFFFFFFu : ((1u << g.depth) - 1u);
    c[axis]             = (pos ? c[axis] + s : c[axis] - s) & wrap;
    const uint64_t pre  = key_prefix(g, k);
    const int      b    = upper_bound_u64(keys, P, key_encode(g, pre, c, 63)) - 1;
    amr_halo_meta  m;
    m.neighbor = -1;
    for (int q = 0; q < 4; ++q) m.finer_ids[q] = -1;
    for (int q = 0; q < 3; ++q) m.quadrant[q] = 0;
    m.relation   = REL_NONE;
    m.padding[0] = m.padding[1] = m.padding[2] = 0;
    const int lb = b >= 0 ? key_level(keys[b]) : -1;
    if (b >= 0 && lb == l) {
        m.relation = REL_SAME;
        m.neighbor = b;
    } else if (b >= 0 && lb == l - 1) {
        uint32_t cb[3];
        key_decode(g, keys[b], cb);
        m.relation = REL_COARSER;
        m.neighbor = b;
        for (int LL = 0; LL < g.rank; ++LL) {
            const int ax   = g.rank - 1 - LL;
            m.quadrant[LL] = static_cast<int32_t>(((c[ax] - cb[ax]) >> (g.depth - l)) & 1u);
        }
    } else if (b >= 0 && lb > l) {
        const uint64_t region  = key_encode(g, pre, c, l);
        const int      opp_pos = 1 - pos;
        bool           found   = true;
        for (int off = 0; off < g.nd; ++off) {
            if (child_coord(g, off, L) != opp_pos) continue;
            int kk = 0, mult = 1; // compute_fine_boundary_linear_index: dim 0 fastest
            for (int LL = 0; LL < g.rank; ++LL) {
                if (LL == L) continue;
                kk += child_coord(g, off, LL) * mult;
                mult *= 2;
            }
            const int f     = find_u64(keys, P, key_child(g, region, off));
            found           = found && f >= 0;
            m.finer_ids[kk] = f;
        }
        if (found) {
            m.relation = REL_FINER;
        } else {
            for (int q = 0; q < 4; ++q) m.finer_ids[q] = -1;
            status[0] = AMR_ERR_UNBALANCED;
        }
    } else {
        status[0] = AMR_ERR_UNBALANCED;
    }
    meta[t] = m;
}

// --------------------------------------------- per-launch re-mesh kernels
static __global__ void k_mark(const uint64_t* __restrict__ keys, const int8_t* __restrict__ flags, int P, Geo g,
                       uint8_t* __restrict__ rmark, uint8_t* __restrict__ chead)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < P) mark_leaf(keys, flags, P, g, rmark, chead, i);
}

static __global__ void k_closure(const amr_halo_meta* __restrict__ meta, int P, Geo g, uint8_t* rmark)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < P) closure_leaf(meta, g, rmark, i);
}

static __global__ void k_veto(const amr_halo_meta* __restrict__ meta, int P, Geo g, const uint8_t* __restrict__ rmark,
                       uint8_t* __restrict__ chead)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < P) veto_leaf(meta, g, rmark, chead, i);
}

static __global__ void k_count(const uint64_t* __restrict__ keys, const uint8_t* __restrict__ rmark,
                        const uint8_t* __restrict__ chead, int P, Geo g, uint32_t* __restrict__ cnt,
                        int32_t* __restrict__ changed)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < P) count_leaf(keys, rmark, chead, g, cnt, changed, i);
}

static __global__ void __launch_bounds__(1024)
k_scan(const uint32_t* __restrict__ cnt, uint32_t* __restrict__ pos, int P, size_t cap, int32_t* __restrict__ status)
{
    __shared__ uint32_t part[1024];
    block_scan(cnt, pos, P, cap, status, part);
}

static __global__ void k_emit(const uint64_t* __restrict__ keys, const uint8_t* __restrict__ rmark,
                       const uint8_t* __restrict__ chead, const uint32_t* __restrict__ pos, int P, Geo g,
                       uint64_t* __restrict__ nkeys, int32_t* __restrict__ nlevels, int32_t* __restrict__ src,
                       int8_t* __restrict__ skind, int32_t* __restrict__ max_level)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < P) emit_leaf(keys, rmark, chead, pos, g, nkeys, nlevels, src, skind, max_level, i);
}

static __global__ void k_neighbors(const uint64_t* __restrict__ keys, int P, Geo g, amr_halo_meta* __restrict__ meta,
                            int32_t* __restrict__ status)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < P * g.ndir) neighbor_entry(keys, P, g, meta, status, t);
}

// --------------------------------------------------- reference drop-ins
template <typename T>
__global__ void __launch_bounds__(256)
k_intergrid(T* __restrict__ buf, const amr_transfer_task* __restrict__ tasks, int ntask, Geo g, int restrict_mode)
{
    const int task = blockIdx.x;
    if (task >= ntask) return;
    const amr_transfer_task tk   = tasks[task];
    const int               half = g.n / 2;
    for (int c = threadIdx.x; c < g.cells; c += blockDim.x) {
        int idx[3];
        interior_coords(g, c, idx);
        int child = 0, base[3] = { 0, 0, 0 };
        for (int L = 0; L < g.rank; ++L) {
            child   = (child << 1) | ((idx[L] - g.h) / half);
            base[L] = ((idx[L] - g.h) % half) * 2 + g.h;
        }
        const int bi = padded_index(g, base);
        const int ci = padded_index(g, idx);
        if (restrict_mode) {
            const T* fp  = buf + static_cast<size_t>(tk.source_patch + child) * g.flat + bi;
            double   sum = 0.0;
            if (g.rank == 2) {
                sum += static_cast<double>(fp[0]);
                sum += static_cast<double>(fp[1]);
                sum += static_cast<double>(fp[g.s[0]]);
                sum += static_cast<double>(fp[g.s[0] + 1]);
                buf[static_cast<size_t>(tk.destination_patch) * g.flat + ci] = static_cast<T>(sum / 4.0);
            } else {
                for (int a = 0; a < 2; ++a)
                    for (int b = 0; b < 2; ++b)
                        for (int e = 0; e < 2; ++e) sum += static_cast<double>(fp[a * g.s[0] + b * g.s[1] + e]);
                buf[static_cast<size_t>(tk.destination_patch) * g.flat + ci] = static_cast<T>(sum / 8.0);
            }
        } else {
            const T v  = buf[static_cast<size_t>(tk.source_patch) * g.flat + ci];
            T*      fp = buf + static_cast<size_t>(tk.destination_patch + child) * g.flat + bi;
            if (g.rank == 2) {
                fp[0]          = v;
                fp[1]          = v;
                fp[g.s[0]]     = v;
                fp[g.s[0] + 1] = v;
            } else {
                for (int a = 0; a < 2; ++a)
                    for (int b = 0; b < 2; ++b)
                        for (int e = 0; e < 2; ++e) fp[a * g.s[0] + b * g.s[1] + e] = v;
            }
        }
    }
}

static __global__ void __launch_bounds__(256)
k_gather(const uint4* __restrict__ src, uint4* __restrict__ dst, size_t words_per_patch,
         const int32_t* __restrict__ sources, int count)
{
    const int j = blockIdx.x;
    if (j >= count) return;
    const uint4* f = src + static_cast<size_t>(sources[j]) * words_per_patch;
    uint4*       t = dst + static_cast<size_t>(j) * words_per_patch;
    for (size_t w = threadIdx.x; w < words_per_patch; w += blockDim.x) t[w] = f[w];
}

static __global__ void k_gather_bytes(const unsigned char* __restrict__ src, unsigned char* __restrict__ dst,
                               size_t bytes, const int32_t* __restrict__ sources, int count)
{
    const int j = blockIdx.x;
    if (j >= count) return;
    const unsigned char* f = src + static_cast<size_t>(sources[j]) * bytes;
    unsigned char*       t = dst + static_cast<size_t>(j) * bytes;
    for (size_t w = threadIdx.x; w < bytes; w += blockDim.x) t[w] = f[w];
}

// finalize_step_dt_kernel semantics (fvm_time_step.cu:204-233) for the
// drop-in dt entry point.
static __global__ void k_finalize_dt(const int32_t* __restrict__ max_level, Geo g, double v0, double v1, double v2,
                              double cfl, double* dt_buf, double* acc, double* remaining, uint32_t* count)
{
    const double v[3]    = { v0, v1, v2 };
    const double step_dt = clamp_step(raw_dt(g, v, *max_level), cfl, *remaining);
    *dt_buf              = step_dt;
    *acc += step_dt;
    if (step_dt > 0.0) {
        *remaining -= step_dt;
        ++(*count);
    }
}

} // namespace amr_gb300

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
// transpose is lin_j + sum_a (contributions - c_a(p) lin_j).  Ghost cells of
// lout are not written (the caller keeps them zero).
template <typename T>
__device__ inline void adjoint_cell(const T* lin, T* lout, const amr_halo_meta* meta, const uint64_t* keys,
                                    const Geo& g, const Coef* coef, const int* up_launch, const double* vel, int p,
                                    int c)
{
    constexpr bool F32 = sizeof(T) == 4;
    int            idx[3];
    interior_coords(g, c, idx);
    const int      nl   = g.depth + 1;
    const uint64_t kp   = keys[p];
    const int      inst = g.inst_shift >= 64 ? 0 : static_cast<int>(kp >> g.inst_shift);
    int            up[3] = { up_launch[0], up_launch[1], up_launch[2] };
    if (vel)
        for (int a = 0; a < 3; ++a) up[a] = a < g.rank ? upwind(vel[3 * inst + a]) : 0;
    const Coef   cp   = coef[inst * nl + key_level(kp)];
    const size_t base = static_cast<size_t>(p) * g.flat;
    const int    li   = padded_index(g, idx);
    const T      lj   = lin[base + li];
    T            acc  = F32 ? lj : static_cast<T>(cp.c0) * lj;
    const int    half = g.n / 2;
    for (int a = 0; a < g.rank; ++a) {
        if (up[a] == 0) continue;
        const int L = g.rank - 1 - a, d = -up[a], pos_d = d > 0 ? 1 : 0;
        const int dist = pos_d ? (g.n + g.h - 1 - idx[L]) : (idx[L] - g.h); // cells to the downwind face
        const T   ca   = static_cast<T>(cp.c[a]);
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
            const Coef cq   = coef[inst * nl + key_level(keys[m.neighbor])];
            const T    w    = static_cast<T>(static_cast<T>(cq.c[a]) / static_cast<T>(1 << g.rank));
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
            const Coef  cf  = coef[inst * nl + key_level(keys[f])];
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
                acc = fma(static_cast<T>(cf.c[a]), s, acc);
            } else {
                T s = T(0);
                for (int b0 = 0; b0 < 2; ++b0)
                    for (int b1 = 0; b1 < 2; ++b1) {
                        int q[3] = { fi[0], fi[1], fi[2] };
                        q[t0] += b0;
                        q[t1] += b1;
                        s += fp[padded_index(g, q)];
                    }
                acc = fma(static_cast<T>(cf.c[a]), s, acc);
            }
        }
    }
    lout[base + li] = acc;
}

template <typename T>
__global__ void __launch_bounds__(256)
k_adjoint(const T* __restrict__ lin, T* __restrict__ lout, const amr_halo_meta* __restrict__ meta,
          const uint64_t* __restrict__ keys, int P, Geo g, const Coef* __restrict__ coef, int up0, int up1, int up2,
          const double* __restrict__ vel, int ppb)
{
    const int up[3] = { up0, up1, up2 };
    const int p0    = blockIdx.x * ppb;
    for (int t = threadIdx.x; t < ppb * g.cells; t += blockDim.x) {
        const int p = p0 + t / g.cells;
        if (p >= P) break;
        adjoint_cell<T>(lin, lout, meta, keys, g, coef, up, vel, p, t - (p - p0) * g.cells);
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
                               int ninst, Coef* __restrict__ coef)
{
    const int nl    = g.depth + 1;
    const int total = steps * ninst * nl;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
        const int    l = e % nl, si = e / nl, inst = si % ninst;
        const double v[3] = { vel[3 * inst], vel[3 * inst + 1], vel[3 * inst + 2] };
        coef[e]           = make_coef(g, dts[si], v, l);
    }
}

} // namespace amr_gb300

namespace amr_gb300 {

// ------------------------------------------------ 3D update, staged
// One step of 3D patches of N^3 cells and one ghost layer, one warp per
// patch (grid-stride).  The patch's interior planes (ghost rows and columns
// included, a contiguous 16-byte-aligned span) move into a per-warp
// shared-memory tile by bulk async copy; each warp owns S tiles in a ring
// and keeps S-1 copies in flight ahead of the patch it works on.  While the
// copy lands the lanes evaluate the upwind ghost faces by the halo rules
// (ghost_value, the values step_cell takes on the fly), then write them into
// the tile, update N^3/32 cells each from the tile with step_cell's
// arithmetic, and store the interior planes back as 16-byte words (ghost
// rows and columns pass through, as in the 2D kernels).  A copy that does
// not land within the wait cap sets *err = AMR_ERR_TIMEOUT; the warp then
// drains its other copies (also capped) and stops.
template <typename T, int N>
struct Step3dShape {
    static constexpr int      P1 = N + 2, PLANE = P1 * P1, FLAT = PLANE * P1;
    static constexpr uint32_t LO    = PLANE * sizeof(T);           // byte span of the interior planes
    static constexpr uint32_t BYTES = N * PLANE * sizeof(T);
    static constexpr int      WORDS = BYTES / 16;
    static constexpr int      PER   = N * N * N / 32;              // cells per lane
    static constexpr int      GPL   = (N * N + 31) / 32;           // ghost cells per lane and face
    static constexpr size_t   TILE  = FLAT * sizeof(T);
    static_assert(LO % 16 == 0 && BYTES % 16 == 0 && TILE % 16 == 0, "planes are whole 16-byte words");
    static_assert(N * N * N % 32 == 0, "a warp's lanes share the cells evenly");
    static constexpr size_t smem(int W, int S) { return static_cast<size_t>(W) * S * (TILE + 8); }
};

template <typename T, int N, int S>
__device__ __forceinline__ void step3d_body(const T* __restrict__ in, T* __restrict__ out,
                                            const amr_halo_meta* __restrict__ meta, const int32_t* __restrict__ levels,
                                            const uint64_t* __restrict__ keys, int P, const Geo& g,
                                            const Coef* __restrict__ coef, const float4* __restrict__ coef4,
                                            int up0, int up1, int up2, const int32_t* __restrict__ upcode,
                                            int32_t* err, T* tiles, uint64_t* bars, int p, int nwarp)
{
    using Sh               = Step3dShape<T, N>;
    constexpr int P1       = Sh::P1, PLANE = Sh::PLANE, FLAT = Sh::FLAT, GPL = Sh::GPL;
    const int     lane     = threadIdx.x & 31;
    const int     nl       = g.depth + 1;
    if (lane == 0) {
        for (int b = 0; b < S; ++b) mbar_init(&bars[b], 1);
        mbar_init_fence();
    }
    __syncwarp();
    const char* in_bytes = reinterpret_cast<const char*>(in);
    auto        request  = [&](int q, int slot) {
        fence_proxy_async_smem();
        mbar_expect_tx(&bars[slot], Sh::BYTES);
        bulk_copy_g2s(reinterpret_cast<char*>(tiles + static_cast<size_t>(slot) * FLAT) + Sh::LO,
                      in_bytes + static_cast<size_t>(q) * Sh::TILE + Sh::LO, Sh::BYTES, &bars[slot]);
    };
    if (lane == 0)
        for (int j = 0; j < S - 1; ++j)
            if (p + j * nwarp < P) request(p + j * nwarp, j);
    uint32_t phase = 0; // bit b: parity of slot b's next completion
    for (int it = 0; p < P; ++it, p += nwarp) {
        const int b  = it % S;
        const int pf = p + (S - 1) * nwarp;
        if (pf < P && lane == 0) request(pf, (it + S - 1) % S);
        const int inst  = keys ? instance_of(g, keys, p) : 0;
        int       up[3] = { up0, up1, up2 };
        if (upcode) { // per-instance upwind sides, packed (integer decode: no FP64 compares)
            const int32_t code = upcode[inst];
            for (int a = 0; a < 3; ++a) up[a] = unpack_upwind(code, a);
        }
        // the row of the leaf's level: FP64 from coef, FP32 from the rows
        // rounded once (coef4)
        const int row = inst * nl + levels[p];
        T         c0, ca[3];
        if constexpr (sizeof(T) == 4) {
            const float4 c4 = coef4[row];
            c0              = c4.w;
            ca[0]           = c4.x;
            ca[1]           = c4.y;
            ca[2]           = c4.z;
        } else {
            const Coef cf = coef[row];
            c0            = cf.c0;
            ca[0]         = cf.c[0];
            ca[1]         = cf.c[1];
            ca[2]         = cf.c[2];
        }
        const T* src = in + static_cast<size_t>(p) * FLAT;
        // the upwind ghost faces (Morton axis a is layout dim 2 - a): ghost
        // cell k of a face has tangential coordinates (k / N + 1, k % N + 1)
        T gv[3][GPL];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const int L = 2 - a, pos = up[a] > 0 ? 1 : 0;
#pragma unroll
            for (int j = 0; j < GPL; ++j) {
                const int k = lane + 32 * j;
                gv[a][j]    = T(0);
                if (up[a] != 0 && k < N * N) {
                    int G[3];
                    G[L]              = pos ? N + 1 : 0;
                    G[L == 0 ? 1 : 0] = k / N + 1;
                    G[L == 2 ? 1 : 2] = k % N + 1;
                    gv[a][j] =
                        ghost_value<T, T>(in, FLAT, meta[static_cast<size_t>(p) * 6 + 2 * L + pos], G, L, pos, g, src);
                }
            }
        }
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
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const int L = 2 - a;
#pragma unroll
            for (int j = 0; j < GPL; ++j) {
                const int k = lane + 32 * j;
                if (up[a] != 0 && k < N * N) {
                    int G[3];
                    G[L]              = up[a] > 0 ? N + 1 : 0;
                    G[L == 0 ? 1 : 0] = k / N + 1;
                    G[L == 2 ? 1 : 2] = k % N + 1;
                    tile[(G[0] * P1 + G[1]) * P1 + G[2]] = gv[a][j];
                }
            }
        }
        __syncwarp();
        T res[Sh::PER];
#pragma unroll
        for (int q = 0; q < Sh::PER; ++q) {
            const int c   = lane + 32 * q;
            const int li  = ((c / (N * N) + 1) * P1 + (c / N) % N + 1) * P1 + c % N + 1;
            const T   u   = tile[li];
            T         acc = sizeof(T) == 4 ? u : c0 * u;
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                if (up[a] == 0) continue;
                const int st  = a == 0 ? 1 : (a == 1 ? P1 : PLANE);
                const T   val = tile[li + up[a] * st];
                acc = fma(ca[a], sizeof(T) == 4 ? static_cast<T>(val - u) : val, acc);
            }
            res[q] = acc;
        }
        __syncwarp();
#pragma unroll
        for (int q = 0; q < Sh::PER; ++q) {
            const int c                                                          = lane + 32 * q;
            tile[((c / (N * N) + 1) * P1 + (c / N) % N + 1) * P1 + c % N + 1] = res[q];
        }
        __syncwarp();
        const uint4* t4  = reinterpret_cast<const uint4*>(reinterpret_cast<const char*>(tile) + Sh::LO);
        uint4*       dst = reinterpret_cast<uint4*>(reinterpret_cast<char*>(out + static_cast<size_t>(p) * FLAT) + Sh::LO);
        for (int w = lane; w < Sh::WORDS; w += 32) dst[w] = t4[w];
        __syncwarp(); // the slot is refilled by a later copy
    }
}

// Tiles and barriers of warp wib in a block of W warps with S slots each.
template <typename T, int N, int W, int S>
__device__ __forceinline__ void step3d_smem(unsigned char* smem, T*& tiles, uint64_t*& bars)
{
    const int wib = threadIdx.x >> 5;
    tiles         = reinterpret_cast<T*>(smem) + static_cast<size_t>(wib) * S * Step3dShape<T, N>::FLAT;
    bars          = reinterpret_cast<uint64_t*>(smem + static_cast<size_t>(W) * S * Step3dShape<T, N>::TILE) + wib * S;
}

// Host-driven launch: W warps per block, one per patch.
template <typename T, int N, int W, int S>
__global__ void __launch_bounds__(W * 32)
k_step3d(const T* __restrict__ in, T* __restrict__ out, const int32_t* __restrict__ levels,
         const amr_halo_meta* __restrict__ meta, int P, Geo g, const Coef* __restrict__ coef,
         const float4* __restrict__ coef4, int up0, int up1, int up2, const uint64_t* __restrict__ keys,
         const int32_t* __restrict__ upcode, int32_t* err)
{
    extern __shared__ __align__(128) unsigned char smem3d[];
    T*        tiles;
    uint64_t* bars;
    step3d_smem<T, N, W, S>(smem3d, tiles, bars);
    const int nwarp = (gridDim.x * blockDim.x) >> 5;
    const int p     = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    step3d_body<T, N, S>(in, out, meta, levels, keys, P, g, coef, coef4, up0, up1, up2, upcode, err, tiles, bars, p,
                         nwarp);
}

} // namespace amr_gb300
