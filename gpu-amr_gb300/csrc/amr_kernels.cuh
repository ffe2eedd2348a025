// Kernels of the GB300 AMR hot path: the per-cell update and halo rules of
// any geometry, the gradient and max-value flags, the step sizes, the re-mesh
// and the reference drop-ins.  The shape-specialised kernels live beside it:
// amr_step2d.cuh (2D updates and passes), amr_flags2d.cuh (2D flags),
// amr_step3d.cuh (the staged 3D update), amr_adjoint.cuh (the adjoint).
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

// The new state, one unit per 16-byte word of each new leaf (grid-stride,
// any grid): a kept leaf moves word by word (ghosts included), a refined or
// coarsened leaf is built cell by cell, each unit taking the same share of
// its cells.  blockIdx.y = field of a multi-field state (fields fstride
// elements apart).
template <typename T>
__global__ void __launch_bounds__(256)
k_remap(const T* __restrict__ old_state, T* __restrict__ new_state, const int32_t* __restrict__ src,
        const int8_t* __restrict__ skind, int P, Geo g, size_t fstride = 0)
{
    old_state += blockIdx.y * fstride;
    new_state += blockIdx.y * fstride;
    const int       words = g.flat * static_cast<int>(sizeof(T)) / 16; // padded sides are even
    const int       per   = (g.cells + words - 1) / words;
    const long long total = static_cast<long long>(P) * words;
    for (long long u = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; u < total;
         u += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int j    = static_cast<int>(u / words);
        const int w    = static_cast<int>(u - static_cast<long long>(j) * words);
        const int kind = skind[j];
        if (kind == 0) {
            const uint4* f4 = reinterpret_cast<const uint4*>(old_state + static_cast<size_t>(src[j]) * g.flat);
            reinterpret_cast<uint4*>(new_state + static_cast<size_t>(j) * g.flat)[w] = f4[w];
        } else {
            const int c1 = min(g.cells, (w + 1) * per);
            for (int c = w * per; c < c1; ++c) remap_cell<T>(old_state, new_state, g, kind, src[j], j, c);
        }
    }
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
