// Persistent AMR cycle on one thread-block cluster.
//
// The reference benchmark loop (bench_fvm_solver_integration_active_amr.b.cpp:
// 220-250: advance a batch of steps, flag, reconstruct, exchange halos) runs
// here as ONE kernel launch: every phase is a loop over the cluster's threads,
// separated by hardware cluster barriers (barrier.cluster, release/acquire),
// so a whole run needs no host round trip.  It is meant for trees small
// enough that launch latency, not bandwidth, sets the pace; the host falls
// back to per-launch kernels when the leaf count passes `leaf_limit`.
//
// Control flow between barriers is uniform over the cluster: every decision
// that ends a loop is taken from values all threads read after a barrier, so
// every thread arrives at every barrier.
#pragma once

#include <cooperative_groups.h>
#include <type_traits>

#include "amr_kernels.cuh"

namespace amr_gb300 {

namespace cg = cooperative_groups;

struct CycleStats {
    uint64_t executed;      // time steps with dt > 0
    double   sum_dt;
    uint64_t cell_updates;  // sum of executed x leaves x n^rank per interval
    uint64_t remeshes;
    uint64_t leaves_sum;    // over intervals, leaves before the re-mesh
    uint64_t intervals;
    int32_t  leaves_min, leaves_max;
    int32_t  P, tb, cur, max_level;
    int32_t  error, stopped;
    uint64_t remeshes_changed; // re-meshes that changed the tree
};

struct CycleArgs {
    Geo            g;
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
    int32_t*       status;
    int32_t*       maxlev;
    CycleStats*    stats;
    double         vel[3];
    double         cfl;
    double         remaining;
    int            up[3];
    long long      steps_total;
    int            interval;
    int            crit;
    double         rthr, cthr;
    GradRule       rule;             // squared-norm thresholds of the gradient rule
    int            min_level, max_level;
    int            P0, tb0, max_level0;
    size_t         cap;
    int            leaf_limit;
};

constexpr int kCycleThreads = 512;

// barrier.cluster.arrive.release / wait.acquire: orders every thread's
// earlier global and shared writes before any thread's later reads.
__device__ __forceinline__ void cluster_barrier()
{
    cg::this_cluster().sync();
}

// Max-value rule over interior and face-ghost cells with the ghosts taken
// from the neighbours by the halo rules; one warp per patch.
template <typename T>
__device__ inline double patch_max_on_the_fly(const T* buf, const amr_halo_meta* meta, const Geo& g, int p, int lane)
{
    const T* u = buf + static_cast<size_t>(p) * g.flat;
    double   m = 0.0;
    for (int c = lane; c < g.cells; c += 32) {
        int idx[3];
        interior_coords(g, c, idx);
        m = fmax(m, static_cast<double>(u[padded_index(g, idx)]));
    }
    const long long per_dir = static_cast<long long>(g.h) * (g.cells / g.n);
    for (long long f0 = lane; f0 < per_dir * g.ndir; f0 += 32) {
        const int d = static_cast<int>(f0 / per_dir);
        int       f = static_cast<int>(f0 - d * per_dir);
        const int L = d / 2, pos = d % 2;
        int       G[3] = { 0, 0, 0 };
        for (int k = g.rank - 1; k >= 0; --k) {
            if (k == L) continue;
            G[k] = f % g.n + g.h;
            f /= g.n;
        }
        G[L]                  = pos ? g.n + g.h + f : f;
        const amr_halo_meta& mm = meta[static_cast<size_t>(p) * g.ndir + d];
        m = fmax(m, static_cast<double>(ghost_value<T, T>(buf, g.flat, mm, G, L, pos, g, u)));
    }
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    return m;
}

template <typename T>
__global__ void __launch_bounds__(kCycleThreads, 1) k_cycle(CycleArgs A)
{
    extern __shared__ unsigned char smem_raw[];
    __shared__ uint32_t part[kCycleThreads];
    __shared__ double   s_ctl[4]; // rem at interval end, executed, sum of dt
    const Geo& g        = A.g;
    const int  nl       = g.depth + 1;
    const int  nthreads = blockDim.x * gridDim.x;
    const int  gtid     = blockIdx.x * blockDim.x + threadIdx.x;
    const int  lane     = threadIdx.x & 31;
    const int  gwarp    = gtid >> 5, nwarps = nthreads >> 5;
    const bool leader   = gtid == 0;
    // coefficient rows in the state type's form (FP32 rows rounded once)
    using CT            = std::conditional_t<sizeof(T) == 4, CoefT<float>, Coef>;
    CT*        coef_s   = reinterpret_cast<CT*>(smem_raw);
    double*    dts_s    = reinterpret_cast<double*>(coef_s + static_cast<size_t>(A.interval) * nl);

    int       P = A.P0, tb = A.tb0, cur = 0, maxlevel = A.max_level0;
    long long done = 0;
    double    sum_dt = 0.0;
    uint64_t  executed_total = 0, cell_updates = 0, remeshes = 0, leaves_sum = 0, intervals = 0, remeshes_changed = 0;
    int       lmin = P, lmax = P, error = 0, stopped = 0;

    while (done < A.steps_total) {
        const int k = static_cast<int>(
            (A.interval > 0 && A.interval < A.steps_total - done) ? A.interval : (A.steps_total - done));
        // ---- step sizes and coefficients of this interval (every block keeps its own copy)
        if (threadIdx.x == 0) {
            const double raw = raw_dt(g, A.vel, maxlevel);
            double       rem = A.remaining - sum_dt;
            double       acc = 0.0;
            double       ex  = 0.0;
            for (int s = 0; s < k; ++s) {
                const double dt = clamp_step(raw, A.cfl, rem);
                acc += dt;
                if (dt > 0.0) {
                    rem -= dt;
                    ex += 1.0;
                }
                dts_s[s] = dt;
            }
            s_ctl[0] = acc;
            s_ctl[1] = ex;
        }
        __syncthreads();
        for (int e = threadIdx.x; e < k * nl; e += blockDim.x) {
            const Coef c = make_coef(g, dts_s[e / nl], A.vel, e % nl);
            if constexpr (sizeof(T) == 4) coef_s[e] = coef_f32(c);
            else coef_s[e] = c;
        }
        __syncthreads();
        const double   batch_dt = s_ctl[0];
        const uint64_t executed = static_cast<uint64_t>(s_ctl[1]);

        // ---- k fused update steps (ghosts on the fly)
        const int32_t*       lv = A.levels[tb];
        const amr_halo_meta* mt = A.meta[tb];
        for (int s = 0; s < k; ++s) {
            const T*    in  = static_cast<const T*>(A.state[cur]);
            T*          out = static_cast<T*>(A.state[cur ^ 1]);
            const CT*   row = coef_s + static_cast<size_t>(s) * nl;
            for (long long t = gtid; t < static_cast<long long>(P) * g.cells; t += nthreads) {
                const int p = static_cast<int>(t / g.cells);
                step_cell<T, true>(in, out, mt, g, row[lv[p]], A.up, p, static_cast<int>(t - static_cast<long long>(p) * g.cells));
            }
            cluster_barrier();
            cur ^= 1;
        }
        done += static_cast<long long>(executed);
        sum_dt += batch_dt;
        executed_total += executed;
        cell_updates += executed * static_cast<uint64_t>(P) * static_cast<uint64_t>(g.cells);
        leaves_sum += static_cast<uint64_t>(P);
        lmin = min(lmin, P);
        lmax = max(lmax, P);
        ++intervals;
        if (A.crit == 0) {
            if (executed == 0) break;
            continue;
        }

        // ---- refinement flags (one warp per patch)
        const T* st = static_cast<const T*>(A.state[cur]);
        for (int p = gwarp; p < P; p += nwarps) {
            int8_t f;
            if (A.crit == 1) {
                int any = 0, all = 1;
                if (g.rank == 2)
                    for (int c = lane; c < g.cells; c += 32)
                        gradient_rule_cell<T, true, 2>(st, mt, g, A.rule, p, c, any, all);
                else
                    for (int c = lane; c < g.cells; c += 32)
                        gradient_rule_cell<T, true, 3>(st, mt, g, A.rule, p, c, any, all);
                any = __any_sync(0xffffffffu, any);
                all = __all_sync(0xffffffffu, all);
                f   = gradient_decision(any, all, lv[p], A.min_level, A.max_level);
            } else {
                const double mx = patch_max_on_the_fly<T>(st, mt, g, p, lane);
                f               = max_decision(mx, lv[p], A.rthr, A.cthr, A.min_level, A.max_level);
            }
            if (lane == 0) A.flags[p] = f;
        }
        if (leader) {
            A.status[0] = A.status[1] = A.status[2] = 0;
            *A.maxlev = 0;
        }
        cluster_barrier();

        // ---- re-mesh (C2-C9): the O(P) decisions run in block 0 with block
        // barriers; the per-cell remap and the neighbour search use the cluster
        const uint64_t* keys = A.keys[tb];
        if (blockIdx.x == 0) {
            for (int i = threadIdx.x; i < P; i += blockDim.x) mark_leaf(keys, A.flags, P, g, A.rmark, A.chead, i);
            __syncthreads();
            for (int rr = 0; rr < (maxlevel > 1 ? maxlevel : 1); ++rr) {
                for (int i = threadIdx.x; i < P; i += blockDim.x) closure_leaf(mt, g, A.rmark, i);
                __syncthreads();
            }
            for (int i = threadIdx.x; i < P; i += blockDim.x) veto_leaf(mt, g, A.rmark, A.chead, i);
            __syncthreads();
            for (int i = threadIdx.x; i < P; i += blockDim.x) count_leaf(keys, A.rmark, A.chead, g, A.cnt, A.status + 1, i);
            __syncthreads();
            block_scan(A.cnt, A.pos, P, A.cap, A.status, part);
            if (A.status[1] && !A.status[0])
                for (int i = threadIdx.x; i < P; i += blockDim.x)
                    emit_leaf(keys, A.rmark, A.chead, A.pos, g, A.keys[tb ^ 1], A.levels[tb ^ 1], A.src, A.skind,
                              A.maxlev, i);
        }
        cluster_barrier();
        const int err = A.status[0], changed = A.status[1], NP = A.status[2];
        ++remeshes;
        if (err) {
            error = err;
            break;
        }
        if (changed) {
            ++remeshes_changed;
            const T* old_state = static_cast<const T*>(A.state[cur]);
            T*       new_state = static_cast<T*>(A.state[cur ^ 1]);
            for (long long t = gtid; t < static_cast<long long>(NP) * g.cells; t += nthreads) {
                const int j = static_cast<int>(t / g.cells);
                remap_cell<T>(old_state, new_state, g, A.skind[j], A.src[j], j,
                              static_cast<int>(t - static_cast<long long>(j) * g.cells));
            }
            for (int t = gtid; t < NP * g.ndir; t += nthreads)
                neighbor_entry(A.keys[tb ^ 1], NP, g, A.meta[tb ^ 1], A.status, t);
            cluster_barrier();
            P        = NP;
            tb ^= 1;
            cur ^= 1;
            maxlevel = *A.maxlev;
            if (A.status[0]) {
                error = A.status[0];
                break;
            }
        }
        if (executed == 0) break;
        if (P > A.leaf_limit) {
            stopped = 1;
            break;
        }
    }
    if (leader) {
        CycleStats s;
        s.executed     = executed_total;
        s.sum_dt       = sum_dt;
        s.cell_updates = cell_updates;
        s.remeshes     = remeshes;
        s.leaves_sum   = leaves_sum;
        s.intervals    = intervals;
        s.leaves_min   = lmin;
        s.leaves_max   = lmax;
        s.P            = P;
        s.tb           = tb;
        s.cur          = cur;
        s.max_level    = maxlevel;
        s.error        = error;
        s.stopped      = stopped;
        s.remeshes_changed = remeshes_changed;
        *A.stats       = s;
    }
}

} // namespace amr_gb300
