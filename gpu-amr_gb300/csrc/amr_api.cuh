// Internal header of the C-ABI translation units (amr_tree.cu, amr_physics_api.cu,
// amr_adjoint_api.cu, amr_dropins.cu, amr_noalloc.cu): the error helpers,
// the geometry check and the device-resident tree object.  Not installed;
// callers of the library see include/amr_gb300.h only.
#pragma once

#include <algorithm>
#include <atomic>
#include <climits>
#include <cmath>
#include <map>
#include <limits>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "amr_gb300.h"
#include "amr_adjoint.cuh"
#include "amr_cycle.cuh"
#include "amr_euler.cuh"
#include "amr_ssprk.cuh"
#include "amr_dg.cuh"
#include "amr_graph.cuh"
#include "amr_vtk.cuh"

using namespace amr_gb300;

namespace amr_api {

// the last error message of this host thread, and the count of kernel
// launches (defined in amr_tree.cu)
extern thread_local std::string g_last_error;
extern std::atomic<uint64_t>    g_launches;

inline amr_status fail(amr_status s, const std::string& what)
{
    g_last_error = what;
    return s;
}

inline amr_status cuda_fail(cudaError_t e, const char* where)
{
    return fail(AMR_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define AMR_CUDA(call)                                          \
    do {                                                        \
        cudaError_t e_ = (call);                                \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call);     \
    } while (0)

#define AMR_LAUNCHED(where)                                     \
    do {                                                        \
        g_launches.fetch_add(1, std::memory_order_relaxed);     \
        cudaError_t e_ = cudaGetLastError();                    \
        if (e_ != cudaSuccess) return cuda_fail(e_, where);     \
    } while (0)

inline bool make_geo(const amr_patch_geometry* pg, Geo& g)
{
    if (!pg) return false;
    const int rank = pg->rank, n = pg->n, h = pg->halo, depth = pg->depth;
    if (rank != 2 && rank != 3) return false;
    if (h < 1 || n < 2 * h || n % 2 != 0) return false;
    if (depth < 0 || rank * depth + 6 > 64 || depth > 30) return false;
    g.rank  = rank;
    g.n     = n;
    g.h     = h;
    g.P1    = n + 2 * h;
    g.depth = depth;
    g.nd    = 1 << rank;
    g.nf    = 1 << (rank - 1);
    g.ndir  = 2 * rank;
    g.flat  = 1;
    g.cells = 1;
    for (int k = 0; k < rank; ++k) {
        g.flat *= g.P1;
        g.cells *= n;
    }
    g.s[0] = g.s[1] = g.s[2] = 0;
    int st = 1;
    for (int L = rank - 1; L >= 0; --L) {
        g.s[L] = st;
        st *= g.P1;
    }
    g.inst_shift  = 64;
    g.morton_mask = (rank * depth >= 64) ? ~0ull : ((1ull << (rank * depth)) - 1ull);
    for (int a = 0; a < 3; ++a) {
        const double len = (a < rank) ? pg->lengths[a] : 1.0;
        if (!(len > 0.0)) return false;
        // physics_system::cell_sizes at level 0: L*2^D/2^D/n == L/n exactly
        g.dx_root[a] = len / static_cast<double>(n);
    }
    return true;
}

inline unsigned grid_for(long long work, int block)
{
    long long b = (work + block - 1) / block;
    if (b < 1) b = 1;
    return static_cast<unsigned>(b);
}

} // namespace amr_api

namespace amr_api {
// One captured interval: the launch sequence of amr_tree_run's graph path for
// a fixed set of parameters.
struct GraphKey {
    int    k = 0, crit = 0, min_level = 0, max_level = 0, rounds = 0, bounds = 0, vel = 0, W = 0, S = 0, grid = 0;
    int    pair = 0; // several steps per pass (same-level trees)
    int    fused = 0; // the whole interval (steps and gradient flags) in one kernel
    int    up[3] = { 0, 0, 0 };
    double rthr = 0.0, cthr = 0.0, cfl = 0.0;
    bool   operator==(const GraphKey& o) const
    {
        return k == o.k && crit == o.crit && min_level == o.min_level && max_level == o.max_level &&
               rounds == o.rounds && bounds == o.bounds && vel == o.vel && W == o.W && S == o.S && grid == o.grid &&
               pair == o.pair && fused == o.fused &&
               up[0] == o.up[0] && up[1] == o.up[1] && up[2] == o.up[2] && std::memcmp(&rthr, &o.rthr, 8) == 0 &&
               std::memcmp(&cthr, &o.cthr, 8) == 0 && std::memcmp(&cfl, &o.cfl, 8) == 0;
    }
};
struct GraphEntry {
    GraphKey        key;
    cudaGraph_t     graph   = nullptr;
    cudaGraphExec_t exec    = nullptr;
    uint64_t        kernels = 0; // kernel nodes of one replay
};
// Launch configuration of the 2D update kernel: W warps per block, S tiles
// per warp, `grid` blocks (0 = one warp per patch up to full residency).
struct StepCfg {
    int W = 8, S = 2, grid = 0;
};
} // namespace amr_api
using namespace amr_api;

struct amr_tree {
    Geo          g{};
    double       lengths[3] = { 1.0, 1.0, 1.0 }; // domain lengths per Morton axis
    int          ninst    = 1;
    size_t       cap      = 0;
    int          dtype    = AMR_F64;
    size_t       esize    = 8;
    int          nvar     = 1; // state fields; field f of a buffer starts at f * fstride() elements
    cudaStream_t stream   = nullptr;
    size_t       size     = 0;
    int          max_level_host = 0;
    bool         ghosts_valid   = false;
    bool         uniform        = true; // every neighbour relation is "same level" (multi-step passes apply)
    bool         fused_off      = false; // a fused interval found leaves that are not 4x4 blocks: not again this run
    long long    pair_chunk     = 1;     // intervals of the next same-level graph chunk whose re-mesh may change the tree

    void*          sbuf[2]{};   // the two state buffers (fixed addresses)
    void*          cur = nullptr; // one of sbuf
    void*          nxt = nullptr;
    uint64_t*      keys[2]{};
    int32_t*       levels[2]{};
    amr_halo_meta* meta[2]{};
    int4*          prec = nullptr; // pass records, one per leaf (multi-step passes)
    int4*          frec = nullptr; // face records, one per leaf (flags of same-level graph intervals)
    bool           dg_state = false; // the re-mesh in progress carries a DG state (polynomial remap)
    int            dg_equation = AMR_DG_ADVECTION;
    double*        dg_prims    = nullptr; // DG Euler: p, u, v per node, eigenvalues x, y per padded cell (14 fields)
    size_t         dg_prims_cap = 0;       // leaves dg_prims holds
    double*        dg_scalars  = nullptr; // DG Euler: [0] step size, [1] time
    unsigned long long* dg_dtmin = nullptr; // DG Euler: smallest CFL step of the last stage (bit pattern)
    int            tb = 0;

    int8_t*   flags  = nullptr;
    uint8_t*  rmark  = nullptr;
    uint8_t*  chead  = nullptr;
    uint32_t* cnt    = nullptr;
    uint32_t* pos    = nullptr;
    int32_t*  src    = nullptr;
    int8_t*   skind  = nullptr;
    int32_t*  status = nullptr; // [0] error, [1] changed, [2] new size
    int32_t*  maxlev = nullptr; // per instance
    int32_t*  maxlev_new = nullptr; // per instance, zero between graph re-meshes
    double*   vel    = nullptr; // per instance, 3 each: the velocities in use
    double*   vel_inst = nullptr; // per instance, as set by amr_tree_set_instance_params
    int32_t*  bounds = nullptr; // per instance (min, max) level bounds
    int32_t*  target = nullptr; // per instance target levels (refine_to_levels)
    unsigned long long* offs = nullptr; // instance offsets, ninst + 1
    uint32_t* tile_sums = nullptr;
    RunCtl*   ctl       = nullptr;
    bool      vel_inst_set = false;
    std::vector<double> vel_inst_host;
    std::vector<int32_t> bounds_host; // per instance (min, max), as set (no device readback on a run)
    uint64_t  topo = 0; // changes whenever the leaves may have changed
    StepCfg   last_cfg{}; // launch shape of the last 2D update
    bool      bounds_set   = false;
    bool      vel_per_leaf = false; // the current advance uses per-instance velocities
    cudaStream_t          cap_stream = nullptr; // private stream for graph capture
    std::vector<GraphEntry> graphs;
    size_t    pinned_bytes = 0;

    double*   dt_acc = nullptr;
    double*   dt_rem = nullptr;
    uint32_t* dt_cnt = nullptr;
    double*   dt_tot = nullptr;
    uint32_t* dt_ctot = nullptr;
    DtState   dts() const { return DtState{ dt_acc, dt_rem, dt_cnt, dt_tot, dt_ctot }; }
    double*   dt_scratch = nullptr; // time bookkeeping of the autotuner's prologue (5 x instances)
    DtState   scratch_dts() const
    {
        const int K = ninst;
        return DtState{ dt_scratch, dt_scratch + K, reinterpret_cast<uint32_t*>(dt_scratch + 2 * K), dt_scratch + 3 * K,
                        reinterpret_cast<uint32_t*>(dt_scratch + 4 * K) };
    }
    double*   step_dt = nullptr;
    Coef*     coef    = nullptr;
    float2*   coef32  = nullptr; // (c_x, c_y) rows of the FP32 2D update
    int32_t*  upcode  = nullptr; // per instance packed upwind offsets
    size_t    coef_steps = 0;
    bool      batch_open = false;

    void* pinned = nullptr; // readback space (pinned_bytes)
    CycleStats* cstats = nullptr;

    // opt-in launch timing of the update kernel
    bool                                          timing = false;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> events;
    std::vector<uint64_t>                         event_cells;
    size_t                                        events_used = 0;

    // Euler solver scratch: per-step minima of dx / (|u| + a) as ordered
    // bit patterns (two slots, alternating) and the step size in use
    unsigned long long* euler_min = nullptr;
    double*             euler_dt  = nullptr;
    int32_t*            euler_ctl = nullptr;
    double*             prim[2]{}; // one-side flux terms beside sbuf[0] / sbuf[1]
    size_t              prim_cap = 0;
    void*               stage_buf = nullptr; // SSPRK intermediate stage (capacity patches)
    size_t              stage_cap = 0;

    size_t fstride() const { return cap * static_cast<size_t>(g.flat); }
    size_t field_bytes(size_t patches) const { return patches * static_cast<size_t>(g.flat) * esize; }
};

namespace amr_api {

// Streaming multiprocessors of the current device (cached per device).
inline int num_sms()
{
    static int sms[64] = {};
    int        dev     = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return 152;
    if (!sms[dev]) {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) v = 152;
        sms[dev] = v;
    }
    return sms[dev];
}

template <typename F>
amr_status dispatch_dtype(int dtype, F&& f)
{
    if (dtype == AMR_F64) return f(double{});
    if (dtype == AMR_F32) return f(float{});
    return fail(AMR_ERR_INVALID, "unknown dtype");
}

// Totals of a solver loop (amr_tree_run, amr_tree_euler_run).
struct RunTotals {
    long long done     = 0;
    double    sum_dt   = 0.0;
    uint64_t  executed = 0, cells = 0, remeshes = 0, intervals = 0, leaves_sum = 0, persistent = 0, graphs = 0;
    uint64_t  remeshes_changed = 0; // re-meshes that changed the tree
    uint64_t  lmin = ~0ull, lmax = 0;
};

// Defined in amr_tree.cu, used by the physics entry points.
amr_status halo_buffer(amr_tree* t, void* buf, const double* step_dt = nullptr);
// Device-to-device copy of `words` 8-byte words by an SM kernel on stream s.
amr_status copy_words8(void* dst, const void* src, size_t words, cudaStream_t s);
amr_status launch_halo(amr_tree* t);
// Defined in amr_tree.cu: `steps` forward-Euler steps with the batch mode
// first_mode (BATCH_RESET or BATCH_CONTINUE), used by the adjoint's forward.
amr_status advance_impl(amr_tree* t, size_t steps, const double* velocity3, double cfl, double remaining,
                        int first_mode);

} // namespace amr_api
