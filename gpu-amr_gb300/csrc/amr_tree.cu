// C-ABI of the GB300 AMR path: the device-resident tree and the reference
// drop-in launchers.  Host code only orchestrates launches; every per-leaf
// or per-cell loop runs in a kernel from amr_kernels.cuh.
#include <atomic>
#include <cmath>
#include <limits>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "amr_gb300.h"
#include "amr_cycle.cuh"

using namespace amr_gb300;

namespace {

thread_local std::string g_last_error;
std::atomic<uint64_t>    g_launches{ 0 };

amr_status fail(amr_status s, const std::string& what)
{
    g_last_error = what;
    return s;
}

amr_status cuda_fail(cudaError_t e, const char* where)
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

bool make_geo(const amr_patch_geometry* pg, Geo& g)
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

} // namespace

struct amr_tree {
    Geo          g{};
    size_t       cap      = 0;
    int          dtype    = AMR_F64;
    size_t       esize    = 8;
    cudaStream_t stream   = nullptr;
    size_t       size     = 0;
    int          max_level_host = 0;
    bool         ghosts_valid   = false;

    void*          cur = nullptr;
    void*          nxt = nullptr;
    uint64_t*      keys[2]{};
    int32_t*       levels[2]{};
    amr_halo_meta* meta[2]{};
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
    double*   vel    = nullptr; // per instance, 3 each

    double*   dt_acc = nullptr;
    double*   dt_rem = nullptr;
    uint32_t* dt_cnt = nullptr;
    double*   step_dt = nullptr;
    Coef*     coef    = nullptr;
    size_t    coef_steps = 0;
    bool      batch_open = false;

    void* pinned = nullptr; // 64 bytes of readback space
    CycleStats* cstats = nullptr;

    // opt-in launch timing of the update kernel
    bool                                          timing = false;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> events;
    std::vector<uint64_t>                         event_cells;
    size_t                                        events_used = 0;
};

namespace {

constexpr size_t kMaxBatch = 1024;


template <typename T, int N, int H>
amr_status launch_step2d(const T* in, T* out, const int32_t* levels, const amr_halo_meta* meta, int P, const Geo& g,
                         const Coef* coef, const int* up, int32_t* err, cudaStream_t s)
{
    // one warp per patch, 8 warps per block, at most 16 resident blocks per SM
    const unsigned grid = static_cast<unsigned>(std::min<long long>(grid_for(P, 8), 152LL * 16));
    k_step2d<T, N, H><<<grid, 256, 0, s>>>(in, out, levels, meta, P, g, coef, up[0], up[1], err);
    AMR_LAUNCHED("k_step2d");
    return AMR_OK;
}

template <typename F>
amr_status dispatch_dtype(int dtype, F&& f)
{
    if (dtype == AMR_F64) return f(double{});
    if (dtype == AMR_F32) return f(float{});
    return fail(AMR_ERR_INVALID, "unknown dtype");
}

void free_tree(amr_tree* t)
{
    if (!t) return;
    for (auto& e : t->events) {
        cudaEventDestroy(e.first);
        cudaEventDestroy(e.second);
    }
    cudaFree(t->cur);
    cudaFree(t->nxt);
    for (int b = 0; b < 2; ++b) {
        cudaFree(t->keys[b]);
        cudaFree(t->levels[b]);
        cudaFree(t->meta[b]);
    }
    cudaFree(t->flags);
    cudaFree(t->rmark);
    cudaFree(t->chead);
    cudaFree(t->cnt);
    cudaFree(t->pos);
    cudaFree(t->src);
    cudaFree(t->skind);
    cudaFree(t->status);
    cudaFree(t->maxlev);
    cudaFree(t->vel);
    cudaFree(t->dt_acc);
    cudaFree(t->dt_rem);
    cudaFree(t->dt_cnt);
    cudaFree(t->step_dt);
    cudaFree(t->coef);
    cudaFree(t->cstats);
    if (t->pinned) cudaFreeHost(t->pinned);
    delete t;
}

amr_status launch_halo(amr_tree* t)
{
    const long long total = static_cast<long long>(t->size) * t->g.ndir * t->g.h * (t->g.cells / t->g.n);
    const unsigned  grid  = static_cast<unsigned>(std::min<long long>(grid_for(total, 256), 152LL * 64));
    return dispatch_dtype(t->dtype, [&](auto z) -> amr_status {
        using T = decltype(z);
        k_halo<T><<<grid, 256, 0, t->stream>>>(static_cast<T*>(t->cur), t->meta[t->tb], total, t->g);
        AMR_LAUNCHED("k_halo");
        t->ghosts_valid = true;
        return AMR_OK;
    });
}


// One root leaf: key 0, level 0, periodic self-neighbours (ndtree.hpp:411-421),
// zero state in both buffers.
amr_status init_root(amr_tree* t)
{
    const Geo&                 g = t->g;
    std::vector<amr_halo_meta> root(g.ndir);
    for (auto& m : root) {
        m.neighbor = 0;
        for (int q = 0; q < 4; ++q) m.finer_ids[q] = -1;
        for (int q = 0; q < 3; ++q) m.quadrant[q] = 0;
        m.relation   = REL_SAME;
        m.padding[0] = m.padding[1] = m.padding[2] = 0;
    }
    const uint64_t zero_key = 0;
    const int32_t  zero_lev = 0;
    const size_t   state_bytes = t->cap * g.flat * t->esize;
    t->tb = 0;
    AMR_CUDA(cudaMemsetAsync(t->cur, 0, state_bytes, t->stream));
    AMR_CUDA(cudaMemsetAsync(t->nxt, 0, state_bytes, t->stream));
    AMR_CUDA(cudaMemsetAsync(t->status, 0, 8 * sizeof(int32_t), t->stream));
    AMR_CUDA(cudaMemcpyAsync(t->keys[0], &zero_key, 8, cudaMemcpyHostToDevice, t->stream));
    AMR_CUDA(cudaMemcpyAsync(t->levels[0], &zero_lev, 4, cudaMemcpyHostToDevice, t->stream));
    AMR_CUDA(cudaMemcpyAsync(t->maxlev, &zero_lev, 4, cudaMemcpyHostToDevice, t->stream));
    AMR_CUDA(cudaMemcpyAsync(t->meta[0], root.data(), g.ndir * sizeof(amr_halo_meta), cudaMemcpyHostToDevice,
                             t->stream));
    AMR_CUDA(cudaStreamSynchronize(t->stream));
    t->size           = 1;
    t->max_level_host = 0;
    t->ghosts_valid   = true;
    t->batch_open     = false;
    return AMR_OK;
}



// Smallest non-negative double s whose correctly rounded square root passes
// `v > thr` (strict) or `v >= thr`; NaN when no s does.  Non-negative doubles
// are ordered like their bit patterns, so a bisection over the bits is exact.
double sq_threshold(double thr, bool strict)
{
    auto ok = [&](double s) {
        const double v = std::sqrt(s);
        return strict ? v > thr : v >= thr;
    };
    if (ok(0.0)) return 0.0;
    if (!ok(std::numeric_limits<double>::infinity())) return std::numeric_limits<double>::quiet_NaN();
    uint64_t lo = 0, hi = 0x7FF0000000000000ull; // ok(lo) false, ok(hi) true
    while (hi - lo > 1) {
        const uint64_t mid = lo + (hi - lo) / 2;
        double         v;
        std::memcpy(&v, &mid, sizeof v);
        if (ok(v)) hi = mid;
        else lo = mid;
    }
    double r;
    std::memcpy(&r, &hi, sizeof r);
    return r;
}

// ------------------------------------------------------------ persistent run
constexpr int kPersistentLeaves = 1024; // above this, per-launch kernels keep all SMs busy
constexpr int kMaxInterval      = 256;

template <typename T>
int cycle_cluster_size(size_t smem)
{
    static int cached[2] = { -1, -1 };
    const int  slot      = sizeof(T) == 8 ? 0 : 1;
    if (cached[slot] >= 0) return cached[slot];
    int best = 0;
    if (cudaFuncSetAttribute(k_cycle<T>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess &&
        cudaFuncSetAttribute(k_cycle<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024) == cudaSuccess) {
        for (int c : { 16, 8, 4 }) {
            cudaLaunchConfig_t  cfg{};
            cudaLaunchAttribute at[1];
            at[0].id               = cudaLaunchAttributeClusterDimension;
            at[0].val.clusterDim.x = c;
            at[0].val.clusterDim.y = 1;
            at[0].val.clusterDim.z = 1;
            cfg.gridDim            = dim3(c, 1, 1);
            cfg.blockDim           = dim3(kCycleThreads, 1, 1);
            cfg.dynamicSmemBytes   = smem;
            cfg.attrs              = at;
            cfg.numAttrs           = 1;
            int clusters           = 0;
            if (cudaOccupancyMaxActiveClusters(&clusters, k_cycle<T>, &cfg) == cudaSuccess && clusters >= 1) {
                best = c;
                break;
            }
        }
    }
    cudaGetLastError(); // a refused query leaves no sticky error
    cached[slot] = best;
    return best;
}

template <typename T>
amr_status launch_cycle(amr_tree* t, CycleArgs& A, int cluster)
{
    const size_t smem = static_cast<size_t>(A.interval) * (A.g.depth + 1) * sizeof(Coef) +
                        static_cast<size_t>(A.interval) * sizeof(double);
    cudaLaunchConfig_t  cfg{};
    cudaLaunchAttribute at[1];
    at[0].id               = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = cluster;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim            = dim3(cluster, 1, 1);
    cfg.blockDim           = dim3(kCycleThreads, 1, 1);
    cfg.dynamicSmemBytes   = smem;
    cfg.stream             = t->stream;
    cfg.attrs              = at;
    cfg.numAttrs           = 1;
    AMR_CUDA(cudaLaunchKernelEx(&cfg, k_cycle<T>, A));
    AMR_LAUNCHED("k_cycle");
    return AMR_OK;
}

} // namespace

extern "C" {

const char* amr_last_error(void) { return g_last_error.c_str(); }
int         amr_version(void) { return 1; }
uint64_t    amr_launch_count(void) { return g_launches.load(); }

amr_status amr_tree_create(const amr_tree_desc* desc, amr_tree** out)
{
    if (!desc || !out) return fail(AMR_ERR_INVALID, "null argument");
    *out = nullptr;
    Geo g;
    if (!make_geo(&desc->geom, g)) return fail(AMR_ERR_INVALID, "bad patch geometry");
    if (desc->capacity < 1 || desc->capacity > (1ull << 30)) return fail(AMR_ERR_INVALID, "bad capacity");
    if (desc->dtype != AMR_F64 && desc->dtype != AMR_F32) return fail(AMR_ERR_INVALID, "bad dtype");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(AMR_ERR_NO_DEVICE, "no CUDA device");
    amr_tree* t = new amr_tree();
    t->g      = g;
    t->cap    = desc->capacity;
    t->dtype  = desc->dtype;
    t->esize  = desc->dtype == AMR_F64 ? 8 : 4;
    t->stream = static_cast<cudaStream_t>(desc->stream);
    const size_t cap = t->cap, state_bytes = cap * g.flat * t->esize;
    cudaError_t  e   = cudaSuccess;
    auto         al  = [&](void** p, size_t bytes) {
        if (e == cudaSuccess) e = cudaMalloc(p, bytes);
    };
    al(&t->cur, state_bytes);
    al(&t->nxt, state_bytes);
    for (int b = 0; b < 2; ++b) {
        al(reinterpret_cast<void**>(&t->keys[b]), cap * sizeof(uint64_t));
        al(reinterpret_cast<void**>(&t->levels[b]), cap * sizeof(int32_t));
        al(reinterpret_cast<void**>(&t->meta[b]), cap * g.ndir * sizeof(amr_halo_meta));
    }
    al(reinterpret_cast<void**>(&t->flags), cap);
    al(reinterpret_cast<void**>(&t->rmark), cap);
    al(reinterpret_cast<void**>(&t->chead), cap);
    al(reinterpret_cast<void**>(&t->cnt), (cap + 1) * sizeof(uint32_t));
    al(reinterpret_cast<void**>(&t->pos), (cap + 1) * sizeof(uint32_t));
    al(reinterpret_cast<void**>(&t->src), cap * sizeof(int32_t));
    al(reinterpret_cast<void**>(&t->skind), cap);
    al(reinterpret_cast<void**>(&t->status), 8 * sizeof(int32_t));
    al(reinterpret_cast<void**>(&t->maxlev), sizeof(int32_t));
    al(reinterpret_cast<void**>(&t->vel), 3 * sizeof(double));
    al(reinterpret_cast<void**>(&t->dt_acc), sizeof(double));
    al(reinterpret_cast<void**>(&t->dt_rem), sizeof(double));
    al(reinterpret_cast<void**>(&t->dt_cnt), sizeof(uint32_t));
    al(reinterpret_cast<void**>(&t->step_dt), kMaxBatch * sizeof(double));
    al(reinterpret_cast<void**>(&t->coef), kMaxBatch * (g.depth + 1) * sizeof(Coef));
    al(reinterpret_cast<void**>(&t->cstats), sizeof(CycleStats));
    if (e == cudaSuccess) e = cudaMallocHost(&t->pinned, 256);
    if (e != cudaSuccess) {
        free_tree(t);
        return cuda_fail(e, "amr_tree_create allocation");
    }
    t->coef_steps = kMaxBatch;
    amr_status rs = init_root(t);
    if (rs != AMR_OK) {
        free_tree(t);
        return rs;
    }
    *out = t;
    return AMR_OK;
}

amr_status amr_tree_destroy(amr_tree* t)
{
    if (!t) return AMR_OK;
    cudaStreamSynchronize(t->stream);
    free_tree(t);
    return AMR_OK;
}

amr_status amr_tree_size(const amr_tree* t, size_t* out)
{
    if (!t || !out) return fail(AMR_ERR_INVALID, "null argument");
    *out = t->size;
    return AMR_OK;
}

amr_status amr_tree_patch_cells(const amr_tree* t, size_t* out)
{
    if (!t || !out) return fail(AMR_ERR_INVALID, "null argument");
    *out = static_cast<size_t>(t->g.flat);
    return AMR_OK;
}

amr_status amr_tree_upload_state(amr_tree* t, const void* host, size_t num)
{
    if (!t || !host) return fail(AMR_ERR_INVALID, "null argument");
    if (num != t->size) return fail(AMR_ERR_INVALID, "patch count does not match tree size");
    AMR_CUDA(cudaMemcpyAsync(t->cur, host, num * t->g.flat * t->esize, cudaMemcpyHostToDevice, t->stream));
    AMR_CUDA(cudaStreamSynchronize(t->stream));
    t->ghosts_valid = true; // caller's ghosts, as in sync_current_to_device
    return AMR_OK;
}

amr_status amr_tree_download_state(amr_tree* t, void* host, size_t num)
{
    if (!t || !host) return fail(AMR_ERR_INVALID, "null argument");
    if (num != t->size) return fail(AMR_ERR_INVALID, "patch count does not match tree size");
    AMR_CUDA(cudaMemcpyAsync(host, t->cur, num * t->g.flat * t->esize, cudaMemcpyDeviceToHost, t->stream));
    AMR_CUDA(cudaStreamSynchronize(t->stream));
    return AMR_OK;
}

amr_status amr_tree_load_state_device(amr_tree* t, const void* device_state, size_t num)
{
    if (!t || !device_state) return fail(AMR_ERR_INVALID, "null argument");
    if (num != t->size) return fail(AMR_ERR_INVALID, "patch count does not match tree size");
    AMR_CUDA(cudaMemcpyAsync(t->cur, device_state, num * t->g.flat * t->esize, cudaMemcpyDeviceToDevice, t->stream));
    t->ghosts_valid = true;
    return AMR_OK;
}

amr_status amr_tree_reset(amr_tree* t)
{
    if (!t) return fail(AMR_ERR_INVALID, "null argument");
    return init_root(t);
}

amr_status amr_tree_device_state(amr_tree* t, void** current, void** next)
{
    if (!t) return fail(AMR_ERR_INVALID, "null argument");
    if (current) *current = t->cur;
    if (next) *next = t->nxt;
    return AMR_OK;
}

amr_status amr_tree_get_ids(const amr_tree* t, uint64_t* host, size_t num)
{
    if (!t || !host || num != t->size) return fail(AMR_ERR_INVALID, "bad argument");
    AMR_CUDA(cudaMemcpyAsync(host, t->keys[t->tb], num * 8, cudaMemcpyDeviceToHost, t->stream));
    AMR_CUDA(cudaStreamSynchronize(t->stream));
    return AMR_OK;
}

amr_status amr_tree_get_levels(const amr_tree* t, int32_t* host, size_t num)
{
    if (!t || !host || num != t->size) return fail(AMR_ERR_INVALID, "bad argument");
    AMR_CUDA(cudaMemcpyAsync(host, t->levels[t->tb], num * 4, cudaMemcpyDeviceToHost, t->stream));
    AMR_CUDA(cudaStreamSynchronize(t->stream));
    return AMR_OK;
}

amr_status amr_tree_get_neighbors(const amr_tree* t, amr_halo_meta* host, size_t num)
{
    if (!t || !host || num != t->size) return fail(AMR_ERR_INVALID, "bad argument");
    AMR_CUDA(cudaMemcpyAsync(host, t->meta[t->tb], num * t->g.ndir * sizeof(amr_halo_meta), cudaMemcpyDeviceToHost,
                             t->stream));
    AMR_CUDA(cudaStreamSynchronize(t->stream));
    return AMR_OK;
}

amr_status amr_tree_halo_exchange(amr_tree* t)
{
    if (!t) return fail(AMR_ERR_INVALID, "null argument");
    return launch_halo(t);
}

amr_status amr_tree_flags_gradient(amr_tree* t, double rthr, double cthr, int min_level, int max_level)
{
    if (!t) return fail(AMR_ERR_INVALID, "null argument");
    if (!t->ghosts_valid) {
        amr_status s = launch_halo(t);
        if (s != AMR_OK) return s;
    }
    const int P = static_cast<int>(t->size);
    return dispatch_dtype(t->dtype, [&](auto z) -> amr_status {
        using T = decltype(z);
        k_flags_gradient<T><<<P, 128, 0, t->stream>>>(static_cast<const T*>(t->cur), t->levels[t->tb], P, t->g, rthr,
                                                     cthr, min_level, max_level, t->flags);
        AMR_LAUNCHED("k_flags_gradient");
        return AMR_OK;
    });
}

amr_status amr_tree_flags_max(amr_tree* t, double rthr, double cthr, int min_level, int max_level)
{
    if (!t) return fail(AMR_ERR_INVALID, "null argument");
    if (!t->ghosts_valid) {
        amr_status s = launch_halo(t);
        if (s != AMR_OK) return s;
    }
    const int P = static_cast<int>(t->size);
    return dispatch_dtype(t->dtype, [&](auto z) -> amr_status {
        using T = decltype(z);
        k_flags_max<T><<<P, 128, 0, t->stream>>>(static_cast<const T*>(t->cur), t->levels[t->tb], P, t->g, rthr, cthr,
                                                min_level, max_level, t->flags);
        AMR_LAUNCHED("k_flags_max");
        return AMR_OK;
    });
}

amr_status amr_tree_set_flags(amr_tree* t, const int8_t* host, size_t num)
{
    if (!t || !host || num != t->size) return fail(AMR_ERR_INVALID, "bad argument");
    AMR_CUDA(cudaMemcpyAsync(t->flags, host, num, cudaMemcpyHostToDevice, t->stream));
    AMR_CUDA(cudaStreamSynchronize(t->stream));
    return AMR_OK;
}

amr_status amr_tree_get_flags(const amr_tree* t, int8_t* host, size_t num)
{
    if (!t || !host || num != t->size) return fail(AMR_ERR_INVALID, "bad argument");
    AMR_CUDA(cudaMemcpyAsync(host, t->flags, num, cudaMemcpyDeviceToHost, t->stream));
    AMR_CUDA(cudaStreamSynchronize(t->stream));
    return AMR_OK;
}

amr_status amr_tree_remesh(amr_tree* t, int* changed)
{
    if (!t) return fail(AMR_ERR_INVALID, "null argument");
    if (changed) *changed = 0;
    const Geo&   g  = t->g;
    const int    P  = static_cast<int>(t->size);
    cudaStream_t s  = t->stream;
    const int    tb = t->tb, nb = 1 - t->tb;
    AMR_CUDA(cudaMemsetAsync(t->status, 0, 3 * sizeof(int32_t), s)); // [7] is the update kernels' wait flag
    k_mark<<<grid_for(P, 256), 256, 0, s>>>(t->keys[tb], t->flags, P, g, t->rmark, t->chead);
    AMR_LAUNCHED("k_mark");
    const int rounds = std::max(1, t->max_level_host);
    for (int r = 0; r < rounds; ++r) {
        k_closure<<<grid_for(P, 256), 256, 0, s>>>(t->meta[tb], P, g, t->rmark);
        AMR_LAUNCHED("k_closure");
    }
    k_veto<<<grid_for(P, 256), 256, 0, s>>>(t->meta[tb], P, g, t->rmark, t->chead);
    AMR_LAUNCHED("k_veto");
    k_count<<<grid_for(P, 256), 256, 0, s>>>(t->keys[tb], t->rmark, t->chead, P, g, t->cnt, t->status + 1);
    AMR_LAUNCHED("k_count");
    k_scan<<<1, 1024, 0, s>>>(t->cnt, t->pos, P, t->cap, t->status);
    AMR_LAUNCHED("k_scan");
    int32_t* hs = static_cast<int32_t*>(t->pinned);
    AMR_CUDA(cudaMemcpyAsync(hs, t->status, 3 * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    AMR_CUDA(cudaStreamSynchronize(s));
    if (hs[0] != 0) return fail(static_cast<amr_status>(hs[0]), "re-mesh would exceed the tree capacity");
    if (!hs[1]) return AMR_OK; // reconstruction_is_noop (ndtree.hpp:1242-1246)
    const int NP = hs[2];
    AMR_CUDA(cudaMemsetAsync(t->maxlev, 0, sizeof(int32_t), s));
    k_emit<<<grid_for(P, 256), 256, 0, s>>>(t->keys[tb], t->rmark, t->chead, t->pos, P, g, t->keys[nb], t->levels[nb],
                                            t->src, t->skind, t->maxlev);
    AMR_LAUNCHED("k_emit");
    amr_status st = dispatch_dtype(t->dtype, [&](auto z) -> amr_status {
        using T = decltype(z);
        k_remap<T><<<NP, 256, 0, s>>>(static_cast<const T*>(t->cur), static_cast<T*>(t->nxt), t->src, t->skind, NP, g);
        AMR_LAUNCHED("k_remap");
        return AMR_OK;
    });
    if (st != AMR_OK) return st;
    k_neighbors<<<grid_for(static_cast<long long>(NP) * g.ndir, 128), 128, 0, s>>>(t->keys[nb], NP, g, t->meta[nb],
                                                                                  t->status);
    AMR_LAUNCHED("k_neighbors");
    AMR_CUDA(cudaMemcpyAsync(hs + 4, t->status, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    AMR_CUDA(cudaMemcpyAsync(hs + 5, t->maxlev, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    AMR_CUDA(cudaStreamSynchronize(s));
    std::swap(t->cur, t->nxt);
    t->tb             = nb;
    t->size           = static_cast<size_t>(NP);
    t->max_level_host = hs[5];
    t->ghosts_valid   = false;
    if (changed) *changed = 1;
    if (hs[4] != 0) return fail(static_cast<amr_status>(hs[4]), "neighbour rebuild found a non-2:1 face");
    return AMR_OK;
}

amr_status amr_tree_refine_uniform(amr_tree* t, int levels)
{
    if (!t || levels < 0) return fail(AMR_ERR_INVALID, "bad argument");
    for (int l = 0; l < levels; ++l) {
        AMR_CUDA(cudaMemsetAsync(t->flags, FLAG_REFINE, t->size, t->stream));
        int        changed = 0;
        amr_status s       = amr_tree_remesh(t, &changed);
        if (s != AMR_OK) return s;
    }
    return AMR_OK;
}

amr_status amr_tree_advance(amr_tree* t, size_t steps, const double* velocity3, double cfl, double remaining)
{
    if (!t || !velocity3) return fail(AMR_ERR_INVALID, "null argument");
    cudaStream_t s = t->stream;
    AMR_CUDA(cudaMemcpyAsync(t->vel, velocity3, 3 * sizeof(double), cudaMemcpyHostToDevice, s));
    int up[3] = { 0, 0, 0 };
    for (int a = 0; a < t->g.rank; ++a) up[a] = velocity3[a] > 0.0 ? -1 : (velocity3[a] < 0.0 ? 1 : 0);
    const int P     = static_cast<int>(t->size);
    const int ppb   = std::max(1, 256 / t->g.cells);
    const unsigned grid = grid_for(P, ppb);
    const int nl    = t->g.depth + 1;
    bool      first = true;
    size_t    done  = 0;
    while (done < steps || (first && steps == 0)) {
        const int chunk = static_cast<int>(std::min(kMaxBatch, steps - done));
        k_batch_begin<<<1, 256, 0, s>>>(t->maxlev, t->g, t->vel, cfl, chunk, first ? 1 : 0, remaining, t->dt_acc,
                                        t->dt_rem, t->dt_cnt, t->step_dt, t->coef);
        AMR_LAUNCHED("k_batch_begin");
        first = false;
        for (int k = 0; k < chunk; ++k) {
            std::pair<cudaEvent_t, cudaEvent_t>* ev = nullptr;
            if (t->timing) {
                if (t->events_used == t->events.size()) {
                    std::pair<cudaEvent_t, cudaEvent_t> e;
                    AMR_CUDA(cudaEventCreate(&e.first));
                    AMR_CUDA(cudaEventCreate(&e.second));
                    t->events.push_back(e);
                    t->event_cells.push_back(0);
                }
                ev = &t->events[t->events_used];
                t->event_cells[t->events_used] = static_cast<uint64_t>(P) * t->g.cells;
                ++t->events_used;
                AMR_CUDA(cudaEventRecord(ev->first, s));
            }
            amr_status st = dispatch_dtype(t->dtype, [&](auto z) -> amr_status {
                using T        = decltype(z);
                const Coef* cf = t->coef + static_cast<size_t>(k) * nl;
                const T*    in = static_cast<const T*>(t->cur);
                T*          out = static_cast<T*>(t->nxt);
                if (t->g.rank == 2 && t->g.n == 16 && t->g.h == 1)
                    return launch_step2d<T, 16, 1>(in, out, t->levels[t->tb], t->meta[t->tb], P, t->g, cf, up,
                                                   t->status + 7, s);
                if (t->g.rank == 2 && t->g.n == 8 && t->g.h == 1)
                    return launch_step2d<T, 8, 1>(in, out, t->levels[t->tb], t->meta[t->tb], P, t->g, cf, up,
                                                  t->status + 7, s);
                k_step<T, true><<<grid, 256, 0, s>>>(in, out, t->levels[t->tb], t->meta[t->tb], P, t->g, cf, up[0],
                                                     up[1], up[2], ppb);
                AMR_LAUNCHED("k_step");
                return AMR_OK;
            });
            if (st != AMR_OK) return st;
            if (ev) AMR_CUDA(cudaEventRecord(ev->second, s));
            std::swap(t->cur, t->nxt);
        }
        done += chunk;
        if (steps == 0) break;
    }
    t->ghosts_valid = false;
    t->batch_open   = true;
    return AMR_OK;
}

amr_status amr_tree_finish_advance(amr_tree* t, double* sum_dt, size_t* executed)
{
    if (!t) return fail(AMR_ERR_INVALID, "null argument");
    char* hp = static_cast<char*>(t->pinned);
    AMR_CUDA(cudaMemcpyAsync(hp + 32, t->dt_acc, sizeof(double), cudaMemcpyDeviceToHost, t->stream));
    AMR_CUDA(cudaMemcpyAsync(hp + 40, t->dt_cnt, sizeof(uint32_t), cudaMemcpyDeviceToHost, t->stream));
    AMR_CUDA(cudaMemcpyAsync(hp + 48, t->status + 7, sizeof(int32_t), cudaMemcpyDeviceToHost, t->stream));
    AMR_CUDA(cudaStreamSynchronize(t->stream));
    int32_t wait_err = 0;
    std::memcpy(&wait_err, hp + 48, sizeof wait_err);
    if (wait_err != 0) {
        AMR_CUDA(cudaMemsetAsync(t->status + 7, 0, sizeof(int32_t), t->stream));
        return fail(AMR_ERR_TIMEOUT, "a bulk copy did not complete within the wait limit");
    }
    double   acc;
    uint32_t cnt;
    std::memcpy(&acc, hp + 32, sizeof acc);
    std::memcpy(&cnt, hp + 40, sizeof cnt);
    if (!t->batch_open) {
        acc = 0.0;
        cnt = 0;
    }
    if (sum_dt) *sum_dt = acc;
    if (executed) *executed = cnt;
    return AMR_OK;
}

amr_status amr_tree_run(amr_tree* t, const amr_cycle_params* p, amr_cycle_stats* out)
{
    if (!t || !p) return fail(AMR_ERR_INVALID, "null argument");
    if (p->criterion < 0 || p->criterion > 2) return fail(AMR_ERR_INVALID, "unknown criterion");
    const Geo&  g = t->g;
    long long   done = 0;
    double      sum_dt = 0.0;
    uint64_t    executed = 0, cells = 0, remeshes = 0, intervals = 0, leaves_sum = 0, persistent = 0;
    uint64_t    lmin = ~0ull, lmax = 0;
    const long long total = static_cast<long long>(p->steps);
    int up[3] = { 0, 0, 0 };
    for (int a = 0; a < g.rank; ++a) up[a] = p->velocity[a] > 0.0 ? -1 : (p->velocity[a] < 0.0 ? 1 : 0);
    const size_t smem = static_cast<size_t>(p->remesh_interval) * (g.depth + 1) * sizeof(Coef) +
                        static_cast<size_t>(p->remesh_interval) * sizeof(double);
    while (done < total) {
        const bool small = !(p->options & AMR_RUN_PER_LAUNCH) && t->size <= static_cast<size_t>(kPersistentLeaves) &&
                           p->remesh_interval >= 1 &&
                           p->remesh_interval <= static_cast<uint64_t>(kMaxInterval) && smem <= 64 * 1024;
        int cluster = small ? (t->dtype == AMR_F64 ? cycle_cluster_size<double>(smem)
                                                   : cycle_cluster_size<float>(smem))
                            : 0;
        const int forced = (p->options >> 8) & 0xFF;
        if (cluster > 0 && forced > 0) cluster = std::min(cluster, forced);
        if (cluster > 0) {
            CycleArgs A{};
            A.g        = g;
            A.state[0] = t->cur;
            A.state[1] = t->nxt;
            for (int b = 0; b < 2; ++b) {
                A.keys[b]   = t->keys[b];
                A.levels[b] = t->levels[b];
                A.meta[b]   = t->meta[b];
            }
            A.flags  = t->flags;
            A.rmark  = t->rmark;
            A.chead  = t->chead;
            A.cnt    = t->cnt;
            A.pos    = t->pos;
            A.src    = t->src;
            A.skind  = t->skind;
            A.status = t->status;
            A.maxlev = t->maxlev;
            A.stats  = t->cstats;
            for (int a = 0; a < 3; ++a) {
                A.vel[a] = p->velocity[a];
                A.up[a]  = up[a];
            }
            A.cfl         = p->cfl;
            A.remaining   = p->remaining_time - sum_dt;
            A.steps_total = total - done;
            A.interval    = static_cast<int>(p->remesh_interval);
            A.crit        = p->criterion;
            A.rthr        = p->refine_threshold;
            A.cthr        = p->coarsen_threshold;
            A.rthr_sq     = sq_threshold(p->refine_threshold, true);
            A.cthr_sq     = sq_threshold(p->coarsen_threshold, false);
            A.min_level   = p->min_level;
            A.max_level   = p->max_level;
            A.P0          = static_cast<int>(t->size);
            A.tb0         = t->tb;
            A.max_level0  = t->max_level_host;
            A.cap         = t->cap;
            A.leaf_limit  = kPersistentLeaves;
            size_t ev_slot = SIZE_MAX;
            if (t->timing) {
                if (t->events_used == t->events.size()) {
                    std::pair<cudaEvent_t, cudaEvent_t> e;
                    AMR_CUDA(cudaEventCreate(&e.first));
                    AMR_CUDA(cudaEventCreate(&e.second));
                    t->events.push_back(e);
                    t->event_cells.push_back(0);
                }
                ev_slot = t->events_used++;
                AMR_CUDA(cudaEventRecord(t->events[ev_slot].first, t->stream));
            }
            amr_status st = t->dtype == AMR_F64 ? launch_cycle<double>(t, A, cluster) : launch_cycle<float>(t, A, cluster);
            if (st != AMR_OK) return st;
            if (ev_slot != SIZE_MAX) AMR_CUDA(cudaEventRecord(t->events[ev_slot].second, t->stream));
            CycleStats* hs = static_cast<CycleStats*>(t->pinned);
            AMR_CUDA(cudaMemcpyAsync(hs, t->cstats, sizeof(CycleStats), cudaMemcpyDeviceToHost, t->stream));
            AMR_CUDA(cudaStreamSynchronize(t->stream));
            const CycleStats cs = *hs;
            if (ev_slot != SIZE_MAX) t->event_cells[ev_slot] = cs.cell_updates;
            t->size             = static_cast<size_t>(cs.P);
            t->tb               = cs.tb;
            if (cs.cur) std::swap(t->cur, t->nxt);
            t->max_level_host = cs.max_level;
            t->ghosts_valid   = false;
            done += static_cast<long long>(cs.executed);
            sum_dt += cs.sum_dt;
            executed += cs.executed;
            cells += cs.cell_updates;
            remeshes += cs.remeshes;
            intervals += cs.intervals;
            persistent += cs.intervals;
            leaves_sum += cs.leaves_sum;
            if (cs.intervals) {
                lmin = std::min<uint64_t>(lmin, static_cast<uint64_t>(cs.leaves_min));
                lmax = std::max<uint64_t>(lmax, static_cast<uint64_t>(cs.leaves_max));
            }
            if (cs.error) return fail(static_cast<amr_status>(cs.error), "persistent re-mesh failed");
            if (!cs.stopped) break;
            continue;
        }
        // one interval with per-launch kernels
        const long long k = (p->remesh_interval > 0 && static_cast<long long>(p->remesh_interval) < total - done)
                                ? static_cast<long long>(p->remesh_interval)
                                : total - done;
        const size_t P = t->size;
        amr_status   st = amr_tree_advance(t, static_cast<size_t>(k), p->velocity, p->cfl, p->remaining_time - sum_dt);
        if (st != AMR_OK) return st;
        double acc = 0.0;
        size_t ex  = 0;
        st         = amr_tree_finish_advance(t, &acc, &ex);
        if (st != AMR_OK) return st;
        done += static_cast<long long>(ex);
        sum_dt += acc;
        executed += ex;
        cells += static_cast<uint64_t>(ex) * P * static_cast<uint64_t>(g.cells);
        leaves_sum += P;
        lmin = std::min<uint64_t>(lmin, P);
        lmax = std::max<uint64_t>(lmax, P);
        ++intervals;
        if (p->criterion != 0) {
            st = p->criterion == 1 ? amr_tree_flags_gradient(t, p->refine_threshold, p->coarsen_threshold,
                                                             p->min_level, p->max_level)
                                   : amr_tree_flags_max(t, p->refine_threshold, p->coarsen_threshold, p->min_level,
                                                        p->max_level);
            if (st != AMR_OK) return st;
            int changed = 0;
            st          = amr_tree_remesh(t, &changed);
            if (st != AMR_OK) return st;
            ++remeshes;
        }
        if (ex == 0) break;
    }
    if (out) {
        out->executed_steps       = executed;
        out->sum_dt               = sum_dt;
        out->cell_updates         = cells;
        out->remeshes             = remeshes;
        out->intervals            = intervals;
        out->leaves_min           = intervals ? lmin : t->size;
        out->leaves_max           = intervals ? lmax : t->size;
        out->leaves_mean          = intervals ? static_cast<double>(leaves_sum) / static_cast<double>(intervals) : 0.0;
        out->persistent_intervals = persistent;
    }
    return AMR_OK;
}

amr_status amr_tree_set_timing(amr_tree* t, int enabled)
{
    if (!t) return fail(AMR_ERR_INVALID, "null argument");
    t->timing = enabled != 0;
    return AMR_OK;
}

amr_status amr_tree_get_timing(amr_tree* t, double* ms, uint64_t* launches, uint64_t* cells)
{
    if (!t) return fail(AMR_ERR_INVALID, "null argument");
    AMR_CUDA(cudaStreamSynchronize(t->stream));
    double   total = 0.0;
    uint64_t c     = 0;
    for (size_t i = 0; i < t->events_used; ++i) {
        float e = 0.f;
        AMR_CUDA(cudaEventElapsedTime(&e, t->events[i].first, t->events[i].second));
        total += e;
        c += t->event_cells[i];
    }
    if (ms) *ms = total;
    if (launches) *launches = t->events_used;
    if (cells) *cells = c;
    t->events_used = 0;
    return AMR_OK;
}

amr_status amr_tree_synchronize(amr_tree* t)
{
    if (!t) return fail(AMR_ERR_INVALID, "null argument");
    AMR_CUDA(cudaStreamSynchronize(t->stream));
    return AMR_OK;
}

} // extern "C"

// ------------------------------------------------------------ drop-ins

namespace {

template <typename T>
amr_status halo_dropin(T* patches, const amr_halo_meta* meta, size_t meta_count, size_t num,
                              const amr_patch_geometry* geom, void* stream)
{
    Geo g;
    if (!patches || !meta || !make_geo(geom, g)) return fail(AMR_ERR_INVALID, "bad argument");
    // the reference validates metadata_count == P * 2 * rank (halo_exchange.cu:363-367)
    if (meta_count != num * static_cast<size_t>(g.ndir)) return fail(AMR_ERR_INVALID, "metadata count mismatch");
    if (num == 0) return AMR_OK;
    const long long total = static_cast<long long>(num) * g.ndir * g.h * (g.cells / g.n);
    const unsigned  grid  = static_cast<unsigned>(std::min<long long>(grid_for(total, 256), 152LL * 64));
    k_halo<T><<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(patches, meta, total, g);
    AMR_LAUNCHED("k_halo");
    return AMR_OK;
}

amr_status intergrid_dropin(double* p, const amr_transfer_task* tasks, size_t n,
                                   const amr_patch_geometry* geom, void* stream, int mode)
{
    Geo g;
    if (!p || (!tasks && n) || !make_geo(geom, g)) return fail(AMR_ERR_INVALID, "bad argument");
    if (n == 0) return AMR_OK;
    k_intergrid<double><<<static_cast<unsigned>(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        p, tasks, static_cast<int>(n), g, mode);
    AMR_LAUNCHED("k_intergrid");
    return AMR_OK;
}

} // namespace

extern "C" {

amr_status amr_halo_exchange_f64(double* p, const amr_halo_meta* m, size_t mc, size_t num,
                                 const amr_patch_geometry* geom, void* stream)
{
    return halo_dropin<double>(p, m, mc, num, geom, stream);
}

amr_status amr_halo_exchange_f32(float* p, const amr_halo_meta* m, size_t mc, size_t num,
                                 const amr_patch_geometry* geom, void* stream)
{
    return halo_dropin<float>(p, m, mc, num, geom, stream);
}

amr_status amr_interpolate_patches_f64(double* p, const amr_transfer_task* tasks, size_t n,
                                       const amr_patch_geometry* geom, void* stream)
{
    return intergrid_dropin(p, tasks, n, geom, stream, 0);
}

amr_status amr_restrict_patches_f64(double* p, const amr_transfer_task* tasks, size_t n,
                                    const amr_patch_geometry* geom, void* stream)
{
    return intergrid_dropin(p, tasks, n, geom, stream, 1);
}

amr_status amr_gather_patches(void* dst, const void* src, size_t patch_bytes, const int32_t* sources, size_t count,
                              void* stream)
{
    if (!dst || !src || (!sources && count) || patch_bytes == 0) return fail(AMR_ERR_INVALID, "bad argument");
    if (count == 0) return AMR_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const bool aligned = patch_bytes % 16 == 0 && reinterpret_cast<uintptr_t>(dst) % 16 == 0 &&
                         reinterpret_cast<uintptr_t>(src) % 16 == 0;
    if (aligned) {
        k_gather<<<static_cast<unsigned>(count), 256, 0, s>>>(static_cast<const uint4*>(src), static_cast<uint4*>(dst),
                                                             patch_bytes / 16, sources, static_cast<int>(count));
    } else {
        k_gather_bytes<<<static_cast<unsigned>(count), 256, 0, s>>>(static_cast<const unsigned char*>(src),
                                                                   static_cast<unsigned char*>(dst), patch_bytes,
                                                                   sources, static_cast<int>(count));
    }
    AMR_LAUNCHED("k_gather");
    return AMR_OK;
}

amr_status amr_compute_step_dt(const int32_t* levels, size_t num, const amr_patch_geometry* geom,
                               const double* v, double cfl, double* dt, double* acc, double* remaining,
                               uint32_t* count, void* stream)
{
    Geo g;
    if (!levels || !v || !dt || !acc || !remaining || !count || !make_geo(geom, g) || num == 0)
        return fail(AMR_ERR_INVALID, "bad argument");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // the maximum level lands in *dt first, then the finalize kernel reads it
    int32_t* lmax = reinterpret_cast<int32_t*>(dt);
    AMR_CUDA(cudaMemsetAsync(lmax, 0, sizeof(int32_t), s));
    k_max_level<<<std::min<unsigned>(grid_for(static_cast<long long>(num), 256), 1024), 256, 0, s>>>(
        levels, static_cast<int>(num), lmax);
    AMR_LAUNCHED("k_max_level");
    k_finalize_dt<<<1, 1, 0, s>>>(lmax, g, v[0], v[1], v[2], cfl, dt, acc, remaining, count);
    AMR_LAUNCHED("k_finalize_dt");
    return AMR_OK;
}

amr_status amr_time_step_f64(const double* in, double* out, const int32_t* levels, size_t num,
                             const amr_patch_geometry* geom, const double* v, const double* dt, void* stream)
{
    Geo g;
    if (!in || !out || !levels || !v || !dt || !make_geo(geom, g)) return fail(AMR_ERR_INVALID, "bad argument");
    if (num == 0) return AMR_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int          up[3] = { 0, 0, 0 };
    for (int a = 0; a < g.rank; ++a) up[a] = v[a] > 0.0 ? -1 : (v[a] < 0.0 ? 1 : 0);
    const int ppb = std::min(64, std::max(1, 256 / g.cells));
    k_step<double, false, true><<<grid_for(static_cast<long long>(num), ppb), 256, 0, s>>>(
        in, out, levels, nullptr, static_cast<int>(num), g, nullptr, up[0], up[1], up[2], ppb, dt, v[0], v[1], v[2]);
    AMR_LAUNCHED("k_step");
    return AMR_OK;
}

amr_status amr_flags_max_f64(const double* patches, const int32_t* levels, size_t num, const amr_patch_geometry* geom,
                             double rthr, double cthr, int min_level, int max_level, int8_t* flags, void* stream)
{
    Geo g;
    if (!patches || !levels || !flags || !make_geo(geom, g)) return fail(AMR_ERR_INVALID, "bad argument");
    if (num == 0) return AMR_OK;
    k_flags_max<double><<<static_cast<unsigned>(num), 128, 0, static_cast<cudaStream_t>(stream)>>>(
        patches, levels, static_cast<int>(num), g, rthr, cthr, min_level, max_level, flags);
    AMR_LAUNCHED("k_flags_max");
    return AMR_OK;
}

} // extern "C"

// ---------------------------------------------------- allocation-free re-mesh
// The tree's re-mesh keeps its working arrays in buffers the tree allocated.
// amr_remesh_noalloc runs the same kernels with those arrays carved out of one
// file-scope device array instead, for callers that may not allocate.
namespace {

constexpr size_t kNoAllocMax = AMR_NOALLOC_MAX_LEAVES;

constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// byte offsets of the working arrays inside the scratch array
constexpr size_t kOffRmark  = 0;
constexpr size_t kOffChead  = kOffRmark + align256(kNoAllocMax);
constexpr size_t kOffCnt    = kOffChead + align256(kNoAllocMax);
constexpr size_t kOffPos    = kOffCnt + align256((kNoAllocMax + 1) * sizeof(uint32_t));
constexpr size_t kOffSrc    = kOffPos + align256((kNoAllocMax + 1) * sizeof(uint32_t));
constexpr size_t kOffSkind  = kOffSrc + align256(kNoAllocMax * sizeof(int32_t));
constexpr size_t kOffStatus = kOffSkind + align256(kNoAllocMax);
constexpr size_t kOffMaxlev = kOffStatus + 256;
constexpr size_t kScratchUsed = kOffMaxlev + 256;
static_assert(kScratchUsed <= AMR_NOALLOC_SCRATCH_BYTES, "scratch layout exceeds the stated size");

} // namespace

// Every GPU that loads the library holds this array until the process exits.
static __device__ __align__(256) unsigned char g_remesh_scratch[AMR_NOALLOC_SCRATCH_BYTES];

namespace {

// In host code the name g_remesh_scratch is a host-side stand-in, not a
// device address; the address comes from cudaGetSymbolAddress, looked up once
// per device with that device current.
amr_status noalloc_scratch(unsigned char** out)
{
    static std::mutex     mu;
    static unsigned char* per_device[128] = {};
    int                   dev             = 0;
    AMR_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 128) return fail(AMR_ERR_INVALID, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(mu);
    if (!per_device[dev]) {
        void*       p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_remesh_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_remesh_scratch)");
        per_device[dev] = static_cast<unsigned char*>(p);
    }
    *out = per_device[dev];
    return AMR_OK;
}

} // namespace

extern "C" amr_status amr_remesh_noalloc(const amr_patch_geometry* geom, size_t num, const uint64_t* ids_in,
                                         const amr_halo_meta* meta_in, const int8_t* flags,
                                         const double* state_in, size_t out_cap, uint64_t* ids_out,
                                         int32_t* levels_out, amr_halo_meta* meta_out, double* state_out,
                                         uint32_t* device_out_count, size_t* host_out_count, void* stream)
{
    Geo g;
    if (!make_geo(geom, g)) return fail(AMR_ERR_INVALID, "bad patch geometry");
    if (!ids_in || !meta_in || !flags || !state_in || !ids_out || !levels_out || !meta_out || !state_out ||
        !device_out_count)
        return fail(AMR_ERR_INVALID, "null argument");
    if (num < 1 || num > kNoAllocMax)
        return fail(AMR_ERR_INVALID, "amr_remesh_noalloc: num_leaves must be in [1, AMR_NOALLOC_MAX_LEAVES]");
    if (out_cap < 1 || out_cap > kNoAllocMax)
        return fail(AMR_ERR_INVALID, "amr_remesh_noalloc: out_capacity must be in [1, AMR_NOALLOC_MAX_LEAVES]");
    unsigned char* base = nullptr;
    amr_status     st   = noalloc_scratch(&base);
    if (st != AMR_OK) return st;
    uint8_t*  rmark  = base + kOffRmark;
    uint8_t*  chead  = base + kOffChead;
    uint32_t* cnt    = reinterpret_cast<uint32_t*>(base + kOffCnt);
    uint32_t* pos    = reinterpret_cast<uint32_t*>(base + kOffPos);
    int32_t*  src    = reinterpret_cast<int32_t*>(base + kOffSrc);
    int8_t*   skind  = reinterpret_cast<int8_t*>(base + kOffSkind);
    int32_t*  status = reinterpret_cast<int32_t*>(base + kOffStatus);
    int32_t*  maxlev = reinterpret_cast<int32_t*>(base + kOffMaxlev);

    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int    P = static_cast<int>(num);
    // the array keeps the previous call's contents: clear what must start at zero
    AMR_CUDA(cudaMemsetAsync(status, 0, 8 * sizeof(int32_t), s));
    AMR_CUDA(cudaMemsetAsync(maxlev, 0, sizeof(int32_t), s));
    k_mark<<<grid_for(P, 256), 256, 0, s>>>(ids_in, flags, P, g, rmark, chead);
    AMR_LAUNCHED("k_mark");
    for (int r = 0; r < std::max(1, g.depth); ++r) {
        k_closure<<<grid_for(P, 256), 256, 0, s>>>(meta_in, P, g, rmark);
        AMR_LAUNCHED("k_closure");
    }
    k_veto<<<grid_for(P, 256), 256, 0, s>>>(meta_in, P, g, rmark, chead);
    AMR_LAUNCHED("k_veto");
    k_count<<<grid_for(P, 256), 256, 0, s>>>(ids_in, rmark, chead, P, g, cnt, status + 1);
    AMR_LAUNCHED("k_count");
    k_scan<<<1, 1024, 0, s>>>(cnt, pos, P, out_cap, status);
    AMR_LAUNCHED("k_scan");
    int32_t hs[3] = { 0, 0, 0 };
    AMR_CUDA(cudaMemcpyAsync(hs, status, sizeof hs, cudaMemcpyDeviceToHost, s));
    AMR_CUDA(cudaStreamSynchronize(s));
    if (hs[0] != 0) return fail(static_cast<amr_status>(hs[0]), "re-mesh would exceed out_capacity");
    const int NP = hs[2];
    k_emit<<<grid_for(P, 256), 256, 0, s>>>(ids_in, rmark, chead, pos, P, g, ids_out, levels_out, src, skind, maxlev);
    AMR_LAUNCHED("k_emit");
    k_remap<double><<<NP, 256, 0, s>>>(state_in, state_out, src, skind, NP, g);
    AMR_LAUNCHED("k_remap");
    k_neighbors<<<grid_for(static_cast<long long>(NP) * g.ndir, 128), 128, 0, s>>>(ids_out, NP, g, meta_out, status);
    AMR_LAUNCHED("k_neighbors");
    const uint32_t count = static_cast<uint32_t>(NP);
    AMR_CUDA(cudaMemcpyAsync(device_out_count, &count, sizeof count, cudaMemcpyHostToDevice, s));
    int32_t err = 0;
    AMR_CUDA(cudaMemcpyAsync(&err, status, sizeof err, cudaMemcpyDeviceToHost, s));
    AMR_CUDA(cudaStreamSynchronize(s));
    if (host_out_count) *host_out_count = static_cast<size_t>(NP);
    if (err != 0) return fail(static_cast<amr_status>(err), "neighbour rebuild found a non-2:1 face");
    return AMR_OK;
}

