// C-ABI of the GB300 AMR path: the device-resident tree and the reference
// drop-in launchers.  Host code only orchestrates launches; every per-leaf
// or per-cell loop runs in a kernel from amr_kernels.cuh.

#include "amr_api.cuh"
#include "amr_interval.cuh"

namespace amr_api {
thread_local std::string g_last_error;
std::atomic<uint64_t>    g_launches{ 0 };
} // namespace amr_api

namespace {

constexpr size_t kMaxBatch = 1024;




// Dynamic shared memory limit of both 2D update kernels of one shape, set
// once per device.
template <typename T, int N, int H, int W, int S>
cudaError_t prepare_step2d()
{
    static std::atomic<uint64_t> done{ 0 };
    int                          dev = 0;
    cudaGetDevice(&dev);
    const uint64_t bit = 1ull << (dev & 63);
    if (done.load() & bit) return cudaSuccess;
    const int   smem = static_cast<int>(Step2dShape<T, N, H>::smem(W, S));
    cudaError_t e    = cudaFuncSetAttribute(k_step2d<T, N, H, W, S>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_run_step2d<T, N, H, W, S>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    const int pass_smem = static_cast<int>(PassShape<T, N, H>::smem(W, S));
    auto      pass_attr = [&]<int D>() {
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_step2d_pass<T, N, H, W, S, D>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     pass_smem);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_run_step2d_pass<T, N, H, W, S, D>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     pass_smem);
    };
    pass_attr.template operator()<2>();
    if constexpr (sizeof(T) == 4) {
        pass_attr.template operator()<3>();
        pass_attr.template operator()<4>();
        pass_attr.template operator()<5>();
    }
    if (e == cudaSuccess) done.fetch_or(bit);
    return e;
}

// Resident blocks per SM of the 2D update kernel (W, S).
template <typename T, int N, int H, int W, int S>
int step2d_occupancy()
{
    if (prepare_step2d<T, N, H, W, S>() != cudaSuccess) return 0;
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_run_step2d<T, N, H, W, S>, W * 32,
                                                      Step2dShape<T, N, H>::smem(W, S)) != cudaSuccess)
        nb = 0;
    cudaGetLastError();
    return nb;
}

// Resident blocks per SM of the D-step pass (W, S), which also holds the
// warps' exchange buffers (registers grow with D).
template <typename T, int N, int H, int W, int S, int D>
int pass2d_occupancy()
{
    static std::atomic<int> cached[64]; // per device, 0 = not yet known
    int                     dev = 0;
    cudaGetDevice(&dev);
    if (const int c = cached[dev & 63].load(); c > 0) return c;
    if (prepare_step2d<T, N, H, W, S>() != cudaSuccess) return 0;
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_run_step2d_pass<T, N, H, W, S, D>, W * 32,
                                                      PassShape<T, N, H>::smem(W, S)) != cudaSuccess)
        nb = 0;
    cudaGetLastError();
    if (nb > 0) cached[dev & 63].store(nb);
    return nb;
}

// Calls f.template operator()<W, S>() for the (W, S) pair of the config; the
// pairs the autotuner searches.
template <typename F>
amr_status with_ws(int W, int S, F&& f)
{
    if (W == 4 && S == 2) return f.template operator()<4, 2>();
    if (W == 4 && S == 3) return f.template operator()<4, 3>();
    if (W == 8 && S == 1) return f.template operator()<8, 1>();
    if (W == 8 && S == 2) return f.template operator()<8, 2>();
    if (W == 8 && S == 3) return f.template operator()<8, 3>();
    if (W == 8 && S == 4) return f.template operator()<8, 4>();
    if (W == 16 && S == 2) return f.template operator()<16, 2>();
    if (W == 16 && S == 3) return f.template operator()<16, 3>();
    if (W == 16 && S == 4) return f.template operator()<16, 4>();
    return fail(AMR_ERR_INVALID, "unsupported update kernel configuration");
}
constexpr int kStepConfigs[][2] = { { 4, 2 }, { 4, 3 }, { 8, 1 }, { 8, 2 }, { 8, 3 }, { 8, 4 }, { 16, 2 }, { 16, 3 }, { 16, 4 } };

// Grid of the 2D update kernel: cfg.grid, or one warp per patch capped at
// full residency.
template <typename T, int N, int H, int W, int S>
unsigned step2d_grid(int P, int grid, int pass_occ = 0)
{
    if (grid > 0) return static_cast<unsigned>(grid);
    const int occ = std::max(1, pass_occ > 0 ? pass_occ : step2d_occupancy<T, N, H, W, S>());
    return static_cast<unsigned>(std::max<long long>(1, std::min<long long>(grid_for(P, W), 1LL * num_sms() * occ)));
}

template <typename T, int N, int H>
amr_status launch_step2d(const T* in, T* out, const amr_halo_meta* meta, int P, const Geo& g, const Coef* coef,
                         const float2* coef32, const int* up, int32_t* err, const uint64_t* keys,
                         const int32_t* upcode, const StepCfg& cfg, cudaStream_t s)
{
    return with_ws(cfg.W, cfg.S, [&]<int W, int S>() -> amr_status {
        AMR_CUDA((prepare_step2d<T, N, H, W, S>()));
        const unsigned grid = step2d_grid<T, N, H, W, S>(P, cfg.grid);
        k_step2d<T, N, H, W, S><<<grid, W * 32, Step2dShape<T, N, H>::smem(W, S), s>>>(
            in, out, meta, P, g, coef, coef32, up[0], up[1], err, keys, upcode);
        AMR_LAUNCHED("k_step2d");
        return AMR_OK;
    });
}

// ---------------------------------------------------------- 3D update
// Staged 3D kernels (one warp per patch, a ring of S bulk-copied tiles per
// warp) serve 4^3 and 8^3 patches with one ghost layer on 16-byte-aligned
// state buffers.
inline bool step3d_shape(const Geo& g, const void* in, const void* out)
{
    return g.rank == 3 && g.h == 1 && (g.n == 8 || g.n == 4) &&
           ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out)) & 15) == 0;
}

// Warps per block and ring depth: 4 x 2 for FP64 8^3 patches (its update is
// FP64-pipe bound; 64 KB of tiles per block), 8 x 2 otherwise (measured on
// uniform level-4 and level-5 trees of 8^3 patches against the other built
// pairs); AMR_GB300_STEP3D="W,S" picks another of (4,2), (4,3), (8,2), (8,3).
inline std::pair<int, int> step3d_config(int n, size_t esize)
{
    static const std::pair<int, int> env = [] {
        const char* e = std::getenv("AMR_GB300_STEP3D");
        int         w = 0, s = 0;
        if (e && std::sscanf(e, "%d,%d", &w, &s) == 2 && (w == 4 || w == 8) && (s == 2 || s == 3))
            return std::make_pair(w, s);
        return std::make_pair(0, 0);
    }();
    if (env.first) return env;
    return n == 8 && esize == 8 ? std::make_pair(4, 2) : std::make_pair(8, 2);
}

template <typename F>
amr_status with_ws3d(int n, size_t esize, F&& f)
{
    const auto [W, S] = step3d_config(n, esize);
    if (W == 4 && S == 2) return f.template operator()<4, 2>();
    if (W == 4 && S == 3) return f.template operator()<4, 3>();
    if (W == 8 && S == 2) return f.template operator()<8, 2>();
    return f.template operator()<8, 3>();
}

// Dynamic shared memory limit of both staged 3D kernels of one shape, set
// once per device; returns the resident blocks per SM (0 on failure).
template <typename T, int N, int W, int S>
int prepare_step3d()
{
    static std::atomic<int> cached[64];
    int                     dev = 0;
    cudaGetDevice(&dev);
    if (const int c = cached[dev & 63].load(); c > 0) return c;
    const int   smem = static_cast<int>(Step3dShape<T, N>::smem(W, S));
    cudaError_t e    = cudaFuncSetAttribute(k_step3d<T, N, W, S>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_run_step3d<T, N, W, S>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    int nb = 0;
    if (e == cudaSuccess &&
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_run_step3d<T, N, W, S>, W * 32, smem) != cudaSuccess)
        nb = 0;
    cudaGetLastError();
    if (nb > 0) cached[dev & 63].store(nb);
    return nb;
}

template <typename T, int N>
amr_status launch_step3d(const T* in, T* out, const int32_t* levels, const amr_halo_meta* meta, int P, const Geo& g,
                         const Coef* coef, const float4* coef4, const int* up, const uint64_t* keys,
                         const int32_t* upcode, int32_t* err, cudaStream_t s)
{
    return with_ws3d(N, sizeof(T), [&]<int W, int S>() -> amr_status {
        const int occ = prepare_step3d<T, N, W, S>();
        if (occ <= 0) return fail(AMR_ERR_CUDA, "staged 3D update kernel: shared-memory configuration failed");
        const unsigned grid = static_cast<unsigned>(
            std::max<long long>(1, std::min<long long>(grid_for(P, W), 1LL * num_sms() * occ)));
        k_step3d<T, N, W, S><<<grid, W * 32, Step3dShape<T, N>::smem(W, S), s>>>(
            in, out, levels, meta, P, g, coef, coef4, up[0], up[1], up[2], keys, upcode, err);
        AMR_LAUNCHED("k_step3d");
        return AMR_OK;
    });
}

// The graph form: the leaf count is read on the device, so the grid is full
// residency and the warps stride over the patches.
template <typename T, int N>
amr_status launch_run_step3d(const RunBufs& B, RunCtl* ctl, const Geo& g, const Coef* coef, const float4* coef4,
                             int parity, const int* up, cudaStream_t s)
{
    return with_ws3d(N, sizeof(T), [&]<int W, int S>() -> amr_status {
        const int occ = prepare_step3d<T, N, W, S>();
        if (occ <= 0) return fail(AMR_ERR_CUDA, "staged 3D update kernel: shared-memory configuration failed");
        k_run_step3d<T, N, W, S><<<static_cast<unsigned>(num_sms() * occ), W * 32, Step3dShape<T, N>::smem(W, S),
                                   s>>>(B, ctl, g, coef, coef4, parity, up[0], up[1], up[2]);
        AMR_LAUNCHED("k_run_step3d");
        return AMR_OK;
    });
}

// Steps per pass on same-level trees: FP32 five (a pass costs a fixed share,
// the state's read and write and the per-patch work, plus a share per step),
// FP64 two (its update is FP64-bound).
template <typename T>
constexpr int kPassSteps = sizeof(T) == 4 ? 5 : 2;

// The pass depths covering k steps: as few passes as depth `deep` allows,
// their depths as equal as possible (10 steps at depth 5: 5 + 5; 6: 3 + 3).
inline void pass_plan(int k, int deep, std::vector<int>& plan)
{
    plan.clear();
    if (k <= 0) return;
    const int np = (k + deep - 1) / deep;
    for (int i = 0; i < np; ++i) plan.push_back(k / np + (i < k % np ? 1 : 0));
}

// Depth D of a pass as a template argument (FP32 2..5, FP64 2).
template <typename T, typename F>
amr_status with_depth(int D, F&& f)
{
    if constexpr (sizeof(T) == 4) {
        if (D == 5) return f.template operator()<5>();
        if (D == 4) return f.template operator()<4>();
        if (D == 3) return f.template operator()<3>();
    }
    if (D == 2) return f.template operator()<2>();
    return fail(AMR_ERR_INVALID, "unsupported pass depth");
}

// D steps per pass (same-level trees, pass records built): coefficient rows
// of step m at coef + m * cstride.
template <typename T, int N, int H, int D>
amr_status launch_step2d_pass(const T* in, T* out, const int4* rec, int P, int nl, const Coef* coef,
                              const float2* coef32, size_t cstride, int32_t* err, const StepCfg& cfg, cudaStream_t s)
{
    return with_ws(cfg.W, cfg.S, [&]<int W, int S>() -> amr_status {
        AMR_CUDA((prepare_step2d<T, N, H, W, S>()));
        const unsigned grid = step2d_grid<T, N, H, W, S>(P, cfg.grid, pass2d_occupancy<T, N, H, W, S, D>());
        k_step2d_pass<T, N, H, W, S, D><<<grid, W * 32, PassShape<T, N, H>::smem(W, S), s>>>(in, out, rec, P, nl, coef,
                                                                                           coef32, cstride, err);
        AMR_LAUNCHED("k_step2d_pass");
        return AMR_OK;
    });
}

// Pass records of the tree's current leaves (host-driven passes and the
// tuner); upwind offsets per instance (upcode) or launch-wide (up).
amr_status build_pass_records(amr_tree* t, const int32_t* upcode, const int* up, cudaStream_t s)
{
    const int P = static_cast<int>(t->size);
    if (P == 0) return AMR_OK;
    const unsigned grid = static_cast<unsigned>(std::min<long long>((P + 255) / 256, 8LL * num_sms()));
    k_pass_records<<<grid, 256, 0, s>>>(t->meta[t->tb], t->keys[t->tb], upcode, up[0], up[1], P, t->g, t->prec,
                                        t->status + 7);
    AMR_LAUNCHED("k_pass_records");
    return AMR_OK;
}

// ------------------------------------------------------------ autotuner
// Picks (W, S, grid) for the 2D update kernel by timing every candidate on
// the tree's current leaves (reads the current state, writes the next
// buffer, which the following step overwrites).  Results are cached per
// device, dtype, patch shape and leaf-count octave.
struct TuneKey {
    int dev, esize, n, h, octave, per_leaf, pair;
    bool operator<(const TuneKey& o) const
    {
        return std::tie(dev, esize, n, h, octave, per_leaf, pair) <
               std::tie(o.dev, o.esize, o.n, o.h, o.octave, o.per_leaf, o.pair);
    }
};
std::mutex                 g_tune_mu;
std::map<TuneKey, StepCfg> g_tuned;
std::atomic<int>           g_tune_mode{ 1 }; // 0 off (defaults), 1 on

TuneKey tune_key(const amr_tree* t, bool per_leaf, bool pair)
{
    int dev = 0;
    cudaGetDevice(&dev);
    int oct = 0;
    while ((static_cast<size_t>(1) << oct) < t->size) ++oct;
    return TuneKey{ dev, static_cast<int>(t->esize), t->g.n, t->g.h, oct, per_leaf ? 1 : 0, pair ? 1 : 0 };
}

bool lookup_tuned(const amr_tree* t, bool per_leaf, bool pair, StepCfg& cfg)
{
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto                        it = g_tuned.find(tune_key(t, per_leaf, pair));
    if (it == g_tuned.end()) return false;
    cfg = it->second;
    return true;
}

// pair: time the multi-step pass instead (same-level trees); every step of
// it reads the prologue's coefficient row (stride 0).
template <typename T, int N, int H>
amr_status tune_step2d(amr_tree* t, const Coef* coef, const float2* coef32, const int* up, const int32_t* upcode,
                       StepCfg& best, bool pair = false)
{
    const TuneKey key = tune_key(t, upcode != nullptr, pair);
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto                        it = g_tuned.find(key);
        if (it != g_tuned.end()) {
            best = it->second;
            return AMR_OK;
        }
    }
    best = StepCfg{};
    if (const char* env = std::getenv("AMR_GB300_STEP_CONFIG")) { // "warps,stages,blocks per SM" (0: full residency)
        int w = 0, st = 0, bps = 0;
        if (std::sscanf(env, "%d,%d,%d", &w, &st, &bps) == 3 &&
            with_ws(w, st, []<int W, int S>() -> amr_status { return AMR_OK; }) == AMR_OK && bps >= 0) {
            best = StepCfg{ w, st, bps > 0 ? bps * num_sms() : 0 };
            std::lock_guard<std::mutex> lk(g_tune_mu);
            g_tuned[key] = best;
            return AMR_OK;
        }
    }
    if (g_tune_mode.load() == 0) return AMR_OK;
    if (const char* env = std::getenv("AMR_GB300_AUTOTUNE"); env && std::strcmp(env, "0") == 0) return AMR_OK;
    const int    P = static_cast<int>(t->size);
    cudaStream_t s = t->stream;
    const int    sms = num_sms();
    if (pair) {
        const amr_status rs = build_pass_records(t, upcode, up, s);
        if (rs != AMR_OK) return rs;
    }
    auto launch = [&](const StepCfg& c) -> amr_status {
        return pair ? launch_step2d_pass<T, N, H, kPassSteps<T>>(static_cast<const T*>(t->cur),
                                                                 static_cast<T*>(t->nxt), t->prec, P, t->g.depth + 1,
                                                                 coef, coef32, 0, t->status + 7, c, s)
                    : launch_step2d<T, N, H>(static_cast<const T*>(t->cur), static_cast<T*>(t->nxt), t->meta[t->tb],
                                             P, t->g, coef, coef32, up, t->status + 7, t->keys[t->tb], upcode, c, s);
    };
    // candidates: every (W, S) with its resident block counts up to full
    // residency or one warp per leaf
    std::vector<StepCfg> cand;
    for (const auto& ws : kStepConfigs) {
        (void)with_ws(ws[0], ws[1], [&]<int W, int S>() -> amr_status {
            const int occ =
                pair ? pass2d_occupancy<T, N, H, W, S, kPassSteps<T>>() : step2d_occupancy<T, N, H, W, S>();
            const int full = static_cast<int>(grid_for(P, W));
            for (int bps : { 1, 2, 3, 4, 6, 8, 12, 16 }) {
                if (bps > occ) break;
                const int grid = std::min(full, sms * bps);
                cand.push_back(StepCfg{ W, S, grid });
                if (grid == full) break; // more blocks would idle
            }
            return AMR_OK;
        });
    }
    // rounds over all candidates, each candidate's best round counts: a
    // candidate's time does not rest on one sample taken during a transient
    cudaEvent_t e0, e1;
    AMR_CUDA(cudaEventCreate(&e0));
    AMR_CUDA(cudaEventCreate(&e1));
    std::vector<float> best_ms(cand.size(), 0.0f);
    amr_status         st = AMR_OK;
    constexpr int      kRounds = 3, kReps = 3;
    for (int round = 0; round < kRounds && st == AMR_OK; ++round) {
        for (size_t i = 0; i < cand.size() && st == AMR_OK; ++i) {
            st = launch(cand[i]); // warm-up
            if (st != AMR_OK) break;
            if (cudaEventRecord(e0, s) != cudaSuccess) st = fail(AMR_ERR_CUDA, "tuner event");
            for (int rep = 0; rep < kReps && st == AMR_OK; ++rep) st = launch(cand[i]);
            if (st != AMR_OK) break;
            float ms = 0.0f;
            if (cudaEventRecord(e1, s) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
                cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess)
                st = fail(AMR_ERR_CUDA, "tuner timing");
            else if (round == 0 || ms < best_ms[i])
                best_ms[i] = ms;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st != AMR_OK) return st;
    size_t bi = 0;
    for (size_t i = 1; i < cand.size(); ++i)
        if (best_ms[i] < best_ms[bi]) bi = i;
    if (!cand.empty()) best = cand[bi];
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tuned[key] = best;
    return AMR_OK;
}



void free_tree(amr_tree* t)
{
    if (!t) return;
    for (auto& e : t->events) {
        cudaEventDestroy(e.first);
        cudaEventDestroy(e.second);
    }
    for (auto& ge : t->graphs) {
        if (ge.exec) cudaGraphExecDestroy(ge.exec);
        if (ge.graph) cudaGraphDestroy(ge.graph);
    }
    if (t->cap_stream) cudaStreamDestroy(t->cap_stream);
    cudaFree(t->sbuf[0]);
    cudaFree(t->sbuf[1]);
    for (int b = 0; b < 2; ++b) {
        cudaFree(t->keys[b]);
        cudaFree(t->levels[b]);
        cudaFree(t->meta[b]);
    }
    cudaFree(t->prec);
    cudaFree(t->frec);
    cudaFree(t->dg_prims);
    cudaFree(t->dg_scalars);
    cudaFree(t->dg_dtmin);
    cudaFree(t->flags);
    cudaFree(t->rmark);
    cudaFree(t->chead);
    cudaFree(t->cnt);
    cudaFree(t->pos);
    cudaFree(t->src);
    cudaFree(t->skind);
    cudaFree(t->status);
    cudaFree(t->maxlev);
    cudaFree(t->maxlev_new);
    cudaFree(t->vel);
    cudaFree(t->vel_inst);
    cudaFree(t->bounds);
    cudaFree(t->target);
    cudaFree(t->offs);
    cudaFree(t->tile_sums);
    cudaFree(t->ctl);
    cudaFree(t->dt_acc);
    cudaFree(t->dt_rem);
    cudaFree(t->dt_cnt);
    cudaFree(t->dt_tot);
    cudaFree(t->dt_ctot);
    cudaFree(t->dt_scratch);
    cudaFree(t->step_dt);
    cudaFree(t->coef);
    cudaFree(t->coef32);
    cudaFree(t->upcode);
    cudaFree(t->cstats);
    cudaFree(t->euler_min);
    cudaFree(t->euler_dt);
    cudaFree(t->euler_ctl);
    cudaFree(t->prim[0]);
    cudaFree(t->prim[1]);
    cudaFree(t->stage_buf);
    if (t->pinned) cudaFreeHost(t->pinned);
    delete t;
}

// One root leaf per instance: key i << inst_shift, level 0, periodic
// self-neighbours (ndtree.hpp:411-421), zero state in both buffers.
amr_status init_root(amr_tree* t)
{
    const Geo&                 g = t->g;
    const int                  K = t->ninst;
    std::vector<amr_halo_meta> root(static_cast<size_t>(K) * g.ndir);
    std::vector<uint64_t>      keys(K);
    std::vector<int32_t>       zeros(K, 0);
    for (int i = 0; i < K; ++i) {
        keys[i] = K > 1 ? static_cast<uint64_t>(i) << g.inst_shift : 0ull;
        for (int d = 0; d < g.ndir; ++d) {
            amr_halo_meta& m = root[static_cast<size_t>(i) * g.ndir + d];
            m.neighbor       = i;
            for (int q = 0; q < 4; ++q) m.finer_ids[q] = -1;
            for (int q = 0; q < 3; ++q) m.quadrant[q] = 0;
            m.relation   = REL_SAME;
            m.padding[0] = m.padding[1] = m.padding[2] = 0;
        }
    }
    const size_t state_bytes = t->nvar * t->field_bytes(t->cap);
    t->tb  = 0;
    t->cur = t->sbuf[0];
    t->nxt = t->sbuf[1];
    AMR_CUDA(cudaMemsetAsync(t->cur, 0, state_bytes, t->stream));
    AMR_CUDA(cudaMemsetAsync(t->nxt, 0, state_bytes, t->stream));
    AMR_CUDA(cudaMemsetAsync(t->status, 0, 8 * sizeof(int32_t), t->stream));
    AMR_CUDA(cudaMemsetAsync(t->maxlev_new, 0, K * sizeof(int32_t), t->stream));
    AMR_CUDA(cudaMemcpyAsync(t->keys[0], keys.data(), K * sizeof(uint64_t), cudaMemcpyHostToDevice, t->stream));
    AMR_CUDA(cudaMemcpyAsync(t->levels[0], zeros.data(), K * sizeof(int32_t), cudaMemcpyHostToDevice, t->stream));
    AMR_CUDA(cudaMemcpyAsync(t->maxlev, zeros.data(), K * sizeof(int32_t), cudaMemcpyHostToDevice, t->stream));
    AMR_CUDA(cudaMemcpyAsync(t->meta[0], root.data(), root.size() * sizeof(amr_halo_meta), cudaMemcpyHostToDevice,
                             t->stream));
    AMR_CUDA(cudaStreamSynchronize(t->stream));
    t->size           = static_cast<size_t>(K);
    t->max_level_host = 0;
    t->ghosts_valid   = true;
    t->batch_open     = false;
    t->uniform        = true; // roots are their own same-level neighbours
    ++t->topo;
    return AMR_OK;
}

// Whether every neighbour record of the current tree is "same level" (the
// condition for two-step passes), read back into t->uniform.
amr_status refresh_uniform(amr_tree* t)
{
    int32_t*        hs = static_cast<int32_t*>(t->pinned);
    const long long n  = static_cast<long long>(t->size) * t->g.ndir;
    AMR_CUDA(cudaMemsetAsync(t->status + 5, 0, sizeof(int32_t), t->stream));
    k_any_not_same<<<std::min<unsigned>(grid_for(n, 256), 1024u), 256, 0, t->stream>>>(t->meta[t->tb], n,
                                                                                          t->status + 5);
    AMR_LAUNCHED("k_any_not_same");
    AMR_CUDA(cudaMemcpyAsync(hs + 8, t->status + 5, sizeof(int32_t), cudaMemcpyDeviceToHost, t->stream));
    AMR_CUDA(cudaStreamSynchronize(t->stream));
    t->uniform = hs[8] == 0;
    return AMR_OK;
}

// Finest level over all leaves of a forest after a re-mesh (one tree: the
// single max_level slot already holds it).
amr_status forest_max_level(amr_tree* t, int* out)
{
    int32_t* hs = static_cast<int32_t*>(t->pinned);
    AMR_CUDA(cudaMemsetAsync(t->status + 3, 0, sizeof(int32_t), t->stream));
    k_max_level<<<std::min<unsigned>(grid_for(static_cast<long long>(t->size), 256), 1024u), 256, 0, t->stream>>>(
        t->levels[t->tb], static_cast<int>(t->size), t->status + 3);
    AMR_LAUNCHED("k_max_level");
    AMR_CUDA(cudaMemcpyAsync(hs + 6, t->status + 3, sizeof(int32_t), cudaMemcpyDeviceToHost, t->stream));
    AMR_CUDA(cudaStreamSynchronize(t->stream));
    *out = hs[6];
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

// The gradient rule's exact squared thresholds and its FP32 pre-filter band.
GradRule make_grad_rule(double rthr, double cthr)
{
    GradRule     r{};
    const double m = 1e-5;
    r.rsq          = sq_threshold(rthr, true);
    r.csq          = sq_threshold(cthr, false);
    auto usable    = [](double t) { return t == 0.0 || (t >= 1e-20 && t <= 1e30); };
    r.fast         = usable(r.rsq) && usable(r.csq) ? 1 : 0;
    auto down      = [](double v) {
        float f = static_cast<float>(v);
        if (static_cast<double>(f) > v) f = std::nextafter(f, -std::numeric_limits<float>::infinity());
        return f;
    };
    auto up = [](double v) {
        float f = static_cast<float>(v);
        if (static_cast<double>(f) < v) f = std::nextafter(f, std::numeric_limits<float>::infinity());
        return f;
    };
    const float ninf = -std::numeric_limits<float>::infinity();
    // s >= 0 always: a zero threshold is decided by s32 >= 0 alone
    r.r_hi = r.rsq == 0.0 ? 0.0f : up(r.rsq * (1.0 + m));
    r.r_lo = r.rsq == 0.0 ? ninf : down(r.rsq * (1.0 - m));
    r.c_hi = r.csq == 0.0 ? 0.0f : up(r.csq * (1.0 + m));
    r.c_lo = r.csq == 0.0 ? ninf : down(r.csq * (1.0 - m));
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

// ------------------------------------------------------------ graph run
RunBufs run_bufs(amr_tree* t, bool per_leaf_vel, bool bounds)
{
    RunBufs B{};
    B.state[0] = t->sbuf[0];
    B.state[1] = t->sbuf[1];
    for (int b = 0; b < 2; ++b) {
        B.keys[b]   = t->keys[b];
        B.levels[b] = t->levels[b];
        B.meta[b]   = t->meta[b];
    }
    B.flags      = t->flags;
    B.rmark      = t->rmark;
    B.chead      = t->chead;
    B.cnt        = t->cnt;
    B.pos        = t->pos;
    B.src        = t->src;
    B.skind      = t->skind;
    B.maxlev     = t->maxlev;
    B.maxlev_new = t->maxlev_new;
    B.vel        = per_leaf_vel ? t->vel : nullptr;
    B.upcode     = per_leaf_vel ? t->upcode : nullptr;
    B.prec       = t->prec;
    B.frec       = t->frec;
    B.bounds     = bounds ? t->bounds : nullptr;
    B.tile_sums  = t->tile_sums;
    B.cap        = t->cap;
    B.ninst      = t->ninst;
    return B;
}

template <typename T, int N, int H>
amr_status launch_run_step2d(const RunBufs& B, RunCtl* ctl, const Geo& g, const Coef* coef, const float2* coef32,
                             int parity, const int* up, const StepCfg& cfg, int P, cudaStream_t s)
{
    return with_ws(cfg.W, cfg.S, [&]<int W, int S>() -> amr_status {
        AMR_CUDA((prepare_step2d<T, N, H, W, S>()));
        const unsigned grid = step2d_grid<T, N, H, W, S>(P, cfg.grid);
        k_run_step2d<T, N, H, W, S><<<grid, W * 32, Step2dShape<T, N, H>::smem(W, S), s>>>(B, ctl, g, coef, coef32,
                                                                                          parity, up[0], up[1]);
        AMR_LAUNCHED("k_run_step2d");
        return AMR_OK;
    });
}

template <typename T, int N, int H, int D>
amr_status launch_run_step2d_pass(const RunBufs& B, RunCtl* ctl, int nl, const Coef* coef, const float2* coef32,
                                  size_t cstride, int parity, const StepCfg& cfg, int P, cudaStream_t s)
{
    return with_ws(cfg.W, cfg.S, [&]<int W, int S>() -> amr_status {
        AMR_CUDA((prepare_step2d<T, N, H, W, S>()));
        const unsigned grid = step2d_grid<T, N, H, W, S>(P, cfg.grid, pass2d_occupancy<T, N, H, W, S, D>());
        k_run_step2d_pass<T, N, H, W, S, D><<<grid, W * 32, PassShape<T, N, H>::smem(W, S), s>>>(B, ctl, nl, coef,
                                                                                               coef32, cstride, parity);
        AMR_LAUNCHED("k_run_step2d_pass");
        return AMR_OK;
    });
}

// Steps per fused interval (the whole re-mesh interval in one kernel).
constexpr int kFusedSteps = 10;

// Grid of the fused interval kernel: every resident CTA, capped by the
// tree's largest block count.
template <bool FLAGS>
unsigned fused_grid(amr_tree* t)
{
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_run_interval2d<kFusedSteps, FLAGS>,
                                                      IntervalShape<kFusedSteps>::THREADS,
                                                      IntervalShape<kFusedSteps>::smem) != cudaSuccess ||
        occ < 1)
        occ = 1;
    cudaGetLastError();
    return static_cast<unsigned>(std::max<long long>(1, std::min<long long>(static_cast<long long>(t->cap) / 16,
                                                                             1LL * num_sms() * occ)));
}

// Shared-memory limit of the fused interval kernel, set once per device.
cudaError_t prepare_fused()
{
    static std::atomic<uint64_t> done{ 0 };
    int                          dev = 0;
    cudaGetDevice(&dev);
    const uint64_t bit = 1ull << (dev & 63);
    if (done.load() & bit) return cudaSuccess;
    const int   smem = static_cast<int>(IntervalShape<kFusedSteps>::smem);
    cudaError_t e    = cudaFuncSetAttribute(k_run_interval2d<kFusedSteps, true>,
                                            cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_run_interval2d<kFusedSteps, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 smem);
    if (e == cudaSuccess) done.fetch_or(bit);
    return e;
}

// Event pair around the next update launch of a timed interval (amr_tree_set_timing).
amr_status timing_slot(amr_tree* t, uint64_t cells, std::pair<cudaEvent_t, cudaEvent_t>** ev)
{
    if (t->events_used == t->events.size()) {
        std::pair<cudaEvent_t, cudaEvent_t> e;
        AMR_CUDA(cudaEventCreate(&e.first));
        AMR_CUDA(cudaEventCreate(&e.second));
        t->events.push_back(e);
        t->event_cells.push_back(0);
    }
    *ev                            = &t->events[t->events_used];
    t->event_cells[t->events_used] = cells;
    ++t->events_used;
    return AMR_OK;
}

// The launch sequence of one interval on stream cs (captured into a graph,
// or launched directly with `timed` > 0: CUDA events around each update
// launch, `timed` being the interval's leaf count for the cell counts).
// Grids are fixed; every kernel takes the leaf count from the control block.
template <typename T>
amr_status record_interval(amr_tree* t, const GraphKey& key, const RunBufs& B, cudaStream_t cs, uint64_t timed = 0)
{
    const Geo& g   = t->g;
    const int  K   = t->ninst, nl = g.depth + 1, sms = num_sms();
    RunCtl*    ctl = t->ctl;
    if (key.pair) { // the interval runs only while the tree is same-level
        k_run_require_uniform<<<1, 32, 0, cs>>>(ctl);
        AMR_LAUNCHED("k_run_require_uniform");
    }
    if (key.fused) { // ... and is made of aligned 4x4 blocks
        k_run_require_blocks<<<grid_for(static_cast<long long>(t->cap) / 16, 256), 256, 0, cs>>>(B, ctl, g, key.up[0],
                                                                                                 key.up[1]);
        AMR_LAUNCHED("k_run_require_blocks");
    }
    k_batch_begin<<<K, 256, 0, cs>>>(t->maxlev, g, t->vel, key.cfl, key.k, BATCH_NEXT, 0.0, t->dts(), t->step_dt,
                                     t->coef, t->coef32, t->upcode, &ctl->err); // nothing after an error
    AMR_LAUNCHED("k_batch_begin");
    if constexpr (sizeof(T) == 4) {
        if (key.fused) { // the whole interval: steps and gradient flags in one kernel
            std::pair<cudaEvent_t, cudaEvent_t>* ev = nullptr;
            if (timed) {
                if (amr_status ts = timing_slot(t, timed * g.cells * key.k, &ev); ts != AMR_OK) return ts;
                AMR_CUDA(cudaEventRecord(ev->first, cs));
            }
            const size_t     cst  = static_cast<size_t>(K) * nl;
            const GradRule   rule = make_grad_rule(key.rthr, key.cthr);
            constexpr size_t smem = IntervalShape<kFusedSteps>::smem;
            constexpr int    nthr = IntervalShape<kFusedSteps>::THREADS;
            if (key.crit == 1)
                k_run_interval2d<kFusedSteps, true><<<fused_grid<true>(t), nthr, smem, cs>>>(
                    B, ctl, g, t->coef32, cst, nl, rule, key.min_level, key.max_level, 0);
            else
                k_run_interval2d<kFusedSteps, false><<<fused_grid<false>(t), nthr, smem, cs>>>(
                    B, ctl, g, t->coef32, cst, nl, rule, key.min_level, key.max_level, 0);
            AMR_LAUNCHED("k_run_interval2d");
            if (timed) AMR_CUDA(cudaEventRecord(ev->second, cs));
            constexpr int sp = 1; // the interval's result is in the other buffer
            if (key.crit != 0) {
                k_run_mark<<<sms * 4, 256, 0, cs>>>(B, ctl, g);
                AMR_LAUNCHED("k_run_mark");
                for (int r = 0; r < key.rounds; ++r) {
                    k_run_closure<<<sms * 4, 256, 0, cs>>>(B, ctl, g);
                    AMR_LAUNCHED("k_run_closure");
                }
                k_run_veto<<<sms * 4, 256, 0, cs>>>(B, ctl, g);
                AMR_LAUNCHED("k_run_veto");
                k_run_count<<<sms * 4, 256, 0, cs>>>(B, ctl, g);
                AMR_LAUNCHED("k_run_count");
                const unsigned ntile = static_cast<unsigned>(
                    std::min<size_t>(1024, std::max<size_t>(1, (t->cap + kScanTile - 1) / kScanTile)));
                k_run_scan_tiles<<<ntile, kScanThreads, 0, cs>>>(B, ctl);
                AMR_LAUNCHED("k_run_scan_tiles");
                k_run_scan_apply<<<ntile, kScanThreads, 0, cs>>>(B, ctl);
                AMR_LAUNCHED("k_run_scan_apply");
                k_run_emit<<<sms * 4, 256, 0, cs>>>(B, ctl, g);
                AMR_LAUNCHED("k_run_emit");
                k_run_remap<T><<<sms * 16, 256, 0, cs>>>(B, ctl, g, sp);
                AMR_LAUNCHED("k_run_remap");
                k_run_neighbors<<<sms * 8, 128, 0, cs>>>(B, ctl, g);
                AMR_LAUNCHED("k_run_neighbors");
            }
            // a fused interval builds no pass or face records (the face-record
            // storage held its block descriptors)
            k_run_commit<<<1, 256, 0, cs>>>(B, ctl, key.k, g.cells, key.crit != 0 ? 1 : 0, sp, 0);
            AMR_LAUNCHED("k_run_commit");
            return AMR_OK;
        }
    }
    if (key.pair) { // records of this interval's tree, with the upwind codes just written
        const unsigned rgrid =
            static_cast<unsigned>(std::min<long long>((static_cast<long long>(t->cap) + 255) / 256, 8LL * sms));
        k_run_pass_records<<<rgrid, 256, 0, cs>>>(B, ctl, g, key.up[0], key.up[1]);
        AMR_LAUNCHED("k_run_pass_records");
    }
    const StepCfg cfg{ key.W, key.S, key.grid };
    const int     ppb = std::max(1, 256 / g.cells);
    // multi-step passes on same-level trees (pass_plan), one launch per step
    // otherwise; the buffers alternate per launch
    std::vector<int> plan;
    if (key.pair) pass_plan(key.k, kPassSteps<T>, plan);
    else plan.assign(static_cast<size_t>(key.k), 1);
    int step = 0;
    for (size_t j = 0; j < plan.size(); ++j) {
        const int     D   = plan[j];
        const int     par = static_cast<int>(j & 1);
        const Coef*   cf  = t->coef + static_cast<size_t>(step) * K * nl;
        const float2* cf2 = t->coef32 + static_cast<size_t>(step) * K * nl;
        const size_t  cst = static_cast<size_t>(K) * nl;
        amr_status    st  = AMR_OK;
        std::pair<cudaEvent_t, cudaEvent_t>* ev = nullptr;
        if (timed) {
            if (amr_status ts = timing_slot(t, timed * g.cells * D, &ev); ts != AMR_OK) return ts;
            AMR_CUDA(cudaEventRecord(ev->first, cs));
        }
        auto pass = [&]<int N>() -> amr_status {
            return with_depth<T>(D, [&]<int DD>() -> amr_status {
                return launch_run_step2d_pass<T, N, 1, DD>(B, ctl, nl, cf, cf2, cst, par, cfg,
                                                           static_cast<int>(t->cap), cs);
            });
        };
        if (D > 1) st = g.n == 16 ? pass.template operator()<16>() : pass.template operator()<8>();
        else if (key.W > 0 && g.n == 16)
            st = launch_run_step2d<T, 16, 1>(B, ctl, g, cf, cf2, par, key.up, cfg, static_cast<int>(t->cap), cs);
        else if (key.W > 0)
            st = launch_run_step2d<T, 8, 1>(B, ctl, g, cf, cf2, par, key.up, cfg, static_cast<int>(t->cap), cs);
        else if (step3d_shape(g, B.state[0], B.state[1])) {
            // float4 rows of the 3D FP32 update
            const float4* cf4 = reinterpret_cast<const float4*>(t->coef32) + static_cast<size_t>(step) * K * nl;
            st = g.n == 8 ? launch_run_step3d<T, 8>(B, ctl, g, cf, cf4, par, key.up, cs)
                          : launch_run_step3d<T, 4>(B, ctl, g, cf, cf4, par, key.up, cs);
        } else {
            k_run_step<T><<<sms * 16, 256, 0, cs>>>(B, ctl, g, cf, par, key.up[0], key.up[1], key.up[2], ppb);
            AMR_LAUNCHED("k_run_step");
        }
        if (st != AMR_OK) return st;
        if (timed) AMR_CUDA(cudaEventRecord(ev->second, cs));
        step += D;
    }
    // parity of the buffer holding the interval's result
    const int sp = static_cast<int>(plan.size() & 1);
    if (key.crit != 0) {
        if (key.crit == 1 && g.rank == 2 && g.h == 1 && (g.n == 16 || g.n == 8)) {
            const GradRule rule = make_grad_rule(key.rthr, key.cthr);
            const unsigned fgrid = static_cast<unsigned>(sms * 4);
            if (key.pair) { // same-level tree: ghosts from the interval's face records
                if (g.n == 16)
                    k_run_flags2d_uniform<T, 16, 1><<<fgrid, 256, Flags2dShape<T, 16, 1, false>::smem(8), cs>>>(
                        B, ctl, rule, key.min_level, key.max_level, sp);
                else
                    k_run_flags2d_uniform<T, 8, 1><<<fgrid, 256, Flags2dShape<T, 8, 1, false>::smem(8), cs>>>(
                        B, ctl, rule, key.min_level, key.max_level, sp);
                AMR_LAUNCHED("k_run_flags2d_uniform");
            } else {
                if (g.n == 16)
                    k_run_flags2d<T, 16, 1><<<fgrid, 256, Flags2dShape<T, 16, 1, false>::smem(8), cs>>>(
                        B, ctl, g, rule, key.min_level, key.max_level, sp);
                else
                    k_run_flags2d<T, 8, 1><<<fgrid, 256, Flags2dShape<T, 8, 1, false>::smem(8), cs>>>(
                        B, ctl, g, rule, key.min_level, key.max_level, sp);
                AMR_LAUNCHED("k_run_flags2d");
            }
        } else if (key.crit == 1) {
            if (g.rank == 2)
                k_run_flags_grad<T, 2><<<sms * 16, 256, 0, cs>>>(B, ctl, g, make_grad_rule(key.rthr, key.cthr),
                                                                 key.min_level, key.max_level, sp);
            else
                k_run_flags_grad<T, 3><<<sms * 16, 256, 0, cs>>>(B, ctl, g, make_grad_rule(key.rthr, key.cthr),
                                                                 key.min_level, key.max_level, sp);
            AMR_LAUNCHED("k_run_flags_grad");
        } else {
            k_run_halo<T><<<sms * 32, 256, 0, cs>>>(B, ctl, g, sp);
            AMR_LAUNCHED("k_run_halo");
            k_run_flags_max<T><<<sms * 16, 128, 0, cs>>>(B, ctl, g, key.rthr, key.cthr, key.min_level, key.max_level,
                                                         sp);
            AMR_LAUNCHED("k_run_flags_max");
        }
        k_run_mark<<<sms * 4, 256, 0, cs>>>(B, ctl, g);
        AMR_LAUNCHED("k_run_mark");
        for (int r = 0; r < key.rounds; ++r) {
            k_run_closure<<<sms * 4, 256, 0, cs>>>(B, ctl, g);
            AMR_LAUNCHED("k_run_closure");
        }
        k_run_veto<<<sms * 4, 256, 0, cs>>>(B, ctl, g);
        AMR_LAUNCHED("k_run_veto");
        k_run_count<<<sms * 4, 256, 0, cs>>>(B, ctl, g);
        AMR_LAUNCHED("k_run_count");
        const unsigned ntile =
            static_cast<unsigned>(std::min<size_t>(1024, std::max<size_t>(1, (t->cap + kScanTile - 1) / kScanTile)));
        k_run_scan_tiles<<<ntile, kScanThreads, 0, cs>>>(B, ctl);
        AMR_LAUNCHED("k_run_scan_tiles");
        k_run_scan_apply<<<ntile, kScanThreads, 0, cs>>>(B, ctl);
        AMR_LAUNCHED("k_run_scan_apply");
        k_run_emit<<<sms * 4, 256, 0, cs>>>(B, ctl, g);
        AMR_LAUNCHED("k_run_emit");
        k_run_remap<T><<<sms * 16, 256, 0, cs>>>(B, ctl, g, sp);
        AMR_LAUNCHED("k_run_remap");
        k_run_neighbors<<<sms * 8, 128, 0, cs>>>(B, ctl, g);
        AMR_LAUNCHED("k_run_neighbors");
    }
    k_run_commit<<<1, 256, 0, cs>>>(B, ctl, key.k, g.cells, key.crit != 0 ? 1 : 0, sp, key.pair ? 1 : 0);
    AMR_LAUNCHED("k_run_commit");
    return AMR_OK;
}

// Executable graph of one interval, captured on first use and cached on the
// tree (buffers have fixed addresses for the tree's lifetime).
amr_status interval_graph(amr_tree* t, const GraphKey& key, const RunBufs& B, cudaGraphExec_t* out,
                          uint64_t* kernels)
{
    for (auto& ge : t->graphs)
        if (ge.key == key) {
            *out     = ge.exec;
            *kernels = ge.kernels;
            return AMR_OK;
        }
    if (!t->cap_stream) AMR_CUDA(cudaStreamCreateWithFlags(&t->cap_stream, cudaStreamNonBlocking));
    AMR_CUDA(cudaStreamBeginCapture(t->cap_stream, cudaStreamCaptureModeThreadLocal));
    const uint64_t before = g_launches.load();
    amr_status st = t->dtype == AMR_F64 ? record_interval<double>(t, key, B, t->cap_stream)
                                        : record_interval<float>(t, key, B, t->cap_stream);
    const uint64_t recorded = g_launches.load() - before;
    g_launches.fetch_sub(recorded); // counted when replayed
    cudaGraph_t graph = nullptr;
    cudaError_t ce    = cudaStreamEndCapture(t->cap_stream, &graph);
    if (st != AMR_OK) {
        if (graph) cudaGraphDestroy(graph);
        return st;
    }
    if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamEndCapture");
    GraphEntry ge;
    ge.key     = key;
    ge.graph   = graph;
    ge.kernels = recorded;
    ce       = cudaGraphInstantiate(&ge.exec, graph, 0);
    if (ce != cudaSuccess) {
        cudaGraphDestroy(graph);
        return cuda_fail(ce, "cudaGraphInstantiate");
    }
    if (t->graphs.size() >= 8) { // keep a handful of shapes
        cudaGraphExecDestroy(t->graphs.front().exec);
        cudaGraphDestroy(t->graphs.front().graph);
        t->graphs.erase(t->graphs.begin());
    }
    t->graphs.push_back(ge);
    *out     = ge.exec;
    *kernels = ge.kernels;
    return AMR_OK;
}

// Whether a run may use the fused interval kernel: AMR_RUN_FUSED asks for it,
// AMR_RUN_NO_FUSED forbids it; otherwise the default (on), which
// AMR_GB300_FUSED=0 in the environment turns off.
bool fused_enabled(int options)
{
    if (options & AMR_RUN_NO_FUSED) return false;
    if (options & AMR_RUN_FUSED) return true;
    static const bool on = [] {
        const char* e = std::getenv("AMR_GB300_FUSED");
        return !(e && e[0] == '0');
    }();
    return on;
}

// True when the run's level bounds pin every instance to one level (min =
// max), so a re-mesh of a same-level tree at those levels changes nothing.
static bool remesh_keeps_levels(const amr_tree* t, const amr_cycle_params* p)
{
    if (!t->bounds_set) return p->min_level == p->max_level;
    for (int i = 0; i < t->ninst; ++i)
        if (t->bounds_host[2 * i] != t->bounds_host[2 * i + 1]) return false;
    return true;
}

// Up to `max_intervals` intervals as graph replays, then one readback of the
// control block.  Requires that no step is clamped by the remaining time.
amr_status run_graph_chunk(amr_tree* t, const amr_cycle_params* p, bool inst_params, long long max_intervals,
                           RunTotals& tot)
{
    const Geo&      g     = t->g;
    const int       K     = t->ninst;
    cudaStream_t    s     = t->stream;
    const long long total = static_cast<long long>(p->steps);
    const long long k     = static_cast<long long>(p->remesh_interval);
    const bool      per_leaf = inst_params && K > 1;
    // velocities in use
    if (inst_params) {
        if (amr_status cs = copy_words8(t->vel, t->vel_inst, 3 * static_cast<size_t>(K), s); cs != AMR_OK) return cs;
    } else {
        std::vector<double> v(3 * static_cast<size_t>(K));
        for (int i = 0; i < K; ++i)
            for (int a = 0; a < 3; ++a) v[3 * i + a] = p->velocity[a];
        AMR_CUDA(cudaMemcpyAsync(t->vel, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice, s));
    }
    const RunBufs B = run_bufs(t, per_leaf, t->bounds_set);
    // control block and per-instance time
    RunCtl c{};
    c.P          = static_cast<int32_t>(t->size);
    c.tb         = t->tb;
    c.sb         = t->cur == t->sbuf[0] ? 0 : 1;
    c.max_level  = t->max_level_host;
    c.leaves_min = INT_MAX;
    c.leaves_max = 0;
    c.uniform    = t->uniform ? 1 : 0;
    RunCtl* hc   = reinterpret_cast<RunCtl*>(static_cast<char*>(t->pinned) + 64);
    *hc          = c;
    AMR_CUDA(cudaMemcpyAsync(t->ctl, hc, sizeof(RunCtl), cudaMemcpyHostToDevice, s));
    // the key of the interval graph(s)
    GraphKey key;
    key.crit      = p->criterion;
    key.min_level = p->min_level;
    key.max_level = p->max_level;
    key.bounds    = t->bounds_set ? 1 : 0;
    key.vel       = per_leaf ? 1 : 0;
    key.rthr      = p->refine_threshold;
    key.cthr      = p->coarsen_threshold;
    key.cfl       = p->cfl;
    for (int a = 0; a < g.rank && !per_leaf; ++a)
        key.up[a] = p->velocity[a] > 0.0 ? -1 : (p->velocity[a] < 0.0 ? 1 : 0);
    int allowed = p->max_level;
    if (t->bounds_set) {
        allowed = 0;
        for (int i = 0; i < K; ++i) allowed = std::max(allowed, static_cast<int>(t->bounds_host[2 * i + 1]));
    }
    key.rounds = std::max(1, std::min(g.depth, std::max(t->max_level_host, allowed)));
    const bool step2d = g.rank == 2 && g.h == 1 && (g.n == 16 || g.n == 8);
    if (step2d) {
        StepCfg cfg;
        if (g.n == 16) {
            // tune on the current leaves with a coefficient table of this run
            // (its own time bookkeeping: the run's totals stay as they are)
            k_batch_begin<<<K, 256, 0, s>>>(t->maxlev, g, t->vel, p->cfl, 1, BATCH_RESET, 1.0, t->scratch_dts(),
                                            t->step_dt, t->coef, t->coef32, t->upcode);
            AMR_LAUNCHED("k_batch_begin");
            int up[3] = { key.up[0], key.up[1], key.up[2] };
            amr_status ts = dispatch_dtype(t->dtype, [&](auto z) -> amr_status {
                using T = decltype(z);
                return tune_step2d<T, 16, 1>(t, t->coef, t->coef32, up, per_leaf ? t->upcode : nullptr, cfg,
                                             t->uniform);
            });
            if (ts != AMR_OK) return ts;
        }
        key.W       = cfg.W;
        key.S       = cfg.S;
        key.grid    = cfg.grid; // 0: full residency
        t->last_cfg = cfg;
        // kernel attributes are set outside the capture
        amr_status ps = dispatch_dtype(t->dtype, [&](auto z) -> amr_status {
            using T = decltype(z);
            return with_ws(key.W, key.S, [&]<int W, int S>() -> amr_status {
                if (g.n == 16) AMR_CUDA((prepare_step2d<T, 16, 1, W, S>()));
                else AMR_CUDA((prepare_step2d<T, 8, 1, W, S>()));
                return AMR_OK;
            });
        });
        if (ps != AMR_OK) return ps;
    } else if (step3d_shape(g, t->sbuf[0], t->sbuf[1])) {
        // the staged 3D kernel's attributes, likewise outside the capture
        amr_status ps = dispatch_dtype(t->dtype, [&](auto z) -> amr_status {
            using T = decltype(z);
            return with_ws3d(g.n, sizeof(T), [&]<int W, int S>() -> amr_status {
                const int occ = g.n == 8 ? prepare_step3d<T, 8, W, S>() : prepare_step3d<T, 4, W, S>();
                return occ > 0 ? AMR_OK
                               : fail(AMR_ERR_CUDA, "staged 3D update kernel: shared-memory configuration failed");
            });
        });
        if (ps != AMR_OK) return ps;
    }
    // per-instance time: one tree carries the run's totals in from the host;
    // a forest starts them at the run's first interval and otherwise keeps
    // its per-instance totals on the device (the next interval folds them)
    if (K == 1 || tot.intervals == 0) {
        k_run_dt_init<<<grid_for(K, 256), 256, 0, s>>>(t->dts(), K, p->remaining_time - tot.sum_dt,
                                                        K == 1 ? tot.sum_dt : 0.0,
                                                        K == 1 ? static_cast<uint32_t>(tot.executed) : 0u);
        AMR_LAUNCHED("k_run_dt_init");
    }
    // same-level trees: two steps per pass, guarded on the device; FP32
    // forests of 16x16 patches whose interval is kFusedSteps long run the
    // whole interval (steps and gradient flags) in one kernel
    const bool pairs = step2d && t->uniform && key.W > 0;
    const bool fused = pairs && t->dtype == AMR_F32 && g.n == 16 && k == kFusedSteps &&
                       (p->criterion == 0 || p->criterion == 1) && !t->fused_off && fused_enabled(p->options);
    if (fused) AMR_CUDA(prepare_fused());
    // A same-level graph is guarded on the device: once a re-mesh has made
    // the tree non-uniform, the replays still queued behind it launch only
    // kernels that find the guard set.  When the re-mesh may change the tree
    // (its level bounds allow it), a chunk of such graphs is short at first
    // and doubles while the tree stays same-level.
    if (pairs && key.crit != 0 && !remesh_keeps_levels(t, p)) {
        max_intervals = std::min(max_intervals, t->pair_chunk);
        t->pair_chunk = std::min<long long>(t->pair_chunk * 2, 1 << 20);
    }
    const long long left  = total - tot.done;
    const long long nfull = std::min(left / k, max_intervals);
    const long long rem   = (nfull < max_intervals) ? left % k : 0;
    cudaGraphExec_t full = nullptr, tail = nullptr;
    uint64_t        nk_full = 0, nk_tail = 0;
    GraphKey key_full = key, key_tail = key;
    if (nfull > 0) {
        key_full.k     = static_cast<int>(k);
        key_full.pair  = pairs && k >= 2 ? 1 : 0;
        key_full.fused = fused ? 1 : 0;
        if (!t->timing) {
            amr_status st = interval_graph(t, key_full, B, &full, &nk_full);
            if (st != AMR_OK) return st;
        }
    }
    if (rem > 0) {
        key_tail.k    = static_cast<int>(rem);
        key_tail.pair = pairs && rem >= 2 ? 1 : 0;
        if (!t->timing) {
            amr_status st = interval_graph(t, key_tail, B, &tail, &nk_tail);
            if (st != AMR_OK) return st;
        }
    }
    if (t->timing) {
        // timed: the same launch sequence issued directly, CUDA events
        // around each update launch; the leaf count of each interval is read
        // back first (it changes with the re-meshes)
        auto direct = [&](const GraphKey& kk) -> amr_status {
            int32_t* hp = reinterpret_cast<int32_t*>(static_cast<char*>(t->pinned) + 64 + sizeof(RunCtl));
            AMR_CUDA(cudaMemcpyAsync(hp, &t->ctl->P, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
            AMR_CUDA(cudaStreamSynchronize(s));
            const uint64_t Pi = static_cast<uint64_t>(std::max(1, *hp));
            return t->dtype == AMR_F64 ? record_interval<double>(t, kk, B, s, Pi)
                                       : record_interval<float>(t, kk, B, s, Pi);
        };
        for (long long i = 0; i < nfull; ++i)
            if (amr_status st = direct(key_full); st != AMR_OK) return st;
        if (rem > 0)
            if (amr_status st = direct(key_tail); st != AMR_OK) return st;
    } else {
        for (long long i = 0; i < nfull; ++i) {
            AMR_CUDA(cudaGraphLaunch(full, s));
            g_launches.fetch_add(nk_full);
        }
        if (tail) {
            AMR_CUDA(cudaGraphLaunch(tail, s));
            g_launches.fetch_add(nk_tail);
        }
    }
    // readback
    AMR_CUDA(cudaMemcpyAsync(hc, t->ctl, sizeof(RunCtl), cudaMemcpyDeviceToHost, s));
    char* hp = static_cast<char*>(t->pinned) + 64 + sizeof(RunCtl);
    AMR_CUDA(cudaMemcpyAsync(hp, t->dt_acc, K * sizeof(double), cudaMemcpyDeviceToHost, s));
    AMR_CUDA(cudaMemcpyAsync(hp + 8 * K, t->dt_tot, K * sizeof(double), cudaMemcpyDeviceToHost, s));
    AMR_CUDA(cudaMemcpyAsync(hp + 16 * K, t->dt_cnt, K * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    AMR_CUDA(cudaMemcpyAsync(hp + 20 * K, t->dt_ctot, K * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    AMR_CUDA(cudaStreamSynchronize(s));
    const RunCtl r = *hc;
    t->size        = static_cast<size_t>(r.P);
    t->tb          = r.tb;
    t->cur         = t->sbuf[r.sb];
    t->nxt         = t->sbuf[r.sb ^ 1];
    t->max_level_host = r.max_level;
    t->ghosts_valid   = false;
    t->batch_open     = true;
    t->uniform        = r.uniform != 0;
    // an interval guarded for two-step passes found the tree non-uniform:
    // it and the rest of the chunk did not run (no state, time or statistic
    // changed); the caller continues with one-step intervals
    // an interval guarded for the fused kernel found leaves that are not
    // aligned 4x4 blocks of one level: the same, with the per-leaf kernels
    const bool retry = r.err == kRetryUniform || r.err == kRetryFused;
    if (r.err == kRetryUniform) t->uniform = false;
    if (r.err == kRetryFused) t->fused_off = true;
    // time of each instance = its batch totals + the open batch
    double   tmax = 0.0;
    uint32_t cmax = 0;
    for (int i = 0; i < K; ++i) {
        double   a, b;
        uint32_t ca, cb;
        std::memcpy(&a, hp + 8 * i, sizeof a);
        std::memcpy(&b, hp + 8 * K + 8 * i, sizeof b);
        std::memcpy(&ca, hp + 16 * K + 4 * i, sizeof ca);
        std::memcpy(&cb, hp + 20 * K + 4 * i, sizeof cb);
        const double ti = b + a;
        if (i == 0 || ti > tmax) tmax = ti;
        cmax = std::max(cmax, ca + cb);
    }
    const long long ran = static_cast<long long>(r.intervals); // intervals committed in this chunk
    tot.done += ran <= nfull ? ran * k : nfull * k + rem;
    // the device totals cover the whole run (carried in or kept on the device)
    tot.sum_dt   = tmax;
    tot.executed = cmax;
    tot.cells += r.cell_updates;
    tot.remeshes += r.remeshes;
    tot.remeshes_changed += r.remeshes_changed;
    tot.intervals += r.intervals;
    tot.graphs += r.intervals;
    tot.leaves_sum += r.leaves_sum;
    if (r.intervals) {
        tot.lmin = std::min<uint64_t>(tot.lmin, static_cast<uint64_t>(r.leaves_min));
        tot.lmax = std::max<uint64_t>(tot.lmax, static_cast<uint64_t>(r.leaves_max));
    }
    if (r.err && !retry) {
        const char* what = r.err == AMR_ERR_CAPACITY     ? "re-mesh would exceed the tree capacity"
                           : r.err == AMR_ERR_UNBALANCED ? "neighbour rebuild found a non-2:1 face"
                           : r.err == AMR_ERR_TIMEOUT    ? "a bulk copy did not complete within the wait limit"
                                                         : "interval graph failed";
        if (r.err == AMR_ERR_TIMEOUT) AMR_CUDA(cudaMemsetAsync(t->ctl, 0, sizeof(RunCtl), s));
        return fail(static_cast<amr_status>(r.err), what);
    }
    return AMR_OK;
}

// Largest CFL step any instance can take (level 0) times the steps left: the
// graph path needs the remaining time to cover it, so no step is clamped.
bool no_clamp(amr_tree* t, const amr_cycle_params* p, bool inst_params, long long steps_left, double sum_dt)
{
    double dmax = 0.0;
    if (inst_params) {
        for (size_t i = 0; i < t->vel_inst_host.size() / 3; ++i)
            dmax = std::max(dmax, p->cfl * raw_dt(t->g, &t->vel_inst_host[3 * i], 0));
    } else {
        dmax = p->cfl * raw_dt(t->g, p->velocity, 0);
    }
    const double need = 2.0 * static_cast<double>(steps_left) * dmax;
    return std::isfinite(need) && p->remaining_time - sum_dt >= need;
}



} // namespace
namespace amr_api {
// Face halo of every field of an arbitrary state buffer of the tree (does
// not touch ghosts_valid); with step_dt, only instances whose step is taken.
// Device-to-device copy of 8-byte words by the SMs (small tables such as the
// velocities a run uses): it never queues behind host transfers on the copy
// engines.
static __global__ void __launch_bounds__(256) k_copy8(uint64_t* __restrict__ dst, const uint64_t* __restrict__ src,
                                                      size_t words)
{
    for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < words;
         i += static_cast<size_t>(gridDim.x) * blockDim.x)
        dst[i] = src[i];
}

amr_status copy_words8(void* dst, const void* src, size_t words, cudaStream_t s)
{
    if (words == 0) return AMR_OK;
    const unsigned grid = static_cast<unsigned>(std::min<size_t>((words + 255) / 256, 8ull * num_sms()));
    k_copy8<<<grid, 256, 0, s>>>(static_cast<uint64_t*>(dst), static_cast<const uint64_t*>(src), words);
    AMR_LAUNCHED("k_copy8");
    return AMR_OK;
}

amr_status halo_buffer(amr_tree* t, void* buf, const double* step_dt)
{
    const long long total = static_cast<long long>(t->size) * t->g.ndir * t->g.h * (t->g.cells / t->g.n);
    const unsigned  grid  = static_cast<unsigned>(std::min<long long>(grid_for(total, 256), 152LL * 64));
    return dispatch_dtype(t->dtype, [&](auto z) -> amr_status {
        using T = decltype(z);
        k_halo<T><<<dim3(grid, t->nvar), 256, 0, t->stream>>>(static_cast<T*>(buf), t->meta[t->tb], total, t->g,
                                                             t->fstride(), t->keys[t->tb], step_dt);
        AMR_LAUNCHED("k_halo");
        return AMR_OK;
    });
}

amr_status launch_halo(amr_tree* t)
{
    const long long total = static_cast<long long>(t->size) * t->g.ndir * t->g.h * (t->g.cells / t->g.n);
    const unsigned  grid  = static_cast<unsigned>(std::min<long long>(grid_for(total, 256), 152LL * 64));
    return dispatch_dtype(t->dtype, [&](auto z) -> amr_status {
        using T = decltype(z);
        k_halo<T><<<dim3(grid, t->nvar), 256, 0, t->stream>>>(static_cast<T*>(t->cur), t->meta[t->tb], total, t->g,
                                                             t->fstride());
        AMR_LAUNCHED("k_halo");
        t->ghosts_valid = true;
        return AMR_OK;
    });
}


} // namespace amr_api

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
    const int K = desc->instances > 1 ? desc->instances : 1;
    if (desc->instances < 0) return fail(AMR_ERR_INVALID, "bad instance count");
    if (K > 1) {
        g.inst_shift = 6 + g.rank * g.depth;
        int bits     = 0;
        while ((1ll << bits) < K) ++bits;
        if (g.inst_shift + bits > 64) return fail(AMR_ERR_INVALID, "too many instances for the tree depth");
    }
    if (static_cast<size_t>(K) > desc->capacity) return fail(AMR_ERR_INVALID, "capacity below the instance count");
    if (desc->fields < 0 || desc->fields > 16) return fail(AMR_ERR_INVALID, "bad field count");
    const int nvar = desc->fields > 1 ? desc->fields : 1;
    if (nvar > 1 && K > 1) return fail(AMR_ERR_INVALID, "forests hold one field");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(AMR_ERR_NO_DEVICE, "no CUDA device");
    amr_tree* t = new amr_tree();
    t->g      = g;
    t->ninst  = K;
    for (int a = 0; a < 3; ++a) t->lengths[a] = a < g.rank ? desc->geom.lengths[a] : 1.0;
    t->cap    = desc->capacity;
    t->dtype  = desc->dtype;
    t->esize  = desc->dtype == AMR_F64 ? 8 : 4;
    t->nvar   = nvar;
    t->stream = static_cast<cudaStream_t>(desc->stream);
    const size_t cap = t->cap, state_bytes = nvar * t->field_bytes(cap);
    cudaError_t  e   = cudaSuccess;
    auto         al  = [&](void** p, size_t bytes) {
        if (e == cudaSuccess) e = cudaMalloc(p, bytes);
    };
    al(&t->sbuf[0], state_bytes);
    al(&t->sbuf[1], state_bytes);
    for (int b = 0; b < 2; ++b) {
        al(reinterpret_cast<void**>(&t->keys[b]), cap * sizeof(uint64_t));
        al(reinterpret_cast<void**>(&t->levels[b]), cap * sizeof(int32_t));
        al(reinterpret_cast<void**>(&t->meta[b]), cap * g.ndir * sizeof(amr_halo_meta));
    }
    al(reinterpret_cast<void**>(&t->prec), cap * sizeof(int4));
    al(reinterpret_cast<void**>(&t->frec), cap * sizeof(int4));
    al(reinterpret_cast<void**>(&t->flags), cap);
    al(reinterpret_cast<void**>(&t->rmark), cap);
    al(reinterpret_cast<void**>(&t->chead), cap);
    al(reinterpret_cast<void**>(&t->cnt), (cap + 1) * sizeof(uint32_t));
    al(reinterpret_cast<void**>(&t->pos), (cap + 1) * sizeof(uint32_t));
    al(reinterpret_cast<void**>(&t->src), cap * sizeof(int32_t));
    al(reinterpret_cast<void**>(&t->skind), cap);
    al(reinterpret_cast<void**>(&t->status), 8 * sizeof(int32_t));
    // coefficient table: up to kMaxBatch steps, at most 16 MiB for a forest
    const size_t nl          = static_cast<size_t>(g.depth + 1);
    const size_t coef_steps  = std::max<size_t>(1, std::min<size_t>(kMaxBatch, (16u << 20) / (K * nl * sizeof(Coef))));
    const size_t ntiles      = (cap + kScanTile - 1) / kScanTile + 1;
    al(reinterpret_cast<void**>(&t->maxlev), K * sizeof(int32_t));
    al(reinterpret_cast<void**>(&t->maxlev_new), K * sizeof(int32_t));
    al(reinterpret_cast<void**>(&t->vel), 3 * K * sizeof(double));
    al(reinterpret_cast<void**>(&t->vel_inst), 3 * K * sizeof(double));
    al(reinterpret_cast<void**>(&t->bounds), 2 * K * sizeof(int32_t));
    al(reinterpret_cast<void**>(&t->target), K * sizeof(int32_t));
    al(reinterpret_cast<void**>(&t->offs), (K + 1) * sizeof(unsigned long long));
    al(reinterpret_cast<void**>(&t->tile_sums), ntiles * sizeof(uint32_t));
    al(reinterpret_cast<void**>(&t->ctl), sizeof(RunCtl));
    al(reinterpret_cast<void**>(&t->dt_acc), K * sizeof(double));
    al(reinterpret_cast<void**>(&t->dt_rem), K * sizeof(double));
    al(reinterpret_cast<void**>(&t->dt_cnt), K * sizeof(uint32_t));
    al(reinterpret_cast<void**>(&t->dt_tot), K * sizeof(double));
    al(reinterpret_cast<void**>(&t->dt_ctot), K * sizeof(uint32_t));
    al(reinterpret_cast<void**>(&t->dt_scratch), 5 * K * sizeof(double));
    al(reinterpret_cast<void**>(&t->step_dt), coef_steps * K * sizeof(double));
    al(reinterpret_cast<void**>(&t->coef), coef_steps * K * nl * sizeof(Coef));
    al(reinterpret_cast<void**>(&t->coef32), coef_steps * K * nl * (t->g.rank == 3 ? sizeof(float4) : sizeof(float2)));
    al(reinterpret_cast<void**>(&t->upcode), K * sizeof(int32_t));
    al(reinterpret_cast<void**>(&t->cstats), sizeof(CycleStats));
    al(reinterpret_cast<void**>(&t->euler_min), 2 * sizeof(unsigned long long));
    al(reinterpret_cast<void**>(&t->euler_dt), sizeof(double));
    al(reinterpret_cast<void**>(&t->euler_ctl), 2 * sizeof(int32_t));
    t->pinned_bytes = std::max<size_t>(1024, 64 + (K + 1) * 32 + sizeof(RunCtl));
    if (e == cudaSuccess) e = cudaMallocHost(&t->pinned, t->pinned_bytes);
    if (e != cudaSuccess) {
        free_tree(t);
        return cuda_fail(e, "amr_tree_create allocation");
    }
    t->coef_steps = coef_steps;
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

amr_status amr_tree_capacity(const amr_tree* t, size_t* out)
{
    if (!t || !out) return fail(AMR_ERR_INVALID, "null argument");
    *out = t->cap;
    return AMR_OK;
}

amr_status amr_tree_reserve(amr_tree* t, size_t cap)
{
    if (!t) return fail(AMR_ERR_INVALID, "null argument");
    if (cap < t->size || cap < static_cast<size_t>(t->ninst) || cap > (1ull << 30))
        return fail(AMR_ERR_INVALID, "capacity does not hold the current leaves");
    if (cap == t->cap) return AMR_OK;
    AMR_CUDA(cudaStreamSynchronize(t->stream));
    const Geo&   g = t->g;
    const size_t P = t->size;
    std::vector<void*> fresh;
    cudaError_t        e  = cudaSuccess;
    auto               al = [&](size_t bytes) -> void* {
        void* q = nullptr;
        if (e == cudaSuccess) e = cudaMalloc(&q, bytes);
        if (q) fresh.push_back(q);
        return q;
    };
    const size_t flat_b = static_cast<size_t>(g.flat) * t->esize;
    void*        sb0    = al(t->nvar * cap * flat_b);
    void*        sb1    = al(t->nvar * cap * flat_b);
    void*        k0     = al(cap * sizeof(uint64_t));
    void*        k1     = al(cap * sizeof(uint64_t));
    void*        l0     = al(cap * sizeof(int32_t));
    void*        l1     = al(cap * sizeof(int32_t));
    void*        m0     = al(cap * g.ndir * sizeof(amr_halo_meta));
    void*        m1     = al(cap * g.ndir * sizeof(amr_halo_meta));
    void*        pr     = al(cap * sizeof(int4)); // pass and face records: rebuilt before every use
    void*        fr     = al(cap * sizeof(int4));
    void*        fl     = al(cap);
    void*        rm     = al(cap);
    void*        ch     = al(cap);
    void*        cn     = al((cap + 1) * sizeof(uint32_t));
    void*        ps     = al((cap + 1) * sizeof(uint32_t));
    void*        sr     = al(cap * sizeof(int32_t));
    void*        sk     = al(cap);
    void*        ts     = al(((cap + kScanTile - 1) / kScanTile + 1) * sizeof(uint32_t));
    if (e != cudaSuccess) {
        for (void* q : fresh) cudaFree(q);
        return cuda_fail(e, "amr_tree_reserve allocation");
    }
    // the current tree and both state buffers (the next buffer may hold the
    // scratch the caller reads through amr_tree_device_state)
    const int cs = t->cur == t->sbuf[0] ? 0 : 1;
    void*     nsb[2] = { sb0, sb1 };
    for (int f = 0; f < t->nvar; ++f) {
        const size_t so = f * t->cap * flat_b, dn = f * cap * flat_b;
        AMR_CUDA(cudaMemcpyAsync(static_cast<char*>(nsb[cs]) + dn, static_cast<const char*>(t->cur) + so, P * flat_b,
                                 cudaMemcpyDeviceToDevice, t->stream));
        AMR_CUDA(cudaMemcpyAsync(static_cast<char*>(nsb[cs ^ 1]) + dn, static_cast<const char*>(t->nxt) + so,
                                 P * flat_b, cudaMemcpyDeviceToDevice, t->stream));
    }
    void* nk[2] = { k0, k1 };
    void* nlv[2] = { l0, l1 };
    void* nm[2] = { m0, m1 };
    AMR_CUDA(cudaMemcpyAsync(nk[t->tb], t->keys[t->tb], P * sizeof(uint64_t), cudaMemcpyDeviceToDevice, t->stream));
    AMR_CUDA(cudaMemcpyAsync(nlv[t->tb], t->levels[t->tb], P * sizeof(int32_t), cudaMemcpyDeviceToDevice, t->stream));
    AMR_CUDA(cudaMemcpyAsync(nm[t->tb], t->meta[t->tb], P * g.ndir * sizeof(amr_halo_meta), cudaMemcpyDeviceToDevice,
                             t->stream));
    AMR_CUDA(cudaMemcpyAsync(fl, t->flags, P, cudaMemcpyDeviceToDevice, t->stream));
    AMR_CUDA(cudaStreamSynchronize(t->stream));
    cudaFree(t->sbuf[0]);
    cudaFree(t->sbuf[1]);
    for (int b = 0; b < 2; ++b) {
        cudaFree(t->keys[b]);
        cudaFree(t->levels[b]);
        cudaFree(t->meta[b]);
    }
    cudaFree(t->prec);
    cudaFree(t->frec);
    t->prec = static_cast<int4*>(pr);
    t->frec = static_cast<int4*>(fr);
    cudaFree(t->flags);
    cudaFree(t->rmark);
    cudaFree(t->chead);
    cudaFree(t->cnt);
    cudaFree(t->pos);
    cudaFree(t->src);
    cudaFree(t->skind);
    cudaFree(t->tile_sums);
    cudaFree(t->prim[0]); // side terms: rebuilt by the next Euler advance
    cudaFree(t->prim[1]);
    t->prim[0] = t->prim[1] = nullptr;
    t->prim_cap = 0;
    cudaFree(t->stage_buf); // SSPRK scratch: allocated again at the next SSPRK advance
    t->stage_buf = nullptr;
    t->stage_cap = 0;
    cudaFree(t->dg_prims); // DG Euler scratch: allocated again at the next DG Euler advance
    t->dg_prims     = nullptr;
    t->dg_prims_cap = 0;
    t->sbuf[0] = sb0;
    t->sbuf[1] = sb1;
    t->cur     = nsb[cs];
    t->nxt     = nsb[cs ^ 1];
    for (int b = 0; b < 2; ++b) {
        t->keys[b]   = static_cast<uint64_t*>(nk[b]);
        t->levels[b] = static_cast<int32_t*>(nlv[b]);
        t->meta[b]   = static_cast<amr_halo_meta*>(nm[b]);
    }
    t->flags     = static_cast<int8_t*>(fl);
    t->rmark     = static_cast<uint8_t*>(rm);
    t->chead     = static_cast<uint8_t*>(ch);
    t->cnt       = static_cast<uint32_t*>(cn);
    t->pos       = static_cast<uint32_t*>(ps);
    t->src       = static_cast<int32_t*>(sr);
    t->skind     = static_cast<int8_t*>(sk);
    t->tile_sums = static_cast<uint32_t*>(ts);
    t->cap       = cap;
    for (auto& ge : t->graphs) { // captured graphs name the old buffers
        if (ge.exec) cudaGraphExecDestroy(ge.exec);
        if (ge.graph) cudaGraphDestroy(ge.graph);
    }
    t->graphs.clear();
    return AMR_OK;
}

amr_status amr_tree_patch_cells(const amr_tree* t, size_t* out)
{
    if (!t || !out) return fail(AMR_ERR_INVALID, "null argument");
    *out = static_cast<size_t>(t->g.flat);
    return AMR_OK;
}

// Device-to-device copy of 16-byte words by the SMs: copies between device
// buffers then never queue behind host transfers on the copy engines.
__global__ void __launch_bounds__(256) k_copy16(uint4* __restrict__ dst, const uint4* __restrict__ src, size_t words)
{
    for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < words;
         i += static_cast<size_t>(gridDim.x) * blockDim.x)
        dst[i] = src[i];
}

// Copies `num` patches of every field between the tree's state (field f at f
// * fstride) and a buffer holding the fields one after another (field f at f *
// num patches).
static amr_status copy_fields(amr_tree* t, void* dst, const void* src, size_t num, cudaMemcpyKind kind, bool to_tree)
{
    const size_t fb = t->field_bytes(num), tstride = t->field_bytes(t->cap);
    for (int f = 0; f < t->nvar; ++f) {
        char*       d = static_cast<char*>(dst) + f * (to_tree ? tstride : fb);
        const char* s = static_cast<const char*>(src) + f * (to_tree ? fb : tstride);
        const bool  words = kind == cudaMemcpyDeviceToDevice && fb % 16 == 0 &&
                           (reinterpret_cast<uintptr_t>(d) | reinterpret_cast<uintptr_t>(s)) % 16 == 0;
        if (words && fb > 0) {
            const size_t   n    = fb / 16;
            const unsigned grid = static_cast<unsigned>(std::min<size_t>((n + 255) / 256, 8ull * num_sms()));
            k_copy16<<<grid, 256, 0, t->stream>>>(reinterpret_cast<uint4*>(d), reinterpret_cast<const uint4*>(s), n);
            AMR_LAUNCHED("k_copy16");
        } else if (fb > 0) {
            AMR_CUDA(cudaMemcpyAsync(d, s, fb, kind, t->stream));
        }
    }
    return AMR_OK;
}

amr_status amr_tree_upload_state(amr_tree* t, const void* host, size_t num)
{
    if (!t || !host) return fail(AMR_ERR_INVALID, "null argument");
    if (num != t->size) return fail(AMR_ERR_INVALID, "patch count does not match tree size");
    if (amr_status s = copy_fields(t, t->cur, host, num, cudaMemcpyHostToDevice, true); s != AMR_OK) return s;
    AMR_CUDA(cudaStreamSynchronize(t->stream));
    t->ghosts_valid = true; // caller's ghosts, as in sync_current_to_device
    return AMR_OK;
}

amr_status amr_tree_download_state(amr_tree* t, void* host, size_t num)
{
    if (!t || !host) return fail(AMR_ERR_INVALID, "null argument");
    if (num != t->size) return fail(AMR_ERR_INVALID, "patch count does not match tree size");
    if (amr_status s = copy_fields(t, host, t->cur, num, cudaMemcpyDeviceToHost, false); s != AMR_OK) return s;
    AMR_CUDA(cudaStreamSynchronize(t->stream));
    return AMR_OK;
}

amr_status amr_tree_load_state_device(amr_tree* t, const void* device_state, size_t num)
{
    if (!t || !device_state) return fail(AMR_ERR_INVALID, "null argument");
    if (num != t->size) return fail(AMR_ERR_INVALID, "patch count does not match tree size");
    if (amr_status s = copy_fields(t, t->cur, device_state, num, cudaMemcpyDeviceToDevice, true); s != AMR_OK)
        return s;
    t->ghosts_valid = true;
    return AMR_OK;
}

amr_status amr_tree_download_state_device(amr_tree* t, void* device_dst, size_t num)
{
    if (!t || !device_dst) return fail(AMR_ERR_INVALID, "null argument");
    if (num != t->size) return fail(AMR_ERR_INVALID, "patch count does not match tree size");
    if (amr_status s = copy_fields(t, device_dst, t->cur, num, cudaMemcpyDeviceToDevice, false); s != AMR_OK)
        return s;
    AMR_CUDA(cudaStreamSynchronize(t->stream));
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
    // ghosts from the buffer when they are current (the caller's or the last
    // exchange's), else evaluated on the fly by the halo rules (same values)
    const bool     fly  = !t->ghosts_valid;
    const int      P    = static_cast<int>(t->size);
    const GradRule rule = make_grad_rule(rthr, cthr);
    const unsigned grid = std::min<unsigned>(grid_for(P, 8), static_cast<unsigned>(num_sms() * 16));
    return dispatch_dtype(t->dtype, [&](auto z) -> amr_status {
        using T = decltype(z);
        const T*       buf = static_cast<const T*>(t->cur);
        const int32_t* bnd = t->bounds_set ? t->bounds : nullptr;
        if (t->g.rank == 2 && t->g.h == 1 && (t->g.n == 16 || t->g.n == 8)) {
            auto sized = [&](auto kern, size_t smem) {
                kern<<<grid, 256, smem, t->stream>>>(buf, t->meta[t->tb], t->keys[t->tb], P, t->g, rule, min_level,
                                                     max_level, bnd, t->flags, t->status + 7);
            };
            if (t->g.n == 16) {
                if (fly) sized(k_flags2d<T, 16, 1, false>, Flags2dShape<T, 16, 1, false>::smem(8));
                else sized(k_flags2d<T, 16, 1, true>, Flags2dShape<T, 16, 1, true>::smem(8));
            } else {
                if (fly) sized(k_flags2d<T, 8, 1, false>, Flags2dShape<T, 8, 1, false>::smem(8));
                else sized(k_flags2d<T, 8, 1, true>, Flags2dShape<T, 8, 1, true>::smem(8));
            }
            AMR_LAUNCHED("k_flags2d");
            return AMR_OK;
        }
        auto launch = [&](auto kern) {
            kern<<<grid, 256, 0, t->stream>>>(buf, t->meta[t->tb], t->levels[t->tb], P, t->g, rule, min_level,
                                              max_level, t->flags, t->keys[t->tb], bnd);
        };
        if (t->g.rank == 2) {
            if (fly) launch(k_flags_grad<T, true, 2>);
            else launch(k_flags_grad<T, false, 2>);
        } else {
            if (fly) launch(k_flags_grad<T, true, 3>);
            else launch(k_flags_grad<T, false, 3>);
        }
        AMR_LAUNCHED("k_flags_grad");
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
                                                min_level, max_level, t->flags,
            t->keys[t->tb], t->bounds_set ? t->bounds : nullptr);
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
    AMR_CUDA(cudaMemsetAsync(t->maxlev, 0, t->ninst * sizeof(int32_t), s));
    k_emit<<<grid_for(P, 256), 256, 0, s>>>(t->keys[tb], t->rmark, t->chead, t->pos, P, g, t->keys[nb], t->levels[nb],
                                            t->src, t->skind, t->maxlev);
    AMR_LAUNCHED("k_emit");
    amr_status st = dispatch_dtype(t->dtype, [&](auto z) -> amr_status {
        using T = decltype(z);
        if constexpr (sizeof(T) == 8) {
            if (t->dg_state) {
                AMR_CUDA(dg_remap(static_cast<const double*>(t->cur), static_cast<double*>(t->nxt), t->src, t->skind,
                                  NP, g, t->fstride(), s));
                AMR_LAUNCHED("k_dg_remap");
                return AMR_OK;
            }
        }
        const long long units = static_cast<long long>(NP) * (g.flat * static_cast<long long>(sizeof(T)) / 16);
        const unsigned  rgrid = static_cast<unsigned>(std::min<long long>((units + 255) / 256, 16LL * num_sms()));
        k_remap<T><<<dim3(std::max(1u, rgrid), t->nvar), 256, 0, s>>>(static_cast<const T*>(t->cur),
                                                                      static_cast<T*>(t->nxt), t->src, t->skind, NP,
                                                                      g, t->fstride());
        AMR_LAUNCHED("k_remap");
        return AMR_OK;
    });
    if (st != AMR_OK) return st;
    k_neighbors<<<grid_for(static_cast<long long>(NP) * g.ndir, 128), 128, 0, s>>>(t->keys[nb], NP, g, t->meta[nb],
                                                                                  t->status);
    AMR_LAUNCHED("k_neighbors");
    AMR_CUDA(cudaMemsetAsync(t->status + 5, 0, sizeof(int32_t), s));
    k_any_not_same<<<std::min<unsigned>(grid_for(static_cast<long long>(NP) * g.ndir, 256), 1024u), 256, 0, s>>>(
        t->meta[nb], static_cast<long long>(NP) * g.ndir, t->status + 5);
    AMR_LAUNCHED("k_any_not_same");
    AMR_CUDA(cudaMemcpyAsync(hs + 8, t->status + 5, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    AMR_CUDA(cudaMemcpyAsync(hs + 4, t->status, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    AMR_CUDA(cudaMemcpyAsync(hs + 5, t->maxlev, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    AMR_CUDA(cudaStreamSynchronize(s));
    const int nerr = hs[4];
    ++t->topo;
    std::swap(t->cur, t->nxt);
    t->tb             = nb;
    t->size           = static_cast<size_t>(NP);
    t->max_level_host = hs[5];
    t->ghosts_valid   = false;
    t->uniform        = hs[8] == 0;
    if (changed) *changed = 1;
    if (t->ninst > 1) {
        int m = 0;
        amr_status ms = forest_max_level(t, &m);
        if (ms != AMR_OK) return ms;
        t->max_level_host = m;
    }
    hs[4] = nerr;
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

} // extern "C"

amr_status amr_api::advance_impl(amr_tree* t, size_t steps, const double* velocity3, double cfl, double remaining,
                        int first_mode)
{
    if (!t) return fail(AMR_ERR_INVALID, "null argument");
    if (t->nvar != 1) return fail(AMR_ERR_INVALID, "the advection update takes a one-field tree");
    if (!velocity3 && !t->vel_inst_set) return fail(AMR_ERR_INVALID, "no velocity given and none set per instance");
    cudaStream_t s = t->stream;
    const int    K = t->ninst;
    int          up[3] = { 0, 0, 0 };
    if (velocity3) {
        std::vector<double> v(3 * static_cast<size_t>(K));
        for (int i = 0; i < K; ++i)
            for (int a = 0; a < 3; ++a) v[3 * i + a] = velocity3[a];
        AMR_CUDA(cudaMemcpyAsync(t->vel, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice, s));
        for (int a = 0; a < t->g.rank; ++a) up[a] = velocity3[a] > 0.0 ? -1 : (velocity3[a] < 0.0 ? 1 : 0);
        t->vel_per_leaf = false;
    } else {
        if (amr_status cs = copy_words8(t->vel, t->vel_inst, 3 * static_cast<size_t>(K), s); cs != AMR_OK) return cs;
        t->vel_per_leaf = true;
    }
    const double*  vleaf = t->vel_per_leaf ? t->vel : nullptr;
    const int32_t* uleaf = t->vel_per_leaf ? t->upcode : nullptr;
    const int P     = static_cast<int>(t->size);
    const int ppb   = std::max(1, 256 / t->g.cells);
    const unsigned grid = grid_for(P, ppb);
    const int nl    = t->g.depth + 1;
    bool      first = true;
    size_t    done  = 0;
    StepCfg   cfg, cfg_pair;
    lookup_tuned(t, uleaf != nullptr, false, cfg);
    if (!lookup_tuned(t, uleaf != nullptr, true, cfg_pair)) cfg_pair = cfg;
    t->last_cfg = t->uniform ? cfg_pair : cfg;
    const bool shape2d = t->g.rank == 2 && t->g.h == 1 && (t->g.n == 16 || t->g.n == 8);
    while (done < steps || (first && steps == 0)) {
        const int chunk = static_cast<int>(std::min(t->coef_steps, steps - done));
        k_batch_begin<<<K, 256, 0, s>>>(t->maxlev, t->g, t->vel, cfl, chunk, first ? first_mode : BATCH_CONTINUE,
                                        remaining, t->dts(), t->step_dt, t->coef, t->coef32, t->upcode);
        AMR_LAUNCHED("k_batch_begin");
        if (first && shape2d && t->uniform && steps > 1) { // records of the multi-step passes (after the
            const amr_status rs = build_pass_records(t, uleaf, up, s); // upwind codes of this advance)
            if (rs != AMR_OK) return rs;
        }
        first = false;
        const int  deep    = t->dtype == AMR_F32 ? kPassSteps<float> : kPassSteps<double>;
        std::vector<int> plan;
        if (shape2d && t->uniform) pass_plan(chunk, deep, plan); // several steps per pass where every relation is same-level
        else plan.assign(static_cast<size_t>(chunk), 1);
        size_t pi = 0;
        for (int k = 0; k < chunk; ++pi) {
            const int  D    = plan[pi];
            const bool pair = D > 1;
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
                t->event_cells[t->events_used] = static_cast<uint64_t>(P) * t->g.cells * D;
                ++t->events_used;
                AMR_CUDA(cudaEventRecord(ev->first, s));
            }
            amr_status st = dispatch_dtype(t->dtype, [&](auto z) -> amr_status {
                using T        = decltype(z);
                const Coef*   cf  = t->coef + static_cast<size_t>(k) * K * nl;
                const float2* cf2 = t->coef32 + static_cast<size_t>(k) * K * nl;
                const T*      in  = static_cast<const T*>(t->cur);
                T*            out = static_cast<T*>(t->nxt);
                if (pair) {
                    const size_t cst  = static_cast<size_t>(K) * nl;
                    auto         pass = [&]<int N>(const StepCfg& c) -> amr_status {
                        return with_depth<T>(D, [&]<int DD>() -> amr_status {
                            return launch_step2d_pass<T, N, 1, DD>(in, out, t->prec, P, nl, cf, cf2, cst,
                                                                   t->status + 7, c, s);
                        });
                    };
                    return t->g.n == 16 ? pass.template operator()<16>(cfg_pair) : pass.template operator()<8>(StepCfg{});
                }
                if (t->g.rank == 2 && t->g.n == 16 && t->g.h == 1)
                    return launch_step2d<T, 16, 1>(in, out, t->meta[t->tb], P, t->g, cf, cf2, up, t->status + 7,
                                                   t->keys[t->tb], uleaf, cfg, s);
                if (t->g.rank == 2 && t->g.n == 8 && t->g.h == 1)
                    return launch_step2d<T, 8, 1>(in, out, t->meta[t->tb], P, t->g, cf, cf2, up, t->status + 7,
                                                  t->keys[t->tb], uleaf, StepCfg{}, s);
                if (step3d_shape(t->g, in, out)) {
                    const float4* cf4 = reinterpret_cast<const float4*>(t->coef32) + static_cast<size_t>(k) * K * nl;
                    return t->g.n == 8 ? launch_step3d<T, 8>(in, out, t->levels[t->tb], t->meta[t->tb], P, t->g, cf,
                                                             cf4, up, t->keys[t->tb], uleaf, t->status + 7, s)
                                       : launch_step3d<T, 4>(in, out, t->levels[t->tb], t->meta[t->tb], P, t->g, cf,
                                                             cf4, up, t->keys[t->tb], uleaf, t->status + 7, s);
                }
                k_step<T, true><<<grid, 256, 0, s>>>(in, out, t->levels[t->tb], t->meta[t->tb], P, t->g, cf, up[0],
                                                     up[1], up[2], ppb, nullptr, 0.0, 0.0, 0.0, t->keys[t->tb],
                                                     vleaf);
                AMR_LAUNCHED("k_step");
                return AMR_OK;
            });
            if (st != AMR_OK) return st;
            if (ev) AMR_CUDA(cudaEventRecord(ev->second, s));
            std::swap(t->cur, t->nxt);
            k += D;
        }
        done += chunk;
        if (steps == 0) break;
    }
    t->ghosts_valid = false;
    t->batch_open   = true;
    return AMR_OK;
}

extern "C" {

amr_status amr_tree_advance(amr_tree* t, size_t steps, const double* velocity3, double cfl, double remaining)
{
    return advance_impl(t, steps, velocity3, cfl, remaining, BATCH_RESET);
}

amr_status amr_tree_finish_advance(amr_tree* t, double* sum_dt, size_t* executed)
{
    if (!t) return fail(AMR_ERR_INVALID, "null argument");
    char*     hp = static_cast<char*>(t->pinned);
    const int K  = t->ninst;
    AMR_CUDA(cudaMemcpyAsync(hp + 48, t->status + 7, sizeof(int32_t), cudaMemcpyDeviceToHost, t->stream));
    AMR_CUDA(cudaMemcpyAsync(hp + 64, t->dt_acc, K * sizeof(double), cudaMemcpyDeviceToHost, t->stream));
    AMR_CUDA(cudaMemcpyAsync(hp + 64 + 8 * K, t->dt_cnt, K * sizeof(uint32_t), cudaMemcpyDeviceToHost, t->stream));
    AMR_CUDA(cudaStreamSynchronize(t->stream));
    int32_t wait_err = 0;
    std::memcpy(&wait_err, hp + 48, sizeof wait_err);
    if (wait_err != 0) {
        AMR_CUDA(cudaMemsetAsync(t->status + 7, 0, sizeof(int32_t), t->stream));
        if (wait_err != AMR_ERR_TIMEOUT)
            return fail(static_cast<amr_status>(wait_err), "a two-step pass met a neighbour of another level");
        return fail(AMR_ERR_TIMEOUT, "a bulk copy did not complete within the wait limit");
    }
    // one tree: its time; a forest: the instance furthest ahead
    double   acc = 0.0;
    uint32_t cnt = 0;
    for (int i = 0; i < K; ++i) {
        double   a;
        uint32_t c;
        std::memcpy(&a, hp + 64 + 8 * i, sizeof a);
        std::memcpy(&c, hp + 64 + 8 * K + 4 * i, sizeof c);
        if (i == 0 || a > acc) acc = a;
        cnt = std::max(cnt, c);
    }
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
    if (t) {
        t->fused_off  = false; // re-evaluated by every run
        t->pair_chunk = 1;
    }
    if (!t || !p) return fail(AMR_ERR_INVALID, "null argument");
    if (p->criterion < 0 || p->criterion > 2) return fail(AMR_ERR_INVALID, "unknown criterion");
    if (t->nvar != 1) return fail(AMR_ERR_INVALID, "the advection run takes a one-field tree");
    const bool inst_params = (p->options & AMR_RUN_INSTANCE_PARAMS) != 0;
    if (inst_params && !t->vel_inst_set) return fail(AMR_ERR_INVALID, "no per-instance velocities set");
    if (p->criterion != 0) ++t->topo;
    const Geo&      g     = t->g;
    const long long total = static_cast<long long>(p->steps);
    RunTotals       tot;
    int up[3] = { 0, 0, 0 };
    for (int a = 0; a < g.rank; ++a) up[a] = p->velocity[a] > 0.0 ? -1 : (p->velocity[a] < 0.0 ? 1 : 0);
    const size_t smem = static_cast<size_t>(p->remesh_interval) * (g.depth + 1) * sizeof(Coef) +
                        static_cast<size_t>(p->remesh_interval) * sizeof(double);
    while (tot.done < total) {
        const bool small = t->ninst == 1 && !(p->options & AMR_RUN_PER_LAUNCH) &&
                           t->size <= static_cast<size_t>(kPersistentLeaves) && p->remesh_interval >= 1 &&
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
            A.remaining   = p->remaining_time - tot.sum_dt;
            A.steps_total = total - tot.done;
            A.interval    = static_cast<int>(p->remesh_interval);
            A.crit        = p->criterion;
            A.rthr        = p->refine_threshold;
            A.cthr        = p->coarsen_threshold;
            A.rule        = make_grad_rule(p->refine_threshold, p->coarsen_threshold);
            A.min_level   = p->min_level;
            A.max_level   = p->max_level;
            if (t->bounds_set) { // one tree: its own (min, max) pair
                A.min_level = t->bounds_host[0];
                A.max_level = t->bounds_host[1];
            }
            if (inst_params) {
                for (int a = 0; a < 3; ++a) {
                    A.vel[a] = t->vel_inst_host[a];
                    A.up[a]  = a < g.rank ? (A.vel[a] > 0.0 ? -1 : (A.vel[a] < 0.0 ? 1 : 0)) : 0;
                }
            }
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
            if (amr_status us = refresh_uniform(t); us != AMR_OK) return us;
            tot.done += static_cast<long long>(cs.executed);
            tot.sum_dt += cs.sum_dt;
            tot.executed += cs.executed;
            tot.cells += cs.cell_updates;
            tot.remeshes += cs.remeshes;
            tot.remeshes_changed += cs.remeshes_changed;
            tot.intervals += cs.intervals;
            tot.persistent += cs.intervals;
            tot.leaves_sum += cs.leaves_sum;
            if (cs.intervals) {
                tot.lmin = std::min<uint64_t>(tot.lmin, static_cast<uint64_t>(cs.leaves_min));
                tot.lmax = std::max<uint64_t>(tot.lmax, static_cast<uint64_t>(cs.leaves_max));
            }
            if (cs.error) return fail(static_cast<amr_status>(cs.error), "persistent re-mesh failed");
            if (!cs.stopped) break;
            continue;
        }
        const bool graph = !(p->options & AMR_RUN_NO_GRAPH) && p->remesh_interval >= 1 &&
                           p->remesh_interval <= t->coef_steps &&
                           no_clamp(t, p, inst_params, total - tot.done, tot.sum_dt);
        if (graph) {
            // a single tree that shrinks below the cluster kernel's limit goes
            // back to it after a short chunk
            const long long chunk = (t->ninst == 1 && !(p->options & AMR_RUN_PER_LAUNCH)) ? 16 : LLONG_MAX;
            amr_status      st    = run_graph_chunk(t, p, inst_params, chunk, tot);
            if (st != AMR_OK) return st;
            continue;
        }
        // one interval with host-driven launches
        const long long k = (p->remesh_interval > 0 && static_cast<long long>(p->remesh_interval) < total - tot.done)
                                ? static_cast<long long>(p->remesh_interval)
                                : total - tot.done;
        const size_t P = t->size;
        // the first batch of the run starts the per-instance totals; later
        // ones fold into them (one tree: remaining time from the host sum, as
        // the reference's loop passes it; a forest: each instance's own)
        const int  mode = tot.intervals == 0 ? BATCH_RESET : (t->ninst == 1 ? BATCH_NEXT_REM : BATCH_NEXT);
        amr_status st   = advance_impl(t, static_cast<size_t>(k), inst_params ? nullptr : p->velocity, p->cfl,
                                       p->remaining_time - tot.sum_dt, mode);
        if (st != AMR_OK) return st;
        double acc = 0.0;
        size_t ex  = 0;
        st         = amr_tree_finish_advance(t, &acc, &ex);
        if (st != AMR_OK) return st;
        tot.done += static_cast<long long>(ex);
        tot.sum_dt += acc;
        tot.executed += ex;
        tot.cells += static_cast<uint64_t>(ex) * P * static_cast<uint64_t>(g.cells);
        tot.leaves_sum += P;
        tot.lmin = std::min<uint64_t>(tot.lmin, P);
        tot.lmax = std::max<uint64_t>(tot.lmax, P);
        ++tot.intervals;
        if (p->criterion != 0) {
            st = p->criterion == 1 ? amr_tree_flags_gradient(t, p->refine_threshold, p->coarsen_threshold,
                                                             p->min_level, p->max_level)
                                   : amr_tree_flags_max(t, p->refine_threshold, p->coarsen_threshold, p->min_level,
                                                        p->max_level);
            if (st != AMR_OK) return st;
            int changed = 0;
            st          = amr_tree_remesh(t, &changed);
            if (st != AMR_OK) return st;
            ++tot.remeshes;
            if (changed) ++tot.remeshes_changed;
        }
        if (ex == 0) break;
    }
    if (out) {
        out->executed_steps       = tot.executed;
        out->sum_dt               = tot.sum_dt;
        out->cell_updates         = tot.cells;
        out->remeshes             = tot.remeshes;
        out->remeshes_changed     = tot.remeshes_changed;
        out->intervals            = tot.intervals;
        out->leaves_min           = tot.intervals ? tot.lmin : t->size;
        out->leaves_max           = tot.intervals ? tot.lmax : t->size;
        out->leaves_mean          = tot.intervals ? static_cast<double>(tot.leaves_sum) / static_cast<double>(tot.intervals)
                                                  : 0.0;
        out->persistent_intervals = tot.persistent;
        out->graph_intervals      = tot.graphs;
    }
    return AMR_OK;
}

amr_status amr_tree_set_instance_params(amr_tree* t, const double* velocity, const int32_t* level_bounds,
                                        size_t instances)
{
    if (!t) return fail(AMR_ERR_INVALID, "null argument");
    if (instances != static_cast<size_t>(t->ninst)) return fail(AMR_ERR_INVALID, "instance count mismatch");
    if (velocity) {
        t->vel_inst_host.assign(velocity, velocity + 3 * instances);
        for (size_t i = 0; i < instances; ++i)
            for (int a = t->g.rank; a < 3; ++a) t->vel_inst_host[3 * i + a] = 0.0;
        AMR_CUDA(cudaMemcpyAsync(t->vel_inst, t->vel_inst_host.data(), 3 * instances * sizeof(double),
                                 cudaMemcpyHostToDevice, t->stream));
        t->vel_inst_set = true;
    }
    if (level_bounds) {
        for (size_t i = 0; i < instances; ++i)
            if (level_bounds[2 * i] < 0 || level_bounds[2 * i + 1] < level_bounds[2 * i])
                return fail(AMR_ERR_INVALID, "bad level bounds");
        t->bounds_host.assign(level_bounds, level_bounds + 2 * instances);
        AMR_CUDA(cudaMemcpyAsync(t->bounds, t->bounds_host.data(), 2 * instances * sizeof(int32_t),
                                 cudaMemcpyHostToDevice, t->stream));
        t->bounds_set = true;
    }
    AMR_CUDA(cudaStreamSynchronize(t->stream));
    return AMR_OK;
}

amr_status amr_tree_refine_to_levels(amr_tree* t, const int32_t* target_levels, size_t instances)
{
    if (!t || !target_levels) return fail(AMR_ERR_INVALID, "null argument");
    if (instances != static_cast<size_t>(t->ninst)) return fail(AMR_ERR_INVALID, "instance count mismatch");
    int top = 0;
    for (size_t i = 0; i < instances; ++i) {
        if (target_levels[i] < 0 || target_levels[i] > t->g.depth) return fail(AMR_ERR_INVALID, "bad target level");
        top = std::max(top, static_cast<int>(target_levels[i]));
    }
    AMR_CUDA(cudaMemcpyAsync(t->target, target_levels, instances * sizeof(int32_t), cudaMemcpyHostToDevice, t->stream));
    for (int l = 0; l < top; ++l) {
        const int P = static_cast<int>(t->size);
        k_flags_to_level<<<grid_for(P, 256), 256, 0, t->stream>>>(t->keys[t->tb], P, t->g, t->target, t->flags);
        AMR_LAUNCHED("k_flags_to_level");
        int        changed = 0;
        amr_status st      = amr_tree_remesh(t, &changed);
        if (st != AMR_OK) return st;
        if (!changed) break;
    }
    return AMR_OK;
}

amr_status amr_tree_instance_offsets(amr_tree* t, uint64_t* offsets, size_t instances_plus_one)
{
    if (!t || !offsets) return fail(AMR_ERR_INVALID, "null argument");
    const int K = t->ninst;
    if (instances_plus_one != static_cast<size_t>(K) + 1) return fail(AMR_ERR_INVALID, "instance count mismatch");
    k_instance_offsets<<<grid_for(K + 1, 256), 256, 0, t->stream>>>(t->keys[t->tb], static_cast<int>(t->size), t->g, K,
                                                                     t->offs);
    AMR_LAUNCHED("k_instance_offsets");
    AMR_CUDA(cudaMemcpyAsync(offsets, t->offs, (K + 1) * sizeof(uint64_t), cudaMemcpyDeviceToHost, t->stream));
    AMR_CUDA(cudaStreamSynchronize(t->stream));
    return AMR_OK;
}

amr_status amr_tree_instance_time(amr_tree* t, double* sum_dt, uint32_t* executed_steps, size_t instances)
{
    if (!t) return fail(AMR_ERR_INVALID, "null argument");
    if (instances != static_cast<size_t>(t->ninst)) return fail(AMR_ERR_INVALID, "instance count mismatch");
    std::vector<double>   acc(instances), tot(instances);
    std::vector<uint32_t> cnt(instances), ctot(instances);
    AMR_CUDA(cudaMemcpyAsync(acc.data(), t->dt_acc, instances * sizeof(double), cudaMemcpyDeviceToHost, t->stream));
    AMR_CUDA(cudaMemcpyAsync(tot.data(), t->dt_tot, instances * sizeof(double), cudaMemcpyDeviceToHost, t->stream));
    AMR_CUDA(cudaMemcpyAsync(cnt.data(), t->dt_cnt, instances * sizeof(uint32_t), cudaMemcpyDeviceToHost, t->stream));
    AMR_CUDA(cudaMemcpyAsync(ctot.data(), t->dt_ctot, instances * sizeof(uint32_t), cudaMemcpyDeviceToHost, t->stream));
    AMR_CUDA(cudaStreamSynchronize(t->stream));
    for (size_t i = 0; i < instances; ++i) {
        if (sum_dt) sum_dt[i] = t->batch_open ? tot[i] + acc[i] : 0.0;
        if (executed_steps) executed_steps[i] = t->batch_open ? ctot[i] + cnt[i] : 0u;
    }
    return AMR_OK;
}

} // extern "C"

extern "C" {

amr_status amr_tree_step_config(const amr_tree* t, int32_t* warps, int32_t* stages, int32_t* blocks)
{
    if (!t) return fail(AMR_ERR_INVALID, "null argument");
    if (warps) *warps = t->last_cfg.W;
    if (stages) *stages = t->last_cfg.S;
    if (blocks) *blocks = t->last_cfg.grid;
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
