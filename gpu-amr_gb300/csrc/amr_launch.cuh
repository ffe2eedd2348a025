// Launch helpers shared by the tree's entry points (amr_tree.cu) and the
// run driver (amr_run.cu): launch shapes and attributes of the 2D and 3D
// update kernels, the multi-step pass plan, the pass records and the
// autotuner (its cache is one per process).
#pragma once

#include "amr_api.cuh"

// The autotuner's cache is one per process (inline variables); the launch
// helpers are internal to each translation unit: a kernel template that two
// translation units instantiate is registered once per unit, so the shared-
// memory attributes each sets (and the flags that record them) must be per
// unit too.
namespace amr_api {
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
inline std::mutex                 g_tune_mu;
inline std::map<TuneKey, StepCfg> g_tuned;
inline std::atomic<int>           g_tune_mode{ 1 }; // 0 off (defaults), 1 on

inline TuneKey tune_key(const amr_tree* t, bool per_leaf, bool pair)
{
    int dev = 0;
    cudaGetDevice(&dev);
    int oct = 0;
    while ((static_cast<size_t>(1) << oct) < t->size) ++oct;
    return TuneKey{ dev, static_cast<int>(t->esize), t->g.n, t->g.h, oct, per_leaf ? 1 : 0, pair ? 1 : 0 };
}

inline bool lookup_tuned(const amr_tree* t, bool per_leaf, bool pair, StepCfg& cfg)
{
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto                        it = g_tuned.find(tune_key(t, per_leaf, pair));
    if (it == g_tuned.end()) return false;
    cfg = it->second;
    return true;
}

// pair: time the multi-step pass instead (same-level trees); every step of
// it reads the prologue's coefficient row (stride 0).

// Defined in amr_tree.cu.
GradRule   make_grad_rule(double rthr, double cthr);
amr_status refresh_uniform(amr_tree* t);

} // namespace amr_api

namespace {


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


} // namespace
