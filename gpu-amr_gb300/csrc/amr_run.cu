// The benchmark loop of the C ABI (amr_tree_run): whole runs of small trees
// in the persistent cluster kernel, otherwise re-mesh intervals as CUDA graph
// replays of a device-resident interval (or host-driven launches where the
// remaining time clamps a step).

#include "amr_interval.cuh"
#include "amr_launch.cuh"

namespace {

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

extern "C" {

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

} // extern "C"
