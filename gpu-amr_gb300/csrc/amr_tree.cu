// C-ABI of the GB300 AMR path: the device-resident tree (creation, state,
// halo exchange, flags, re-mesh, advance) and the forest entry points; the
// run driver (amr_tree_run) is in amr_run.cu.  Host code only orchestrates
// launches; every per-leaf or per-cell loop runs in a kernel.

#include "amr_launch.cuh"

namespace amr_api {
thread_local std::string g_last_error;
std::atomic<uint64_t>    g_launches{ 0 };
} // namespace amr_api

namespace {

constexpr size_t kMaxBatch = 1024;

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
} // namespace

namespace amr_api {
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

// Face halo of every field of an arbitrary state buffer of the tree (does
// not touch ghosts_valid); with step_dt, only instances whose step is taken.
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
