// C-ABI of the discrete adjoint on a frozen mesh, and the bounded-wait self-test.

#include "amr_api.cuh"

namespace {
// The bounded-wait self-test: an mbarrier expects 16 bytes nobody sends.
__global__ void k_selftest_wait(int32_t* status, int polls)
{
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        mbar_init_fence();
        mbar_expect_tx(&bar, 16);
        status[0] = mbar_wait_bounded(&bar, 0, polls) ? AMR_OK : AMR_ERR_TIMEOUT;
    }
}

__global__ void k_selftest_touch(int32_t* status) { status[1] = 1; }
} // namespace

struct amr_adjoint {
    amr_tree*          t = nullptr;
    size_t             steps = 0, every = 1, nseg = 0;
    double             vel3[3] = { 0, 0, 0 };
    bool               per_instance = false;
    double             cfl = 0.0, remaining = 0.0;
    uint64_t           topo = 0;
    std::vector<void*> ckpt;    // nseg + 1 states
    double*            dts = nullptr; // steps * ninst step sizes
    double*            vel = nullptr; // velocities of the run (3 per instance)
    int32_t*           upcode = nullptr; // their packed upwind offsets (per instance)
    void*              lam[2]{};
    bool               forward_done = false;
};

namespace {
void free_adjoint(amr_adjoint* a)
{
    if (!a) return;
    for (void* c : a->ckpt) cudaFree(c);
    cudaFree(a->dts);
    cudaFree(a->vel);
    cudaFree(a->upcode);
    cudaFree(a->lam[0]);
    cudaFree(a->lam[1]);
    delete a;
}
} // namespace

extern "C" {

amr_status amr_adjoint_create(amr_tree* t, size_t steps, const double* velocity3, double cfl, double remaining,
                              size_t every, amr_adjoint** out)
{
    if (!t || !out) return fail(AMR_ERR_INVALID, "null argument");
    *out = nullptr;
    if (t->nvar != 1) return fail(AMR_ERR_INVALID, "the adjoint takes a one-field tree");
    if (every < 1 || every > t->coef_steps) return fail(AMR_ERR_INVALID, "checkpoint interval out of range");
    if (!velocity3 && !t->vel_inst_set) return fail(AMR_ERR_INVALID, "no velocity given and none set per instance");
    amr_adjoint* a = new amr_adjoint();
    a->t           = t;
    a->steps       = steps;
    a->every       = every;
    a->nseg        = (steps + every - 1) / every;
    a->cfl         = cfl;
    a->remaining   = remaining;
    a->topo        = t->topo;
    a->per_instance = velocity3 == nullptr;
    if (velocity3)
        for (int k = 0; k < 3; ++k) a->vel3[k] = velocity3[k];
    const size_t bytes = t->cap * t->g.flat * t->esize; // room for the tree's capacity
    const size_t K     = static_cast<size_t>(t->ninst);
    cudaError_t  e     = cudaSuccess;
    a->ckpt.assign(a->nseg + 1, nullptr);
    for (auto& c : a->ckpt)
        if (e == cudaSuccess) e = cudaMalloc(&c, t->size * t->g.flat * t->esize);
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&a->dts), std::max<size_t>(1, steps) * K * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&a->vel), 3 * K * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&a->upcode), K * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc(&a->lam[0], bytes);
    if (e == cudaSuccess) e = cudaMalloc(&a->lam[1], bytes);
    if (e != cudaSuccess) {
        free_adjoint(a);
        return cuda_fail(e, "amr_adjoint_create allocation");
    }
    *out = a;
    return AMR_OK;
}

amr_status amr_adjoint_destroy(amr_adjoint* a)
{
    if (!a) return AMR_OK;
    cudaStreamSynchronize(a->t->stream);
    free_adjoint(a);
    return AMR_OK;
}

amr_status amr_adjoint_checkpoint_count(const amr_adjoint* a, size_t* count)
{
    if (!a || !count) return fail(AMR_ERR_INVALID, "null argument");
    *count = a->ckpt.size();
    return AMR_OK;
}

amr_status amr_adjoint_forward(amr_adjoint* a)
{
    if (!a) return fail(AMR_ERR_INVALID, "null argument");
    amr_tree* t = a->t;
    if (t->topo != a->topo) return fail(AMR_ERR_INVALID, "the tree was re-meshed after the adjoint was created");
    cudaStream_t s     = t->stream;
    const size_t bytes = t->size * t->g.flat * t->esize;
    const size_t K     = static_cast<size_t>(t->ninst);
    AMR_CUDA(cudaMemcpyAsync(a->ckpt[0], t->cur, bytes, cudaMemcpyDeviceToDevice, s));
    for (size_t m = 0; m < a->nseg; ++m) {
        const size_t k  = std::min(a->every, a->steps - m * a->every);
        amr_status   st = advance_impl(t, k, a->per_instance ? nullptr : a->vel3, a->cfl, a->remaining,
                                       m == 0 ? BATCH_RESET : BATCH_CONTINUE);
        if (st != AMR_OK) return st;
        if (m == 0) { // velocities in use (per instance) and their upwind codes
            AMR_CUDA(cudaMemcpyAsync(a->vel, t->vel, 3 * K * sizeof(double), cudaMemcpyDeviceToDevice, s));
            AMR_CUDA(cudaMemcpyAsync(a->upcode, t->upcode, K * sizeof(int32_t), cudaMemcpyDeviceToDevice, s));
        }
        AMR_CUDA(cudaMemcpyAsync(a->dts + m * a->every * K, t->step_dt, k * K * sizeof(double),
                                 cudaMemcpyDeviceToDevice, s));
        AMR_CUDA(cudaMemcpyAsync(a->ckpt[m + 1], t->cur, bytes, cudaMemcpyDeviceToDevice, s));
    }
    if (a->nseg == 0 && a->per_instance)
        AMR_CUDA(cudaMemcpyAsync(a->vel, t->vel_inst, 3 * K * sizeof(double), cudaMemcpyDeviceToDevice, s));
    int32_t wait_err = 0;
    AMR_CUDA(cudaMemcpyAsync(&wait_err, t->status + 7, sizeof wait_err, cudaMemcpyDeviceToHost, s));
    AMR_CUDA(cudaStreamSynchronize(s));
    if (wait_err) {
        AMR_CUDA(cudaMemsetAsync(t->status + 7, 0, sizeof(int32_t), s));
        return fail(AMR_ERR_TIMEOUT, "a bulk copy did not complete within the wait limit");
    }
    a->forward_done = true;
    return AMR_OK;
}

} // extern "C"

namespace {
// The reverse sweep on the adjoint's own buffers: lambda_T in lam[0] on
// entry; returns the index of the buffer holding lambda_0.
amr_status adjoint_sweep(amr_adjoint* a, int* result)
{
    amr_tree*       t     = a->t;
    cudaStream_t    s     = t->stream;
    const Geo&      g     = t->g;
    const int       P     = static_cast<int>(t->size);
    const int       K     = t->ninst;
    const int       nl    = g.depth + 1;
    const size_t    bytes = static_cast<size_t>(P) * g.flat * t->esize;
    const long long total = static_cast<long long>(P) * g.flat;
    int up[3] = { 0, 0, 0 };
    if (!a->per_instance)
        for (int k = 0; k < g.rank; ++k) up[k] = a->vel3[k] > 0.0 ? -1 : (a->vel3[k] < 0.0 ? 1 : 0);
    const int32_t* uleaf = a->per_instance ? a->upcode : nullptr;
    const int      ppb   = std::max(1, 256 / g.cells);
    const unsigned grid  = grid_for(P, ppb);
    int            cur   = 0;
    amr_status     st    = dispatch_dtype(t->dtype, [&](auto z) -> amr_status {
        using T = decltype(z);
        AMR_CUDA(cudaMemsetAsync(a->lam[1], 0, bytes, s));
        const unsigned zg = static_cast<unsigned>(std::min<long long>(grid_for(total, 256), 152LL * 32));
        k_zero_ghosts<T><<<zg, 256, 0, s>>>(static_cast<T*>(a->lam[0]), total, g);
        AMR_LAUNCHED("k_zero_ghosts");
        for (size_t m = a->nseg; m-- > 0;) {
            const int k = static_cast<int>(std::min(a->every, a->steps - m * a->every));
            k_coef_from_dt<<<grid_for(static_cast<long long>(k) * K * nl, 256), 256, 0, s>>>(
                a->dts + m * a->every * K, g, a->vel, k, K, t->coef, t->coef32);
            AMR_LAUNCHED("k_coef_from_dt");
            for (int j = k - 1; j >= 0; --j) {
                const size_t  row  = static_cast<size_t>(j) * K * nl;
                const Coef*   cf   = t->coef + row;
                const float2* cf32 = g.rank == 3
                                         ? reinterpret_cast<const float2*>(reinterpret_cast<const float4*>(t->coef32) + row)
                                         : t->coef32 + row;
                k_adjoint<T><<<grid, 256, 0, s>>>(static_cast<const T*>(a->lam[cur]), static_cast<T*>(a->lam[cur ^ 1]),
                                                  t->meta[t->tb], t->keys[t->tb], P, g, cf, cf32, up[0], up[1], up[2],
                                                  uleaf, ppb);
                AMR_LAUNCHED("k_adjoint");
                cur ^= 1;
            }
        }
        return AMR_OK;
    });
    *result = cur;
    return st;
}

amr_status adjoint_ready(amr_adjoint* a)
{
    if (a->t->topo != a->topo) return fail(AMR_ERR_INVALID, "the tree was re-meshed after the adjoint was created");
    if (!a->forward_done) return fail(AMR_ERR_INVALID, "amr_adjoint_forward has not run");
    return AMR_OK;
}
} // namespace

extern "C" {

amr_status amr_adjoint_backward(amr_adjoint* a, const void* lam_T, void* lam_0)
{
    if (!a || !lam_T || !lam_0) return fail(AMR_ERR_INVALID, "null argument");
    amr_status st = adjoint_ready(a);
    if (st != AMR_OK) return st;
    amr_tree*    t     = a->t;
    const size_t bytes = t->size * t->g.flat * t->esize;
    AMR_CUDA(cudaMemcpyAsync(a->lam[0], lam_T, bytes, cudaMemcpyDeviceToDevice, t->stream));
    int res = 0;
    st      = adjoint_sweep(a, &res);
    if (st != AMR_OK) return st;
    AMR_CUDA(cudaMemcpyAsync(lam_0, a->lam[res], bytes, cudaMemcpyDeviceToDevice, t->stream));
    AMR_CUDA(cudaStreamSynchronize(t->stream));
    return AMR_OK;
}

amr_status amr_adjoint_backward_host(amr_adjoint* a, const void* lam_T, void* lam_0)
{
    if (!a || !lam_T || !lam_0) return fail(AMR_ERR_INVALID, "null argument");
    amr_status st = adjoint_ready(a);
    if (st != AMR_OK) return st;
    amr_tree*    t     = a->t;
    const size_t bytes = t->size * t->g.flat * t->esize;
    AMR_CUDA(cudaMemcpyAsync(a->lam[0], lam_T, bytes, cudaMemcpyHostToDevice, t->stream));
    int res = 0;
    st      = adjoint_sweep(a, &res);
    if (st != AMR_OK) return st;
    AMR_CUDA(cudaMemcpyAsync(lam_0, a->lam[res], bytes, cudaMemcpyDeviceToHost, t->stream));
    AMR_CUDA(cudaStreamSynchronize(t->stream));
    return AMR_OK;
}

amr_status amr_adjoint_checkpoint(amr_adjoint* a, size_t index, void* dst)
{
    if (!a || !dst) return fail(AMR_ERR_INVALID, "null argument");
    if (index >= a->ckpt.size()) return fail(AMR_ERR_INVALID, "checkpoint index out of range");
    if (!a->forward_done) return fail(AMR_ERR_INVALID, "amr_adjoint_forward has not run");
    amr_tree* t = a->t;
    AMR_CUDA(cudaMemcpyAsync(dst, a->ckpt[index], t->size * t->g.flat * t->esize, cudaMemcpyDeviceToDevice, t->stream));
    AMR_CUDA(cudaStreamSynchronize(t->stream));
    return AMR_OK;
}

amr_status amr_selftest_wait_timeout(int32_t polls, amr_status* observed)
{
    if (polls < 1) return fail(AMR_ERR_INVALID, "polls must be positive");
    int32_t* d = nullptr;
    AMR_CUDA(cudaMalloc(reinterpret_cast<void**>(&d), 2 * sizeof(int32_t)));
    int32_t h[2] = { -1, 0 };
    cudaError_t e = cudaMemcpy(d, h, sizeof h, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        k_selftest_wait<<<1, 32>>>(d, polls);
        g_launches.fetch_add(1);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        k_selftest_touch<<<1, 1>>>(d);
        g_launches.fetch_add(1);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(h, d, sizeof h, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return cuda_fail(e, "amr_selftest_wait_timeout");
    if (observed) *observed = static_cast<amr_status>(h[0]);
    if (h[1] != 1) return fail(AMR_ERR_CUDA, "the context did not run the follow-up kernel");
    if (h[0] != AMR_ERR_TIMEOUT) return fail(AMR_ERR_INVALID, "the wait did not time out");
    return AMR_OK;
}


} // extern "C"
