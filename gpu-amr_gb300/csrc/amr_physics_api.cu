// C-ABI entry points of the physics on the device tree: SSPRK time integration, the DG patch solver
// (advection and Euler) with its printer, compressible Euler and the VTK writer.

#include "amr_api.cuh"

extern "C" {

amr_status amr_tree_advance_ssprk(amr_tree* t, size_t steps, int order, const double* velocity3, double cfl,
                                  double remaining)
{
    if (!t) return fail(AMR_ERR_INVALID, "null argument");
    if (order != 2 && order != 3) return fail(AMR_ERR_INVALID, "SSPRK order is 2 or 3");
    if (t->nvar != 1 || t->dtype != AMR_F64) return fail(AMR_ERR_INVALID, "SSPRK advances a one-field FP64 tree");
    if (!velocity3 && !t->vel_inst_set) return fail(AMR_ERR_INVALID, "no velocity given and none set per instance");
    cudaStream_t s = t->stream;
    const int    K = t->ninst;
    if (velocity3) {
        std::vector<double> v(3 * static_cast<size_t>(K));
        for (int i = 0; i < K; ++i)
            for (int a = 0; a < 3; ++a) v[3 * i + a] = velocity3[a];
        AMR_CUDA(cudaMemcpyAsync(t->vel, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice, s));
    } else {
        if (amr_status cs = copy_words8(t->vel, t->vel_inst, 3 * static_cast<size_t>(K), s); cs != AMR_OK) return cs;
    }
    if (t->stage_cap != t->cap) {
        cudaFree(t->stage_buf);
        t->stage_buf = nullptr;
        t->stage_cap = 0;
        AMR_CUDA(cudaMalloc(&t->stage_buf, t->field_bytes(t->cap)));
        t->stage_cap = t->cap;
    }
    SsprkStage st{};
    st.keys   = t->keys[t->tb];
    st.P      = static_cast<int>(t->size);
    st.g      = t->g;
    st.vel    = t->vel;
    st.stream = s;
    uint64_t launches = 0;
    auto     stage    = [&](const void* in, const void* un, void* out, int mode, const double* dts) -> amr_status {
        st.in      = static_cast<const double*>(in);
        st.un      = static_cast<const double*>(un);
        st.out     = static_cast<double*>(out);
        st.mode    = mode;
        st.step_dt = dts;
        AMR_CUDA(ssprk_stage(st));
        ++launches;
        return AMR_OK;
    };
    bool   first = true;
    size_t done  = 0;
    while (done < steps || (first && steps == 0)) {
        // CFL steps of this chunk (as amr_tree_advance: the finest level,
        // clamped to the remaining time), and the time bookkeeping
        const int chunk = static_cast<int>(std::min(t->coef_steps, steps - done));
        k_batch_begin<<<K, 256, 0, s>>>(t->maxlev, t->g, t->vel, cfl, chunk, first ? BATCH_RESET : BATCH_CONTINUE,
                                        remaining, t->dts(), t->step_dt, t->coef, t->coef32, t->upcode);
        AMR_LAUNCHED("k_batch_begin");
        first = false;
        for (int k = 0; k < chunk; ++k) {
            const double* dts = t->step_dt + static_cast<size_t>(k) * K;
            // (a step past the time limit, step size 0, changes nothing:
            // no halo, and every stage copies)
            if (amr_status hs = halo_buffer(t, t->cur, dts); hs != AMR_OK) return hs;
            amr_status rs = AMR_OK;
            if (order == 2) {
                if ((rs = stage(t->cur, t->cur, t->stage_buf, 0, dts)) != AMR_OK) return rs;
                if ((rs = halo_buffer(t, t->stage_buf, dts)) != AMR_OK) return rs;
                if ((rs = stage(t->stage_buf, t->cur, t->nxt, 2, dts)) != AMR_OK) return rs;
            } else {
                if ((rs = stage(t->cur, t->cur, t->nxt, 0, dts)) != AMR_OK) return rs;
                if ((rs = halo_buffer(t, t->nxt, dts)) != AMR_OK) return rs;
                if ((rs = stage(t->nxt, t->cur, t->stage_buf, 31, dts)) != AMR_OK) return rs;
                if ((rs = halo_buffer(t, t->stage_buf, dts)) != AMR_OK) return rs;
                if ((rs = stage(t->stage_buf, t->cur, t->nxt, 32, dts)) != AMR_OK) return rs;
            }
            std::swap(t->cur, t->nxt);
        }
        done += chunk;
        if (steps == 0) break;
    }
    g_launches.fetch_add(launches, std::memory_order_relaxed);
    // the buffer's ghost cells hold the last stage's combination, which is
    // what the reference's tree holds between steps (no halo exchange follows
    // the last stage); criteria read them from the buffer as it does
    t->ghosts_valid = true;
    t->batch_open   = true;
    return AMR_OK;
}

amr_status amr_tree_dg_set_equation(amr_tree* t, int equation)
{
    if (!t) return fail(AMR_ERR_INVALID, "null argument");
    if (equation != AMR_DG_ADVECTION && equation != AMR_DG_EULER) return fail(AMR_ERR_INVALID, "unknown DG equation");
    if (equation == AMR_DG_EULER) {
        if (!t->dg_scalars) AMR_CUDA(cudaMalloc(&t->dg_scalars, 2 * sizeof(double)));
        if (!t->dg_dtmin) {
            AMR_CUDA(cudaMalloc(&t->dg_dtmin, sizeof(unsigned long long)));
            const unsigned long long inf = 0x7ff0000000000000ull; // +inf: no patch seen
            if (const cudaError_t e = cudaMemcpy(t->dg_dtmin, &inf, sizeof inf, cudaMemcpyHostToDevice);
                e != cudaSuccess) {
                cudaFree(t->dg_dtmin);
                t->dg_dtmin = nullptr;
                return cuda_fail(e, "amr_tree_dg_set_equation");
            }
        }
    }
    t->dg_equation = equation;
    return AMR_OK;
}

namespace
{
// DG Euler steps: the step size lives on the device, set per step from the
// patches' wave speeds (solver.hpp:227-234), so the host reads it back once
// per call
amr_status dg_euler_advance(amr_tree* t, const DgStage& st, size_t steps, double* dt, double* time)
{
    cudaStream_t         s    = t->stream;
    const Geo&           g    = t->g;
    const amr_halo_meta* meta = t->meta[t->tb];
    if (t->dg_prims_cap < t->cap) {
        cudaFree(t->dg_prims);
        t->dg_prims     = nullptr;
        t->dg_prims_cap = 0;
        AMR_CUDA(cudaMalloc(&t->dg_prims, 14 * t->fstride() * sizeof(double)));
        t->dg_prims_cap = t->cap;
    }
    double* hp = static_cast<double*>(t->pinned);
    hp[0]      = *dt;
    hp[1]      = time ? *time : 0.0;
    AMR_CUDA(cudaMemcpyAsync(t->dg_scalars, hp, 2 * sizeof(double), cudaMemcpyHostToDevice, s));
    DgEulerStage es{};
    es.prims   = t->dg_prims;
    es.keys    = st.keys;
    es.P       = st.P;
    es.g       = g;
    es.fstride = st.fstride;
    es.dt      = t->dg_scalars;
    es.dt_min  = t->dg_dtmin;
    es.stream  = s;
    uint64_t launches = 0;
    for (size_t k = 0; k < steps; ++k) {
        AMR_CUDA(dg_halo(static_cast<double*>(t->cur), meta, st.P, g, st.fstride, s));
        AMR_CUDA(dg_euler_prims(static_cast<const double*>(t->cur), t->dg_prims, st.P, g, st.fstride, s));
        es.in   = static_cast<const double*>(t->cur);
        es.un   = static_cast<const double*>(t->cur);
        es.out  = static_cast<double*>(t->nxt);
        es.mode = 0;
        AMR_CUDA(dg_euler_stage(es));
        AMR_CUDA(dg_halo(static_cast<double*>(t->nxt), meta, st.P, g, st.fstride, s));
        AMR_CUDA(dg_euler_prims(static_cast<const double*>(t->nxt), t->dg_prims, st.P, g, st.fstride, s));
        es.in   = static_cast<const double*>(t->nxt);
        es.out  = static_cast<double*>(t->cur); // u^n is read and replaced cell by cell
        es.mode = 1;
        AMR_CUDA(dg_euler_stage(es));
        AMR_CUDA(dg_euler_next(t->dg_scalars, t->dg_scalars + 1, t->dg_dtmin, s));
        launches += 7;
    }
    AMR_CUDA(cudaMemcpyAsync(hp, t->dg_scalars, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
    AMR_CUDA(cudaStreamSynchronize(s));
    g_launches.fetch_add(launches, std::memory_order_relaxed);
    t->ghosts_valid = true;
    *dt             = hp[0];
    if (time) *time = hp[1];
    return AMR_OK;
}
} // namespace

amr_status amr_tree_dg_advance(amr_tree* t, size_t steps, double* dt, double* time)
{
    if (!t || !dt) return fail(AMR_ERR_INVALID, "null argument");
    const Geo& g = t->g;
    if (g.rank != 2 || g.n != kDgPatch || g.h != 1 || t->nvar != kDgFields || t->dtype != AMR_F64)
        return fail(AMR_ERR_INVALID, "the DG advance needs a 2D FP64 tree of 4x4 patches, one ghost cell, 16 fields");
    if (!(*dt > 0.0)) return fail(AMR_ERR_INVALID, "the DG step size must be positive");
    cudaStream_t s = t->stream;
    DgStage      st{};
    st.keys    = t->keys[t->tb];
    st.P       = static_cast<int>(t->size);
    st.g       = g;
    st.fstride = t->fstride();
    st.stream  = s;
    if (t->dg_equation == AMR_DG_EULER) return dg_euler_advance(t, st, steps, dt, time);
    // CFL step of the finest cells (solver.hpp:227-234 with |v| = 1)
    const double edge   = (1.0 / static_cast<double>(1u << t->max_level_host)) / static_cast<double>(kDgPatch);
    const double scale  = 1.0 / (std::pow(static_cast<double>(kDgOrder), 2.0) + 1.0);
    const double dt_cfl = scale * 0.5 * edge / 1.0;
    double       h      = *dt, acc = time ? *time : 0.0;
    uint64_t     launches = 0;
    const amr_halo_meta* meta = t->meta[t->tb];
    for (size_t k = 0; k < steps; ++k) {
        AMR_CUDA(dg_halo(static_cast<double*>(t->cur), meta, st.P, g, st.fstride, s));
        st.in   = static_cast<const double*>(t->cur);
        st.un   = static_cast<const double*>(t->cur);
        st.out  = static_cast<double*>(t->nxt);
        st.dt   = h;
        st.mode = 0;
        AMR_CUDA(dg_stage(st));
        AMR_CUDA(dg_halo(static_cast<double*>(t->nxt), meta, st.P, g, st.fstride, s));
        st.in   = static_cast<const double*>(t->nxt);
        st.out  = static_cast<double*>(t->cur); // u^n is read and replaced cell by cell
        st.mode = 1;
        AMR_CUDA(dg_stage(st));
        launches += 4;
        h = std::min(h, std::min(h, dt_cfl));
        acc += h; // the reference's loop adds the updated step (solver.hpp:129, 134)
    }
    g_launches.fetch_add(launches, std::memory_order_relaxed);
    t->ghosts_valid = true; // the ghosts the reference's tree holds after a step
    *dt             = h;
    if (time) *time = acc;
    return AMR_OK;
}

amr_status amr_tree_dg_remesh(amr_tree* t, double refine_threshold, double coarsen_threshold, int* changed)
{
    if (!t) return fail(AMR_ERR_INVALID, "null argument");
    const Geo& g = t->g;
    if (g.rank != 2 || g.n != kDgPatch || g.h != 1 || t->nvar != kDgFields || t->dtype != AMR_F64)
        return fail(AMR_ERR_INVALID, "the DG re-mesh needs a 2D FP64 tree of 4x4 patches, one ghost cell, 16 fields");
    AMR_CUDA(dg_flags(static_cast<const double*>(t->cur), static_cast<int>(t->size), g, t->fstride(),
                      refine_threshold, coarsen_threshold, t->flags, t->stream));
    g_launches.fetch_add(1, std::memory_order_relaxed);
    t->dg_state         = true;
    const amr_status st = amr_tree_remesh(t, changed);
    t->dg_state         = false;
    return st;
}

amr_status amr_tree_dg_write_vtk(amr_tree* t, const char* path)
{
    if (!t || !path) return fail(AMR_ERR_INVALID, "null argument");
    const Geo& g = t->g;
    if (g.rank != 2 || g.n != kDgPatch || g.h != 1 || t->nvar != kDgFields || t->dtype != AMR_F64)
        return fail(AMR_ERR_INVALID, "the DG printer needs a 2D FP64 tree of 4x4 patches, one ghost cell, 16 fields");
    AMR_CUDA(cudaStreamSynchronize(t->stream));
    std::string      err;
    uint64_t         launches = 0;
    const amr_status st = dg_write_vtk(t->keys[t->tb], static_cast<const double*>(t->cur), t->size, g, t->fstride(),
                                       t->stream, path, err, launches);
    g_launches.fetch_add(launches, std::memory_order_relaxed);
    if (st != AMR_OK) return fail(st, err);
    return AMR_OK;
}

amr_status amr_tree_dg_run(amr_tree* t, double initial_dt, double end_time, int amr_interval,
                           double refine_threshold, double coarsen_threshold, amr_dg_stats* stats)
{
    if (!t || !stats || amr_interval < 0) return fail(AMR_ERR_INVALID, "bad argument");
    *stats                = amr_dg_stats{};
    double    dt          = initial_dt, time = 0.0;
    long long step        = 0, next_amr = 0;
    size_t    leaves_max  = t->size;
    while (time < end_time) {
        stats->cells += static_cast<uint64_t>(t->size) * kDgPatch * kDgPatch;
        if (amr_status st = amr_tree_dg_advance(t, 1, &dt, &time); st != AMR_OK) return st;
        ++step;
        if (step >= next_amr) { // apply_amr (solver.hpp:249-251): an interval of 0 re-meshes every step
            int changed = 0;
            if (amr_status st = amr_tree_dg_remesh(t, refine_threshold, coarsen_threshold, &changed); st != AMR_OK)
                return st;
            ++stats->remeshes;
            next_amr   = step + amr_interval;
            leaves_max = std::max(leaves_max, t->size);
        }
    }
    AMR_CUDA(cudaStreamSynchronize(t->stream));
    stats->steps      = static_cast<uint64_t>(step);
    stats->time       = time;
    stats->next_dt    = dt;
    stats->leaves_max = static_cast<uint64_t>(leaves_max);
    return AMR_OK;
}


// ------------------------------------------------------------------ Euler
static amr_status euler_check(amr_tree* t)
{
    if (!t) return fail(AMR_ERR_INVALID, "null argument");
    if (t->nvar != t->g.rank + 2) return fail(AMR_ERR_INVALID, "the Euler solver takes a tree of rank + 2 fields");
    if (t->dtype != AMR_F64) return fail(AMR_ERR_INVALID, "the Euler solver is FP64");
    if (!euler_supported(t->g)) return fail(AMR_ERR_INVALID, "patch too large for the Euler update");
    return AMR_OK;
}

static amr_status euler_advance_impl(amr_tree* t, size_t steps, double gamma, double cfl, double remaining)
{
    const size_t prim_elems = static_cast<size_t>(t->g.rank * (t->g.rank + 2)) * t->fstride();
    if (t->prim_cap != t->cap) {
        cudaFree(t->prim[0]);
        cudaFree(t->prim[1]);
        t->prim[0] = t->prim[1] = nullptr;
        t->prim_cap = 0;
        AMR_CUDA(cudaMalloc(&t->prim[0], prim_elems * sizeof(double)));
        AMR_CUDA(cudaMalloc(&t->prim[1], prim_elems * sizeof(double)));
        t->prim_cap = t->cap;
    }
    if (!t->ghosts_valid) {
        amr_status s = launch_halo(t);
        if (s != AMR_OK) return s;
    }
    EulerBufs b{};
    b.g        = t->g;
    b.P        = static_cast<int>(t->size);
    b.fstride  = t->fstride();
    b.levels   = t->levels[t->tb];
    b.meta     = t->meta[t->tb];
    b.state[0] = static_cast<double*>(t->sbuf[0]);
    b.state[1] = static_cast<double*>(t->sbuf[1]);
    b.prim[0]  = t->prim[0];
    b.prim[1]  = t->prim[1];
    b.min_slot = t->euler_min;
    b.step_dt  = t->euler_dt;
    b.ctl      = t->euler_ctl;
    b.acc      = t->dt_acc;
    b.rem      = t->dt_rem;
    b.cnt      = t->dt_cnt;
    b.stream   = t->stream;
    int      cur      = t->cur == t->sbuf[0] ? 0 : 1;
    uint64_t launches = 0;
    cudaError_t e = euler_begin(b, cur, gamma, remaining, &launches);
    for (size_t k = 0; k < steps && e == cudaSuccess; ++k) {
        std::pair<cudaEvent_t, cudaEvent_t>* ev = nullptr;
        if (t->timing) { // opt-in timing of the update kernel
            if (t->events_used == t->events.size()) {
                std::pair<cudaEvent_t, cudaEvent_t> pe;
                AMR_CUDA(cudaEventCreate(&pe.first));
                AMR_CUDA(cudaEventCreate(&pe.second));
                t->events.push_back(pe);
                t->event_cells.push_back(0);
            }
            ev = &t->events[t->events_used];
            t->event_cells[t->events_used] = static_cast<uint64_t>(b.P) * t->g.cells;
            ++t->events_used;
        }
        e = euler_step(b, cur, static_cast<int>(k & 1), gamma, cfl, &launches, ev ? ev->first : nullptr,
                       ev ? ev->second : nullptr);
        cur ^= 1;
    }
    g_launches.fetch_add(launches, std::memory_order_relaxed);
    if (e != cudaSuccess) return cuda_fail(e, "Euler step");
    t->cur          = t->sbuf[cur];
    t->nxt          = t->sbuf[cur ^ 1];
    t->ghosts_valid = true; // the last step's halo filled every field
    t->batch_open   = true;
    return AMR_OK;
}

amr_status amr_tree_euler_advance(amr_tree* t, size_t steps, double gamma, double cfl, double remaining)
{
    if (amr_status s = euler_check(t); s != AMR_OK) return s;
    return euler_advance_impl(t, steps, gamma, cfl, remaining);
}

amr_status amr_tree_euler_run(amr_tree* t, const amr_euler_params* p, amr_cycle_stats* out)
{
    if (amr_status s = euler_check(t); s != AMR_OK) return s;
    if (!p) return fail(AMR_ERR_INVALID, "null argument");
    if (p->remesh_interval < 1) return fail(AMR_ERR_INVALID, "re-mesh interval must be positive");
    RunTotals tot;
    double    time = 0.0;
    while (tot.done < static_cast<long long>(p->steps) && time < p->end_time) {
        const size_t k = static_cast<size_t>(
            std::min<long long>(static_cast<long long>(p->remesh_interval), static_cast<long long>(p->steps) - tot.done));
        const size_t leaves = t->size;
        amr_status   st     = euler_advance_impl(t, k, p->gamma, p->cfl, p->end_time - time);
        if (st != AMR_OK) return st;
        // the benchmark's criterion: max Rho over the patch, then re-mesh
        st = amr_tree_flags_max(t, p->refine_threshold, p->coarsen_threshold, p->min_level, p->max_level);
        if (st != AMR_OK) return st;
        int changed = 0;
        st          = amr_tree_remesh(t, &changed);
        if (st != AMR_OK) return st;
        ++tot.remeshes;
        if (changed) ++tot.remeshes_changed;
        double acc = 0.0;
        size_t ex  = 0;
        st         = amr_tree_finish_advance(t, &acc, &ex);
        if (st != AMR_OK) return st;
        time += acc;
        tot.done += static_cast<long long>(ex);
        tot.executed += ex;
        tot.cells += static_cast<uint64_t>(ex) * leaves * t->g.cells;
        ++tot.intervals;
        tot.leaves_sum += leaves;
        tot.lmin = std::min<uint64_t>(tot.lmin, leaves);
        tot.lmax = std::max<uint64_t>(tot.lmax, leaves);
        if (ex == 0) break;
    }
    if (!t->ghosts_valid) {
        amr_status s = launch_halo(t);
        if (s != AMR_OK) return s;
    }
    AMR_CUDA(cudaStreamSynchronize(t->stream));
    if (out) {
        std::memset(out, 0, sizeof(*out));
        out->executed_steps = tot.executed;
        out->sum_dt         = time;
        out->cell_updates   = tot.cells;
        out->remeshes       = tot.remeshes;
        out->remeshes_changed = tot.remeshes_changed;
        out->intervals      = tot.intervals;
        out->leaves_min     = tot.intervals ? tot.lmin : t->size;
        out->leaves_max     = tot.intervals ? tot.lmax : t->size;
        out->leaves_mean    = tot.intervals ? static_cast<double>(tot.leaves_sum) / tot.intervals : 0.0;
    }
    return AMR_OK;
}

amr_status amr_tree_write_vtk(amr_tree* t, const char* path, const char* field_name)
{
    if (!t || !path) return fail(AMR_ERR_INVALID, "null argument");
    VtkTree v{};
    v.g     = t->g;
    for (int a = 0; a < 3; ++a) v.dom.lengths[a] = t->lengths[a];
    v.keys   = t->keys[t->tb];
    v.state  = t->cur;
    v.size   = t->size;
    v.esize  = t->esize;
    v.nvar   = t->nvar;
    v.fstride = t->fstride();
    v.stream = t->stream;
    AMR_CUDA(cudaStreamSynchronize(t->stream));
    std::string      err;
    const amr_status st = vtk_write(v, path, field_name ? field_name : "Scalar", err);
    // five section kernels, and one per field, per chunk of 2^22 cells
    g_launches.fetch_add((5 + t->nvar) * std::max<uint64_t>(1, (t->size * t->g.cells + (1ull << 22) - 1) >> 22));
    if (st != AMR_OK) return fail(st, err);
    return AMR_OK;
}


} // extern "C"
