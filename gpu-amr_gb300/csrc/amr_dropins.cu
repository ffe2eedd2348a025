// Free-function drop-ins: one per amr::cuda:: launcher of the reference, on caller-owned buffers
// in the reference's layout.

#include "amr_api.cuh"

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

