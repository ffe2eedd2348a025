// The allocation-free re-mesh entry point (amr_remesh_noalloc).

#include "amr_api.cuh"

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

