// The staged 3D update of 8^3 and 4^3 patches with one ghost layer.
#pragma once

#include "amr_kernels.cuh"

namespace amr_gb300 {

// ------------------------------------------------ 3D update, staged
// One step of 3D patches of N^3 cells and one ghost layer, one warp per
// patch (grid-stride).  The patch's interior planes (ghost rows and columns
// included, a contiguous 16-byte-aligned span) move into a per-warp
// shared-memory tile by bulk async copy; each warp owns S tiles in a ring
// and keeps S-1 copies in flight ahead of the patch it works on.  While the
// copy lands the lanes evaluate the upwind ghost faces by the halo rules
// (ghost_value, the values step_cell takes on the fly), then write them into
// the tile, update N^3/32 cells each from the tile with step_cell's
// arithmetic, and store the interior planes back as 16-byte words (ghost
// rows and columns pass through, as in the 2D kernels).  A copy that does
// not land within the wait cap sets *err = AMR_ERR_TIMEOUT; the warp then
// drains its other copies (also capped) and stops.
template <typename T, int N>
struct Step3dShape {
    static constexpr int      P1 = N + 2, PLANE = P1 * P1, FLAT = PLANE * P1;
    static constexpr uint32_t LO    = PLANE * sizeof(T);           // byte span of the interior planes
    static constexpr uint32_t BYTES = N * PLANE * sizeof(T);
    static constexpr int      WORDS = BYTES / 16;
    static constexpr int      PER   = N * N * N / 32;              // cells per lane
    static constexpr int      GPL   = (N * N + 31) / 32;           // ghost cells per lane and face
    static constexpr size_t   TILE  = FLAT * sizeof(T);
    static_assert(LO % 16 == 0 && BYTES % 16 == 0 && TILE % 16 == 0, "planes are whole 16-byte words");
    static_assert(N * N * N % 32 == 0, "a warp's lanes share the cells evenly");
    static constexpr size_t smem(int W, int S) { return static_cast<size_t>(W) * S * (TILE + 8); }
};

template <typename T, int N, int S>
__device__ __forceinline__ void step3d_body(const T* __restrict__ in, T* __restrict__ out,
                                            const amr_halo_meta* __restrict__ meta, const int32_t* __restrict__ levels,
                                            const uint64_t* __restrict__ keys, int P, const Geo& g,
                                            const Coef* __restrict__ coef, const float4* __restrict__ coef4,
                                            int up0, int up1, int up2, const int32_t* __restrict__ upcode,
                                            int32_t* err, T* tiles, uint64_t* bars, int p, int nwarp)
{
    using Sh               = Step3dShape<T, N>;
    constexpr int P1       = Sh::P1, PLANE = Sh::PLANE, FLAT = Sh::FLAT, GPL = Sh::GPL;
    const int     lane     = threadIdx.x & 31;
    const int     nl       = g.depth + 1;
    if (lane == 0) {
        for (int b = 0; b < S; ++b) mbar_init(&bars[b], 1);
        mbar_init_fence();
    }
    __syncwarp();
    const char* in_bytes = reinterpret_cast<const char*>(in);
    auto        request  = [&](int q, int slot) {
        fence_proxy_async_smem();
        mbar_expect_tx(&bars[slot], Sh::BYTES);
        bulk_copy_g2s(reinterpret_cast<char*>(tiles + static_cast<size_t>(slot) * FLAT) + Sh::LO,
                      in_bytes + static_cast<size_t>(q) * Sh::TILE + Sh::LO, Sh::BYTES, &bars[slot]);
    };
    if (lane == 0)
        for (int j = 0; j < S - 1; ++j)
            if (p + j * nwarp < P) request(p + j * nwarp, j);
    uint32_t phase = 0; // bit b: parity of slot b's next completion
    for (int it = 0; p < P; ++it, p += nwarp) {
        const int b  = it % S;
        const int pf = p + (S - 1) * nwarp;
        if (pf < P && lane == 0) request(pf, (it + S - 1) % S);
        const int inst  = keys ? instance_of(g, keys, p) : 0;
        int       up[3] = { up0, up1, up2 };
        if (upcode) { // per-instance upwind sides, packed (integer decode: no FP64 compares)
            const int32_t code = upcode[inst];
            for (int a = 0; a < 3; ++a) up[a] = unpack_upwind(code, a);
        }
        // the row of the leaf's level: FP64 from coef, FP32 from the rows
        // rounded once (coef4)
        const int row = inst * nl + levels[p];
        T         c0, ca[3];
        if constexpr (sizeof(T) == 4) {
            const float4 c4 = coef4[row];
            c0              = c4.w;
            ca[0]           = c4.x;
            ca[1]           = c4.y;
            ca[2]           = c4.z;
        } else {
            const Coef cf = coef[row];
            c0            = cf.c0;
            ca[0]         = cf.c[0];
            ca[1]         = cf.c[1];
            ca[2]         = cf.c[2];
        }
        const T* src = in + static_cast<size_t>(p) * FLAT;
        // the upwind ghost faces (Morton axis a is layout dim 2 - a): ghost
        // cell k of a face has tangential coordinates (k / N + 1, k % N + 1)
        T gv[3][GPL];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const int L = 2 - a, pos = up[a] > 0 ? 1 : 0;
#pragma unroll
            for (int j = 0; j < GPL; ++j) {
                const int k = lane + 32 * j;
                gv[a][j]    = T(0);
                if (up[a] != 0 && k < N * N) {
                    int G[3];
                    G[L]              = pos ? N + 1 : 0;
                    G[L == 0 ? 1 : 0] = k / N + 1;
                    G[L == 2 ? 1 : 2] = k % N + 1;
                    gv[a][j] =
                        ghost_value<T, T>(in, FLAT, meta[static_cast<size_t>(p) * 6 + 2 * L + pos], G, L, pos, g, src);
                }
            }
        }
        if (!mbar_wait_bounded(&bars[b], (phase >> b) & 1u)) {
            if (lane == 0) atomicExch(err, static_cast<int32_t>(AMR_ERR_TIMEOUT));
            phase ^= 1u << b;
            for (int j = 1; j < S; ++j) // drain the copies still in flight
                if (p + j * nwarp < P) {
                    const int sl = (it + j) % S;
                    mbar_wait_bounded(&bars[sl], (phase >> sl) & 1u);
                    phase ^= 1u << sl;
                }
            return;
        }
        phase ^= 1u << b;
        T* tile = tiles + static_cast<size_t>(b) * FLAT;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const int L = 2 - a;
#pragma unroll
            for (int j = 0; j < GPL; ++j) {
                const int k = lane + 32 * j;
                if (up[a] != 0 && k < N * N) {
                    int G[3];
                    G[L]              = up[a] > 0 ? N + 1 : 0;
                    G[L == 0 ? 1 : 0] = k / N + 1;
                    G[L == 2 ? 1 : 2] = k % N + 1;
                    tile[(G[0] * P1 + G[1]) * P1 + G[2]] = gv[a][j];
                }
            }
        }
        __syncwarp();
        T res[Sh::PER];
#pragma unroll
        for (int q = 0; q < Sh::PER; ++q) {
            const int c   = lane + 32 * q;
            const int li  = ((c / (N * N) + 1) * P1 + (c / N) % N + 1) * P1 + c % N + 1;
            const T   u   = tile[li];
            T         acc = sizeof(T) == 4 ? u : c0 * u;
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                if (up[a] == 0) continue;
                const int st  = a == 0 ? 1 : (a == 1 ? P1 : PLANE);
                const T   val = tile[li + up[a] * st];
                acc = fma(ca[a], sizeof(T) == 4 ? static_cast<T>(val - u) : val, acc);
            }
            res[q] = acc;
        }
        __syncwarp();
#pragma unroll
        for (int q = 0; q < Sh::PER; ++q) {
            const int c                                                          = lane + 32 * q;
            tile[((c / (N * N) + 1) * P1 + (c / N) % N + 1) * P1 + c % N + 1] = res[q];
        }
        __syncwarp();
        const uint4* t4  = reinterpret_cast<const uint4*>(reinterpret_cast<const char*>(tile) + Sh::LO);
        uint4*       dst = reinterpret_cast<uint4*>(reinterpret_cast<char*>(out + static_cast<size_t>(p) * FLAT) + Sh::LO);
        for (int w = lane; w < Sh::WORDS; w += 32) dst[w] = t4[w];
        __syncwarp(); // the slot is refilled by a later copy
    }
}

// Tiles and barriers of warp wib in a block of W warps with S slots each.
template <typename T, int N, int W, int S>
__device__ __forceinline__ void step3d_smem(unsigned char* smem, T*& tiles, uint64_t*& bars)
{
    const int wib = threadIdx.x >> 5;
    tiles         = reinterpret_cast<T*>(smem) + static_cast<size_t>(wib) * S * Step3dShape<T, N>::FLAT;
    bars          = reinterpret_cast<uint64_t*>(smem + static_cast<size_t>(W) * S * Step3dShape<T, N>::TILE) + wib * S;
}

// Host-driven launch: W warps per block, one per patch.
template <typename T, int N, int W, int S>
__global__ void __launch_bounds__(W * 32)
k_step3d(const T* __restrict__ in, T* __restrict__ out, const int32_t* __restrict__ levels,
         const amr_halo_meta* __restrict__ meta, int P, Geo g, const Coef* __restrict__ coef,
         const float4* __restrict__ coef4, int up0, int up1, int up2, const uint64_t* __restrict__ keys,
         const int32_t* __restrict__ upcode, int32_t* err)
{
    extern __shared__ __align__(128) unsigned char smem3d[];
    T*        tiles;
    uint64_t* bars;
    step3d_smem<T, N, W, S>(smem3d, tiles, bars);
    const int nwarp = (gridDim.x * blockDim.x) >> 5;
    const int p     = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    step3d_body<T, N, S>(in, out, meta, levels, keys, P, g, coef, coef4, up0, up1, up2, upcode, err, tiles, bars, p,
                         nwarp);
}

} // namespace amr_gb300
