// Device-resident VTK writer: vtk_print::print (include/ndtree/vtk_print.hpp:
// 53-257) for the tree's current leaves and state.  Every section of the
// legacy binary file (points, connectivity, cell types, cell_index, is_halo,
// the scalar field) is produced on the device, big-endian, in chunks of
// cells, copied back and appended to the file; the host writes only the
// section header lines.  Corner coordinates use the reference's arithmetic
// (physics_system::patch_coord / cell_sizes, physics_system.hpp:62-104) with
// explicit rounding, so the file is byte-identical to the reference's.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "amr_gb300.h"
#include "amr_vtk.cuh"

namespace amr_gb300 {
namespace {

__device__ __forceinline__ uint32_t bswap32(uint32_t x) { return __byte_perm(x, 0, 0x0123); }

__device__ __forceinline__ void put_be64(unsigned char* dst, double v)
{
    // most significant byte first: the high word, byte-swapped, then the low word
    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(v));
    uint32_t*                d = reinterpret_cast<uint32_t*>(dst);
    d[0]                       = bswap32(static_cast<uint32_t>(b >> 32));
    d[1]                       = bswap32(static_cast<uint32_t>(b));
}
__device__ __forceinline__ void put_be32(unsigned char* dst, uint32_t v)
{
    *reinterpret_cast<uint32_t*>(dst) = bswap32(v);
}

// Interior cell `cell` of the chunk: patch and row-major interior coordinates.
__device__ __forceinline__ void cell_coords(const Geo& g, long long cell, int& p, int* idx)
{
    p          = static_cast<int>(cell / g.cells);
    int c      = static_cast<int>(cell - static_cast<long long>(p) * g.cells);
    idx[2]     = 0;
    for (int L = g.rank - 1; L >= 0; --L) {
        idx[L] = c % g.n + g.h;
        c /= g.n;
    }
}

__global__ void k_vtk_points(const uint64_t* __restrict__ keys, Geo g, VtkDomain dom, long long first,
                             long long count, unsigned char* __restrict__ out)
{
    const int box = 1 << g.rank;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < count;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        int p, idx[3];
        cell_coords(g, first + i, p, idx);
        uint32_t c[3];
        key_decode(g, keys[p], c);
        const int    level = key_level(keys[p]);
        const double maxc  = static_cast<double>(1u << g.depth);
        double       o[3] = { 0, 0, 0 }, cs[3] = { 0, 0, 0 };
        for (int k = 0; k < g.rank; ++k) {
            o[k]              = __ddiv_rn(__dmul_rn(dom.lengths[k], static_cast<double>(c[k])), maxc);
            const double size = __ddiv_rn(__dmul_rn(dom.lengths[k], static_cast<double>(1u << (g.depth - level))), maxc);
            cs[k]             = __ddiv_rn(size, static_cast<double>(g.n));
        }
        unsigned char* d = out + i * box * 24;
        if (g.rank == 2) {
            const double x = __dadd_rn(o[0], __dmul_rn(static_cast<double>(idx[1] - g.h), cs[0]));
            const double y = __dadd_rn(o[1], __dmul_rn(static_cast<double>(idx[0] - g.h), cs[1]));
            const double X = __dadd_rn(x, cs[0]), Y = __dadd_rn(y, cs[1]);
            const double pts[12] = { x, y, 0.0, X, y, 0.0, X, Y, 0.0, x, Y, 0.0 };
            for (int k = 0; k < 12; ++k) put_be64(d + 8 * k, pts[k]);
        } else {
            const double x = __dadd_rn(o[0], __dmul_rn(static_cast<double>(idx[2] - g.h), cs[0]));
            const double y = __dadd_rn(o[1], __dmul_rn(static_cast<double>(idx[1] - g.h), cs[1]));
            const double z = __dadd_rn(o[2], __dmul_rn(static_cast<double>(idx[0] - g.h), cs[2]));
            const double X = __dadd_rn(x, cs[0]), Y = __dadd_rn(y, cs[1]), Z = __dadd_rn(z, cs[2]);
            // VTK_VOXEL corner order of the reference
            const double pts[24] = { x, y, z, X, y, z, x, Y, z, X, Y, z, x, y, Z, X, y, Z, x, Y, Z, X, Y, Z };
            for (int k = 0; k < 24; ++k) put_be64(d + 8 * k, pts[k]);
        }
    }
}

// CELLS: box, then the box corner indices i*box + j (as the reference's int).
__global__ void k_vtk_cells(int box, long long first, long long count, unsigned char* __restrict__ out)
{
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < count;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        unsigned char*  d    = out + i * (box + 1) * 4;
        const long long cell = first + i;
        put_be32(d, static_cast<uint32_t>(box));
        for (int j = 0; j < box; ++j) put_be32(d + 4 * (j + 1), static_cast<uint32_t>(static_cast<int>(cell * box + j)));
    }
}

// mode 0: the constant v; 1: the cell index; 2: is_halo_cell of linear
// index (cell mod n^rank) on the padded layout (the reference's loop).
__global__ void k_vtk_ints(Geo g, int mode, int v, long long first, long long count, unsigned char* __restrict__ out)
{
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < count;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const long long cell = first + i;
        uint32_t        val  = static_cast<uint32_t>(v);
        if (mode == 1) val = static_cast<uint32_t>(static_cast<int>(cell));
        if (mode == 2) {
            long long li   = cell % g.cells;
            long long st   = g.flat / g.P1;
            int       halo = 0;
            for (int k = 0; k < g.rank; ++k) {
                const long long rel = li / st;
                if (rel < g.h || rel >= g.P1 - g.h) {
                    halo = 1;
                    break;
                }
                li %= st;
                st /= g.P1;
            }
            val = static_cast<uint32_t>(halo);
        }
        put_be32(out + 4 * i, val);
    }
}

template <typename T>
__global__ void k_vtk_values(const T* __restrict__ state, Geo g, long long first, long long count,
                             unsigned char* __restrict__ out)
{
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < count;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        int p, idx[3];
        cell_coords(g, first + i, p, idx);
        const T v = state[static_cast<size_t>(p) * g.flat + padded_index(g, idx)];
        if constexpr (sizeof(T) == 8) put_be64(out + 8 * i, v);
        else put_be32(out + 4 * i, __float_as_uint(v));
    }
}

} // namespace

amr_status vtk_write(const VtkTree& v, const char* path, const char* fields, std::string& err)
{
    const Geo&      g     = v.g;
    const long long cells = static_cast<long long>(v.size) * g.cells;
    const int       box   = 1 << g.rank;
    FILE*           f     = std::fopen(path, "wb");
    if (!f) {
        err = std::string("cannot open ") + path;
        return AMR_ERR_INVALID;
    }
    // staging: at most 1 << 22 cells of the widest section (points)
    const long long chunk     = std::min<long long>(std::max<long long>(cells, 1), 1LL << 22);
    const size_t    max_bytes = static_cast<size_t>(chunk) * box * 24;
    unsigned char*  dbuf      = nullptr;
    unsigned char*  hbuf      = nullptr;
    cudaError_t     e         = cudaMalloc(&dbuf, max_bytes);
    if (e == cudaSuccess) e = cudaMallocHost(&hbuf, max_bytes);
    auto section = [&](size_t per_cell, auto&& launch) -> bool {
        for (long long first = 0; first < cells && e == cudaSuccess; first += chunk) {
            const long long n    = std::min(chunk, cells - first);
            const unsigned  grid = static_cast<unsigned>(std::min<long long>((n + 255) / 256, 152LL * 32));
            launch(first, n, grid);
            if (e == cudaSuccess) e = cudaGetLastError();
            if (e == cudaSuccess) e = cudaMemcpyAsync(hbuf, dbuf, n * per_cell, cudaMemcpyDeviceToHost, v.stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(v.stream);
            if (e == cudaSuccess && std::fwrite(hbuf, 1, n * per_cell, f) != static_cast<size_t>(n * per_cell)) {
                err = "short write";
                return false;
            }
        }
        return e == cudaSuccess;
    };
    bool ok = e == cudaSuccess;
    if (ok) {
        std::fprintf(f, "# vtk DataFile Version 3.0\nAMR Tree Structure\nBINARY\nDATASET UNSTRUCTURED_GRID\n");
        std::fprintf(f, "POINTS %lld double\n", cells * box);
        ok = section(static_cast<size_t>(box) * 24, [&](long long first, long long n, unsigned grid) {
            k_vtk_points<<<grid, 256, 0, v.stream>>>(v.keys, g, v.dom, first, n, dbuf);
        });
    }
    if (ok) {
        std::fprintf(f, "CELLS %lld %lld\n", cells, cells * (box + 1));
        ok = section(static_cast<size_t>(box + 1) * 4, [&](long long first, long long n, unsigned grid) {
            k_vtk_cells<<<grid, 256, 0, v.stream>>>(box, first, n, dbuf);
        });
    }
    if (ok) {
        std::fprintf(f, "CELL_TYPES %lld\n", cells);
        ok = section(4, [&](long long first, long long n, unsigned grid) {
            k_vtk_ints<<<grid, 256, 0, v.stream>>>(g, 0, g.rank == 2 ? 9 : 11, first, n, dbuf);
        });
    }
    if (ok) {
        std::fprintf(f, "CELL_DATA %lld\nSCALARS cell_index int 1\nLOOKUP_TABLE default\n", cells);
        ok = section(4, [&](long long first, long long n, unsigned grid) {
            k_vtk_ints<<<grid, 256, 0, v.stream>>>(g, 1, 0, first, n, dbuf);
        });
    }
    if (ok) {
        std::fprintf(f, "SCALARS is_halo int 1\nLOOKUP_TABLE default\n");
        ok = section(4, [&](long long first, long long n, unsigned grid) {
            k_vtk_ints<<<grid, 256, 0, v.stream>>>(g, 2, 0, first, n, dbuf);
        });
    }
    // one SCALARS block per field, in field order (vtk_print.hpp writes the
    // cell type's fields in tuple order)
    const char* name = fields;
    for (int fi = 0; ok && fi < v.nvar; ++fi) {
        size_t len = 0;
        while (name[len] && name[len] != ',') ++len;
        std::fprintf(f, "SCALARS %.*s %s 1\nLOOKUP_TABLE default\n", static_cast<int>(len), name,
                     v.esize == 8 ? "double" : "float");
        name += len + (name[len] == ',' ? 1 : 0);
        const size_t off = fi * v.fstride;
        ok = section(v.esize, [&](long long first, long long n, unsigned grid) {
            if (v.esize == 8)
                k_vtk_values<double><<<grid, 256, 0, v.stream>>>(static_cast<const double*>(v.state) + off, g, first,
                                                                 n, dbuf);
            else
                k_vtk_values<float><<<grid, 256, 0, v.stream>>>(static_cast<const float*>(v.state) + off, g, first, n,
                                                                dbuf);
        });
    }
    if (dbuf) cudaFree(dbuf);
    if (hbuf) cudaFreeHost(hbuf);
    const bool closed = std::fclose(f) == 0;
    if (e != cudaSuccess) {
        err = std::string("vtk writer: ") + cudaGetErrorString(e);
        return AMR_ERR_CUDA;
    }
    if (!ok || !closed) {
        if (err.empty()) err = "vtk writer: write failed";
        return AMR_ERR_INVALID;
    }
    return AMR_OK;
}

} // namespace amr_gb300
