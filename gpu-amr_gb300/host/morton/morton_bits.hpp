// Bit interleave of Morton (Z-order) codes: coordinate k of a rank-r point
// sits at bit r*b + k (x lowest), the layout of libmorton's 64-bit encoders
// used by gpu-amr's morton_id (include/morton/morton_id.hpp:118-140, 334-359).
// Spread/compact by binary magic numbers; usable from host and device code.
#pragma once

#include <cstdint>

#if defined(__CUDACC__)
#    define AMR_HD __host__ __device__
#else
#    define AMR_HD
#endif

namespace amr::morton_bits
{

AMR_HD inline std::uint64_t spread2(std::uint64_t v)
{
    v &= 0xFFFFFFFFull;
    v = (v | (v << 16)) & 0x0000FFFF0000FFFFull;
    v = (v | (v << 8)) & 0x00FF00FF00FF00FFull;
    v = (v | (v << 4)) & 0x0F0F0F0F0F0F0F0Full;
    v = (v | (v << 2)) & 0x3333333333333333ull;
    v = (v | (v << 1)) & 0x5555555555555555ull;
    return v;
}

AMR_HD inline std::uint32_t compact2(std::uint64_t v)
{
    v &= 0x5555555555555555ull;
    v = (v | (v >> 1)) & 0x3333333333333333ull;
    v = (v | (v >> 2)) & 0x0F0F0F0F0F0F0F0Full;
    v = (v | (v >> 4)) & 0x00FF00FF00FF00FFull;
    v = (v | (v >> 8)) & 0x0000FFFF0000FFFFull;
    v = (v | (v >> 16)) & 0x00000000FFFFFFFFull;
    return static_cast<std::uint32_t>(v);
}

AMR_HD inline std::uint64_t spread3(std::uint64_t v)
{
    v &= 0x1FFFFFull;
    v = (v | (v << 32)) & 0x001F00000000FFFFull;
    v = (v | (v << 16)) & 0x001F0000FF0000FFull;
    v = (v | (v << 8)) & 0x100F00F00F00F00Full;
    v = (v | (v << 4)) & 0x10C30C30C30C30C3ull;
    v = (v | (v << 2)) & 0x1249249249249249ull;
    return v;
}

AMR_HD inline std::uint32_t compact3(std::uint64_t v)
{
    v &= 0x1249249249249249ull;
    v = (v | (v >> 2)) & 0x10C30C30C30C30C3ull;
    v = (v | (v >> 4)) & 0x100F00F00F00F00Full;
    v = (v | (v >> 8)) & 0x001F0000FF0000FFull;
    v = (v | (v >> 16)) & 0x001F00000000FFFFull;
    v = (v | (v >> 32)) & 0x00000000001FFFFFull;
    return static_cast<std::uint32_t>(v);
}

} // namespace amr::morton_bits
