// Morton patch index with the interface of gpu-amr's
// amr::ndt::morton::morton_id<Depth, Rank> (include/morton/morton_id.hpp):
// id = interleave(x, y[, z]) << 6 | level, coordinates on a 2^Depth grid,
// ordering by the raw 64-bit id.
#pragma once

#include "morton/morton_bits.hpp"

#include <array>
#include <bitset>
#include <climits>
#include <concepts>
#include <cstdint>
#include <functional>
#include <optional>
#include <string>
#include <utility>

namespace amr::ndt::morton
{

template <std::unsigned_integral auto Depth, std::unsigned_integral auto Rank>
    requires(Rank == 2u || Rank == 3u) && (Rank * Depth + 6u <= 64u)
class morton_id
{
public:
    enum direction { left, right, top, bottom, front, back };

    using depth_t     = decltype(Depth);
    using mask_t      = std::uint64_t;
    using coord_array = std::array<std::uint32_t, Rank>;
    using offset_t    = std::uint32_t;
    using size_type   = std::uint32_t;
    using direction_t = direction;
    using level_t     = std::uint8_t;

    static constexpr size_type s_depth = Depth;
    static constexpr size_type s_rank  = Rank;

    constexpr morton_id() : m_id(0) {}
    constexpr morton_id(mask_t id) : m_id(id) {}

    static constexpr auto decode(mask_t id) -> std::pair<coord_array, level_t>
    {
        const mask_t m = id >> 6;
        coord_array  c{};
        if constexpr (Rank == 2u) {
            c[0] = amr::morton_bits::compact2(m);
            c[1] = amr::morton_bits::compact2(m >> 1);
        } else {
            c[0] = amr::morton_bits::compact3(m);
            c[1] = amr::morton_bits::compact3(m >> 1);
            c[2] = amr::morton_bits::compact3(m >> 2);
        }
        return { c, static_cast<level_t>(id & 0x3Fu) };
    }

    static constexpr auto encode(coord_array const& c, level_t level) -> mask_t
    {
        mask_t m;
        if constexpr (Rank == 2u)
            m = amr::morton_bits::spread2(c[0]) | (amr::morton_bits::spread2(c[1]) << 1);
        else
            m = amr::morton_bits::spread3(c[0]) | (amr::morton_bits::spread3(c[1]) << 1) |
                (amr::morton_bits::spread3(c[2]) << 2);
        return (m << 6) | (level & 0x3Fu);
    }

    static constexpr auto isvalid_coord(coord_array c, level_t level) -> bool
    {
        const std::uint32_t grid = 1u << (s_depth - level), maxc = 1u << s_depth;
        for (auto v : c)
            if (v % grid != 0 || v >= maxc) return false;
        return true;
    }

    static constexpr auto offset_of(morton_id id) -> offset_t
    {
        auto [c, level]       = decode(id.m_id);
        const std::uint32_t d = 1u << (s_depth - level + 1);
        offset_t            o = 0;
        for (std::size_t k = 0; k != Rank; ++k)
            if (c[k] % d != 0) o |= 1u << k;
        return o;
    }

    static constexpr auto offset(morton_id id, offset_t off) -> morton_id
    {
        auto [c, level]       = decode(id.m_id);
        const std::uint32_t d = 1u << (s_depth - level);
        for (std::size_t k = 0; k != Rank; ++k) c[k] += ((off >> k) & 1u) * d;
        return morton_id(encode(c, level));
    }

    static constexpr auto root() -> morton_id { return morton_id(0); }
    static constexpr auto bits() -> std::size_t { return sizeof(mask_t) * CHAR_BIT; }
    static constexpr auto parent_of(morton_id id) -> morton_id
    {
        auto [c, level]         = decode(id.id());
        const std::uint32_t off = 1u << (s_depth - level);
        for (auto& v : c) v &= ~off;
        return morton_id(encode(c, static_cast<level_t>(level - 1)));
    }
    static constexpr auto child_of(morton_id parent, offset_t off) -> morton_id { return offset(parent.id() + 1, off); }
    static constexpr auto level(morton_id id) -> level_t { return decode(id.id()).second; }
    static constexpr auto neighbor_at(morton_id id, direction dir) -> std::optional<morton_id>
    {
        auto [c, level]         = decode(id.id());
        const std::uint32_t off = 1u << (s_depth - level);
        switch (dir) {
        case left: c[0] -= off; break;
        case right: c[0] += off; break;
        case bottom: c[1] += off; break;
        case top: c[1] -= off; break;
        case front:
            if constexpr (Rank == 3u) c[2] -= off;
            break;
        case back:
            if constexpr (Rank == 3u) c[2] += off;
            break;
        }
        if (!isvalid_coord(c, level)) return std::nullopt;
        return morton_id(encode(c, level));
    }

    constexpr auto id() const noexcept -> mask_t { return m_id; }
    auto           repr() const -> std::string { return std::bitset<64>(m_id).to_string(); }
    constexpr auto level() const noexcept -> level_t { return static_cast<level_t>(m_id & 0x3Fu); }
    static constexpr auto rank() -> size_type { return s_rank; }
    static constexpr auto nd_fanout() -> size_type { return 1u << Rank; }
    static constexpr auto fanout() -> size_type { return 2; }
    static constexpr auto max_depth() -> size_type { return s_depth; }

    auto operator==(morton_id const&) const noexcept -> bool = default;

private:
    mask_t m_id;
};

template <std::unsigned_integral auto D, std::unsigned_integral auto R>
constexpr auto operator<(morton_id<D, R> const& a, morton_id<D, R> const& b) noexcept -> bool
{
    return a.id() < b.id();
}

} // namespace amr::ndt::morton

template <std::unsigned_integral auto D, std::unsigned_integral auto R>
struct std::hash<amr::ndt::morton::morton_id<D, R>>
{
    auto operator()(amr::ndt::morton::morton_id<D, R> const& id) const noexcept -> std::size_t { return id.id(); }
};
