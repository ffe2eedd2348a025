// Patch and cell geometry with the interface of gpu-amr's
// amr::ndt::solver::physics_system<Patch_Index, Patch_Layout, Domain_Sizes>
// (include/solver/physics_system.hpp): Morton axis k (x, y, z) is layout
// dimension rank-1-k.
#pragma once

#include "ndtree/patch_layout.hpp"

#include <array>
#include <cstdint>

namespace amr::ndt::solver
{

template <typename Patch_Index, typename Patch_Layout, auto Domain_Sizes>
class physics_system
{
public:
    using patch_index_t       = Patch_Index;
    using patch_layout_t      = Patch_Layout;
    using physics_coord_t     = double;
    static constexpr std::size_t n_dimension = Patch_Index::rank();
    using physics_coord_arr_t = std::array<physics_coord_t, n_dimension>;

    static constexpr auto patch_sizes(patch_index_t const& id) noexcept -> physics_coord_arr_t
    {
        const auto [c, level]     = patch_index_t::decode(id.id());
        const std::uint32_t psize = 1u << (patch_index_t::max_depth() - level);
        physics_coord_arr_t r{};
        for (std::size_t i = 0; i != n_dimension; ++i)
            r[i] = static_cast<double>(Domain_Sizes[i]) * static_cast<double>(psize) /
                   static_cast<double>(1u << patch_index_t::max_depth());
        return r;
    }

    static constexpr auto cell_sizes(patch_index_t const& id) noexcept -> physics_coord_arr_t
    {
        const auto          ps = patch_sizes(id);
        physics_coord_arr_t r{};
        for (std::size_t i = 0; i != n_dimension; ++i)
            r[i] = ps[i] / static_cast<double>(patch_layout_t::data_layout_t::sizes()[n_dimension - 1 - i]);
        return r;
    }

    static constexpr auto patch_coord(patch_index_t const& id) noexcept -> physics_coord_arr_t
    {
        const auto [c, level] = patch_index_t::decode(id.id());
        physics_coord_arr_t r{};
        for (std::size_t i = 0; i != n_dimension; ++i)
            r[i] = static_cast<double>(Domain_Sizes[i]) * static_cast<double>(c[i]) /
                   static_cast<double>(1u << patch_index_t::max_depth());
        return r;
    }

    static constexpr auto cell_coord(patch_index_t const& id, typename patch_layout_t::padded_layout_t::index_t li) noexcept
        -> physics_coord_arr_t
    {
        const auto origin = patch_coord(id);
        const auto cs     = cell_sizes(id);
        const auto multi  = patch_layout_t::padded_layout_t::multi_index(li);
        physics_coord_arr_t r{};
        for (std::size_t i = 0; i != n_dimension; ++i) {
            const double data_cell = static_cast<double>(multi[n_dimension - 1 - i]) -
                                     static_cast<double>(patch_layout_t::halo_width());
            r[i] = origin[i] + data_cell * cs[i];
        }
        return r;
    }

    static constexpr auto domain_length(std::size_t d) noexcept -> physics_coord_t
    {
        return static_cast<physics_coord_t>(Domain_Sizes[d]);
    }
};

} // namespace amr::ndt::solver
