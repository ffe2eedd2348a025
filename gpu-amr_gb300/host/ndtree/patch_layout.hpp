// Padded patch layout with the interface of gpu-amr's
// amr::ndt::patches::patch_layout<Data_Layout, Halo_Width>
// (include/ndtree/patch_layout.hpp): (n + 2h)^rank cells, row-major.
#pragma once

#include "containers/static_layout.hpp"

namespace amr::ndt::patches
{

namespace detail
{
template <typename Shape, std::size_t Pad, typename Seq>
struct padded_shape;
template <typename Shape, std::size_t Pad, std::size_t... I>
struct padded_shape<Shape, Pad, std::index_sequence<I...>>
{
    using type = containers::static_shape<static_cast<typename Shape::size_type>(Shape::sizes()[I] + Pad)...>;
};
} // namespace detail

template <typename Data_Layout, std::integral auto Halo_Width>
class patch_layout
{
public:
    using data_layout_t   = Data_Layout;
    using size_type       = typename data_layout_t::size_type;
    using index_t         = typename data_layout_t::index_t;
    using rank_t          = typename data_layout_t::rank_t;
    using shape_t         = typename data_layout_t::shape_t;
    using padded_layout_t = containers::static_layout<typename detail::padded_shape<
        shape_t, static_cast<std::size_t>(2 * Halo_Width), std::make_index_sequence<shape_t::rank()>>::type>;

    static constexpr auto rank() noexcept -> rank_t { return data_layout_t::rank(); }
    static constexpr auto halo_width() noexcept -> size_type { return static_cast<size_type>(Halo_Width); }
    static constexpr auto flat_size() noexcept -> size_type { return padded_layout_t::flat_size(); }
};

} // namespace amr::ndt::patches

namespace amr::ndt::utils::patches
{

// is_halo_cell (include/ndtree/patch_utils.hpp:33-58)
template <typename Layout>
constexpr auto is_halo_cell(typename Layout::index_t linear_index) noexcept -> bool
{
    using padded      = typename Layout::padded_layout_t;
    const auto multi  = padded::multi_index(linear_index);
    const auto h      = Layout::halo_width();
    for (std::size_t d = 0; d != Layout::rank(); ++d)
        if (multi[d] < h || multi[d] >= padded::sizes()[d] - h) return true;
    return false;
}

} // namespace amr::ndt::utils::patches
