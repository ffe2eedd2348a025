// One padded patch of one field, the interface of gpu-amr's
// amr::ndt::patches::patch<T, Patch_Layout> (include/ndtree/patch.hpp): a
// contiguous array of flat_size() values.
#pragma once

#include "ndtree/patch_layout.hpp"

#include <array>

namespace amr::ndt::patches
{

template <typename T, typename Patch_Layout>
class patch
{
public:
    using patch_layout_t  = Patch_Layout;
    using value_type      = T;
    using index_t         = typename Patch_Layout::index_t;
    using container_t     = std::array<T, Patch_Layout::flat_size()>;

    static constexpr auto rank() noexcept { return Patch_Layout::rank(); }
    static constexpr auto halo_width() noexcept { return Patch_Layout::halo_width(); }

    constexpr auto data() noexcept -> container_t& { return m_data; }
    constexpr auto data() const noexcept -> container_t const& { return m_data; }
    constexpr auto operator[](index_t i) noexcept -> T& { return m_data[static_cast<std::size_t>(i)]; }
    constexpr auto operator[](index_t i) const noexcept -> T const& { return m_data[static_cast<std::size_t>(i)]; }

private:
    container_t m_data;
};

} // namespace amr::ndt::patches
