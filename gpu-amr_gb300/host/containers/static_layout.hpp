// Row-major layout (last index fastest) with the interface of gpu-amr's
// amr::containers::static_layout (include/containers/static_layout.hpp).
#pragma once

#include "containers/static_shape.hpp"

namespace amr::containers
{

template <typename Shape>
class static_layout
{
public:
    using shape_t       = Shape;
    using size_type     = typename Shape::size_type;
    using index_t       = typename Shape::index_t;
    using rank_t        = typename Shape::rank_t;
    using multi_index_t = std::array<index_t, Shape::rank()>;

    static constexpr auto rank() noexcept -> rank_t { return Shape::rank(); }
    static constexpr auto flat_size() noexcept -> size_type { return Shape::elements(); }
    static constexpr auto elements() noexcept -> size_type { return Shape::elements(); }
    static constexpr auto sizes() noexcept -> auto const& { return Shape::sizes(); }
    static constexpr auto size(index_t i) noexcept -> size_type { return Shape::size(i); }
    static constexpr std::array<size_type, Shape::rank()> s_strides = [] {
        std::array<size_type, Shape::rank()> st{};
        size_type                            acc = 1;
        for (std::size_t d = Shape::rank(); d-- > 0;) {
            st[d] = acc;
            acc *= Shape::sizes()[d];
        }
        return st;
    }();
    static constexpr auto strides() noexcept -> std::array<size_type, Shape::rank()> const& { return s_strides; }
    static constexpr auto stride(index_t i) noexcept -> size_type { return strides()[static_cast<std::size_t>(i)]; }

    template <std::integral... I>
        requires(sizeof...(I) == Shape::rank())
    static constexpr auto linear_index(I... idxs) noexcept -> index_t
    {
        const std::array<index_t, Shape::rank()> a{ static_cast<index_t>(idxs)... };
        return linear_index(a);
    }
    static constexpr auto linear_index(multi_index_t const& a) noexcept -> index_t
    {
        index_t li = 0;
        for (std::size_t d = 0; d != Shape::rank(); ++d) li += a[d] * strides()[d];
        return li;
    }
    static constexpr auto multi_index(index_t li) noexcept -> multi_index_t
    {
        multi_index_t m{};
        for (std::size_t d = 0; d != Shape::rank(); ++d) {
            m[d] = li / strides()[d];
            li %= strides()[d];
        }
        return m;
    }
};

} // namespace amr::containers
