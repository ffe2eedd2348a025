// Compile-time patch shape with the interface of gpu-amr's
// amr::containers::static_shape (include/containers/static_shape.hpp).
#pragma once

#include <array>
#include <concepts>
#include <cstddef>
#include <type_traits>

namespace amr::containers
{

template <std::integral auto N, std::integral auto... Ns>
    requires(N > 0) && ((Ns > 0) && ...)
class static_shape
{
public:
    using size_type = std::common_type_t<decltype(N), decltype(Ns)...>;
    using rank_t    = size_type;
    using index_t   = size_type;

    static constexpr std::array<size_type, sizeof...(Ns) + 1> s_sizes{ N, Ns... };

    static constexpr auto rank() noexcept -> rank_t { return sizeof...(Ns) + 1; }
    static constexpr auto elements() noexcept -> size_type { return (N * ... * Ns); }
    static constexpr auto sizes() noexcept -> std::array<size_type, sizeof...(Ns) + 1> const& { return s_sizes; }
    static constexpr auto size(index_t i) noexcept -> size_type { return sizes()[static_cast<std::size_t>(i)]; }
};

} // namespace amr::containers
