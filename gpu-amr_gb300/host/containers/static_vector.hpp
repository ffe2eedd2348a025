// Fixed-size vector with the interface of gpu-amr's
// amr::containers::static_vector (include/containers/static_vector.hpp).
#pragma once

#include <array>
#include <concepts>
#include <cstddef>
#include <initializer_list>

namespace amr::containers
{

template <typename T, std::integral auto N>
struct static_vector
{
    using value_type = T;
    std::array<T, static_cast<std::size_t>(N)> m_data{};

    constexpr static_vector() = default;
    constexpr static_vector(std::initializer_list<T> l)
    {
        std::size_t i = 0;
        for (auto const& v : l)
            if (i < m_data.size()) m_data[i++] = v;
    }
    constexpr auto operator[](std::size_t i) noexcept -> T& { return m_data[i]; }
    constexpr auto operator[](std::size_t i) const noexcept -> T const& { return m_data[i]; }
    static constexpr auto size() noexcept -> std::size_t { return static_cast<std::size_t>(N); }
    constexpr auto begin() noexcept { return m_data.begin(); }
    constexpr auto end() noexcept { return m_data.end(); }
    constexpr auto begin() const noexcept { return m_data.begin(); }
    constexpr auto end() const noexcept { return m_data.end(); }
};

} // namespace amr::containers
