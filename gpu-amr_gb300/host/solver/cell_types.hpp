// Field tags and cell types of gpu-amr's FV solver
// (include/solver/cell_types.hpp) for the scalar advection path.
#pragma once

#include <cstddef>
#include <string_view>
#include <tuple>

namespace amr::cell
{

struct Scalar
{
    using type = double;
    static constexpr auto index() noexcept -> std::size_t { return 0; }
    static constexpr auto name() noexcept -> std::string_view { return "Scalar"; }
    type value;
};

struct AdvectionCell
{
    using deconstructed_types_map_t = std::tuple<Scalar>;
    explicit AdvectionCell(double v) { std::get<Scalar>(m_data).value = v; }
    auto data_tuple() -> auto& { return m_data; }
    auto data_tuple() const -> auto const& { return m_data; }
    deconstructed_types_map_t m_data;
};

} // namespace amr::cell
