// Field tags and cell types of gpu-amr's FV solver
// (include/solver/cell_types.hpp): the scalar advection cell and the Euler
// cells (rho, rho u, rho v, [rho w], E), one FP64 field per tag.
#pragma once

#include <cstddef>
#include <string_view>
#include <tuple>

namespace amr::cell
{

#define AMR_GB300_FIELD_TAG(Name, Index)                                                   \
    struct Name                                                                            \
    {                                                                                      \
        using type = double;                                                               \
        static constexpr auto index() noexcept -> std::size_t { return Index; }            \
        static constexpr auto name() noexcept -> std::string_view { return #Name; }        \
        type value;                                                                        \
    };

AMR_GB300_FIELD_TAG(Scalar, 0)
AMR_GB300_FIELD_TAG(Rho, 0)
AMR_GB300_FIELD_TAG(Rhou, 1)
AMR_GB300_FIELD_TAG(Rhov, 2)
AMR_GB300_FIELD_TAG(Rhow, 3)
AMR_GB300_FIELD_TAG(E2D, 3)
AMR_GB300_FIELD_TAG(E3D, 4)

#undef AMR_GB300_FIELD_TAG

struct AdvectionCell
{
    using deconstructed_types_map_t = std::tuple<Scalar>;
    explicit AdvectionCell(double v) { std::get<Scalar>(m_data).value = v; }
    auto data_tuple() -> auto& { return m_data; }
    auto data_tuple() const -> auto const& { return m_data; }
    deconstructed_types_map_t m_data;
};

struct EulerCell2D
{
    using deconstructed_types_map_t = std::tuple<Rho, Rhou, Rhov, E2D>;
    EulerCell2D(double rho, double rhou, double rhov, double e)
    {
        std::get<Rho>(m_data).value  = rho;
        std::get<Rhou>(m_data).value = rhou;
        std::get<Rhov>(m_data).value = rhov;
        std::get<E2D>(m_data).value  = e;
    }
    auto data_tuple() -> auto& { return m_data; }
    auto data_tuple() const -> auto const& { return m_data; }
    deconstructed_types_map_t m_data;
};

struct EulerCell3D
{
    using deconstructed_types_map_t = std::tuple<Rho, Rhou, Rhov, Rhow, E3D>;
    EulerCell3D(double rho, double rhou, double rhov, double rhow, double e)
    {
        std::get<Rho>(m_data).value  = rho;
        std::get<Rhou>(m_data).value = rhou;
        std::get<Rhov>(m_data).value = rhov;
        std::get<Rhow>(m_data).value = rhow;
        std::get<E3D>(m_data).value  = e;
    }
    auto data_tuple() -> auto& { return m_data; }
    auto data_tuple() const -> auto const& { return m_data; }
    deconstructed_types_map_t m_data;
};

} // namespace amr::cell
