// gpu-amr's compile-time DG configuration (include/config/generated_config.hpp,
// generated there from config.yaml): the same names and values, so code
// written against the reference's DG solver (dg_helpers/solver.hpp) compiles
// unchanged against this library.  The device DG path implements exactly this
// configuration (order 2, 2D, 4 variables per node, 4x4 cells per patch with
// one ghost cell, SSPRK2, Courant number 0.5) for both equations;
// DGSolver<Policy> checks a policy against it at compile time.
#pragma once

#include <cstddef>

namespace amr::config
{

enum class EquationType
{
    Advection,
    Euler
};

enum class TimeIntegratorType
{
    Euler,
    SSPRK2,
    SSPRK3
};

constexpr double CourantNumber = 0.5;

struct GlobalConfigPolicy
{
    static constexpr double             EndTime    = 1.0;
    static constexpr std::size_t        Order      = 2;
    static constexpr std::size_t        Dim        = 2;
    static constexpr std::size_t        DOFs       = 4;
    static constexpr std::size_t        PatchSize  = 4;
    static constexpr std::size_t        HaloWidth  = 1;
    static constexpr unsigned int       MaxDepth   = 6;
    static constexpr EquationType       equation   = EquationType::Advection;
    static constexpr TimeIntegratorType integrator = TimeIntegratorType::SSPRK2;
};

} // namespace amr::config
