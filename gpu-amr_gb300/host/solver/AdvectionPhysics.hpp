// Linear advection equation plug-in with the static interface of gpu-amr's
// AdvectionPhysics<DIM> (include/solver/AdvectionPhysics.hpp:17-91).  The
// update itself runs in the CUDA kernels (upwind form of the Rusanov flux);
// this type supplies NVAR, the field tags, the velocity and the primitive ->
// conservative map.  Velocity is the reference's {1.0, 0.5, 0.0}; a solver
// can override it at run time (amr_solver::set_velocity).
#pragma once

#include "containers/static_vector.hpp"
#include "solver/cell_types.hpp"

#include <cmath>
#include <tuple>

template <int DIM>
class AdvectionPhysics
{
public:
    static constexpr int    NVAR        = 1;
    static constexpr double Velocity[3] = { 1.0, 0.5, 0.0 };
    using FieldTags                     = std::tuple<amr::cell::Scalar>;

    static void primitiveToConservative(const amr::containers::static_vector<double, NVAR>& prim,
                                        amr::containers::static_vector<double, NVAR>& cons, double)
    {
        cons[0] = prim[0];
    }

    static constexpr int getNumVars() { return NVAR; }
};
